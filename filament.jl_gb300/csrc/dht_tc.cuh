// dht_tc.cuh -- the Hankel transforms of the linear step as tcgen05
// tensor-core GEMMs on exact FP16 slices (kind::f16, FP32 accumulation in
// tensor memory).
//
// Reference: src/modules/linear_propagators/spectral.jl:16-26
// (PS * E; E .*= exp(i KZ dz); spectral guard; PS \ E) with the order-0
// QDHT pair written as E <- M2 D M1 E, M1 = T diag(s), M2 = diag(1/s) T and
// D = exp(i KZ dz) * guard.  One launch computes C[M x N] = A[M x K] B[K x N]
// with A = M1 or M2 (fixed) and B the field, K-major: B^T row n is one real
// column (re or im of one frequency) of the half spectrum, index k = radial
// point contiguous.
//
// Numerics.  The tensor core adds FP32 products rounding toward zero; summed
// over K = 1024 that biases every output by ~ -7e-6 relative, and the field
// would be damped step after step.  Here the dominant product is exact:
//   A[i][k] = qa_i (a0 + a1 + a2),     a0 integer, |a0| <= 1024,
//   B[k][j] = qb_cj (b0 + b1 + b2),    b0 integer, |b0| <= 128,
// a1 = fp16(rest), a2 = fp16(rest - a1), likewise b1, b2; qa_i is a power of
// two from the row maximum of A, qb_cj one from the maximum of column j over
// the 64-wide K chunk c.  All slices are exact FP16 values.  Over one chunk
// the head sum sum_k a0 b0 is an integer below 2^23, which the tensor core
// computes exactly.  The five correction products
// a0 b1 + a1 b0 + a1 b1 + a0 b2 + a2 b0 (together below 2^-8 of the head) go
// to a second accumulator, whose round-toward-zero error is ~2^-28 of the
// result; the dropped products a1 b2, a2 b1, a2 b2 are below 2^-29.  (Also
// dropping a2 b0, below 2^-22 of the head, made the transforms 3-6% faster
// but raised the 1000 x 4096 workload's field error against the FP64 oracle
// at z = 2.1 m from 3.1e-5 to 4.0e-5: the filament amplifies it.)  The
// consumer warps add each chunk's two accumulators times qb_cj into FP32
// registers (round to nearest) and apply qa_i in the epilogue.
//
// k_slice cuts the FP32 operand B (written by the row kernel) into its
// slices and chunk scales once, so the GEMM streams FP16 tiles with TMA
// only; k_slice_prop does the same for the forward transform's output after
// applying the linear propagator exp(i KZ dz) * guard.
//
// GEMM roles (320 threads): warps 0-7 drain the accumulators and run the
// epilogue; warp 8 issues the TMA loads; warp 9 issues the MMAs.  Tile
// 128 x 128, K stage 32 (four stages of six 8 KB slice tiles, 64-byte
// swizzle), accumulation chunk 64, two accumulator pairs in 512
// tensor-memory columns (ping-pong between chunks).  Every mbarrier wait is
// bounded and also gives up once another role has failed; a failure sets
// *err.
#pragma once
#include <cuda_fp16.h>
#include "tc_ptx.cuh"
#include "rowkernels.cuh"
#include "tc_params.h"

#define TC_BM 128
#define TC_BN 128
#define TC_BK 32                               // K per shared-memory stage
#define TC_CHUNK 64                            // K per exact chunk (scale block of B)
#define TC_STAGES 4
#define TC_CONSUMERS 256
#define TC_THREADS (TC_CONSUMERS + 64)
#define TC_SLICE_BYTES (TC_BM * TC_BK * 2)     // one FP16 slice tile, 64-byte swizzle
#define TC_STAGE_BYTES (6 * TC_SLICE_BYTES)   // a0, a1, a2, b0, b1, b2
#define TC_SMEM_BYTES (TC_STAGES * TC_STAGE_BYTES + 1024 + 256)
#define TC_WAIT_LIMIT (1u << 26)
#define TC_OFF_A(s) ((s) * TC_SLICE_BYTES)
// the barrier block of k_dht_tc, 8 bytes each: full[S] empty[S] accf[2]
// acce[2] done, then the tensor-memory address slot; it must fit the 256
// bytes reserved after the stages
#define TC_BAR_FULL(s) (8u * (s))
#define TC_BAR_EMPTY(s) (8u * (TC_STAGES + (s)))
#define TC_BAR_ACCF(b) (8u * (2 * TC_STAGES + (b)))
#define TC_BAR_ACCE(b) (8u * (2 * TC_STAGES + 2 + (b)))
#define TC_BAR_DONE (8u * (2 * TC_STAGES + 4))
#define TC_BAR_SLOT (8u * (2 * TC_STAGES + 5))
static_assert(TC_BAR_SLOT + 4 <= 256, "k_dht_tc barrier block overflows its 256 bytes");
static_assert(TC_STAGE_BYTES % 1024 == 0, "stage pitch keeps the 1024-byte alignment of the slices");
#define TC_OFF_B(s) ((3 + (s)) * TC_SLICE_BYTES)

// bounded wait that also stops when *fail is set by another role
__device__ __forceinline__ bool tc_wait(uint32_t bar, uint32_t parity, volatile int* fail) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *fail) return false;
  }
  *fail = 1;
  return false;
}
__device__ __forceinline__ void tc_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

// ---------------------------------------------------------------------------
// B [N][K] FP32 (K contiguous) -> slices b0, b1, b2 [N][K] FP16 and chunk
// scales qb [K/64][N].  One warp per (column n, CH consecutive chunks);
// lane l holds k = 64c + 2l, 2l + 1 of each chunk c.  All loads of a warp
// are issued before the first use.  qb = 2^(E-6) for a chunk maximum f 2^E,
// so |B / qb| < 128.
template <int CH>
__global__ void __launch_bounds__(256) k_slice(const float* __restrict__ B, __half2* b0, __half2* b1, __half2* b2,
                                               float* qb, int N, int K, const DevCtl* ctl) {
  if (ctl && ctl->done) return;
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int nch = K / TC_CHUNK, ngrp = nch / CH;
  if (g >= N * ngrp) return;
  const int n = g / ngrp, c0 = (g - n * ngrp) * CH;
  const size_t base = ((size_t)n * K + (size_t)c0 * TC_CHUNK) / 2 + lane;   // half2 / float2 index
  float2 v[CH];
#pragma unroll
  for (int u = 0; u < CH; ++u) v[u] = __ldg(reinterpret_cast<const float2*>(B) + base + u * (TC_CHUNK / 2));
#pragma unroll
  for (int u = 0; u < CH; ++u) {
    const unsigned m =
        __reduce_max_sync(0xffffffffu, max(__float_as_uint(fabsf(v[u].x)), __float_as_uint(fabsf(v[u].y))));
    float q = 0.f, iq = 0.f;
    if (m != 0u) {
      int e = (int)((m >> 23) & 0xFFu) - 127;
      e = min(max(e, -100), 120);
      q = __uint_as_float((unsigned)(e - 6 + 127) << 23);
      iq = __uint_as_float((unsigned)(6 - e + 127) << 23);
    }
    float hd[2], m1[2], m2[2];
    const float x[2] = {v[u].x * iq, v[u].y * iq};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const float i0 = rintf(x[i]);               // |i0| <= 128, exact
      const float r = x[i] - i0;                  // exact, |r| <= 1/2
      const float r1 = __half2float(__float2half_rn(r));
      hd[i] = i0;
      m1[i] = r1;
      m2[i] = r - r1;                             // exact
    }
    const size_t e2 = base + u * (TC_CHUNK / 2);
    b0[e2] = __floats2half2_rn(hd[0], hd[1]);
    b1[e2] = __floats2half2_rn(m1[0], m1[1]);
    b2[e2] = __floats2half2_rn(m2[0], m2[1]);
    if (lane == 0) qb[(size_t)(c0 + u) * N + n] = q;
  }
}

// The same for the output of the forward transform, with the linear
// propagator applied first (spectral.jl:21-24: E .*= exp(i KZ dz), spectral
// guard): W [2 nh][K] holds (re, im) of frequency w in rows 2w, 2w + 1; kz, gd
// are [nh][K] (radial index contiguous).  One warp per (frequency w,
// CH consecutive chunks); both rows of w are sliced with their own chunk
// scales.
// MUL = false: the linear propagator exp(i KZ dz) gd from kz = KZ (zu
// units) and the guard gd; MUL = true: a plain complex factor kz (the
// non-paraxial QZ(kt, w) / QZ(w) times the spectral guard), gd unused.
template <int CH, bool MUL>
__global__ void __launch_bounds__(256) k_slice_prop(const float* __restrict__ W, const float2* __restrict__ kz,
                                                    const float* __restrict__ gd, __half2* b0, __half2* b1,
                                                    __half2* b2, float* qb, int nh, int K, const DevCtl* ctl,
                                                    float dz_fixed) {
  if (ctl && ctl->done) return;
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * 8 + (threadIdx.x >> 5);
  const int nch = K / TC_CHUNK, ngrp = nch / CH;
  if (g >= nh * ngrp) return;
  const int w = g / ngrp, c0 = (g - w * ngrp) * CH;
  const float dz = ctl ? (float)ctl->dz : dz_fixed;
  const size_t kb = (size_t)c0 * TC_CHUNK / 2 + lane;                   // float2 index inside a row
  const float2* re = reinterpret_cast<const float2*>(W + (size_t)(2 * w) * K) + kb;
  const float2* im = reinterpret_cast<const float2*>(W + (size_t)(2 * w + 1) * K) + kb;
  const float4* kq = reinterpret_cast<const float4*>(kz + (size_t)w * K) + kb;
  const float2* gq = MUL ? nullptr : reinterpret_cast<const float2*>(gd + (size_t)w * K) + kb;
  float2 vr[CH], vi[CH], gg[CH];
  float4 kk[CH];
#pragma unroll
  for (int u = 0; u < CH; ++u) {
    vr[u] = __ldg(re + u * (TC_CHUNK / 2));
    vi[u] = __ldg(im + u * (TC_CHUNK / 2));
    kk[u] = __ldg(kq + u * (TC_CHUNK / 2));
    gg[u] = MUL ? make_float2(1.f, 1.f) : __ldg(gq + u * (TC_CHUNK / 2));
  }
#pragma unroll
  for (int u = 0; u < CH; ++u) {
    // two radial points per lane: (vr.x, vi.x) and (vr.y, vi.y)
    float xr[2], xi[2];
    const float kx[2] = {kk[u].x, kk[u].z}, ky[2] = {kk[u].y, kk[u].w}, gv[2] = {gg[u].x, gg[u].y};
    const float ar[2] = {vr[u].x, vr[u].y}, ai[2] = {vi[u].x, vi[u].y};
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      float amp, sn, cs;
      if (MUL) {
        amp = 1.f;
        cs = kx[i];
        sn = ky[i];
      } else {
        amp = gv[i] * expf(-ky[i] * dz);
        sincosf(kx[i] * dz, &sn, &cs);
      }
      xr[i] = amp * (ar[i] * cs - ai[i] * sn);
      xi[i] = amp * (ar[i] * sn + ai[i] * cs);
    }
#pragma unroll
    for (int part = 0; part < 2; ++part) {
      const float* x = part ? xi : xr;
      const unsigned m = __reduce_max_sync(0xffffffffu, max(__float_as_uint(fabsf(x[0])), __float_as_uint(fabsf(x[1]))));
      float q = 0.f, iq = 0.f;
      if (m != 0u) {
        int e = (int)((m >> 23) & 0xFFu) - 127;
        e = min(max(e, -100), 120);
        q = __uint_as_float((unsigned)(e - 6 + 127) << 23);
        iq = __uint_as_float((unsigned)(6 - e + 127) << 23);
      }
      float hd[2], m1[2], m2[2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const float y = x[i] * iq;
        const float i0 = rintf(y);
        const float r = y - i0;
        const float r1 = __half2float(__float2half_rn(r));
        hd[i] = i0;
        m1[i] = r1;
        m2[i] = r - r1;
      }
      const int n = 2 * w + part;
      const size_t e2 = ((size_t)n * K) / 2 + kb + u * (TC_CHUNK / 2);
      b0[e2] = __floats2half2_rn(hd[0], hd[1]);
      b1[e2] = __floats2half2_rn(m1[0], m1[1]);
      b2[e2] = __floats2half2_rn(m2[0], m2[1]);
      if (lane == 0) qb[(size_t)(c0 + u) * (2 * nh) + n] = q;
    }
  }
}

// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(TC_THREADS, 1)
    k_dht_tc(const __grid_constant__ CUtensorMap tA0, const __grid_constant__ CUtensorMap tA1,
             const __grid_constant__ CUtensorMap tA2, const __grid_constant__ CUtensorMap tB0,
             const __grid_constant__ CUtensorMap tB1, const __grid_constant__ CUtensorMap tB2, TcGemmParams p) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  __shared__ volatile int s_fail;
  if (p.ctl && p.ctl->done) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(tc_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = tc_smem + (sbase - raw);
  const uint32_t bars = sbase + TC_STAGES * TC_STAGE_BYTES;
  auto full_bar = [&](int s) { return bars + TC_BAR_FULL(s); };
  auto empty_bar = [&](int s) { return bars + TC_BAR_EMPTY(s); };
  auto accf_bar = [&](int b) { return bars + TC_BAR_ACCF(b); };
  auto acce_bar = [&](int b) { return bars + TC_BAR_ACCE(b); };
  const uint32_t done_bar = bars + TC_BAR_DONE;   // all issued MMAs complete
  const uint32_t tmem_slot = bars + TC_BAR_SLOT;
  volatile uint32_t* tmem_slot_g =
      reinterpret_cast<volatile uint32_t*>(gbase + TC_STAGES * TC_STAGE_BYTES + TC_BAR_SLOT);

  const int bm = blockIdx.y * TC_BM, bn = blockIdx.x * TC_BN;
  if (tid == 0) s_fail = 0;
  if (warp == 0) tc::tmem_alloc(tmem_slot, 512);
  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      tc::mbar_init(full_bar(s), 1);
      tc::mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(accf_bar(b), 1);
      tc::mbar_init(acce_bar(b), 8);
    }
    tc::mbar_init(done_bar, 1);
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot_g;
  const int nk = p.K / TC_BK;              // stages; two per chunk
  const int nc = p.K / TC_CHUNK;

  float acc[64];
#pragma unroll
  for (int i = 0; i < 64; ++i) acc[i] = 0.f;

  if (warp == 8) {
    // ---------------- producer: TMA loads, refills a stage once its MMAs finished
    if (lane == 0) {
      for (int kb = 0; kb < nk; ++kb) {
        const int s = kb % TC_STAGES;
        const int use = kb / TC_STAGES;
        if (use > 0 && !tc_wait(empty_bar(s), (use - 1) & 1, &s_fail)) break;
        const uint32_t st = sbase + s * TC_STAGE_BYTES;
        tc::mbar_expect_tx(full_bar(s), TC_STAGE_BYTES);
        tc::tma_load_2d(st + TC_OFF_A(0), &tA0, kb * TC_BK, bm, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_A(1), &tA1, kb * TC_BK, bm, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_A(2), &tA2, kb * TC_BK, bm, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_B(0), &tB0, kb * TC_BK, bn, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_B(1), &tB1, kb * TC_BK, bn, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_B(2), &tB2, kb * TC_BK, bn, full_bar(s));
      }
      // wait for the last loads so no copy lands after the block exits
      for (int kb = (nk > TC_STAGES ? nk - TC_STAGES : 0); kb < nk; ++kb)
        tc_wait(full_bar(kb % TC_STAGES), (kb / TC_STAGES) & 1, &s_fail);
    }
  } else if (warp == 9) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_f16(TC_BM, TC_BN);
      for (int kb = 0; kb < nk && !s_fail; ++kb) {
        const int s = kb % TC_STAGES;
        if (!tc_wait(full_bar(s), (kb / TC_STAGES) & 1, &s_fail)) break;
        const int c = kb >> 1, b = c & 1;
        const bool first = (kb & 1) == 0;
        if (first && (c >> 1) > 0 && !tc_wait(acce_bar(b), ((c >> 1) - 1) & 1, &s_fail)) break;
        tc::tc_fence_after();
        const uint64_t ds = tc::desc_k64(sbase + s * TC_STAGE_BYTES);
        const uint32_t big = tmem + (uint32_t)(b * 256), small = big + 128u;
#pragma unroll
        for (int kk = 0; kk < TC_BK / 16; ++kk) {
          const uint32_t ko = (uint32_t)(kk * 32);   // 16 FP16 = 32 bytes
          const uint64_t a0 = tc::desc_add(ds, TC_OFF_A(0) + ko), a1 = tc::desc_add(ds, TC_OFF_A(1) + ko),
                         a2 = tc::desc_add(ds, TC_OFF_A(2) + ko);
          const uint64_t b0 = tc::desc_add(ds, TC_OFF_B(0) + ko), b1 = tc::desc_add(ds, TC_OFF_B(1) + ko),
                         b2 = tc::desc_add(ds, TC_OFF_B(2) + ko);
          const uint32_t accum = (first && kk == 0) ? 0u : 1u;
          tc::mma_f16(big, a0, b0, idesc, accum);
          tc::mma_f16(small, a0, b1, idesc, accum);
          tc::mma_f16(small, a1, b0, idesc, 1);
          tc::mma_f16(small, a1, b1, idesc, 1);
          tc::mma_f16(small, a0, b2, idesc, 1);
          tc::mma_f16(small, a2, b0, idesc, 1);
        }
        tc::mma_commit(empty_bar(s));
        if (!first) tc::mma_commit(accf_bar(b));
      }
      // no MMA may still write tensor memory when it is released, also after
      // a failure
      tc::mma_commit(done_bar);
      tc::mbar_wait(done_bar, 0, TC_WAIT_LIMIT);
    }
  } else {
    // ---------------- consumers: chunk accumulators -> FP32 registers
    const int q = warp & 3, hcol = warp >> 2;
    const float* qcol = p.qb + bn + 64 * hcol;
    for (int c = 0; c < nc; ++c) {
      const int b = c & 1;
      const float4* qv = reinterpret_cast<const float4*>(qcol + (size_t)c * p.ldqb);
      float4 sc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) sc[i] = __ldg(qv + i);
      if (!tc_wait(accf_bar(b), (c >> 1) & 1, &s_fail)) break;
      tc::tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 256 + 64 * hcol);
#pragma unroll
      for (int qq = 0; qq < 4; ++qq) {
        uint32_t rb[16], rs[16];
        tc::tmem_ld16_async(taddr + 16u * qq, rb);
        tc::tmem_ld16_async(taddr + 128u + 16u * qq, rs);
        tc::tmem_wait_ld16(rb, rs);
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          const float sq[4] = {sc[i].x, sc[i].y, sc[i].z, sc[i].w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int j = 4 * i + e;
            acc[16 * qq + j] = fmaf(__uint_as_float(rb[j]) + __uint_as_float(rs[j]), sq[e], acc[16 * qq + j]);
          }
        }
        if (qq < 3) {
#pragma unroll
          for (int i = 0; i < 4; ++i) sc[i] = __ldg(qv + 4 * (qq + 1) + i);
        }
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) tc_arrive(acce_bar(b));
    }
  }
  __syncthreads();
  // ---------------- epilogue (consumers hold one row x 64 columns each)
  if (warp < 8 && !s_fail) {
    const int q = warp & 3, hcol = warp >> 2;
    const int row = bm + 32 * q + lane;
    const int col0 = bn + 64 * hcol;
    const float sa = p.qa[row];
#pragma unroll
    for (int i = 0; i < 64; ++i) acc[i] *= sa;
    if (p.mode == 1) {
#pragma unroll
      for (int i = 0; i < 64; ++i) p.out[(size_t)(col0 + i) * p.ldo + row] = acc[i];
    } else {
      float4* dst = reinterpret_cast<float4*>(p.out + (size_t)row * p.ldo + col0);
#pragma unroll
      for (int i = 0; i < 16; ++i) dst[i] = make_float4(acc[4 * i], acc[4 * i + 1], acc[4 * i + 2], acc[4 * i + 3]);
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
  }
  if (s_fail && tid == 0) atomicExch(p.err, 1);
  if (p.mode == 2 && p.ctl && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0 && !s_fail)
    p.ctl->guard_pending = 1;   // mode 3: the same store without the flag
}
