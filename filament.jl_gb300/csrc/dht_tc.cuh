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
//   A[i][k] = qa_i (a0 + a1 + a2),  a0 integer, |a0| <= 1024,
//   B[k][j] = qb_j (b0 + b1 + b2),  b0 integer, |b0| <= 256,
// a1 = fp16(rest), a2 = fp16(rest - a1), likewise b1, b2; qa_i and qb_j are
// powers of two from the row maximum of A and the column maximum of B.  All
// slices are exact FP16 values.  Over one 32-wide K chunk the head sum
// sum_k a0 b0 is an integer below 2^23, which the tensor core computes
// exactly.  The five correction products a0 b1 + a1 b0 + a1 b1 + a0 b2 + a2 b0
// (together below 2^-9 of the head) go to a second accumulator; its
// round-toward-zero error is ~2^-30 of the result, and the dropped products
// a1 b2, a2 b1, a2 b2 are below 2^-31.  The consumer warps add each chunk's
// two accumulators into FP32 registers (round to nearest) and apply
// qa_i qb_j in the epilogue.
//
// Column maxima of B come from the producer of B (the row kernel, or the
// epilogue of the forward transform) through atomicMax on the bit patterns of
// |value|; the inverse transform clears the row kernel's array for the next
// step, the row kernel clears the forward transform's.
//
// Roles (320 threads): warps 0-7 convert each stage's FP32 B tile into its
// three slices, drain the accumulators and run the epilogue; warp 8 issues
// the TMA loads (three A slices and the FP32 B tile); warp 9 issues the MMAs.
// Tile 128 x 128, K chunk 32, three shared-memory stages of
// {B fp32, a0, a1, a2, b0, b1, b2} = 64 KB, two accumulator pairs in 512
// tensor-memory columns (ping-pong between chunks).  Every mbarrier wait is
// bounded and also gives up once another role has failed; a failure sets *err.
#pragma once
#include <cuda_fp16.h>
#include "tc_ptx.cuh"
#include "rowkernels.cuh"
#include "tc_params.h"

#define TC_BM 128
#define TC_BN 128
#define TC_BK 32
#define TC_STAGES 3
#define TC_CONSUMERS 256
#define TC_THREADS (TC_CONSUMERS + 64)
#define TC_RAW_BYTES (TC_BN * TC_BK * 4)       // FP32 B tile, 128-byte swizzle
#define TC_SLICE_BYTES (TC_BM * TC_BK * 2)     // one FP16 slice tile, 64-byte swizzle
#define TC_STAGE_BYTES (TC_RAW_BYTES + 6 * TC_SLICE_BYTES)
#define TC_SMEM_BYTES (TC_STAGES * TC_STAGE_BYTES + 1024 + 256 + 2 * TC_BN * 4)
#define TC_WAIT_LIMIT (1u << 26)
// byte offsets inside a stage
#define TC_OFF_A(s) (TC_RAW_BYTES + (s) * TC_SLICE_BYTES)
#define TC_OFF_B(s) (TC_RAW_BYTES + (3 + (s)) * TC_SLICE_BYTES)


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

// column scale qb = 2^(E-7) for a column maximum m = f 2^E (|B / qb| < 256);
// returns 1/qb, or 0 for an all-zero column
__device__ __forceinline__ float tc_inv_scale(unsigned mbits, float* qb) {
  int e = (int)((mbits >> 23) & 0xFFu) - 127;
  if ((mbits & 0x7FFFFFFFu) == 0u) { *qb = 0.f; return 0.f; }
  e = max(e, -100);
  e = min(e, 120);
  *qb = __uint_as_float((unsigned)(e - 7 + 127) << 23);
  return __uint_as_float((unsigned)(7 - e + 127) << 23);
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    k_dht_tc(const __grid_constant__ CUtensorMap tA0, const __grid_constant__ CUtensorMap tA1,
             const __grid_constant__ CUtensorMap tA2, const __grid_constant__ CUtensorMap tB, TcGemmParams p) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  __shared__ volatile int s_fail;
  if (p.ctl && p.ctl->done) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(tc_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = tc_smem + (sbase - raw);
  const uint32_t bars = sbase + TC_STAGES * TC_STAGE_BYTES;
  // barrier block: full[3] conv[3] empty[3] accf[2] acce[2] tmem_slot done
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto conv_bar = [&](int s) { return bars + 24u + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 48u + 8u * s; };
  auto accf_bar = [&](int b) { return bars + 72u + 8u * b; };
  auto acce_bar = [&](int b) { return bars + 88u + 8u * b; };
  const uint32_t tmem_slot = bars + 104u;
  const uint32_t done_bar = bars + 112u;   // all issued MMAs complete
  volatile uint32_t* tmem_slot_g = reinterpret_cast<volatile uint32_t*>(gbase + TC_STAGES * TC_STAGE_BYTES + 104);
  float* qb_s = reinterpret_cast<float*>(gbase + TC_STAGES * TC_STAGE_BYTES + 256);
  float* iqb_s = qb_s + TC_BN;

  const int bm = blockIdx.y * TC_BM, bn = blockIdx.x * TC_BN;
  if (tid == 0) s_fail = 0;
  if (tid < TC_BN) iqb_s[tid] = tc_inv_scale(p.cm_in[bn + tid], &qb_s[tid]);
  if (warp == 0) tc::tmem_alloc(tmem_slot, 512);
  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      tc::mbar_init(full_bar(s), 1);
      tc::mbar_init(conv_bar(s), 8);
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
  const int nk = p.K / TC_BK;

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
        tc::mbar_expect_tx(full_bar(s), TC_RAW_BYTES + 3 * TC_SLICE_BYTES);
        tc::tma_load_2d(st, &tB, kb * TC_BK, bn, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_A(0), &tA0, kb * TC_BK, bm, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_A(1), &tA1, kb * TC_BK, bm, full_bar(s));
        tc::tma_load_2d(st + TC_OFF_A(2), &tA2, kb * TC_BK, bm, full_bar(s));
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
        if (!tc_wait(conv_bar(s), (kb / TC_STAGES) & 1, &s_fail)) break;
        const int b = kb & 1;
        const int use = kb >> 1;
        if (use > 0 && !tc_wait(acce_bar(b), (use - 1) & 1, &s_fail)) break;
        tc::tc_fence_after();
        const uint32_t st = sbase + s * TC_STAGE_BYTES;
        const uint32_t big = tmem + (uint32_t)(b * 256), small = big + 128u;
#pragma unroll
        for (int kk = 0; kk < TC_BK / 16; ++kk) {
          const uint32_t ko = (uint32_t)(kk * 32);   // 16 FP16 = 32 bytes
          const uint64_t a0 = tc::desc_k64(st + TC_OFF_A(0) + ko), a1 = tc::desc_k64(st + TC_OFF_A(1) + ko),
                         a2 = tc::desc_k64(st + TC_OFF_A(2) + ko);
          const uint64_t b0 = tc::desc_k64(st + TC_OFF_B(0) + ko), b1 = tc::desc_k64(st + TC_OFF_B(1) + ko),
                         b2 = tc::desc_k64(st + TC_OFF_B(2) + ko);
          tc::mma_f16(big, a0, b0, idesc, kk != 0);
          tc::mma_f16(small, a0, b1, idesc, kk != 0);
          tc::mma_f16(small, a1, b0, idesc, 1);
          tc::mma_f16(small, a1, b1, idesc, 1);
          tc::mma_f16(small, a0, b2, idesc, 1);
          tc::mma_f16(small, a2, b0, idesc, 1);
        }
        tc::mma_commit(accf_bar(b));
        tc::mma_commit(empty_bar(s));
      }
      // no MMA may still write tensor memory when it is released, also after
      // a failure
      tc::mma_commit(done_bar);
      tc::mbar_wait(done_bar, 0, TC_WAIT_LIMIT);
    }
  } else {
    // ---------------- consumers
    const int q = warp & 3, hcol = warp >> 2;
    // thread -> (B^T row n = output column, half h of the 32-wide chunk)
    const int n = tid >> 1, h = tid & 1;
    const float iq = iqb_s[n];
    auto convert = [&](int kb) -> bool {
      const int s = kb % TC_STAGES;
      if (!tc_wait(full_bar(s), (kb / TC_STAGES) & 1, &s_fail)) return false;
      uint8_t* st = gbase + s * TC_STAGE_BYTES;
      float y[16];
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        // 128-byte swizzle: 16-byte unit u of row n sits at unit u ^ (n & 7)
        const int u = (4 * h + j) ^ (n & 7);
        const float4 v = *reinterpret_cast<const float4*>(st + n * 128 + u * 16);
        y[4 * j] = v.x * iq;
        y[4 * j + 1] = v.y * iq;
        y[4 * j + 2] = v.z * iq;
        y[4 * j + 3] = v.w * iq;
      }
      __half2 s0[8], s1[8], s2[8];
#pragma unroll
      for (int e = 0; e < 8; ++e) {
        float hd[2], m1[2], m2[2];
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const float x = y[2 * e + c];
          const float i0 = rintf(x);                 // |i0| <= 256, exact
          const float r = x - i0;                    // exact, |r| <= 1/2
          const float r1 = __half2float(__float2half_rn(r));
          hd[c] = i0;
          m1[c] = r1;
          m2[c] = r - r1;                            // exact
        }
        s0[e] = __floats2half2_rn(hd[0], hd[1]);
        s1[e] = __floats2half2_rn(m1[0], m1[1]);
        s2[e] = __floats2half2_rn(m2[0], m2[1]);
      }
#pragma unroll
      for (int w = 0; w < 2; ++w) {
        // 64-byte swizzle: 16-byte unit u of row n sits at unit u ^ ((n >> 1) & 3)
        const int u = (2 * h + w) ^ ((n >> 1) & 3);
        const int off = n * 64 + u * 16;
        *reinterpret_cast<uint4*>(st + TC_OFF_B(0) + off) = *reinterpret_cast<const uint4*>(&s0[4 * w]);
        *reinterpret_cast<uint4*>(st + TC_OFF_B(1) + off) = *reinterpret_cast<const uint4*>(&s1[4 * w]);
        *reinterpret_cast<uint4*>(st + TC_OFF_B(2) + off) = *reinterpret_cast<const uint4*>(&s2[4 * w]);
      }
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) tc_arrive(conv_bar(s));
      return true;
    };
    bool ok = convert(0);
    for (int kb = 0; kb < nk && ok; ++kb) {
      if (kb + 1 < nk) ok = convert(kb + 1);
      if (!ok) break;
      const int b = kb & 1;
      if (!tc_wait(accf_bar(b), (kb >> 1) & 1, &s_fail)) { ok = false; break; }
      tc::tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 256 + 64 * hcol);
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        float vb[32], vs[32];
        tc::tmem_ld32(taddr + 32u * half, vb);
        tc::tmem_ld32(taddr + 128u + 32u * half, vs);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[32 * half + i] += vb[i] + vs[i];
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
    const int c0 = 64 * hcol;
    const float sa = p.qa[row];
#pragma unroll
    for (int i = 0; i < 64; ++i) acc[i] *= sa * qb_s[c0 + i];
    const int col0 = bn + c0;
    if (p.mode == 1) {
      const float dz = p.ctl ? (float)p.ctl->dz : p.dz_fixed;
      const int w0 = col0 >> 1;
      const float2* kzr = p.kz + (size_t)row * p.nh + w0;
      const float* gr = p.gd + (size_t)row * p.nh + w0;
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        float2 k = kzr[i];
        float amp = gr[i] * expf(-k.y * dz);
        float sn, cs;
        sincosf(k.x * dz, &sn, &cs);
        float re = acc[2 * i], im = acc[2 * i + 1];
        acc[2 * i] = amp * (re * cs - im * sn);
        acc[2 * i + 1] = amp * (re * sn + im * cs);
      }
#pragma unroll
      for (int i = 0; i < 64; ++i) {
        p.out[(size_t)(col0 + i) * p.ldo + row] = acc[i];
        if (p.cm_out) {
          const unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(fabsf(acc[i])));
          if (lane == 0) atomicMax(&p.cm_out[col0 + i], m);
        }
      }
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
  if (!s_fail && p.cm_clear && blockIdx.y == 0 && tid < TC_BN) p.cm_clear[bn + tid] = 0u;
  if (p.mode == 2 && p.ctl && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0 && !s_fail)
    p.ctl->guard_pending = 1;
}
