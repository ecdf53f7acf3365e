// dht_tc2.cuh -- Hankel transform GEMM on tcgen05 tensor cores with
// round-to-nearest accumulation across K.
//
// C = A B with A one of the two fixed Hankel matrices, split on the host into
// three TF32 pieces A = Ah + Am + Al (33 significant bits: the matrix is
// applied every z-step, so its representation error would add up
// coherently), and B split per tile into a TF32 head and rounded remainder;
// C ~ Ah Bh + Ah Bl + Am Bh + Al Bh.  The tensor memory accumulator only
// ever holds one 16-wide K chunk: the tensor core's FP32 accumulation rounds toward
// zero, which over a long K chain biases every output toward zero by
// ~7e-6 relative at K = 1024 and would damp the field step after step.
// Each chunk lands in a fresh accumulator (two sets, ping-pong: the Th*Bh
// product in one, the two small cross products in another) and eight
// consumer warps add it into FP32 registers, where rounding is unbiased.
// The head-product chunk itself still carries the round-toward-zero of the
// tensor core's own sum (about -2^-23 relative on average); the consumers
// add it as fma(v, 1 + 2^-23, acc), which removes that mean error (residual
// bias ~5e-9 relative per GEMM in the random-matrix check, the same as
// sequential FP32 summation).
//
// Warp roles (320 threads): warps 0-7 split the B tiles into head and
// remainder and accumulate chunks into registers, then run the epilogue;
// warp 8 issues the TMA loads; warp 9 issues the MMAs.  Tile 128 x 128,
// K step 32, two shared-memory stages {Ah, Am, Al, B, Bl} of 80 KB.
// Every mbarrier wait is bounded and also gives up as soon as another role
// has failed; failures set *err.
#pragma once
#include "tc_ptx.cuh"
#include "dht_tc.cuh"

#define T2_BM 128
#define T2_BN 128
#define T2_BK 32
#ifndef T2_CHUNK
#define T2_CHUNK 16
#endif
#define T2_STAGES 2
#define T2_CONSUMERS 256
#define T2_THREADS (T2_CONSUMERS + 64)
#define T2_A_BYTES (T2_BM * T2_BK * 4)
#define T2_B_BYTES (T2_BN * T2_BK * 4)
#define T2_STAGE_BYTES (3 * T2_A_BYTES + 2 * T2_B_BYTES)
#define T2_SMEM_BYTES (T2_STAGES * T2_STAGE_BYTES + 1024 + 256)

// bounded wait that also stops when *fail is set by another role
__device__ __forceinline__ bool t2_wait(uint32_t bar, uint32_t parity, volatile int* fail) {
  for (uint32_t i = 0; i < TC_WAIT_LIMIT; ++i) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *fail) return false;
  }
  *fail = 1;
  return false;
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

__global__ void __launch_bounds__(T2_THREADS, 1)
    k_dht_tc2(const __grid_constant__ CUtensorMap tTh, const __grid_constant__ CUtensorMap tTm,
              const __grid_constant__ CUtensorMap tTl, const __grid_constant__ CUtensorMap tB, TcGemmParams p) {
  extern __shared__ __align__(1024) uint8_t t2_smem[];
  __shared__ volatile int s_fail;
  if (p.ctl && p.ctl->done) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(t2_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = t2_smem + (sbase - raw);
  const uint32_t bars = sbase + T2_STAGES * T2_STAGE_BYTES;
  // barrier block: full[3] conv[3] empty[3] accf[2] acce[2] tmem_slot
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto conv_bar = [&](int s) { return bars + 24u + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 48u + 8u * s; };
  auto accf_bar = [&](int b) { return bars + 72u + 8u * b; };
  auto acce_bar = [&](int b) { return bars + 88u + 8u * b; };
  const uint32_t tmem_slot = bars + 104u;
  volatile uint32_t* tmem_slot_g = reinterpret_cast<volatile uint32_t*>(gbase + T2_STAGES * T2_STAGE_BYTES + 104);

  if (tid == 0) s_fail = 0;
  if (warp == 0) tc::tmem_alloc(tmem_slot, 512);
  if (tid == 0) {
    for (int s = 0; s < T2_STAGES; ++s) {
      tc::mbar_init(full_bar(s), 1);
      tc::mbar_init(conv_bar(s), 8);
      tc::mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(accf_bar(b), 1);
      tc::mbar_init(acce_bar(b), 8);
    }
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot_g;
  const int bm = blockIdx.y * T2_BM, bn = blockIdx.x * T2_BN;
  const int nk = p.K / T2_BK;
  const int chunks_per_kb = T2_BK / T2_CHUNK;
  const int nchunks = nk * chunks_per_kb;

  float acc[64];
#pragma unroll
  for (int i = 0; i < 64; ++i) acc[i] = 0.f;

  if (warp == 8) {
    // ---------------- producer: TMA loads, refills a stage once its MMAs finished
    if (lane == 0) {
      for (int kb = 0; kb < nk; ++kb) {
        const int s = kb % T2_STAGES;
        const int use = kb / T2_STAGES;
        if (use > 0 && !t2_wait(empty_bar(s), (use - 1) & 1, &s_fail)) break;
        const uint32_t st = sbase + s * T2_STAGE_BYTES;
        tc::mbar_expect_tx(full_bar(s), 3 * T2_A_BYTES + T2_B_BYTES);
        tc::tma_load_2d(st, &tTh, kb * T2_BK, bm, full_bar(s));
        tc::tma_load_2d(st + T2_A_BYTES, &tTm, kb * T2_BK, bm, full_bar(s));
        tc::tma_load_2d(st + 2 * T2_A_BYTES, &tTl, kb * T2_BK, bm, full_bar(s));
        tc::tma_load_2d(st + 3 * T2_A_BYTES, &tB, kb * T2_BK, bn, full_bar(s));
      }
      // wait for the last loads so no copy lands after the block exits
      for (int kb = (nk > T2_STAGES ? nk - T2_STAGES : 0); kb < nk; ++kb)
        t2_wait(full_bar(kb % T2_STAGES), (kb / T2_STAGES) & 1, &s_fail);
    }
  } else if (warp == 9) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_tf32(T2_BM, T2_BN);
      int chunk = 0;
      for (int kb = 0; kb < nk && !s_fail; ++kb) {
        const int s = kb % T2_STAGES;
        if (!t2_wait(conv_bar(s), (kb / T2_STAGES) & 1, &s_fail)) break;
        tc::tc_fence_after();
        const uint32_t st = sbase + s * T2_STAGE_BYTES;
        for (int c = 0; c < chunks_per_kb; ++c, ++chunk) {
          const int b = chunk & 1;
          const int use = chunk >> 1;
          if (use > 0 && !t2_wait(acce_bar(b), (use - 1) & 1, &s_fail)) break;
          tc::tc_fence_after();
          const uint32_t big = tmem + (uint32_t)(b * 256), small = big + 128u;
#pragma unroll
          for (int kk = 0; kk < T2_CHUNK / 8; ++kk) {
            const uint32_t koff = (uint32_t)((c * T2_CHUNK + kk * 8) * 4);
            const uint64_t ah = tc::desc_k128(st + koff);
            const uint64_t am = tc::desc_k128(st + T2_A_BYTES + koff);
            const uint64_t al = tc::desc_k128(st + 2 * T2_A_BYTES + koff);
            const uint64_t bh = tc::desc_k128(st + 3 * T2_A_BYTES + koff);
            const uint64_t bl = tc::desc_k128(st + 3 * T2_A_BYTES + T2_B_BYTES + koff);
            tc::mma_tf32(big, ah, bh, idesc, kk != 0);
            tc::mma_tf32(small, ah, bl, idesc, kk != 0);
            tc::mma_tf32(small, am, bh, idesc, 1);
            tc::mma_tf32(small, al, bh, idesc, 1);
          }
          tc::mma_commit(accf_bar(b));
        }
        tc::mma_commit(empty_bar(s));
      }
    }
  } else {
    // ---------------- consumers: split B, accumulate chunks in registers
    const int q = warp & 3, hcol = warp >> 2;
    auto convert = [&](int kb) -> bool {
      const int s = kb % T2_STAGES;
      if (!t2_wait(full_bar(s), (kb / T2_STAGES) & 1, &s_fail)) return false;
      float4* Bp = reinterpret_cast<float4*>(gbase + s * T2_STAGE_BYTES + 3 * T2_A_BYTES);
      float4* Bl = reinterpret_cast<float4*>(gbase + s * T2_STAGE_BYTES + 3 * T2_A_BYTES + T2_B_BYTES);
#pragma unroll
      for (int i = tid; i < T2_B_BYTES / 16; i += T2_CONSUMERS) {
        float4 v = Bp[i];
        float4 h = tf32_head(v);
        Bp[i] = h;
        Bl[i] = tf32_round(make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w));
      }
      tc::fence_proxy_async_smem();
      __syncwarp();
      if (lane == 0) mbar_arrive(conv_bar(s));
      return true;
    };
    bool ok = convert(0);
    int chunk = 0;
    for (int kb = 0; kb < nk && ok; ++kb) {
      if (kb + 1 < nk) ok = convert(kb + 1);
      if (!ok) break;
      for (int c = 0; c < chunks_per_kb; ++c, ++chunk) {
        const int b = chunk & 1;
        if (!t2_wait(accf_bar(b), (chunk >> 1) & 1, &s_fail)) { ok = false; break; }
        tc::tc_fence_after();
        const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)(b * 256 + 64 * hcol);
        float v[32];
        const float kap = p.rz_fix;
        tc::tmem_ld32(taddr, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] = fmaf(v[i], kap, acc[i]);
        tc::tmem_ld32(taddr + 32u, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[32 + i] = fmaf(v[i], kap, acc[32 + i]);
        tc::tmem_ld32(taddr + 128u, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[i] += v[i];
        tc::tmem_ld32(taddr + 160u, v);
#pragma unroll
        for (int i = 0; i < 32; ++i) acc[32 + i] += v[i];
        tc::tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(acce_bar(b));
      }
    }
    (void)nchunks;
  }
  __syncthreads();
  // ---------------- epilogue (consumers hold one row x 64 columns each)
  if (warp < 8 && !s_fail) {
    const int q = warp & 3, hcol = warp >> 2;
    const int row = bm + 32 * q + lane;
    const int col0 = bn + 64 * hcol;
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
      for (int i = 0; i < 64; ++i) p.out[(size_t)(col0 + i) * p.ldo + row] = acc[i];
    } else {
      const float sc = (p.mode == 2 && p.inv_s) ? p.inv_s[row] : 1.0f;
      float4* dst = reinterpret_cast<float4*>(p.out + (size_t)row * p.ldo + col0);
#pragma unroll
      for (int i = 0; i < 16; ++i)
        dst[i] = make_float4(sc * acc[4 * i], sc * acc[4 * i + 1], sc * acc[4 * i + 2], sc * acc[4 * i + 3]);
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
    p.ctl->guard_pending = 1;
}
