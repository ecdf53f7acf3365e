// dht_tc.cuh -- the Hankel transforms of the linear step as tcgen05 tensor-core
// GEMMs (kind::tf32, FP32 accumulation in tensor memory).
//
// Reference: src/modules/linear_propagators/spectral.jl:16-26
// (PS * E; E .*= exp(i KZ dz); spectral guard; PS \ E) with the order-0
// QDHT pair written as E <- diag(1/s) T D T diag(s) E; the row kernel applies
// diag(s) when it writes the spectrum, this kernel applies T (twice) and
// D = exp(i KZ dz) * guard, and the second launch applies diag(1/s).
//
// C[M x N] = T[M x K] * B[K x N] with T symmetric and both operands stored
// K-major: T row-major, B as B^T (row n = one real column of the complex
// half spectrum, index k = transverse point contiguous).  FP32 accuracy
// comes from a three-product TF32 split: T = Th + Tl (exact TF32 head plus
// remainder, prepared once on the host), B = Bh + Bl (split in shared memory
// per tile), C ~ Th Bh + Th Bl + Tl Bh.
//
// Tile 128 x 256 x 32, two pipeline stages of {Th, Tl, B, Bl} filled by TMA
// with 128-byte swizzle, one thread issues the MMAs, 256 threads split B and
// run the epilogue (tcgen05.ld of the 128 x 256 FP32 accumulator).
// All mbarrier waits are bounded; a timeout sets *err and the block leaves
// after releasing its tensor memory.
#pragma once
#include "tc_ptx.cuh"
#include "rowkernels.cuh"

#define TC_BM 128
#define TC_BN 256
#define TC_BK 32
#define TC_STAGES 2
#define TC_THREADS 256
#define TC_A_BYTES (TC_BM * TC_BK * 4)
#define TC_B_BYTES (TC_BN * TC_BK * 4)
#define TC_STAGE_BYTES (2 * TC_A_BYTES + 2 * TC_B_BYTES)
#define TC_SMEM_BYTES (TC_STAGES * TC_STAGE_BYTES + 1024 + 256)
#define TC_WAIT_LIMIT (1u << 26)

struct TcGemmParams {
  float* out;
  int ldo;           // leading dimension of out (floats)
  int K;             // contraction length, multiple of TC_BK
  int mode;          // 0 row-major store; 1 propagator + transposed store;
                     // 2 row scale + row-major store (+ guard pending)
  const float2* kz;  // mode 1: [M][nh] KZ in zu units
  const float* gd;   // mode 1: [M][nh] spectral guard
  int nh;
  const float* inv_s;  // mode 2: [M] row scale
  DevCtl* ctl;       // NULL: no controller (dz = dz_fixed)
  float dz_fixed;
  int* err;          // set to 1 on a timed-out wait
  float rz_fix;      // factor applied to each chunk of the head product as it
                     // is summed (de-biasing of round-toward-zero), see dht_tc2.cuh
};

// nearest TF32 value (ties away from zero); exact TF32 operands are not
// altered by the tensor core's conversion, so rounding here keeps the
// remainder terms unbiased
__device__ __forceinline__ float tf32_round1(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
__device__ __forceinline__ float4 tf32_round(float4 v) {
  return make_float4(tf32_round1(v.x), tf32_round1(v.y), tf32_round1(v.z), tf32_round1(v.w));
}

__device__ __forceinline__ float4 tf32_head(float4 v) {
  const unsigned m = 0xFFFFE000u;
  return make_float4(__uint_as_float(__float_as_uint(v.x) & m), __uint_as_float(__float_as_uint(v.y) & m),
                     __uint_as_float(__float_as_uint(v.z) & m), __uint_as_float(__float_as_uint(v.w) & m));
}

static __global__ void __launch_bounds__(TC_THREADS, 1)
    k_dht_tc(const __grid_constant__ CUtensorMap tTh, const __grid_constant__ CUtensorMap tTl,
             const __grid_constant__ CUtensorMap tB, TcGemmParams p) {
  extern __shared__ __align__(1024) uint8_t tc_smem[];
  __shared__ int s_fail;
  if (p.ctl && p.ctl->done) return;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(tc_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = tc_smem + (sbase - raw);
  const uint32_t bars = sbase + TC_STAGES * TC_STAGE_BYTES;
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 16u + 8u * s; };
  const uint32_t accum_bar = bars + 32u;
  const uint32_t tmem_slot = bars + 40u;
  volatile uint32_t* tmem_slot_g = reinterpret_cast<volatile uint32_t*>(gbase + TC_STAGES * TC_STAGE_BYTES + 40);

  if (tid == 0) s_fail = 0;
  if (warp == 0) tc::tmem_alloc(tmem_slot, TC_BN);
  if (tid == 0) {
    for (int s = 0; s < TC_STAGES; ++s) {
      tc::mbar_init(full_bar(s), 1);
      tc::mbar_init(empty_bar(s), 1);
    }
    tc::mbar_init(accum_bar, 1);
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot_g;

  const int bm = blockIdx.y * TC_BM, bn = blockIdx.x * TC_BN;
  const int nk = p.K / TC_BK;
  auto issue = [&](int kb, int s) {
    const uint32_t st = sbase + s * TC_STAGE_BYTES;
    tc::mbar_expect_tx(full_bar(s), 2 * TC_A_BYTES + TC_B_BYTES);
    tc::tma_load_2d(st, &tTh, kb * TC_BK, bm, full_bar(s));
    tc::tma_load_2d(st + TC_A_BYTES, &tTl, kb * TC_BK, bm, full_bar(s));
    tc::tma_load_2d(st + 2 * TC_A_BYTES, &tB, kb * TC_BK, bn, full_bar(s));
  };
  int issued = 0;   // loads issued (thread 0)
  if (tid == 0)
    for (int s = 0; s < TC_STAGES && s < nk; ++s) { issue(s, s); ++issued; }

  const uint32_t idesc = tc::idesc_tf32(TC_BM, TC_BN);
  int done_kb = 0;
  for (int kb = 0; kb < nk; ++kb) {
    const int s = kb & 1;
    const uint32_t ph = (kb >> 1) & 1;
    if (!tc::mbar_wait(full_bar(s), ph, TC_WAIT_LIMIT)) s_fail = 1;
    __syncthreads();
    if (s_fail) break;
    // split B into an exact TF32 head (in place) and the remainder
    float4* Bp = reinterpret_cast<float4*>(gbase + s * TC_STAGE_BYTES + 2 * TC_A_BYTES);
    float4* Bl = reinterpret_cast<float4*>(gbase + s * TC_STAGE_BYTES + 2 * TC_A_BYTES + TC_B_BYTES);
#pragma unroll 4
    for (int i = tid; i < TC_B_BYTES / 16; i += TC_THREADS) {
      float4 v = Bp[i];
      float4 h = tf32_head(v);
      Bp[i] = h;
      Bl[i] = make_float4(v.x - h.x, v.y - h.y, v.z - h.z, v.w - h.w);
    }
    tc::fence_proxy_async_smem();
    __syncthreads();
    if (tid == 0) {
      tc::tc_fence_after();
      const uint32_t st = sbase + s * TC_STAGE_BYTES;
#pragma unroll
      for (int kk = 0; kk < TC_BK / 8; ++kk) {
        const uint64_t ah = tc::desc_k128(st + kk * 32);
        const uint64_t al = tc::desc_k128(st + TC_A_BYTES + kk * 32);
        const uint64_t bh = tc::desc_k128(st + 2 * TC_A_BYTES + kk * 32);
        const uint64_t bl = tc::desc_k128(st + 2 * TC_A_BYTES + TC_B_BYTES + kk * 32);
        tc::mma_tf32(tmem, ah, bh, idesc, (kb | kk) != 0);
        tc::mma_tf32(tmem, ah, bl, idesc, 1);
        tc::mma_tf32(tmem, al, bh, idesc, 1);
      }
      tc::mma_commit(empty_bar(s));
      if (kb + TC_STAGES < nk) {
        // the stage is refilled once the MMAs reading it are complete
        if (tc::mbar_wait(empty_bar(s), ph, TC_WAIT_LIMIT)) { issue(kb + TC_STAGES, s); ++issued; }
        else s_fail = 1;
      }
    }
    done_kb = kb + 1;
  }
  if (tid == 0 && !s_fail) tc::mma_commit(accum_bar);
  __syncthreads();
  bool have = false;
  if (!s_fail) {
    have = tc::mbar_wait(accum_bar, 0, TC_WAIT_LIMIT);
    if (!have) s_fail = 1;
  } else if (tid == 0) {
    // let loads still in flight land before the block's shared memory goes away
    for (int kb = done_kb; kb < issued; ++kb) tc::mbar_wait(full_bar(kb & 1), (kb >> 1) & 1, TC_WAIT_LIMIT);
  }
  __syncthreads();
  tc::tc_fence_after();

  if (!s_fail) {
    const int q = warp & 3, hcol = warp >> 2;
    const int row = bm + 32 * q + lane;
    const float dz = p.ctl ? (float)p.ctl->dz : p.dz_fixed;
#pragma unroll 1
    for (int c = 0; c < 4; ++c) {
      const int col0 = 128 * hcol + 32 * c;
      float v[32];
      tc::tmem_ld32(tmem + ((uint32_t)(32 * q) << 16) + (uint32_t)col0, v);
      if (p.mode == 1) {
        const int w0 = (bn + col0) >> 1;
        const float2* kzr = p.kz + (size_t)row * p.nh + w0;
        const float* gr = p.gd + (size_t)row * p.nh + w0;
#pragma unroll
        for (int i = 0; i < 16; ++i) {
          float2 k = kzr[i];
          float amp = gr[i] * expf(-k.y * dz);
          float sn, cs;
          sincosf(k.x * dz, &sn, &cs);
          float re = v[2 * i], im = v[2 * i + 1];
          v[2 * i] = amp * (re * cs - im * sn);
          v[2 * i + 1] = amp * (re * sn + im * cs);
        }
#pragma unroll
        for (int i = 0; i < 32; ++i) p.out[(size_t)(bn + col0 + i) * p.ldo + row] = v[i];
      } else {
        const float sc = (p.mode == 2) ? p.inv_s[row] : 1.0f;
        float4* dst = reinterpret_cast<float4*>(p.out + (size_t)row * p.ldo + bn + col0);
#pragma unroll
        for (int i = 0; i < 8; ++i)
          dst[i] = make_float4(sc * v[4 * i], sc * v[4 * i + 1], sc * v[4 * i + 2], sc * v[4 * i + 3]);
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, TC_BN);
  }
  if (s_fail && tid == 0) atomicExch(p.err, 1);
  if (p.mode == 2 && p.ctl && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0 && !s_fail)
    p.ctl->guard_pending = 1;
}
