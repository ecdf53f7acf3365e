// nn_tc.cu -- inference kernels of the learned plasma surrogate
// (surrogate.cuh) with channel-last activations [row][t][64]:
//
//   layer 0 (3 -> 64)   k_nn_l0_cl   CUDA cores, 1728 MAC per point
//   layer 1 (64 -> 64)  k_nn_conv_tc tcgen05, 36864 MAC per point
//   layer 2 (64 -> 64)  k_nn_conv_tc
//   layer 3 (64 -> 1)   k_nn_l3_cl   CUDA cores, 576 MAC per point
//
// The 64 -> 64 convolution is an implicit GEMM per tile of 128 time points:
//   Y[t][co] = sum_k sum_ci X[t + k - 4][ci] W_k[co][ci],
// M = 128 (time points, one tensor-memory lane each), N = 64 (channels),
// K = 9 taps x 64 channels.  For every tap one TMA load brings the shifted
// tile X[t0 + k - 4 .. t0 + k + 123][0..63] (128 B rows, 128-byte swizzle,
// K-major A); rows outside [0, T) are zero-filled by the copy, which is the
// convolution's "same" padding.  The nine weight matrices W_k[co][ci]
// (K-major B, 72 KB) stay in shared memory for the whole launch.  Four MMAs
// of K = 16 per tap accumulate in FP32 in tensor memory; two 64-column
// accumulators alternate between tiles so that the epilogue of one tile
// (bias, tanh, BF16, 128 B store per time point) overlaps the MMAs of the
// next.  Persistent grid: one block per SM walks the tiles of all rows.
//
// Roles (192 threads): warps 0-3 epilogue (warp w owns tensor-memory lanes
// 32w .. 32w+31), warp 4 TMA producer, warp 5 MMA issuer.  Every mbarrier
// wait is bounded and gives up once another role failed; a failure sets
// *err and the block releases its tensor memory after its MMAs completed.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "nn_tc.h"
#include "surrogate_consts.h"
#include "tc_host.h"
#include "tc_ptx.cuh"

#define NT_BM 128                      // time points per tile
#define NT_STAGES 4
#define NT_A_BYTES (NT_BM * 128)       // one tap's activation tile
#define NT_W_BYTES (64 * 128)          // one tap's weights
#define NT_W_OFF 0
#define NT_A_OFF (NN_K * NT_W_BYTES)
#define NT_BAR_OFF (NT_A_OFF + NT_STAGES * NT_A_BYTES)
#define NT_SMEM (NT_BAR_OFF + 256 + 1024)
#define NT_THREADS 192
#define NT_WAIT_LIMIT (1u << 26)

static __device__ __forceinline__ bool nt_wait(uint32_t bar, uint32_t parity, volatile int* fail) {
  for (uint32_t i = 0; i < NT_WAIT_LIMIT; ++i) {
    if (tc::mbar_try_wait(bar, parity)) return true;
    if ((i & 255u) == 255u && *fail) return false;
  }
  *fail = 1;
  return false;
}
static __device__ __forceinline__ void nt_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}

struct NtParams {
  const float* bias;       // [64]
  __nv_bfloat16* out;      // [rows][T][64]
  int T, tiles_per_row, maxrows;
  const int* count;
  const int* stop;
  int* err;
};

__global__ void __launch_bounds__(NT_THREADS, 1)
    k_nn_conv_tc(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, NtParams p) {
  extern __shared__ __align__(1024) uint8_t nt_smem[];
  __shared__ volatile int s_fail;
  if (p.stop && *p.stop) return;
  const int nrows = p.count ? min(*p.count, p.maxrows) : p.maxrows;
  const int ntiles = nrows * p.tiles_per_row;
  if ((int)blockIdx.x >= ntiles) return;   // block-uniform, before any barrier
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(nt_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = nt_smem + (sbase - raw);
  const uint32_t bars = sbase + NT_BAR_OFF;
  // barrier block: full[4] empty[4] accf[2] acce[2] wbar done tmem_slot
  auto full_bar = [&](int s) { return bars + 8u * s; };
  auto empty_bar = [&](int s) { return bars + 32u + 8u * s; };
  auto accf_bar = [&](int b) { return bars + 64u + 8u * b; };
  auto acce_bar = [&](int b) { return bars + 80u + 8u * b; };
  const uint32_t wbar = bars + 96u, done_bar = bars + 104u, tmem_slot = bars + 112u;
  volatile uint32_t* tmem_slot_g = reinterpret_cast<volatile uint32_t*>(gbase + NT_BAR_OFF + 112);

  if (tid == 0) s_fail = 0;
  if (warp == 0) tc::tmem_alloc(tmem_slot, 128);
  if (tid == 0) {
    for (int s = 0; s < NT_STAGES; ++s) {
      tc::mbar_init(full_bar(s), 1);
      tc::mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(accf_bar(b), 1);
      tc::mbar_init(acce_bar(b), 4);
    }
    tc::mbar_init(wbar, 1);
    tc::mbar_init(done_bar, 1);
    tc::fence_mbar_init();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot_g;
  const int tpr = p.tiles_per_row;

  if (warp == 4) {
    // ---------------- producer: weights once, then one activation tile per tap
    if (lane == 0) {
      tc::mbar_expect_tx(wbar, NN_K * NT_W_BYTES);
      for (int k = 0; k < NN_K; ++k) tc::tma_load_2d(sbase + NT_W_OFF + k * NT_W_BYTES, &tw, 0, 64 * k, wbar);
      int it = 0;
      for (int tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x) {
        const int b = tile / tpr, t0 = (tile - b * tpr) * NT_BM;
        for (int k = 0; k < NN_K; ++k, ++it) {
          const int s = it % NT_STAGES, use = it / NT_STAGES;
          if (use > 0 && !nt_wait(empty_bar(s), (use - 1) & 1, &s_fail)) break;
          tc::mbar_expect_tx(full_bar(s), NT_A_BYTES);
          tc::tma_load_3d(sbase + NT_A_OFF + s * NT_A_BYTES, &tx, 0, t0 + k - NN_HALF, b, full_bar(s));
        }
      }
      // wait for the last loads so that no copy lands after the block exits
      nt_wait(wbar, 0, &s_fail);
      for (int i = (it > NT_STAGES ? it - NT_STAGES : 0); i < it; ++i)
        nt_wait(full_bar(i % NT_STAGES), (i / NT_STAGES) & 1, &s_fail);
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_bf16(NT_BM, 64);
      if (nt_wait(wbar, 0, &s_fail)) {
        int it = 0, lt = 0;
        for (int tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x, ++lt) {
          const int buf = lt & 1, ub = lt >> 1;
          if (ub > 0 && !nt_wait(acce_bar(buf), (ub - 1) & 1, &s_fail)) break;
          tc::tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)(buf * 64);
          bool ok = true;
          for (int k = 0; k < NN_K; ++k, ++it) {
            const int s = it % NT_STAGES;
            if (!nt_wait(full_bar(s), (it / NT_STAGES) & 1, &s_fail)) { ok = false; break; }
            tc::tc_fence_after();
            const uint32_t a = sbase + NT_A_OFF + s * NT_A_BYTES, w = sbase + NT_W_OFF + k * NT_W_BYTES;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {   // 16 channels = 32 bytes per MMA
              tc::mma_f16(acc, tc::desc_k128(a + 32u * kk), tc::desc_k128(w + 32u * kk), idesc,
                          (k | kk) ? 1u : 0u);
            }
            tc::mma_commit(empty_bar(s));
          }
          if (!ok) break;
          tc::mma_commit(accf_bar(buf));
        }
      }
      // no MMA may still write tensor memory when it is released
      tc::mma_commit(done_bar);
      tc::mbar_wait(done_bar, 0, NT_WAIT_LIMIT);
    }
  } else {
    // ---------------- epilogue: warp w owns time points 32w .. 32w+31 of the tile
    int lt = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++lt) {
      const int buf = lt & 1;
      if (!nt_wait(accf_bar(buf), (lt >> 1) & 1, &s_fail)) break;
      tc::tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16) + (uint32_t)(buf * 64);
      uint32_t r0[32], r1[32];
      tc::tmem_ld32_async(taddr, r0);
      tc::tmem_ld32_async(taddr + 32u, r1);
      tc::tmem_wait_ld(r0);
      tc::tmem_wait_ld(r1);
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) nt_arrive(acce_bar(buf));
      const int b = tile / tpr, t = (tile - b * tpr) * NT_BM + 32 * warp + lane;
      if (t < p.T) {
        uint4* dst = reinterpret_cast<uint4*>(p.out + ((size_t)b * p.T + t) * 64);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          uint32_t pk[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int c = 8 * q + 2 * e;
            const float v0 = __uint_as_float(c < 32 ? r0[c] : r1[c - 32]) + __ldg(&p.bias[c]);
            const float v1 = __uint_as_float(c + 1 < 32 ? r0[c + 1] : r1[c + 1 - 32]) + __ldg(&p.bias[c + 1]);
            const __nv_bfloat162 h = __floats2bfloat162_rn(tanhf(v0), tanhf(v1));
            pk[e] = *reinterpret_cast<const uint32_t*>(&h);
          }
          dst[q] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 128);
  }
  if (s_fail && tid == 0) atomicExch(p.err, 1);
}

// ---------------------------------------------------------------------------
// Layer 0 (3 -> 64, tanh): x [rows][3][T] -> y [rows][T][64].  Block: 32 time
// points x 8 channel groups of 8; rows b = blockIdx.y, + gridDim.y, ...
__global__ void __launch_bounds__(256) k_nn_l0_cl(const __nv_bfloat16* __restrict__ x,
                                                  const __nv_bfloat16* __restrict__ w,   // [ci][k][co]
                                                  const float* __restrict__ bias, __nv_bfloat16* y, int T,
                                                  int maxrows, const int* count, const int* stop) {
  constexpr int TT = 32, W2 = TT + NN_K - 1;
  __shared__ float xs[NN_IN][W2];
  __shared__ float ws[NN_IN * NN_K][64];
  if (stop && *stop) return;
  const int nb = count ? min(*count, maxrows) : maxrows;
  const int tid = threadIdx.x, tl = tid & 31, cg = tid >> 5;
  for (int i = tid; i < NN_IN * NN_K * 64; i += 256) ws[i / 64][i % 64] = __bfloat162float(w[i]);
  const int t0 = blockIdx.x * TT;
  for (int b = blockIdx.y; b < nb; b += gridDim.y) {
    __syncthreads();
    for (int i = tid; i < NN_IN * W2; i += 256) {
      const int ci = i / W2, j = i - ci * W2, t = t0 + j - NN_HALF;
      xs[ci][j] = (t >= 0 && t < T) ? __bfloat162float(x[((size_t)b * NN_IN + ci) * T + t]) : 0.f;
    }
    __syncthreads();
    float acc[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] = bias[8 * cg + c];
#pragma unroll
    for (int ci = 0; ci < NN_IN; ++ci)
#pragma unroll
      for (int k = 0; k < NN_K; ++k) {
        const float xv = xs[ci][tl + k];
#pragma unroll
        for (int c = 0; c < 8; ++c) acc[c] = fmaf(ws[ci * NN_K + k][8 * cg + c], xv, acc[c]);
      }
    const int t = t0 + tl;
    if (t < T) {
      uint32_t pk[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        const __nv_bfloat162 h = __floats2bfloat162_rn(tanhf(acc[2 * e]), tanhf(acc[2 * e + 1]));
        pk[e] = *reinterpret_cast<const uint32_t*>(&h);
      }
      *reinterpret_cast<uint4*>(y + ((size_t)b * T + t) * 64 + 8 * cg) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}

// Layer 3 (64 -> 1, no activation): y [rows][T][64] -> out [rows][T] (FP32).
// Block: 128 time points; the tile with its halo is staged in shared memory
// with a row pitch of 33 words (conflict-free column reads).
__global__ void __launch_bounds__(128) k_nn_l3_cl(const __nv_bfloat16* __restrict__ y,
                                                  const __nv_bfloat16* __restrict__ w,   // [ci][k]
                                                  const float* __restrict__ bias, float* out, int T, int maxrows,
                                                  const int* count, const int* stop) {
  constexpr int TT = 128, W2 = TT + NN_K - 1, PITCH = 33;
  __shared__ uint32_t ys[W2 * PITCH];   // bf16 pairs
  __shared__ float ws[NN_K][64];
  if (stop && *stop) return;
  const int nb = count ? min(*count, maxrows) : maxrows;
  const int tid = threadIdx.x;
  for (int i = tid; i < 64 * NN_K; i += TT) ws[i % NN_K][i / NN_K] = __bfloat162float(w[i]);
  const int t0 = blockIdx.x * TT;
  for (int b = blockIdx.y; b < nb; b += gridDim.y) {
    __syncthreads();
    // W2 rows x 32 words, 4 words per 16-byte load
    for (int i = tid; i < W2 * 8; i += TT) {
      const int r = i >> 3, q = i & 7, t = t0 + r - NN_HALF;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (t >= 0 && t < T) v = *reinterpret_cast<const uint4*>(y + ((size_t)b * T + t) * 64 + 8 * q);
      uint32_t* d = ys + r * PITCH + 4 * q;
      d[0] = v.x;
      d[1] = v.y;
      d[2] = v.z;
      d[3] = v.w;
    }
    __syncthreads();
    float acc = bias[0];
#pragma unroll
    for (int k = 0; k < NN_K; ++k) {
      const uint32_t* row = ys + (tid + k) * PITCH;
#pragma unroll 8
      for (int c2 = 0; c2 < 32; ++c2) {
        const uint32_t u = row[c2];
        const __nv_bfloat162 h = *reinterpret_cast<const __nv_bfloat162*>(&u);
        acc = fmaf(ws[k][2 * c2], __low2float(h), acc);
        acc = fmaf(ws[k][2 * c2 + 1], __high2float(h), acc);
      }
    }
    const int t = t0 + tid;
    if (t < T) out[(size_t)b * T + t] = acc;
  }
}

// ---------------------------------------------------------------------------
int nn_plan_init(NnRowsPlan* p) {
  if (p->T % NT_BM) return -3;
  const unsigned long long d1[3] = {64ull, (unsigned long long)p->T, (unsigned long long)p->maxrows};
  const unsigned box[3] = {64u, (unsigned)NT_BM, 1u};
  int rc = tc_make_map_bf16(&p->map_a1, p->a1, 3, d1, box);
  if (!rc) rc = tc_make_map_bf16(&p->map_a2, p->a2, 3, d1, box);
  if (rc) return rc;
  int dev = 0;
  cudaGetDevice(&dev);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 148;
  p->sms = sms;
  return 0;
}

int nn_weight_map(CUtensorMap* m, const __nv_bfloat16* wt) {
  const unsigned long long d[2] = {64ull, (unsigned long long)NN_K * 64ull};
  const unsigned box[2] = {64u, 64u};
  return tc_make_map_bf16(m, wt, 2, d, box);
}

cudaError_t nn_launch_l0_cl(const __nv_bfloat16* x, const __nv_bfloat16* w, const float* bias, __nv_bfloat16* y,
                            int T, int maxrows, const int* count, const int* stop, cudaStream_t st) {
  const int gx = (T + 31) / 32, gy = std::max(1, std::min(maxrows, (152 * 8 + gx - 1) / gx));
  k_nn_l0_cl<<<dim3(gx, gy), 256, 0, st>>>(x, w, bias, y, T, maxrows, count, stop);
  return cudaGetLastError();
}

cudaError_t nn_launch_l3_cl(const __nv_bfloat16* y, const __nv_bfloat16* w, const float* bias, float* out, int T,
                            int maxrows, const int* count, const int* stop, cudaStream_t st) {
  const int gx = (T + 127) / 128, gy = std::max(1, std::min(maxrows, (152 * 16 + gx - 1) / gx));
  k_nn_l3_cl<<<dim3(gx, gy), 128, 0, st>>>(y, w, bias, out, T, maxrows, count, stop);
  return cudaGetLastError();
}

cudaError_t nn_launch_conv_tc(const CUtensorMap& tx, const CUtensorMap& tw, const float* bias, __nv_bfloat16* out,
                              const NnRowsPlan& p, cudaStream_t st) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_nn_conv_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, NT_SMEM);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  NtParams q;
  q.bias = bias;
  q.out = out;
  q.T = p.T;
  q.tiles_per_row = p.T / NT_BM;
  q.maxrows = p.maxrows;
  q.count = p.count;
  q.stop = p.stop;
  q.err = p.err;
  const int tiles = p.maxrows * q.tiles_per_row;
  const int grid = std::max(1, std::min(p.sms, tiles));
  k_nn_conv_tc<<<grid, NT_THREADS, NT_SMEM, st>>>(tx, tw, q);
  return cudaGetLastError();
}
