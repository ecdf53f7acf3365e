// nn_tc.cu -- inference kernels of the learned plasma surrogate
// (surrogate.cuh) with channel-last activations [row][t][64]:
//
//   layer 0 (3 -> 64)   CUDA cores, 1728 MAC per point, inside layer 1's kernel
//   layer 1 (64 -> 64)  k_nn_conv_tc<false, true> tcgen05, 36864 MAC per point
//   layer 2 (64 -> 64)  k_nn_conv_tc<true, false> tcgen05, 36864 MAC per point
//   layer 3 (64 -> 1)   layer 2's epilogue (nine per-tap partial sums, 576
//                       MAC per point), summed where the density is formed
//
// The 64 -> 64 convolution is an implicit GEMM per tile of 128 time points:
//   Y[t][co] = sum_k sum_ci X[t + k - 4][ci] W_k[co][ci],
// M = 128 (time points, one tensor-memory lane each), N = 64 (channels),
// K = 9 taps x 64 channels.  One TMA load per tile brings the halo tile
// X[t0 - 4 .. t0 + 131][0..63] (136 rows of 128 B, 128-byte swizzle, K-major
// A); the A operand of tap k starts k rows (k * 128 B) into it -- the swizzle
// is a function of the shared-memory address, so the shifted operand reads
// the rows as the copy wrote them.  Rows outside [0, T) are zero-filled by the
// copy, which is the convolution's "same" padding.  The nine weight matrices W_k[co][ci]
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
//
// Layer 1 with layer 0 fused (L0): its input tile is not loaded but computed.
// Eight more warps (6-13) form the 136-row halo tile of layer-0 activations
// of each tile from the three input channels, tanh(b0 + sum_ci sum_k
// w0[ci][k][co] x[ci][t + k - 4]) rounded to BF16 (zero for rows outside
// [0, T), the "same" padding of layer 1), and write it into the stage in
// the layout the 128-byte swizzle gives a TMA copy (16-byte chunk c of row r
// at chunk c ^ (r mod 8) of the 1024-byte aligned stage).  Warp q owns halo
// rows 17q .. 17q + 16, lane l the channel pair (2l, 2l + 1) with its 54
// weights in registers; the warp stages its 25-point input window per
// channel in its own shared buffer and walks the rows with a rolling 9-tap
// window; a row is one 128-byte store by the warp.  Every lane fences its
// writes for the tensor core's proxy and arrives on the stage's full barrier
// (count 256).  Layer 0's activations never reach HBM.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "nn_tc.h"
#include "surrogate_consts.h"
#include "tc_host.h"
#include "tc_ptx.cuh"

#define NT_BM 128                      // time points per tile
#define NT_STAGES 6
#define NT_HALO (NT_BM + NN_K - 1)     // rows of one tile with its halo
#define NT_A_BYTES (NT_HALO * 128)     // the halo tile as loaded
#define NT_A_STRIDE 18432              // stage pitch: NT_A_BYTES rounded up to 1024
#define NT_W_BYTES (64 * 128)          // one tap's weights
#define NT_W_OFF 0
#define NT_A_OFF (NN_K * NT_W_BYTES)
#define NT_BAR_OFF (NT_A_OFF + NT_STAGES * NT_A_STRIDE)
#define NT_BAR_BYTES 256               // barrier block (layout below) + tensor-memory slot
#define NT_SMEM (NT_BAR_OFF + NT_BAR_BYTES + 1024)
// barrier block, 8 bytes each: full[S] empty[S] accf[2] acce[2] wbar done, then the
// tensor-memory address slot
#define NT_FULL(s) (8u * (s))
#define NT_EMPTY(s) (8u * (NT_STAGES + (s)))
#define NT_ACCF(b) (8u * (2 * NT_STAGES + (b)))
#define NT_ACCE(b) (8u * (2 * NT_STAGES + 2 + (b)))
#define NT_WBAR (8u * (2 * NT_STAGES + 4))
#define NT_DONE (8u * (2 * NT_STAGES + 5))
#define NT_SLOT (8u * (2 * NT_STAGES + 6))
static_assert(NT_SLOT + 4 <= NT_BAR_BYTES, "barrier block overflows its reserved bytes");
static_assert(NT_A_STRIDE % 1024 == 0 && NT_A_STRIDE >= NT_A_BYTES, "stage pitch");
#define NT_THREADS 192
#define NT_L0_WARPS 8                  // layer-0 warps of the fused kernel
#define NT_THREADS_L0 (NT_THREADS + 32 * NT_L0_WARPS)
#define NT_L0_ROWS (NT_HALO / NT_L0_WARPS)   // halo rows per layer-0 warp
static_assert(NT_L0_ROWS * NT_L0_WARPS == NT_HALO, "the halo rows split evenly over the layer-0 warps");
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
// hardware tanh (tanh.approx.f32, relative error about 2^-11, below the
// BF16 rounding of the activations it feeds)
static __device__ __forceinline__ float nt_tanh(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// two FP32 FMAs in one instruction (fma.rn.f32x2): lane-wise
// round-to-nearest, the same results as fmaf on each lane
static __device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) {
  float2 d;
  asm("{\n .reg .b64 a, b, c, d;\n mov.b64 a, {%2, %3};\n mov.b64 b, {%4, %5};\n mov.b64 c, {%6, %7};\n"
      " fma.rn.f32x2 d, a, b, c;\n mov.b64 {%0, %1}, d;\n}"
      : "=f"(d.x), "=f"(d.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y), "f"(c.x), "f"(c.y));
  return d;
}

struct NtParams {
  const float* bias;       // [64]
  const __nv_bfloat16* x0; // L0: network inputs [rows][3][T]
  const __nv_bfloat16* w0; // L0: layer-0 weights [ci][k][co]
  const float* b0;         // L0: layer-0 bias [64]
  __nv_bfloat16* out;      // [rows][T][64] (layer 1)
  const __nv_bfloat16* w3; // layer 3 weights [ci][k] (FINAL)
  float* part;             // [rows][9][T] layer-3 partial sums (FINAL)
  int T, tiles_per_row, maxrows;
  const int* count;
  const int* stop;
  int* err;
};

// FINAL (layer 2): the epilogue applies layer 3 to its own point instead of
// storing the activations: P_k[t] = sum_ci w3[ci][k] y[t][ci] for the nine
// taps k (the BF16-rounded activations, as stored between layers), so that
// out[t] = b3 + sum_k P_k[t + k - 4] (nn_out_at).
template <bool FINAL, bool L0>
__global__ void __launch_bounds__(L0 ? NT_THREADS_L0 : NT_THREADS, 1)
    k_nn_conv_tc(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, NtParams p) {
  static_assert(!(FINAL && L0), "layer 0 is fused into layer 1 only");
  extern __shared__ __align__(1024) uint8_t nt_smem[];
  __shared__ volatile int s_fail;
  __shared__ __align__(16) float s_bias[64];
  // L0: each layer-0 warp's input window (three channels x 25 points)
  __shared__ float s_xw[L0 ? NT_L0_WARPS : 1][NN_IN][L0 ? NT_L0_ROWS + NN_K - 1 : 1];
  // layer-3 weights as tap pairs: s_w3[(kp * 64 + ci) * 2 + u] = w3[ci][2 kp + u]
  // (kp < 5; the tenth tap is zero)
  __shared__ __align__(16) float s_w3[FINAL ? 5 * 64 * 2 : 4];
  if (p.stop && *p.stop) return;
  const int nrows = p.count ? min(*p.count, p.maxrows) : p.maxrows;
  const int ntiles = nrows * p.tiles_per_row;
  if ((int)blockIdx.x >= ntiles) return;   // block-uniform, before any barrier
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(nt_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = nt_smem + (sbase - raw);
  const uint32_t bars = sbase + NT_BAR_OFF;
  auto full_bar = [&](int s) { return bars + NT_FULL(s); };
  auto empty_bar = [&](int s) { return bars + NT_EMPTY(s); };
  auto accf_bar = [&](int b) { return bars + NT_ACCF(b); };
  auto acce_bar = [&](int b) { return bars + NT_ACCE(b); };
  const uint32_t wbar = bars + NT_WBAR, done_bar = bars + NT_DONE, tmem_slot = bars + NT_SLOT;
  volatile uint32_t* tmem_slot_g = reinterpret_cast<volatile uint32_t*>(gbase + NT_BAR_OFF + NT_SLOT);

  if (tid == 0) s_fail = 0;
  if (tid < 64) s_bias[tid] = p.bias[tid];
  if (FINAL)
    for (int i = tid; i < 5 * 64 * 2; i += NT_THREADS) {
      const int u = i & 1, ci = (i >> 1) & 63, k = 2 * (i >> 7) + u;
      s_w3[i] = k < NN_K ? __bfloat162float(p.w3[ci * NN_K + k]) : 0.f;
    }
  if (warp == 0) tc::tmem_alloc(tmem_slot, 128);
  if (tid == 0) {
    for (int s = 0; s < NT_STAGES; ++s) {
      tc::mbar_init(full_bar(s), L0 ? 32 * NT_L0_WARPS : 1);
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
      for (int tile = blockIdx.x; tile < ntiles && !s_fail && !L0; tile += gridDim.x, ++it) {
        const int b = tile / tpr, t0 = (tile - b * tpr) * NT_BM;
        const int s = it % NT_STAGES, use = it / NT_STAGES;
        if (use > 0 && !nt_wait(empty_bar(s), (use - 1) & 1, &s_fail)) break;
        tc::mbar_expect_tx(full_bar(s), NT_A_BYTES);
        tc::tma_load_3d(sbase + NT_A_OFF + s * NT_A_STRIDE, &tx, 0, t0 - NN_HALF, b, full_bar(s));
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
        int lt = 0;
        for (int tile = blockIdx.x; tile < ntiles && !s_fail; tile += gridDim.x, ++lt) {
          const int buf = lt & 1, ub = lt >> 1;
          if (ub > 0 && !nt_wait(acce_bar(buf), (ub - 1) & 1, &s_fail)) break;
          const int s = lt % NT_STAGES;
          if (!nt_wait(full_bar(s), (lt / NT_STAGES) & 1, &s_fail)) break;
          tc::tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)(buf * 64);
          const uint32_t a = sbase + NT_A_OFF + s * NT_A_STRIDE;
#pragma unroll 1
          for (int k = 0; k < NN_K; ++k) {
            const uint32_t ak = a + 128u * k, w = sbase + NT_W_OFF + k * NT_W_BYTES;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {   // 16 channels = 32 bytes per MMA
              tc::mma_f16(acc, tc::desc_k128(ak + 32u * kk), tc::desc_k128(w + 32u * kk), idesc,
                          (k | kk) ? 1u : 0u);
            }
          }
          tc::mma_commit(empty_bar(s));
          tc::mma_commit(accf_bar(buf));
        }
      }
      // no MMA may still write tensor memory when it is released
      tc::mma_commit(done_bar);
      tc::mbar_wait(done_bar, 0, NT_WAIT_LIMIT);
    }
  } else if (L0 && warp >= 6) {
    // ---------------- layer 0 into the stages (see the header).  Lane 0
    // decides each stage wait and the warp follows it (no divergence); no
    // barrier across warps, so a warp that stops holds no other up.
    const int q = warp - 6, c2 = 2 * lane, r0 = NT_L0_ROWS * q;
    float2 wv[NN_IN][NN_K];
#pragma unroll
    for (int ci = 0; ci < NN_IN; ++ci)
#pragma unroll
      for (int k = 0; k < NN_K; ++k) {
        const __nv_bfloat162 w = *reinterpret_cast<const __nv_bfloat162*>(p.w0 + (ci * NN_K + k) * 64 + c2);
        wv[ci][k] = __bfloat1622float2(w);
      }
    const float2 bias0 = make_float2(p.b0[c2], p.b0[c2 + 1]);
    float* xw = &s_xw[q][0][0];
    constexpr int XW = NT_L0_ROWS + NN_K - 1;
    constexpr int XL = (NN_IN * XW + 31) / 32;        // window values per lane
    // this lane's window values x[ci][t0 - 8 + r0 + j] of a tile (zero
    // outside [0, T)), loaded one tile ahead of their use
    auto load_window = [&](int tile, float (&v)[XL]) {
      const int b = tile / tpr, t0 = (tile - b * tpr) * NT_BM;
      const __nv_bfloat16* xb = p.x0 + (size_t)b * NN_IN * p.T;
#pragma unroll
      for (int u = 0; u < XL; ++u) {
        const int i = lane + 32 * u;
        v[u] = 0.f;
        if (i < NN_IN * XW) {
          const int ci = i / XW, j = i - ci * XW, tt = t0 - 2 * NN_HALF + r0 + j;
          if (tt >= 0 && tt < p.T) v[u] = __bfloat162float(xb[(size_t)ci * p.T + tt]);
        }
      }
    };
    float nxt[XL];
    if ((int)blockIdx.x < ntiles) load_window(blockIdx.x, nxt);
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int b = tile / tpr, t0 = (tile - b * tpr) * NT_BM;
      const int s = it % NT_STAGES, use = it / NT_STAGES;
      int ok = 1;
      if (lane == 0) ok = !s_fail && (use == 0 || nt_wait(empty_bar(s), (use - 1) & 1, &s_fail));
      if (!__shfl_sync(0xffffffffu, ok, 0)) break;
      (void)b;
#pragma unroll
      for (int u = 0; u < XL; ++u)
        if (lane + 32 * u < NN_IN * XW) xw[lane + 32 * u] = nxt[u];
      __syncwarp();
      if (tile + (int)gridDim.x < ntiles) load_window(tile + gridDim.x, nxt);   // in flight during the rows
      uint8_t* st = gbase + NT_A_OFF + s * NT_A_STRIDE;
      float win[NN_IN][NN_K];
#pragma unroll
      for (int ci = 0; ci < NN_IN; ++ci)
#pragma unroll
        for (int k = 0; k < NN_K - 1; ++k) win[ci][k + 1] = xw[ci * XW + k];
#pragma unroll
      for (int j = 0; j < NT_L0_ROWS; ++j) {
        // window of row r0 + j: x at tau - 4 .. tau + 4, tau = t0 - 4 + r0 + j
#pragma unroll
        for (int ci = 0; ci < NN_IN; ++ci) {
#pragma unroll
          for (int k = 0; k < NN_K - 1; ++k) win[ci][k] = win[ci][k + 1];
          win[ci][NN_K - 1] = xw[ci * XW + j + NN_K - 1];
        }
        const int r = r0 + j, tau = t0 - NN_HALF + r;
        // one independent chain per input channel, joined at the end
        float2 a[NN_IN];
#pragma unroll
        for (int ci = 0; ci < NN_IN; ++ci) {
          a[ci] = ci == 0 ? bias0 : make_float2(0.f, 0.f);
#pragma unroll
          for (int k = 0; k < NN_K; ++k) a[ci] = fma2(wv[ci][k], make_float2(win[ci][k], win[ci][k]), a[ci]);
        }
        const float vx = (a[0].x + a[1].x) + a[2].x, vy = (a[0].y + a[1].y) + a[2].y;
        uint32_t pk = 0u;
        if (tau >= 0 && tau < p.T) {
          const __nv_bfloat162 h = __floats2bfloat162_rn(nt_tanh(vx), nt_tanh(vy));
          pk = *reinterpret_cast<const uint32_t*>(&h);
        }
        // channels c2, c2 + 1: byte 4 lane of the row, 16-byte chunk lane / 4
        *reinterpret_cast<uint32_t*>(st + r * 128 + (((lane >> 2) ^ (r & 7)) << 4) + ((lane & 3) << 2)) = pk;
      }
      __syncwarp();                   // xw free for the next tile
      tc::fence_proxy_async_smem();   // this lane's writes, for the MMAs
      nt_arrive(full_bar(s));
    }
  } else if (warp < 4) {
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
      if (FINAL && t < p.T) {
        float y[64];
        const float4* bv = reinterpret_cast<const float4*>(s_bias);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          const float4 bq = bv[q];
          const float bb[4] = {bq.x, bq.y, bq.z, bq.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int c = 4 * q + e;
            const float v = __uint_as_float(c < 32 ? r0[c] : r1[c - 32]) + bb[e];
            y[c] = __bfloat162float(__float2bfloat16_rn(nt_tanh(v)));
          }
        }
        float* dst = p.part + (size_t)b * NN_K * p.T + t;
        // P_k = sum_ci w3[ci][k] y[ci], taps k and k+1 in one fma.rn.f32x2;
        // two chains per tap pair (even and odd ci), joined at the end
#pragma unroll
        for (int kp = 0; kp < 5; ++kp) {
          const float4* wk = reinterpret_cast<const float4*>(s_w3 + kp * 128);
          float2 a0 = make_float2(0.f, 0.f), a1 = make_float2(0.f, 0.f);
#pragma unroll
          for (int ci = 0; ci < 64; ci += 2) {
            const float4 w = wk[ci / 2];   // (w3[ci][2kp], w3[ci][2kp+1], w3[ci+1][2kp], w3[ci+1][2kp+1])
            a0 = fma2(make_float2(w.x, w.y), make_float2(y[ci], y[ci]), a0);
            a1 = fma2(make_float2(w.z, w.w), make_float2(y[ci + 1], y[ci + 1]), a1);
          }
          dst[(size_t)(2 * kp) * p.T] = a0.x + a1.x;
          if (2 * kp + 1 < NN_K) dst[(size_t)(2 * kp + 1) * p.T] = a0.y + a1.y;
        }
      } else if (t < p.T) {
        uint4* dst = reinterpret_cast<uint4*>(p.out + ((size_t)b * p.T + t) * 64);
        const float4* bv = reinterpret_cast<const float4*>(s_bias);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
          const float4 b0 = bv[2 * q], b1 = bv[2 * q + 1];
          const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
          uint32_t pk[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int c = 8 * q + 2 * e;
            const float v0 = __uint_as_float(c < 32 ? r0[c] : r1[c - 32]) + bb[2 * e];
            const float v1 = __uint_as_float(c + 1 < 32 ? r0[c + 1] : r1[c + 1 - 32]) + bb[2 * e + 1];
            const __nv_bfloat162 h = __floats2bfloat162_rn(nt_tanh(v0), nt_tanh(v1));
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


// Network output from the layer-3 partial sums (the inference path outside
// the row kernel): out[b][t] = b3 + sum_k P_k[t + k - 4].
__global__ void __launch_bounds__(256) k_nn_out(const float* __restrict__ part, const float* __restrict__ b3,
                                                float* out, int T, int rows) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i >= (long)rows * T) return;
  const int b = (int)(i / T), t = (int)(i - (long)b * T);
  out[i] = nn_out_at(part + (size_t)b * NN_K * T, b3[0], t, T);
}

// ---------------------------------------------------------------------------
int nn_plan_init(NnRowsPlan* p) {
  if (p->T % NT_BM) return -3;
  const unsigned long long d1[3] = {64ull, (unsigned long long)p->T, (unsigned long long)p->maxrows};
  const unsigned box[3] = {64u, (unsigned)NT_HALO, 1u};
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

cudaError_t nn_launch_out(const float* part, const float* b3, float* out, int T, int rows, cudaStream_t st) {
  const long n = (long)rows * T;
  k_nn_out<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(part, b3, out, T, rows);
  return cudaGetLastError();
}

cudaError_t nn_launch_conv_tc(const CUtensorMap& tx, const CUtensorMap& tw, const float* bias, __nv_bfloat16* out,
                              const __nv_bfloat16* w3, float* part, const NnRowsPlan& p, cudaStream_t st,
                              const __nv_bfloat16* x0, const __nv_bfloat16* w0, const float* b0) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e =
        cudaFuncSetAttribute(k_nn_conv_tc<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, NT_SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_nn_conv_tc<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, NT_SMEM);
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_nn_conv_tc<false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, NT_SMEM);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  if (x0 && part) return cudaErrorInvalidValue;   // layer 0 is fused into layer 1 only
  NtParams q;
  q.bias = bias;
  q.x0 = x0;
  q.w0 = w0;
  q.b0 = b0;
  q.out = out;
  q.w3 = w3;
  q.part = part;
  q.T = p.T;
  q.tiles_per_row = p.T / NT_BM;
  q.maxrows = p.maxrows;
  q.count = p.count;
  q.stop = p.stop;
  q.err = p.err;
  const int tiles = p.maxrows * q.tiles_per_row;
  const int grid = std::max(1, std::min(p.sms, tiles));
  if (part)
    k_nn_conv_tc<true, false><<<grid, NT_THREADS, NT_SMEM, st>>>(tx, tw, q);
  else if (x0)
    k_nn_conv_tc<false, true><<<grid, NT_THREADS_L0, NT_SMEM, st>>>(tx, tw, q);
  else
    k_nn_conv_tc<false, false><<<grid, NT_THREADS, NT_SMEM, st>>>(tx, tw, q);
  return cudaGetLastError();
}
