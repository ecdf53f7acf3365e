// nn_tc.cu -- inference kernels of the learned plasma surrogate
// (surrogate.cuh) with channel-last activations [row][t][64]:
//
//   layer 0 (3 -> 64)   k_nn_l01_tc tcgen05 (im2col of the inputs, K = 27
//                       padded to 32), 1728 MAC per point
//   layer 1 (64 -> 64)  k_nn_l01_tc tcgen05, 36864 MAC per point
//   layer 2 (64 -> 64)  k_nn_conv_tc<true> tcgen05, 36864 MAC per point
//   layer 3 (64 -> 1)   layer 2's epilogue (nine per-tap partial sums, 576
//                       MAC per point), summed where the density is formed
//
// The 64 -> 64 convolution is an implicit GEMM per tile of 128 time points:
//   Y[t][co] = sum_k sum_ci X[t + k - 4][ci] W_k[co][ci],
// M = 128 (time points, one tensor-memory lane each), N = 64 (channels),
// K = 9 taps x 64 channels.  The halo tile X[t0 - 4 .. t0 + 131][0..63] (136
// rows of 128 B, 128-byte swizzle, K-major A) is in shared memory; the A
// operand of tap k starts k rows (k * 128 B) into it -- the swizzle is a
// function of the shared-memory address, so the shifted operand reads the
// rows as they were written.  Rows outside [0, T) are zero, the
// convolution's "same" padding.  The nine weight matrices W_k[co][ci]
// (K-major B, 72 KB) stay in shared memory for the whole launch.  Four MMAs
// of K = 16 per tap accumulate in FP32 in tensor memory; two 64-column
// accumulators alternate between tiles so that the epilogue of one tile
// (bias, tanh, BF16, 128 B store per time point) overlaps the MMAs of the
// next.  Persistent grid: one block per SM walks the tiles of all rows.
//
// k_nn_conv_tc (layer 2, and a plain layer 1): one TMA load per tile brings
// the halo tile (the copy zero-fills rows outside [0, T)).  Roles (192
// threads): warps 0-3 epilogue (warp w owns tensor-memory lanes 32w ..
// 32w+31), warp 4 TMA producer, warp 5 MMA issuer.  k_nn_l01_tc computes
// the halo tile itself from layer 0 (see there).  Every mbarrier wait is
// bounded and gives up once another role failed; a failure sets *err and
// the block releases its tensor memory after its MMAs completed.
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
  const __nv_bfloat16* x0; // k_nn_l01_tc: network inputs [rows][3][T]
  const __nv_bfloat16* w0; // k_nn_l01_tc: layer-0 weights [ci][k][co]
  const float* b0;         // k_nn_l01_tc: layer-0 bias [64]
  __nv_bfloat16* out;      // [rows][T][64] (layer 1)
  const __nv_bfloat16* w3; // layer 3 weights [ci][k] (FINAL)
  float* part;             // [rows][9][T] layer-3 partial sums (FINAL)
  int T, tiles_per_row, maxrows;
  const int* count;
  const int* stop;
  int* err;
  const int* tlist;        // the tiles to run: the first *tcount entries (NULL: every tile)
  const int* tcount;
};

// The tiles a block runs: entries blockIdx.x + i gridDim.x of the tile list
// (or of all tiles without one), i < ntl.  Every role of the block walks the
// same sequence.  Entries are clamped to the tiles of the counted rows.
struct NtTiles {
  const int* list;
  int total, ntl, last;
  __device__ NtTiles(const NtParams& p, int ntiles) {
    list = p.tlist;
    total = p.tlist ? min(*p.tcount, ntiles) : ntiles;
    ntl = (int)blockIdx.x < total ? (total - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    last = ntiles - 1;
  }
  __device__ int at(int i) const {
    const int k = (int)blockIdx.x + i * (int)gridDim.x;
    return list ? max(0, min(__ldg(&list[k]), last)) : k;
  }
};

// FINAL (layer 2): the epilogue applies layer 3 to its own point instead of
// storing the activations: P_k[t] = sum_ci w3[ci][k] y[t][ci] for the nine
// taps k (the BF16-rounded activations, as stored between layers), so that
// out[t] = b3 + sum_k P_k[t + k - 4] (nn_out_at).
template <bool FINAL>
__global__ void __launch_bounds__(NT_THREADS, 1)
    k_nn_conv_tc(const __grid_constant__ CUtensorMap tx, const __grid_constant__ CUtensorMap tw, NtParams p) {
  extern __shared__ __align__(1024) uint8_t nt_smem[];
  __shared__ volatile int s_fail;
  __shared__ __align__(16) float s_bias[64];
  // layer-3 weights as tap pairs: s_w3[(kp * 64 + ci) * 2 + u] = w3[ci][2 kp + u]
  // (kp < 5; the tenth tap is zero)
  __shared__ __align__(16) float s_w3[FINAL ? 5 * 64 * 2 : 4];
  if (p.stop && *p.stop) return;
  const int nrows = p.count ? min(*p.count, p.maxrows) : p.maxrows;
  const NtTiles tiles(p, nrows * p.tiles_per_row);
  const int ntl = tiles.ntl;
  if (ntl == 0) return;   // block-uniform, before any barrier
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
      for (; it < ntl && !s_fail; ++it) {
        const int tile = tiles.at(it);
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
        for (int lt = 0; lt < ntl && !s_fail; ++lt) {
          const int buf = lt & 1, ub = lt >> 1;
          if (ub > 0 && !nt_wait(acce_bar(buf), (ub - 1) & 1, &s_fail)) break;
          const int s = lt % NT_STAGES;
          if (!nt_wait(full_bar(s), (lt / NT_STAGES) & 1, &s_fail)) break;
          tc::tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)(buf * 64);
          // tap k: A k rows into the halo tile, W_k; 16 channels = 32 bytes per MMA
          const uint64_t da = tc::desc_k128(sbase + NT_A_OFF + s * NT_A_STRIDE), dw = tc::desc_k128(sbase + NT_W_OFF);
#pragma unroll
          for (int k = 0; k < NN_K; ++k)
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              tc::mma_f16(acc, tc::desc_add(da, 128u * k + 32u * kk), tc::desc_add(dw, k * NT_W_BYTES + 32u * kk),
                          idesc, (k | kk) ? 1u : 0u);
          tc::mma_commit(empty_bar(s));
          tc::mma_commit(accf_bar(buf));
        }
      }
      // no MMA may still write tensor memory when it is released
      tc::mma_commit(done_bar);
      tc::mbar_wait(done_bar, 0, NT_WAIT_LIMIT);
    }
  } else if (warp < 4) {
    // ---------------- epilogue: warp w owns time points 32w .. 32w+31 of the tile
    for (int lt = 0; lt < ntl; ++lt) {
      const int tile = tiles.at(lt);
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


// ---------------------------------------------------------------------------
// Layers 0 and 1, both on the tensor cores (the network's first launch).
// Per tile of 128 time points t0 .. t0 + 127 of a row:
//   im2col (warps 14-17): A0[r][kk] = x[ci][t0 - 8 + r + k] for kk = 9 ci + k
//     < 27 (zero for kk = 27 .. 31 and for times outside [0, T), layer 0's
//     "same" padding), r = 0 .. 135 the 136 halo rows of layer 1; BF16 rows of
//     128 B in the 128-byte swizzle (only the first 64 bytes are read), two
//     buffers.  Each warp stages the tile's input window x[ci][t0 - 8 ..
//     t0 + 135] in its own shared slice and writes 34 rows.
//   MMA (warp 5): layer 0 as two M = 128, N = 64, K = 32 products, rows 0 ..
//     127 and 8 .. 135 of A0 (1024 bytes in, a whole swizzle atom), against
//     W0[co][kk] (shared memory, written once) into a tensor-memory pair; the
//     layer-0 products of tile i + 1 are issued before layer 1's of tile i.
//     Layer 1 as in k_nn_conv_tc: nine taps, each a 128-byte row shift into
//     the halo tile.
//   layer-0 epilogue (warps 6-13, two per tensor-memory lane quadrant q, one
//     per half of the channels): bias, tanh, BF16 of row r = lane + 32 q (the
//     quadrant-3 warps also rows 128 .. 135 from the second product's lanes
//     120 .. 127), zero where t0 - 4 + r is outside [0, T) (layer 1's
//     padding), written into the layer-1 stage in the 128-byte swizzle; proxy
//     fence; arrive on the stage's barrier.
//   layer-1 epilogue (warps 0-3) and the layer-1 weights (warp 4): as in
//   k_nn_conv_tc.
// Every wait is bounded and gives up once another role failed.
#define L1_STAGES 5
#define L01_WARPS 18
#define L01_THREADS (32 * L01_WARPS)
#define L01_A0_BYTES (NT_HALO * 128)                         // 17408, a multiple of 1024
#define L01_A_OFF (NN_K * NT_W_BYTES)                         // layer-1 stages
#define L01_A0_OFF (L01_A_OFF + L1_STAGES * NT_A_STRIDE)      // two im2col buffers
#define L01_W0_OFF (L01_A0_OFF + 2 * L01_A0_BYTES)            // W0 [64][128 B]
#define L01_XW_OFF (L01_W0_OFF + 64 * 128)                    // 4 warps x 3 x 144 BF16 windows
#define L01_XW 144                                            // window points per channel
#define L01_BAR_OFF (L01_XW_OFF + 4096)
#define L01_SMEM (L01_BAR_OFF + 256 + 1024)
// barriers, 8 bytes each: full[S] empty[S] accf[2] acce[2] a0f[2] c0f[2] c0e[2] wbar done, then the slot
#define L01_FULL(s) (8u * (s))
#define L01_EMPTY(s) (8u * (L1_STAGES + (s)))
#define L01_ACCF(b) (8u * (2 * L1_STAGES + (b)))
#define L01_ACCE(b) (8u * (2 * L1_STAGES + 2 + (b)))
#define L01_A0F(b) (8u * (2 * L1_STAGES + 4 + (b)))
#define L01_C0F(b) (8u * (2 * L1_STAGES + 6 + (b)))
#define L01_C0E(b) (8u * (2 * L1_STAGES + 8 + (b)))
#define L01_WBAR (8u * (2 * L1_STAGES + 10))
#define L01_DONE (8u * (2 * L1_STAGES + 11))
#define L01_SLOT (8u * (2 * L1_STAGES + 12))
static_assert(L01_SLOT + 4 <= 256, "barrier block overflows its reserved bytes");
static_assert(L01_A0_BYTES % 1024 == 0 && L01_A0_OFF % 1024 == 0 && L01_W0_OFF % 1024 == 0, "swizzle atoms");
static_assert(4 * 3 * L01_XW * 2 <= 4096, "input windows");
static_assert(L01_SMEM + 1024 <= 232448, "shared memory of one block (with static)");
static_assert(NT_HALO == 4 * 34, "four im2col warps of 34 rows");

__global__ void __launch_bounds__(L01_THREADS, 1)
    k_nn_l01_tc(const __grid_constant__ CUtensorMap tw, NtParams p) {
  extern __shared__ __align__(1024) uint8_t nt_smem[];
  __shared__ volatile int s_fail;
  __shared__ __align__(16) float s_bias[64];    // layer 1
  __shared__ __align__(16) float s_b0[64];      // layer 0
  if (p.stop && *p.stop) return;
  const int nrows = p.count ? min(*p.count, p.maxrows) : p.maxrows;
  const NtTiles tiles(p, nrows * p.tiles_per_row);
  const int ntl = tiles.ntl;
  if (ntl == 0) return;   // block-uniform, before any barrier
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t raw = tc::smem_u32(nt_smem);
  const uint32_t sbase = (raw + 1023u) & ~1023u;
  uint8_t* gbase = nt_smem + (sbase - raw);
  const uint32_t bars = sbase + L01_BAR_OFF;
  auto full_bar = [&](int s) { return bars + L01_FULL(s); };
  auto empty_bar = [&](int s) { return bars + L01_EMPTY(s); };
  auto accf_bar = [&](int b) { return bars + L01_ACCF(b); };
  auto acce_bar = [&](int b) { return bars + L01_ACCE(b); };
  auto a0f_bar = [&](int b) { return bars + L01_A0F(b); };
  auto c0f_bar = [&](int b) { return bars + L01_C0F(b); };
  auto c0e_bar = [&](int b) { return bars + L01_C0E(b); };
  const uint32_t wbar = bars + L01_WBAR, done_bar = bars + L01_DONE, tmem_slot = bars + L01_SLOT;
  volatile uint32_t* tmem_slot_g = reinterpret_cast<volatile uint32_t*>(gbase + L01_BAR_OFF + L01_SLOT);

  if (tid == 0) s_fail = 0;
  if (tid < 64) {
    s_bias[tid] = p.bias[tid];
    s_b0[tid] = p.b0[tid];
  }
  // W0[co][kk] = w0[ci][k][co] for kk = 9 ci + k < 27, zero up to kk = 63; row
  // co of 128 B, 16-byte chunk j at j ^ (co & 7)
  for (int i = tid; i < 64 * 32; i += L01_THREADS) {
    const int co = i >> 5, pr = i & 31, kk = 2 * pr;
    auto w = [&](int q) -> __nv_bfloat16 {
      return q < NN_IN * NN_K ? p.w0[(size_t)q * 64 + co] : __float2bfloat16_rn(0.f);
    };
    __nv_bfloat162 v;
    v.x = w(kk);
    v.y = w(kk + 1);
    *reinterpret_cast<__nv_bfloat162*>(gbase + L01_W0_OFF + co * 128 + (((pr >> 2) ^ (co & 7)) << 4) + ((pr & 3) << 2)) = v;
  }
  tc::fence_proxy_async_smem();   // W0 for the tensor core
  if (warp == 0) tc::tmem_alloc(tmem_slot, 512);
  if (tid == 0) {
    for (int s = 0; s < L1_STAGES; ++s) {
      tc::mbar_init(full_bar(s), 256);
      tc::mbar_init(empty_bar(s), 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(accf_bar(b), 1);
      tc::mbar_init(acce_bar(b), 4);
      tc::mbar_init(a0f_bar(b), 128);
      tc::mbar_init(c0f_bar(b), 1);
      tc::mbar_init(c0e_bar(b), 8);
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
  auto tile_of = [&](int tile, int* b, int* t0) {
    *b = tile / tpr;
    *t0 = (tile - *b * tpr) * NT_BM;
  };

  if (warp == 4) {
    // ---------------- layer-1 weights once (TMA); waited for before exit
    if (lane == 0) {
      tc::mbar_expect_tx(wbar, NN_K * NT_W_BYTES);
      for (int k = 0; k < NN_K; ++k) tc::tma_load_2d(sbase + k * NT_W_BYTES, &tw, 0, 64 * k, wbar);
      nt_wait(wbar, 0, &s_fail);
    }
  } else if (warp == 5) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = tc::idesc_bf16(NT_BM, 64);
      auto layer0 = [&](int i) -> bool {
        const int b = i & 1, u = i >> 1;
        if (!nt_wait(a0f_bar(b), u & 1, &s_fail)) return false;            // im2col of tile i
        if (u > 0 && !nt_wait(c0e_bar(b), (u - 1) & 1, &s_fail)) return false;   // acc0[b] drained
        tc::tc_fence_after();
        const uint64_t da = tc::desc_k128(sbase + L01_A0_OFF + b * L01_A0_BYTES), dw = tc::desc_k128(sbase + L01_W0_OFF);
        const uint32_t acc = tmem + 128u + 128u * b;
#pragma unroll
        for (int h = 0; h < 2; ++h)          // rows 0 .. 127, rows 8 .. 135
#pragma unroll
          for (int kk = 0; kk < 2; ++kk)     // K = 32 in two steps of 16
            tc::mma_f16(acc + 64u * h, tc::desc_add(da, 1024u * h + 32u * kk), tc::desc_add(dw, 32u * kk), idesc,
                        kk ? 1u : 0u);
        tc::mma_commit(c0f_bar(b));
        return true;
      };
      if (nt_wait(wbar, 0, &s_fail) && (ntl == 0 || layer0(0))) {
        for (int i = 0; i < ntl && !s_fail; ++i) {
          if (i + 1 < ntl && !layer0(i + 1)) break;
          const int buf = i & 1, ub = i >> 1;
          if (ub > 0 && !nt_wait(acce_bar(buf), (ub - 1) & 1, &s_fail)) break;
          const int s = i % L1_STAGES;
          if (!nt_wait(full_bar(s), (i / L1_STAGES) & 1, &s_fail)) break;
          tc::tc_fence_after();
          const uint32_t acc = tmem + (uint32_t)(buf * 64);
          const uint64_t da = tc::desc_k128(sbase + L01_A_OFF + s * NT_A_STRIDE), dw = tc::desc_k128(sbase);
#pragma unroll
          for (int k = 0; k < NN_K; ++k)
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
              tc::mma_f16(acc, tc::desc_add(da, 128u * k + 32u * kk), tc::desc_add(dw, k * NT_W_BYTES + 32u * kk),
                          idesc, (k | kk) ? 1u : 0u);
          tc::mma_commit(empty_bar(s));
          tc::mma_commit(accf_bar(buf));
        }
      }
      // no MMA may still write tensor memory when it is released
      tc::mma_commit(done_bar);
      tc::mbar_wait(done_bar, 0, NT_WAIT_LIMIT);
    }
  } else if (warp >= 14) {
    // ---------------- im2col of layer 0's input.  Lane l writes the BF16
    // pair kk = 2 (l mod 16), + 1 (fixed channel and tap offsets) of the rows
    // 34 w + (l / 16) + 2 m of its warp's 34; the next tile's window is
    // loaded into registers while this tile's rows are written.
    const int w = warp - 14;
    uint16_t* xw = reinterpret_cast<uint16_t*>(gbase + L01_XW_OFF) + w * NN_IN * L01_XW;
    const uint16_t* x0 = reinterpret_cast<const uint16_t*>(p.x0);
    const int pr = lane & 15, r1 = lane >> 4;
    const int kk0 = 2 * pr, kk1 = kk0 + 1;
    const bool v0 = kk0 < NN_IN * NN_K, v1 = kk1 < NN_IN * NN_K;
    const int o0 = v0 ? (kk0 / NN_K) * L01_XW + kk0 % NN_K : 0;
    const int o1 = v1 ? (kk1 / NN_K) * L01_XW + kk1 % NN_K : 0;
    constexpr int XM = (L01_XW + 31) / 32;
    uint16_t nx[NN_IN][XM];
    auto load_window = [&](int tile) {
      int row, t0;
      tile_of(tile, &row, &t0);
      const uint16_t* xr = x0 + (size_t)row * NN_IN * p.T;
#pragma unroll
      for (int ci = 0; ci < NN_IN; ++ci)
#pragma unroll
        for (int m = 0; m < XM; ++m) {
          const int j = lane + 32 * m, t = t0 - 2 * NN_HALF + j;
          nx[ci][m] = (j < L01_XW && t >= 0 && t < p.T) ? xr[(size_t)ci * p.T + t] : (uint16_t)0;
        }
    };
    load_window(tiles.at(0));
    for (int i = 0; i < ntl; ++i) {
      const int b = i & 1, u = i >> 1;
      int ok = 1;
      if (lane == 0) ok = !s_fail && (u == 0 || nt_wait(c0f_bar(b), (u - 1) & 1, &s_fail));   // A0[b] free
      if (!__shfl_sync(0xffffffffu, ok, 0)) break;
#pragma unroll
      for (int ci = 0; ci < NN_IN; ++ci)
#pragma unroll
        for (int m = 0; m < XM; ++m)
          if (lane + 32 * m < L01_XW) xw[ci * L01_XW + lane + 32 * m] = nx[ci][m];
      __syncwarp();
      if (i + 1 < ntl) load_window(tiles.at(i + 1));   // in flight while the rows are written
      uint8_t* a0 = gbase + L01_A0_OFF + b * L01_A0_BYTES;
#pragma unroll
      for (int m = 0; m < 17; ++m) {
        const int r = 34 * w + r1 + 2 * m;
        const uint32_t lo = v0 ? (uint32_t)xw[o0 + r] : 0u, hi = v1 ? (uint32_t)xw[o1 + r] : 0u;
        *reinterpret_cast<uint32_t*>(a0 + r * 128 + (((pr >> 2) ^ (r & 7)) << 4) + ((pr & 3) << 2)) = lo | (hi << 16);
      }
      __syncwarp();                   // xw free for the next tile
      tc::fence_proxy_async_smem();
      nt_arrive(a0f_bar(b));
    }
  } else if (warp >= 6) {
    // ---------------- layer-0 epilogue into the layer-1 stages: warps
    // 6-13, two per tensor-memory lane quadrant q, warp half h taking the
    // channels 32 h .. 32 h + 31 (16-byte chunks 4 h .. 4 h + 3 of a row)
    const int q = warp & 3, h = (warp - 6) >> 2;
    // 32 layer-0 outputs of one row (accumulator columns of this warp's
    // half) -> row r of stage st, 16-byte chunk j at j ^ (r & 7)
    auto put_row = [&](uint8_t* st, int r, int tau, const uint32_t (&v)[32]) {
      const bool in = tau >= 0 && tau < p.T;
      const float4* bv = reinterpret_cast<const float4*>(s_b0 + 32 * h);
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        uint32_t pk[4] = {0u, 0u, 0u, 0u};
        if (in) {
          const float4 b0 = bv[2 * j], b1 = bv[2 * j + 1];
          const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int c = 8 * j + 2 * e;
            const __nv_bfloat162 hv = __floats2bfloat162_rn(nt_tanh(__uint_as_float(v[c]) + bb[2 * e]),
                                                            nt_tanh(__uint_as_float(v[c + 1]) + bb[2 * e + 1]));
            pk[e] = *reinterpret_cast<const uint32_t*>(&hv);
          }
        }
        *reinterpret_cast<uint4*>(st + r * 128 + (((4 * h + j) ^ (r & 7)) << 4)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    };
    for (int i = 0; i < ntl; ++i) {
      const int b = i & 1, u = i >> 1;
      const int cur = tiles.at(i);
      if (!nt_wait(c0f_bar(b), u & 1, &s_fail)) break;
      tc::tc_fence_after();
      int row, t0;
      tile_of(cur, &row, &t0);
      (void)row;
      const uint32_t taddr = tmem + ((uint32_t)(32 * q) << 16) + 128u + 128u * b + 32u * h;
      uint32_t v[32];
      tc::tmem_ld32_async(taddr, v);
      tc::tmem_wait_ld(v);
      const int s = i % L1_STAGES, use = i / L1_STAGES;
      if (use > 0 && !nt_wait(empty_bar(s), (use - 1) & 1, &s_fail)) break;
      uint8_t* st = gbase + L01_A_OFF + s * NT_A_STRIDE;
      const int r = 32 * q + lane;
      put_row(st, r, t0 - NN_HALF + r, v);
      if (q == 3) {
        // rows 128 .. 135: the second product's rows 8 + l, lanes l = 120 .. 127
        tc::tmem_ld32_async(taddr + 64u, v);
        tc::tmem_wait_ld(v);
        if (lane >= 24) put_row(st, 104 + lane, t0 - NN_HALF + 104 + lane, v);
      }
      tc::tc_fence_before();
      __syncwarp();
      if (lane == 0) nt_arrive(c0e_bar(b));
      tc::fence_proxy_async_smem();   // this lane's writes, for the MMAs
      nt_arrive(full_bar(s));
    }
  } else {
    // ---------------- layer-1 epilogue: warp w owns time points 32w .. 32w+31 of the tile
    for (int i = 0; i < ntl; ++i) {
      const int buf = i & 1;
      const int cur = tiles.at(i);
      if (!nt_wait(accf_bar(buf), (i >> 1) & 1, &s_fail)) break;
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
      int row, t0;
      tile_of(cur, &row, &t0);
      const int t = t0 + 32 * warp + lane;
      if (t < p.T) {
        uint4* dst = reinterpret_cast<uint4*>(p.out + ((size_t)row * p.T + t) * 64);
        const float4* bv = reinterpret_cast<const float4*>(s_bias);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          const float4 b0 = bv[2 * j], b1 = bv[2 * j + 1];
          const float bb[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
          uint32_t pk[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const int c = 8 * j + 2 * e;
            const float v0 = __uint_as_float(c < 32 ? r0[c] : r1[c - 32]) + bb[2 * e];
            const float v1 = __uint_as_float(c + 1 < 32 ? r0[c + 1] : r1[c + 1 - 32]) + bb[2 * e + 1];
            const __nv_bfloat162 h = __floats2bfloat162_rn(nt_tanh(v0), nt_tanh(v1));
            pk[e] = *reinterpret_cast<const uint32_t*>(&h);
          }
          dst[j] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
        }
      }
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc::tc_fence_after();
    tc::tmem_dealloc(tmem, 512);
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
  if (x0 && part) return cudaErrorInvalidValue;   // layer 0 is fused into layer 1 only
  // the launched kernel's shared-memory limit, set on every launch (a host
  // call, legal under stream capture): the attribute belongs to the current
  // device's context
  cudaError_t e;
  if (part)
    e = cudaFuncSetAttribute(k_nn_conv_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, NT_SMEM);
  else if (x0)
    e = cudaFuncSetAttribute(k_nn_l01_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, L01_SMEM);
  else
    e = cudaFuncSetAttribute(k_nn_conv_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, NT_SMEM);
  if (e != cudaSuccess) return e;
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
  q.tlist = p.tlist;
  q.tcount = p.tcount;
  const int tiles = p.maxrows * q.tiles_per_row;
  const int grid = std::max(1, std::min(p.sms, tiles));
  if (part)
    k_nn_conv_tc<true><<<grid, NT_THREADS, NT_SMEM, st>>>(tx, tw, q);
  else if (x0)
    k_nn_l01_tc<<<grid, L01_THREADS, L01_SMEM, st>>>(tw, q);
  else
    k_nn_conv_tc<false><<<grid, NT_THREADS, NT_SMEM, st>>>(tx, tw, q);
  return cudaGetLastError();
}
