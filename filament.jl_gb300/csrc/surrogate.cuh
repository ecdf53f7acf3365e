// surrogate.cuh -- the learned plasma surrogate: a 4-layer 1-D convolutional
// network (3 -> 64 -> 64 -> 64 -> 1 channels, kernel 9, "same" padding, tanh
// after the first three layers) evaluated on the time row of one transverse
// point, in place of the ODE solve of plasma_equations.jl:46-72.  The density
// follows in closed form from the effective rate of every step t_j -> t_{j+1},
//   w_j = Wb_j + kappa A_j (1 - e^{-S_j}) e^{g_j},
//   rho_j = rho0 + (rho_nt - rho0) (1 - exp(-dt sum_{i<j} w_i)),
// which is exact for photoionisation with any time-dependent rate: Wb_j is
// the medium's rate averaged with the time integrator's quadrature over the
// stage points of the step, A_j the same quadrature of E^2, kappa the summed
// avalanche coefficient and S_j = dt sum_{i<j} Wb_i, so that the second term is
// the avalanche rate of the photoionised density.  The network's output g_j
// is the log of that term's amplification by the avalanche itself (the
// density history beyond photoionisation), learned from the ODE.
//
// Inputs per time point: f0 = ln(max(I, 1e-30)) / 16, f1 = Re(E)^2 / max(I, 1e-30)
// (the carrier phase, which drives the avalanche term) and
// f2 = ln(max(S_j, 1e-30)) / 16 (the density history beyond the network's
// 33-point receptive field).  Weights and hidden activations are stored in
// BF16, every product is accumulated in FP32 and the output layer is written
// in FP32; training keeps FP32 master weights (Adam).
#pragma once
#include <cuda_bf16.h>
#include "common.cuh"
#include "surrogate_consts.h"

// layer l: ci_l -> co_l
__host__ __device__ constexpr int nn_ci(int l) { return l == 0 ? NN_IN : NN_CH; }
__host__ __device__ constexpr int nn_co(int l) { return l == 3 ? 1 : NN_CH; }
// FP32 parameter offsets: weights [co][ci][k] then bias [co], layer by layer
__host__ __device__ constexpr int nn_wsize(int l) { return nn_co(l) * nn_ci(l) * NN_K; }
__host__ __device__ constexpr int nn_psize(int l) { return nn_wsize(l) + nn_co(l); }
__host__ __device__ constexpr int nn_poff(int l) { return l == 0 ? 0 : nn_poff(l - 1) + nn_psize(l - 1); }
__host__ __device__ constexpr int nn_nparams() { return nn_poff(NN_LAYERS); }

FIL_DEV float nn_ld(const __nv_bfloat16* p) { return __bfloat162float(*p); }
FIL_DEV float nn_ld(const float* p) { return *p; }
FIL_DEV void nn_st(__nv_bfloat16* p, float v) { *p = __float2bfloat16_rn(v); }
FIL_DEV void nn_st(float* p, float v) { *p = v; }

// 1-D convolution, y[b][co][t] = act(bias[co] + sum_ci,k w[ci][k][co] x[b][ci][t + k - 4]),
// x outside [0, T) is zero.  Weights in BF16, layout [ci][k][co] (the COW
// outputs of a thread are contiguous).  Block: TT time points x CO/COW
// output groups; lane = time point, so the weight loads of a warp are
// uniform.  ACT 1: tanh.  XT, YT: BF16 activations, FP32 gradients and
// output.  Rows b = blockIdx.y, blockIdx.y + gridDim.y, ... below the row
// count (*count when given, a device value, else B); `stop` (optional)
// non-zero skips the launch.
template <int CI, int CO, int TT, int COW, int ACT, typename XT, typename YT>
__global__ void __launch_bounds__(TT*(CO / COW)) k_nn_conv(const XT* __restrict__ x,
                                                             const __nv_bfloat16* __restrict__ w,
                                                             const float* __restrict__ bias, YT* y, int T, int B,
                                                             const int* count, const int* stop) {
  constexpr int W2 = TT + NN_K - 1;
  __shared__ float xs[CI][W2];
  if (stop && *stop) return;
  const int nb = count ? *count : B;
  const int t0 = blockIdx.x * TT;
  const int tid = threadIdx.x, nth = TT * (CO / COW);
  const int tl = tid % TT, cg = tid / TT;
  for (int b = blockIdx.y; b < nb; b += gridDim.y) {
    __syncthreads();   // xs free
    for (int i = tid; i < CI * W2; i += nth) {
      const int ci = i / W2, j = i - ci * W2, t = t0 + j - NN_HALF;
      xs[ci][j] = (t >= 0 && t < T) ? nn_ld(x + ((size_t)b * CI + ci) * T + t) : 0.f;
    }
    __syncthreads();
    float acc[COW];
#pragma unroll
    for (int c = 0; c < COW; ++c) acc[c] = bias ? bias[cg * COW + c] : 0.f;
    for (int ci = 0; ci < CI; ++ci) {
#pragma unroll
      for (int k = 0; k < NN_K; ++k) {
        const float xv = xs[ci][tl + k];
        const __nv_bfloat16* wr = w + ((size_t)ci * NN_K + k) * CO + cg * COW;
#pragma unroll
        for (int c = 0; c < COW; ++c) acc[c] = fmaf(__bfloat162float(wr[c]), xv, acc[c]);
      }
    }
    const int t = t0 + tl;
    if (t < T) {
#pragma unroll
      for (int c = 0; c < COW; ++c) {
        const float v = ACT ? tanhf(acc[c]) : acc[c];
        nn_st(y + ((size_t)b * CO + cg * COW + c) * T + t, v);
      }
    }
  }
}

// Weight gradient: dw[co][ci][k] += sum_b,t g[b][co][t] x[b][ci][t + k - 4],
// dbias[co] += sum g.  Block (co group of COG, ci); threads stride over
// (b, t); FP32 partial sums reduced in shared memory, one atomic per weight.
template <int CI, int CO, int COG>
__global__ void __launch_bounds__(256) k_nn_wgrad(const __nv_bfloat16* __restrict__ x,
                                                  const float* __restrict__ g, float* dw, float* dbias, int B,
                                                  int T) {
  __shared__ float red[8][COG * NN_K + COG];
  const int cg = blockIdx.x, ci = blockIdx.y;
  float a[COG][NN_K], ab[COG];
#pragma unroll
  for (int c = 0; c < COG; ++c) {
    ab[c] = 0.f;
#pragma unroll
    for (int k = 0; k < NN_K; ++k) a[c][k] = 0.f;
  }
  const long n = (long)B * T;
  for (long i = threadIdx.x; i < n; i += 256) {
    const int b = (int)(i / T), t = (int)(i - (long)b * T);
    float xv[NN_K];
#pragma unroll
    for (int k = 0; k < NN_K; ++k) {
      const int tt = t + k - NN_HALF;
      xv[k] = (tt >= 0 && tt < T) ? __bfloat162float(x[((size_t)b * CI + ci) * T + tt]) : 0.f;
    }
#pragma unroll
    for (int c = 0; c < COG; ++c) {
      const float gv = g[((size_t)b * CO + cg * COG + c) * T + t];
      ab[c] += gv;
#pragma unroll
      for (int k = 0; k < NN_K; ++k) a[c][k] = fmaf(gv, xv[k], a[c][k]);
    }
  }
  // warp sums, then one partial per warp in shared memory
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < COG; ++c) {
#pragma unroll
    for (int k = 0; k < NN_K; ++k) {
      const float v = warp_sum<float>(a[c][k]);
      if (lane == 0) red[wp][c * NN_K + k] = v;
    }
    const float v = warp_sum<float>(ab[c]);
    if (lane == 0) red[wp][COG * NN_K + c] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < COG * NN_K + COG; i += 256) {
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += red[q][i];
    if (i < COG * NN_K) {
      const int c = i / NN_K, k = i - c * NN_K;
      atomicAdd(&dw[((size_t)(cg * COG + c) * CI + ci) * NN_K + k], s);
    } else if (ci == 0) {
      atomicAdd(&dbias[cg * COG + (i - COG * NN_K)], s);
    }
  }
}

// g[i] = d[i] (1 - y[i]^2): back through tanh
__global__ void k_nn_tanh_bwd(const float* __restrict__ d, const __nv_bfloat16* __restrict__ y, float* g, long n) {
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (i < n) {
    const float v = __bfloat162float(y[i]);
    g[i] = d[i] * (1.f - v * v);
  }
}

// loss = sum m (out - tgt)^2 / sum m (m: the point weights); g = d loss / d out
__global__ void k_nn_loss(const float* __restrict__ out, const float* __restrict__ tgt,
                          const float* __restrict__ mask, float* g, float* acc, long n, float inv_count) {
  __shared__ float sm[32];
  const long i = blockIdx.x * 256L + threadIdx.x;
  float l = 0.f;
  if (i < n) {
    const float e = out[i] - tgt[i], me = mask[i] * e;
    g[i] = 2.f * me * inv_count;
    l = me * e * inv_count;
  }
  l = block_sum<float>(l, sm);
  if (threadIdx.x == 0) atomicAdd(acc, l);
}

// Adam on the FP32 master parameters, then the BF16 compute copies:
// forward layout [ci][k][co] and the flipped transpose [co][k][ci] with
// k -> 8 - k used by the input-gradient convolution.
struct NnAdam {
  float lr, b1, b2, eps, c1, c2;   // c1 = 1 - b1^t, c2 = 1 - b2^t
};
__global__ void k_nn_adam(float* p, float* m, float* v, const float* g, int n, NnAdam a) {
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float mi = a.b1 * m[i] + (1.f - a.b1) * gi, vi = a.b2 * v[i] + (1.f - a.b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= a.lr * (mi / a.c1) / (sqrtf(vi / a.c2) + a.eps);
}
// wt (optional): the tensor-core layout [k][co][ci] of the 64 -> 64 layers
__global__ void k_nn_pack(const float* __restrict__ p, __nv_bfloat16* wf, __nv_bfloat16* wb, __nv_bfloat16* wt,
                          int l) {
  const int ci_n = nn_ci(l), co_n = nn_co(l), n = co_n * ci_n * NN_K;
  const int i = blockIdx.x * 256 + threadIdx.x;
  if (i >= n) return;
  const int co = i / (ci_n * NN_K), r = i - co * ci_n * NN_K, ci = r / NN_K, k = r - ci * NN_K;
  const __nv_bfloat16 v = __float2bfloat16_rn(p[nn_poff(l) + i]);
  wf[((size_t)ci * NN_K + k) * co_n + co] = v;
  wb[((size_t)co * NN_K + (NN_K - 1 - k)) * ci_n + ci] = v;
  if (wt) wt[((size_t)k * co_n + co) * ci_n + ci] = v;
}
