// dht_vec.cu -- the linear step of the R geometry (no time axis):
// E <- g_r * M2 (P * (M1 E)) on one complex column E(r), as two
// matrix-vector products with the Hankel pair M1 = T diag(s),
// M2 = diag(1/s) T and P = exp(i KZ(k, w0) dz) * Kguard(k).
//
// Reference: src/modules/linear_propagators/spectral.jl:16-26 (PS * E;
// E .*= exp(i KZ dz); spectral guard; PS \ E) with the R tables of
// spectral.jl:28-52 and Guards.jl:41-58; the field guard that ends the step
// (Models.jl:116-118) is applied on the inverse product's store.
#include "launch.h"
#include "dht_simt.cuh"

// One warp per output row i: out[i] = sum_k M[i][k] in[k] (the lanes stride
// over k, then a warp sum), then mode 1: times the propagator of row i
// (transverse wave number kt2[i], the one frequency w0); mode 2: times the
// field guard g_row[i].
template <typename R>
__global__ void __launch_bounds__(256) k_dht_vec(const R* __restrict__ M, const typename C2T<R>::type* __restrict__ in,
                                                 typename C2T<R>::type* __restrict__ out, int n, int ldm,
                                                 PropParams<R> pp, const R* __restrict__ g_row, DevCtl* ctl,
                                                 int mode) {
  typedef typename C2T<R>::type C;
  if (ctl->done) return;
  const int lane = threadIdx.x & 31;
  const int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= n) return;
  const R* mi = M + (size_t)i * ldm;
  R ar = 0, ai = 0;
  for (int k = lane; k < n; k += 32) {
    const R m = mi[k];
    const C v = in[k];
    ar = fma(m, v.x, ar);
    ai = fma(m, v.y, ai);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ar += __shfl_xor_sync(0xffffffffu, ar, o);
    ai += __shfl_xor_sync(0xffffffffu, ai, o);
  }
  if (lane) return;
  C v = mk<R>(ar, ai);
  if (mode == 1) v = cmul(v, propagator<R>(pp, pp.kt2[i], 0, (R)ctl->dz));
  else v = g_row[i] * v;
  out[i] = v;
}

template <typename R>
cudaError_t launch_dht_vec(const R* M, const typename C2T<R>::type* in, typename C2T<R>::type* out, int n, int ldm,
                           const PropParams<R>& pp, const R* g_row, DevCtl* ctl, int mode, cudaStream_t st) {
  k_dht_vec<R><<<(n + 7) / 8, 256, 0, st>>>(M, in, out, n, ldm, pp, g_row, ctl, mode);
  return cudaGetLastError();
}

template cudaError_t launch_dht_vec<float>(const float*, const float2*, float2*, int, int, const PropParams<float>&,
                                           const float*, DevCtl*, int, cudaStream_t);
template cudaError_t launch_dht_vec<double>(const double*, const double2*, double2*, int, int,
                                            const PropParams<double>&, const double*, DevCtl*, int, cudaStream_t);
