// xyfft.cu -- the transverse 2-D transform of the XYT linear step:
// E <- ifft2(exp(i KZ(kx, ky, w) dz) * guards * fft2(E)) on every frequency
// column of the half spectrum.
//
// Reference: src/modules/linear_propagators/spectral.jl:104-156 (XY/XYT
// propagator: PS = plan_fft over dims (1, 2), KZ from
// sqrt(beta^2 - kx^2 - ky^2) in the moving frame) with the spectral guards of
// Guards.jl:162-193, 218-262.
//
// The field is S[p][k], p = ix * Ny + iy, k < Nt/2 contiguous.  A transform
// along one transverse axis is a batch of 1-D FFTs along a strided line; a
// block takes KT consecutive frequency columns of one line group, so that
// every row of the tile it loads is KT contiguous complex values.  Three
// launches per step:
//   y pass   : fft along y                     (lines p = ix*Ny + iy, stride Nt/2)
//   x pass   : fft along x, propagator, ifft   (stride Ny*Nt/2; the k-space
//              point (kx, ky) of every element is known here)
//   y pass   : ifft along y, scaled by 1/(Nx Ny), into the state
#include "launch.h"
#include "rowkernels.cuh"
#include "dht_simt.cuh"
#include "xyfft.h"

// KT frequency columns per block: KT * NL / 16 threads, KT * NL complex in
// shared memory (69.6 KB for both precisions).
template <typename R, int NL> constexpr int xy_kt() {
  constexpr int cap = (sizeof(R) == 4 ? 8192 : 4096) / NL;
  return cap >= 16 ? 16 : cap;
}

// MODE 0: forward transform.  MODE 1: forward, propagator, inverse (x pass).
// MODE 2: inverse transform into `out`, marks the field guard pending.
template <typename R, int NL, int MODE>
__global__ void __launch_bounds__(xy_kt<R, NL>() * (NL / 16)) k_xylines(XyParams<R> p) {
  typedef typename C2T<R>::type C;
  constexpr int KT = xy_kt<R, NL>();
  constexpr int T = NL / 16, NP = NL + NL / 16, NTH = KT * T;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* tile = reinterpret_cast<C*>(smem_raw);
  if (p.ctl && p.ctl->done) return;
  const int tid = threadIdx.x;
  const int k0 = blockIdx.x * KT;
  const int o = blockIdx.y;
  const size_t base = (size_t)o * p.outer_stride + k0;
#pragma unroll 4
  for (int i = tid; i < NL * KT; i += NTH) {
    const int l = i / KT, c = i - l * KT;
    tile[c * NP + pad16(l)] = p.in[base + (size_t)l * p.line_stride + c];
  }
  const int g = tid / T, gt = tid - g * T;
  C* s = tile + g * NP;
  if (MODE == 2) {
    filfft::group_fft<C, NL, +1>(s, p.tw, gt);
  } else {
    filfft::group_fft<C, NL, -1>(s, p.tw, gt);
  }
  if (MODE == 1) {
    // element (l = ix, column k0 + g) of outer line o = iy
    const int k = k0 + g;
    const R ky2 = p.kt2_outer[o], sgo = p.sg_outer[o];
    const R dz = p.ctl ? (R)p.ctl->dz : p.dz_fixed;
    PropParams<R> pp = p.pp;
    R wgk = (R)1;
    if (p.wg) wgk = p.wg[p.wg_bug ? o : k];
    pp.wg = nullptr;
    for (int l = gt; l < NL; l += T) {
      C f = propagator<R>(pp, p.kt2_line[l] + ky2, k, dz);
      const R gg = p.sg_line[l] * sgo * wgk;
      s[pad16(l)] = cmul(s[pad16(l)], mk<R>(gg * f.x, gg * f.y));
    }
    filfft::group_fft<C, NL, +1>(s, p.tw, gt);
  }
  __syncthreads();
#pragma unroll 4
  for (int i = tid; i < NL * KT; i += NTH) {
    const int l = i / KT, c = i - l * KT;
    p.out[base + (size_t)l * p.line_stride + c] = p.scale * tile[c * NP + pad16(l)];
  }
  if (MODE == 2 && p.ctl && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) p.ctl->guard_pending = 1;
}

template <typename R, int NL>
static cudaError_t launch_xy_n(const XyParams<R>& p, int mode, int nh, int nouter, cudaStream_t st) {
  typedef typename C2T<R>::type C;
  constexpr int KT = xy_kt<R, NL>();
  if (nh % KT) return cudaErrorInvalidValue;
  const size_t sm = (size_t)KT * (NL + NL / 16) * sizeof(C);
  dim3 grid(nh / KT, nouter);
  cudaError_t e = cudaSuccess;
  if (mode == 0) {
    e = cudaFuncSetAttribute(k_xylines<R, NL, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) k_xylines<R, NL, 0><<<grid, KT * (NL / 16), sm, st>>>(p);
  } else if (mode == 1) {
    e = cudaFuncSetAttribute(k_xylines<R, NL, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) k_xylines<R, NL, 1><<<grid, KT * (NL / 16), sm, st>>>(p);
  } else {
    e = cudaFuncSetAttribute(k_xylines<R, NL, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e == cudaSuccess) k_xylines<R, NL, 2><<<grid, KT * (NL / 16), sm, st>>>(p);
  }
  if (e != cudaSuccess) return e;
  return cudaGetLastError();
}

template <typename R>
cudaError_t launch_xylines(const XyParams<R>& p, int nl, int mode, int nh, int nouter, cudaStream_t st) {
  switch (nl) {
    case 64: return launch_xy_n<R, 64>(p, mode, nh, nouter, st);
    case 128: return launch_xy_n<R, 128>(p, mode, nh, nouter, st);
    case 256: return launch_xy_n<R, 256>(p, mode, nh, nouter, st);
    case 512: return launch_xy_n<R, 512>(p, mode, nh, nouter, st);
    case 1024: return launch_xy_n<R, 1024>(p, mode, nh, nouter, st);
  }
  return cudaErrorInvalidValue;
}

template cudaError_t launch_xylines<float>(const XyParams<float>&, int, int, int, int, cudaStream_t);
template cudaError_t launch_xylines<double>(const XyParams<double>&, int, int, int, int, cudaStream_t);
