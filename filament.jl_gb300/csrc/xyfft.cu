// xyfft.cu -- the transverse 2-D transform of the XYT linear step:
// E <- ifft2(exp(i KZ(kx, ky, w) dz) * guards * fft2(E)) on every frequency
// column (both halves of the spectrum, as the reference's plan over the
// full array; only the analytic half with the projection option).
//
// Reference: src/modules/linear_propagators/spectral.jl:104-156 (XY/XYT
// propagator: PS = plan_fft over dims (1, 2), KZ from
// sqrt(beta^2 - kx^2 - ky^2) in the moving frame) with the spectral guards of
// Guards.jl:162-193, 218-262.
//
// The field is S[p][k], p = ix * Ny + iy, k < Nt contiguous.  A transform
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
// MODE 2: inverse transform into `out`, marks the field guard pending (XYT).
// MODE 3: inverse transform into `out` times the field guard g1[ix] g2[iy]
// (XY, whose step ends with the guard, Models.jl:116-118).
template <typename R, int NL, int KT, int MODE>
__global__ void __launch_bounds__(KT * (NL / 16)) k_xylines(XyParams<R> p) {
  typedef typename C2T<R>::type C;
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
  if (MODE >= 2) {
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
    const C cph = colphase<R>(p.kcol[k], p.ctl ? p.ctl->dz : (double)p.dz_fixed);
    for (int l = gt; l < NL; l += T) {
      C f = propagator_cd<R>(pp, p.kt2_line[l] + ky2, k, dz, cph);
      const R gg = p.sg_line[l] * sgo * wgk;
      s[pad16(l)] = cmul(s[pad16(l)], mk<R>(gg * f.x, gg * f.y));
    }
    filfft::group_fft<C, NL, +1>(s, p.tw, gt);
  }
  __syncthreads();
#pragma unroll 4
  for (int i = tid; i < NL * KT; i += NTH) {
    const int l = i / KT, c = i - l * KT;
    R sc = p.scale;
    if (MODE == 3) sc *= p.g_outer[o] * p.g_line[l];
    p.out[base + (size_t)l * p.line_stride + c] = sc * tile[c * NP + pad16(l)];
  }
  if (MODE == 2 && p.ctl && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) p.ctl->guard_pending = 1;
}

template <typename R, int NL, int KT, int MODE>
static cudaError_t launch_xy_k(const XyParams<R>& p, int nh, int nouter, cudaStream_t st) {
  typedef typename C2T<R>::type C;
  const size_t sm = (size_t)KT * (NL + NL / 16) * sizeof(C);
  cudaError_t e = cudaFuncSetAttribute(k_xylines<R, NL, KT, MODE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  dim3 grid(nh / KT, nouter);
  k_xylines<R, NL, KT, MODE><<<grid, KT * (NL / 16), sm, st>>>(p);
  return cudaGetLastError();
}

// XYT: KT frequency columns per block (nh a multiple of KT); XY (nh = 1):
// one column, modes 0, 1 and 3
template <typename R, int NL>
static cudaError_t launch_xy_n(const XyParams<R>& p, int mode, int nh, int nouter, cudaStream_t st) {
  constexpr int KT = xy_kt<R, NL>();
  if (nh == 1) {
    if (mode == 0) return launch_xy_k<R, NL, 1, 0>(p, nh, nouter, st);
    if (mode == 1) return launch_xy_k<R, NL, 1, 1>(p, nh, nouter, st);
    if (mode == 3) return launch_xy_k<R, NL, 1, 3>(p, nh, nouter, st);
    return cudaErrorInvalidValue;
  }
  if constexpr (NL <= 1024) {
    if (nh % KT) return cudaErrorInvalidValue;
    if (mode == 0) return launch_xy_k<R, NL, KT, 0>(p, nh, nouter, st);
    if (mode == 1) return launch_xy_k<R, NL, KT, 1>(p, nh, nouter, st);
    if (mode == 2) return launch_xy_k<R, NL, KT, 2>(p, nh, nouter, st);
  }
  return cudaErrorInvalidValue;
}

template <typename R>
cudaError_t launch_xylines(const XyParams<R>& p, int nl, int mode, int nh, int nouter, cudaStream_t st) {
  switch (nl) {
    case 64: return launch_xy_n<R, 64>(p, mode, nh, nouter, st);
    case 128: return launch_xy_n<R, 128>(p, mode, nh, nouter, st);
    case 256: return launch_xy_n<R, 256>(p, mode, nh, nouter, st);
    case 512: return launch_xy_n<R, 512>(p, mode, nh, nouter, st);
    case 1024: return launch_xy_n<R, 1024>(p, mode, nh, nouter, st);
    case 2048: return launch_xy_n<R, 2048>(p, mode, nh, nouter, st);
    case 4096: return launch_xy_n<R, 4096>(p, mode, nh, nouter, st);
  }
  return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// XY geometry (no time axis): the state is E(x, y) itself.
// Nonlinear step (nonlinear_propagators.jl:38-74 with cubic.jl:49-54,
// F = 3/4 |E|^2 E): dE/dz = C0 * g(x, y) * F(E), C0 = i QZ(w0) Rnl(w0), an
// explicit RK step per point; writes the result into `out`.  With the
// adaptive Tsitouras pair each point chooses its own substeps (its error
// norm is |e| / (atol + rtol max(|y0|, |y1|))).  Also the R geometry (one
// column, ny = 1).
template <typename R>
__global__ void __launch_bounds__(256) k_xy_nonlinear(const typename C2T<R>::type* in, typename C2T<R>::type* out,
                                                      XyNlParams<R> p) {
  typedef typename C2T<R>::type C;
  const long i = blockIdx.x * 256L + threadIdx.x;
  if (p.ctl && p.ctl->done) return;
  const bool live = i < p.n;
  const R dz = p.ctl ? (R)p.ctl->dz : p.dz_fixed;
  const long ii = live ? i : 0;
  const int ix = (int)(ii / p.ny), iy = (int)(ii - (long)ix * p.ny);
  const R g = p.g1[ix] * p.g2[iy];
  auto rhs = [&](C u) -> C {
    const R f = g * (R)0.75 * (u.x * u.x + u.y * u.y);
    return cmul(p.c0, mk<R>(f * u.x, f * u.y));
  };
  C y = in[ii];
  C k[7];
  if (p.tsit != 2) {
    C acc = mk<R>(0, 0);
#pragma unroll
    for (int s = 0; s < 7; ++s) {
      if (s < p.ns) {
        C u = y;
#pragma unroll
        for (int l = 0; l < s; ++l) u = u + (dz * p.a[s][l]) * k[l];
        k[s] = rhs(u);
        acc = acc + p.b[s] * k[s];
      }
    }
    if (live) out[i] = y + dz * acc;
    return;
  }
  OdeStep o;
  ode_begin(o, p.ctl ? p.ctl->dz : (double)p.dz_fixed);
  const double dzd = o.h;
  unsigned rejects = 0;
  int fin = 0;
  k[0] = rhs(y);
  while (live) {
    const R h = (R)o.h;
    C acc = mk<R>(0, 0);
#pragma unroll
    for (int s = 1; s < 7; ++s) {
      acc = acc + p.b[s - 1] * k[s - 1];
      C u = y;
      if (s < 6) {
#pragma unroll
        for (int l = 0; l < s; ++l) u = u + (h * p.a[s][l]) * k[l];
      } else {
        u = u + h * acc;
      }
      k[s] = rhs(u);
    }
    C e = mk<R>(0, 0);
#pragma unroll
    for (int j = 0; j < 7; ++j) e = e + p.bt[j] * k[j];
    e = h * e;
    const C y1 = y + h * acc;
    const double sc = p.atol + p.rtol * fmax(sqrt((double)cabs2(y)), sqrt((double)cabs2(y1)));
    const int ok = ode_after(o, sqrt((double)cabs2(e)) / sc, dzd, &fin);
    if (ok) {
      y = y1;
      k[0] = k[6];
    } else {
      ++rejects;
    }
    if (fin) break;
  }
  if (live) out[i] = y;
  // counts: one atomic per warp
  unsigned long long na = live ? (unsigned long long)o.attempts : 0ull, nr = rejects;
#pragma unroll
  for (int d = 16; d > 0; d >>= 1) {
    na += __shfl_xor_sync(0xffffffffu, na, d);
    nr += __shfl_xor_sync(0xffffffffu, nr, d);
  }
  const unsigned gave_up = __ballot_sync(0xffffffffu, fin == 2);
  if ((threadIdx.x & 31) == 0 && p.ctl) {
    atomicAdd(&p.ctl->ode_attempts, na);
    atomicAdd(&p.ctl->ode_rejects, nr);
    if (gave_up) atomicOr(&p.ctl->flags, FIL_FLAG_ODE);
  }
}

// Reductions of the XY field (FieldAnalyzers.jl:240-255): F = |E|^2 per
// point, Imax.
template <typename R>
__global__ void __launch_bounds__(256) k_xy_reduce(const typename C2T<R>::type* E, double* fluence, DevCtl* ctl,
                                                   long n, int check_done) {
  typedef typename C2T<R>::type C;
  __shared__ double sm[32];
  if (check_done && ctl->done) return;
  const long i = blockIdx.x * 256L + threadIdx.x;
  double I = 0;
  if (i < n) {
    const C e = E[i];
    I = (double)(e.x * e.x + e.y * e.y);
    fluence[i] = I;
  }
  const double m = block_max<double>(I, sm);
  if (threadIdx.x == 0) {
    if (!isfinite(m)) atomicOr(&ctl->flags, FIL_FLAG_NAN);
    else atomic_max_nonneg(&ctl->imax_acc, m);
  }
}

template <typename R>
cudaError_t launch_xy_nonlinear(const typename C2T<R>::type* in, typename C2T<R>::type* out, const XyNlParams<R>& p,
                                cudaStream_t st) {
  k_xy_nonlinear<R><<<(unsigned)((p.n + 255) / 256), 256, 0, st>>>(in, out, p);
  return cudaGetLastError();
}
template <typename R>
cudaError_t launch_xy_reduce(const typename C2T<R>::type* E, double* fluence, DevCtl* ctl, long n, int check_done,
                             cudaStream_t st) {
  k_xy_reduce<R><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(E, fluence, ctl, n, check_done);
  return cudaGetLastError();
}

#define XY_INST(R)                                                                                              \
  template cudaError_t launch_xylines<R>(const XyParams<R>&, int, int, int, int, cudaStream_t);              \
  template cudaError_t launch_xy_nonlinear<R>(const C2T<R>::type*, C2T<R>::type*, const XyNlParams<R>&,     \
                                              cudaStream_t);                                                 \
  template cudaError_t launch_xy_reduce<R>(const C2T<R>::type*, double*, DevCtl*, long, int, cudaStream_t);
XY_INST(float)
XY_INST(double)
