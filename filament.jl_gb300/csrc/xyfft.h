// xyfft.h -- launch parameters of the XYT transverse transform (xyfft.cu).
#pragma once
#include "dht_simt.cuh"

template <typename R> struct XyParams {
  typedef typename C2T<R>::type C;
  const C* in;
  C* out;                 // may equal in
  size_t line_stride;     // elements between consecutive points of a line
  size_t outer_stride;    // elements between consecutive lines
  const C* tw;            // per-pass FFT twiddles of the line length
  R scale;                // applied on store
  // propagator (x pass)
  PropParams<R> pp;       // beta, dfr, kparaxial (kmax2, wg unused here)
  const double* kcol;     // [columns] Re C(w) of KZ = C(w) + D(kt, w) in FP64 (propagator_cd)
  const R* wg;            // frequency guard [nh] or NULL
  int wg_bug;             // XYT: frequency guard indexed by iy (Guards.jl:314)
  const R* kt2_line;      // kx^2 along the line
  const R* kt2_outer;     // ky^2 of the line
  const R* sg_line;       // spectral guard along the line
  const R* sg_outer;
  const R* g_line;        // field guard along the line (mode 3)
  const R* g_outer;
  DevCtl* ctl;
  R dz_fixed;
};

// XY nonlinear step parameters
template <typename R> struct XyNlParams {
  typedef typename C2T<R>::type C;
  long n;                 // nx * ny
  int ny, ns;
  R a[7][6], b[7];        // explicit RK tableau (ns stages)
  // Tsitouras 5(4) (tsit5.h): 1 one step of dz (ns = 6), 2 adaptive
  // substeps per point (first same as last, bt = b - bhat)
  int tsit;
  R bt[7];
  double atol, rtol;
  C c0;                   // i QZ(w0) Rnl_cubic(w0)
  const R* g1;            // field guard along x, y
  const R* g2;
  DevCtl* ctl;
  R dz_fixed;
};

template <typename R>
cudaError_t launch_xylines(const XyParams<R>& p, int nl, int mode, int nh, int nouter, cudaStream_t st);
template <typename R>
cudaError_t launch_xy_nonlinear(const typename C2T<R>::type* in, typename C2T<R>::type* out, const XyNlParams<R>& p,
                                cudaStream_t st);
template <typename R>
cudaError_t launch_xy_reduce(const typename C2T<R>::type* E, double* fluence, DevCtl* ctl, long n, int check_done,
                             cudaStream_t st);
