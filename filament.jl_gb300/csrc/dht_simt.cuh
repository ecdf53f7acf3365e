// dht_simt.cuh -- the Hankel transform pair of the linear step as two real
// GEMMs on CUDA cores (FP32 or FP64), with the linear propagator fused into
// the first one's epilogue.
//
// Reference: src/modules/linear_propagators/spectral.jl:16-26
//   PS * E;  E .*= exp(i KZ dz);  spectral guard;  PS \ E
// with the QDHT pair folded to two real matrices M1 = T diag(s) and
// M2 = diag(1/s) T acting on the r index of the [Nr][Nt/2] half spectrum
// (complex columns = pairs of real columns).
#pragma once
#include "common.cuh"
#include "rowkernels.cuh"

template <typename R> struct PropParams {
  typedef typename C2T<R>::type C;
  const R* kt2;     // [Mpad] transverse wave number squared (zu units)
  const C* beta;    // [nh]
  const C* dfr;     // [nh] (beta - w/vf) zu
  const R* kmax2;   // [nh] k-guard cut-off squared; NULL: no k guard
  const R* wg;      // [nh] frequency guard; NULL: none
  int kparaxial;
};

// principal complex square root; a -0 imaginary part is treated as +0
// (the reference takes sqrt(beta^2 - kt^2 + 0im))
template <typename R> FIL_DEV typename C2T<R>::type csqrt_p(typename C2T<R>::type z) {
  R x = z.x, y = z.y + (R)0;
  R r = hypot(x, y);
  if (x >= (R)0) {
    R t = sqrt((r + x) * (R)0.5);
    return mk<R>(t, t > (R)0 ? y / (2 * t) : (R)0);
  } else {
    R t = sqrt((r - x) * (R)0.5);
    return mk<R>(fabs(y) / (2 * t), copysign(t, y));
  }
}

template <typename R> FIL_DEV typename C2T<R>::type cdiv(typename C2T<R>::type a, typename C2T<R>::type b) {
  R d = b.x * b.x + b.y * b.y;
  return mk<R>((a.x * b.x + a.y * b.y) / d, (a.y * b.x - a.x * b.y) / d);
}

// exp(i KZ dz) * guard for transverse index i (kt2) and frequency column j
template <typename R>
FIL_DEV typename C2T<R>::type propagator(const PropParams<R>& P, R kt2, int j, R dz) {
  typedef typename C2T<R>::type C;
  C b = P.beta[j];
  C kz = P.dfr[j];
  if (P.kparaxial) {
    if (b.x != (R)0 || b.y != (R)0) kz = kz - cdiv<R>(mk<R>(kt2, 0), (R)2 * b);
  } else {
    C b2 = cmul(b, b);
    C s = csqrt_p<R>(mk<R>(b2.x - kt2, b2.y));
    C den = b + s;
    if (den.x != (R)0 || den.y != (R)0) kz = kz - cdiv<R>(mk<R>(kt2, 0), den);
  }
  R g = (R)1;
  if (P.kmax2) {
    R km2 = P.kmax2[j];
    if (km2 == (R)0) {
      g = 0;
    } else {
      R q = kt2 / km2, q2 = q * q, q4 = q2 * q2, q5 = q4 * q, q10 = q5 * q5;
      g = exp(-(q10 * q10));
    }
  }
  if (P.wg) g *= P.wg[j];
  R amp = g * exp(-kz.y * dz);
  R sn, cs;
  sincos(kz.x * dz, &sn, &cs);
  return mk<R>(amp * cs, amp * sn);
}

// Factor of the non-paraxial prefactor for transverse index i (kt2) and
// frequency column j: QZ(kt, w) / QZ(w) = beta / kz, kz = sqrt(beta^2 - kt^2)
// (0 where kz = 0, as Qfunc_nonparaxial, nonlinear_propagators.jl:232-241),
// times the spectral guard Kguard Wguard.
template <typename R>
FIL_DEV typename C2T<R>::type qz_ratio(const PropParams<R>& P, R kt2, int j) {
  typedef typename C2T<R>::type C;
  const C b = P.beta[j];
  const C b2 = cmul(b, b);
  const C kz = csqrt_p<R>(mk<R>(b2.x - kt2, b2.y));
  if (kz.x == (R)0 && kz.y == (R)0) return mk<R>(0, 0);
  C q = cdiv<R>(b, kz);
  R g = (R)1;
  if (P.kmax2) {
    R km2 = P.kmax2[j];
    if (km2 == (R)0) {
      g = 0;
    } else {
      R x = kt2 / km2, x2 = x * x, x4 = x2 * x2, x5 = x4 * x, x10 = x5 * x5;
      g = exp(-(x10 * x10));
    }
  }
  if (P.wg) g *= P.wg[j];
  return mk<R>(g * q.x, g * q.y);
}

// exp(i KZ dz) * guard on both sides of w = 0 (the XY/XYT transverse
// passes, which also propagate the negative frequencies), with
//   KZ = C(w) + D(kt, w),
//   paraxial:      C = dfr,                D = -kt^2 / (2 beta)
//   non-paraxial:  C = dfr + (c - beta),   D = -kt^2 / (sqrt(beta^2 - kt^2) + c),
// c = beta where Re beta >= 0 and -beta otherwise: the same
// sqrt(beta^2 - kt^2) - w/vf as the reference's Kfunc (spectral.jl:160-184),
// but without the cancellation in sqrt + beta that the rationalised form
// meets for beta < 0.  Re C dz (up to ~1e4 rad for w < 0, moving frame) is
// reduced by the caller in FP64 and passed as cph = exp(i Re C dz).
template <typename R>
FIL_DEV typename C2T<R>::type propagator_cd(const PropParams<R>& P, R kt2, int j, R dz, typename C2T<R>::type cph) {
  typedef typename C2T<R>::type C;
  const C b = P.beta[j];
  const C df = P.dfr[j];
  C d = mk<R>(0, 0);
  R cim = df.y;
  if (P.kparaxial) {
    if (b.x != (R)0 || b.y != (R)0) d = cdiv<R>(mk<R>(-kt2, 0), (R)2 * b);
  } else {
    const bool neg = b.x < (R)0;
    const C c = neg ? mk<R>(-b.x, -b.y) : b;
    const C b2 = cmul(b, b);
    const C sq = csqrt_p<R>(mk<R>(b2.x - kt2, b2.y));
    const C den = sq + c;
    if (den.x != (R)0 || den.y != (R)0) d = cdiv<R>(mk<R>(-kt2, 0), den);
    if (neg) cim -= (R)2 * b.y;
  }
  R g = (R)1;
  if (P.kmax2) {
    R km2 = P.kmax2[j];
    if (km2 == (R)0) {
      g = 0;
    } else {
      R q = kt2 / km2, q2 = q * q, q4 = q2 * q2, q5 = q4 * q, q10 = q5 * q5;
      g = exp(-(q10 * q10));
    }
  }
  if (P.wg) g *= P.wg[j];
  const R amp = g * exp(-(cim + d.y) * dz);
  R sn, cs;
  sincos(d.x * dz, &sn, &cs);
  const C r = cmul(cph, mk<R>(cs, sn));
  return mk<R>(amp * r.x, amp * r.y);
}

// exp(i kc dz) for a column term kc given in FP64: the phase reduced to
// [-pi, pi] in FP64 (in units of pi, exact), then sin/cos of pi x
template <typename R> FIL_DEV typename C2T<R>::type colphase(double kc, double dz) {
  const double t = kc * dz * 0.3183098861837907;
  const R x = (R)(t - 2.0 * rint(0.5 * t));
  R sn, cs;
  sincospi(x, &sn, &cs);
  return mk<R>(cs, sn);
}

template <typename R> struct GemmVec;
template <> struct GemmVec<float> {
  static FIL_DEV void ld4(const float* p, float (&v)[4]) {
    float4 t = *reinterpret_cast<const float4*>(p);
    v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
  }
  static FIL_DEV void st4(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
  }
};
template <> struct GemmVec<double> {
  static FIL_DEV void ld4(const double* p, double (&v)[4]) {
    double2 a = *reinterpret_cast<const double2*>(p), b = *reinterpret_cast<const double2*>(p + 2);
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  static FIL_DEV void st4(double* p, const double (&v)[4]) {
    *reinterpret_cast<double2*>(p) = make_double2(v[0], v[1]);
    *reinterpret_cast<double2*>(p + 2) = make_double2(v[2], v[3]);
  }
};

// C[M x N] = A[M x K] B[K x N], row-major, M,K multiples of 128 / 8,
// N multiple of 128.  256 threads, 128x128 tile, 8x8 outputs per thread.
// EPI = 1: multiply complex pairs of C by the propagator (row i, column
// j = col/2); EPI = 2: plain store and mark the field guard pending;
// EPI = 3: multiply by the non-paraxial prefactor's factor (qz_ratio);
// EPI = 4: plain store.
template <typename R, int EPI>
__global__ void __launch_bounds__(256) k_dht_simt(const R* __restrict__ A, const R* __restrict__ B,
                                                  R* __restrict__ C, int M, int N, int K,
                                                  PropParams<R> pp, DevCtl* ctl) {
  constexpr int BM = 128, BN = 128, BK = 8;
  __shared__ __align__(16) R As[2][BK][BM + 4];
  __shared__ __align__(16) R Bs[2][BK][BN];
  if (ctl->done) return;
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  const int bm = blockIdx.y * BM, bn = blockIdx.x * BN;
  const R* Ab = A + (size_t)bm * K;
  const R* Bb = B + bn;
  // loader indices: A: row tid/2, k-quad (tid&1)*4 ; B: k row tid/32, col (tid&31)*4
  const int arow = tid >> 1, akq = (tid & 1) * 4;
  const int bk = tid >> 5, bcol = (tid & 31) * 4;
  R acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0;
  R ra[4], rb[4];
  GemmVec<R>::ld4(Ab + (size_t)arow * K + akq, ra);
  GemmVec<R>::ld4(Bb + (size_t)bk * N + bcol, rb);
#pragma unroll
  for (int q = 0; q < 4; ++q) As[0][akq + q][arow] = ra[q];
  GemmVec<R>::st4(&Bs[0][bk][bcol], rb);
  __syncthreads();
  int buf = 0;
  for (int k0 = 0; k0 < K; k0 += BK) {
    const bool more = (k0 + BK) < K;
    if (more) {
      GemmVec<R>::ld4(Ab + (size_t)arow * K + k0 + BK + akq, ra);
      GemmVec<R>::ld4(Bb + (size_t)(k0 + BK + bk) * N + bcol, rb);
    }
#pragma unroll
    for (int kk = 0; kk < BK; ++kk) {
      R a[8], b[8];
      R t4[4];
      GemmVec<R>::ld4(&As[buf][kk][ty * 4], t4);
      a[0] = t4[0]; a[1] = t4[1]; a[2] = t4[2]; a[3] = t4[3];
      GemmVec<R>::ld4(&As[buf][kk][64 + ty * 4], t4);
      a[4] = t4[0]; a[5] = t4[1]; a[6] = t4[2]; a[7] = t4[3];
      GemmVec<R>::ld4(&Bs[buf][kk][tx * 4], t4);
      b[0] = t4[0]; b[1] = t4[1]; b[2] = t4[2]; b[3] = t4[3];
      GemmVec<R>::ld4(&Bs[buf][kk][64 + tx * 4], t4);
      b[4] = t4[0]; b[5] = t4[1]; b[6] = t4[2]; b[7] = t4[3];
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    if (more) {
      const int nb = buf ^ 1;
#pragma unroll
      for (int q = 0; q < 4; ++q) As[nb][akq + q][arow] = ra[q];
      GemmVec<R>::st4(&Bs[nb][bk][bcol], rb);
      __syncthreads();
      buf = nb;
    }
  }
  // epilogue
  const R dz = (R)ctl->dz;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int row = bm + (i < 4 ? ty * 4 + i : 64 + ty * 4 + (i - 4));
    R kt2 = (EPI == 1 || EPI == 3) ? pp.kt2[row] : (R)0;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int col = bn + h * 64 + tx * 4;
      R v[4] = {acc[i][h * 4 + 0], acc[i][h * 4 + 1], acc[i][h * 4 + 2], acc[i][h * 4 + 3]};
      if (EPI == 1 || EPI == 3) {
#pragma unroll
        for (int p = 0; p < 2; ++p) {
          typename C2T<R>::type pr = EPI == 1 ? propagator<R>(pp, kt2, (col >> 1) + p, dz)
                                              : qz_ratio<R>(pp, kt2, (col >> 1) + p);
          R re = v[2 * p], im = v[2 * p + 1];
          v[2 * p] = re * pr.x - im * pr.y;
          v[2 * p + 1] = re * pr.y + im * pr.x;
        }
      }
      GemmVec<R>::st4(C + (size_t)row * N + col, v);
    }
  }
  if (EPI == 2 && blockIdx.x == 0 && blockIdx.y == 0 && tid == 0) ctl->guard_pending = 1;
  (void)M;
}
