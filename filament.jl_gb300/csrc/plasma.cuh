// plasma.cuh -- parallel-in-time solve of the multiphoton/avalanche plasma
// equation of one transverse point (one row of E(t) in shared memory).
//
// Reference: src/modules/plasma_equations.jl:46-72 (sequential RK over t per
// point) with the right-hand sides of
// src/modules/plasma_equations/photoionization_avalanche.jl:119-205:
//   drho_i/dt  = W_i(I) (rho_nt,i - rho_i) + Rava_i E^2 (rho_nt,i - rho_i)/rho_nt,i * sum(rho)
//   drho'_i/dt = W_i(I) (rho_nt,i - rho'_i)                 (photoionisation only)
//   Kdrho(t_j) = sum_i K_i(I_j) W_i(I_j) (rho_nt,i - rho'_i(t_{j+1}))
// with E linearly interpolated at the stage times t_j + c_s dt.
//
// Instead of one thread walking 4095 steps, every explicit-RK step is written
// as a map u_{j+1} = Phi_j(u_j).  For the photoionisation-only equation Phi_j
// is affine, so u_j for all j follows from one block-wide associative scan of
// affine maps (each thread composes a 16-step chunk, a warp/block scan joins
// the chunks, each thread re-applies its chunk from its incoming prefix).
// With avalanche the map is polynomial; Newton's method on the whole
// sequence linearises every Phi_j around the previous iterate, which is again
// an affine scan.  Iteration starts from the photoionisation-only solution
// (avalanche is a small correction) and stops when the update is below a
// relative tolerance; its fixed point is the sequential RK solution.
//
// Affine maps are stored as u -> (I - L) u + B with L = I - dPhi/du kept
// explicitly, so products of thousands of near-identity maps do not lose the
// small deviations to rounding.
#pragma once
#include "common.cuh"

#define FIL_MAXCOMP 4
#define FIL_MAXRATE 32

// Scalars in the working precision R: the FP32 kernels then issue no FP64
// instruction (the FP64 pipe of this part runs at 1/64 of the FP32 rate).
// The rate tables stay FP64 here and are converted once per block into
// shared memory.
template <typename R> struct PlasmaParams {
  int nc;                 // species
  int ns;                 // RK stages
  int kdep, ereal, powerlaw, rate_n;
  int pidx[4];            // stage time: 0 = t_j, 1 = midpoint, 2 = t_{j+1}
  R a[4][4], b[4];        // RK tableau
  R dt, rho0;
  R rho_nt[FIL_MAXCOMP], rava_nt[FIL_MAXCOMP], kfix[FIL_MAXCOMP];
  double lx[FIL_MAXCOMP][FIL_MAXRATE], ly[FIL_MAXCOMP][FIL_MAXRATE], sl[FIL_MAXCOMP][FIL_MAXRATE];
  int avalanche;          // any rava != 0
  int maxit;              // Newton iteration cap
  R tol;                  // Newton: stop when update^2 <= tol |u|^2
  R skip;                 // rows with max W * window below this keep rho0
  // relative skip (0: off): a row whose density rise is bounded by
  // skip_rel * (largest density of the previous solve) keeps rho0.  With
  // g = rava_sum * max E^2 * window the rise is bounded (Gronwall) by
  // (max W * window * rhont_sum + nc * rho0 * g) * exp(g): photoionisation at
  // the largest rate plus avalanche of the initial density, amplified by the
  // largest avalanche growth.
  R skip_rel, rhont_sum, rava_sum;
  // plasma-channel skip of a row left at rho0 = 0: its losses response
  // |Kdrho E / |E|^2| <= K rho_nt W(Imax) / sqrt(Imax) changes the step by at
  // most dz * max|C_losses| * that, and the row's spectrum is at least
  // sqrt(Imax) / (Nt/2); the channel is dropped when
  // dz * ychan_coef * max W <= 2^-30 Imax, ychan_coef = max|C_losses| K
  // rho_nt (Nt/2).  0: never (FP64, rho0 != 0, tabulated or sub-linear rates,
  // E_real losses).
  R ychan_coef;
  // power law with an integer order m (multiphoton rate sigma_m I^m):
  // W(I) = (wscale I)^m by repeated squaring instead of exp/log; 0 = no
  int ipow[FIL_MAXCOMP];
  R wscale[FIL_MAXCOMP];
};

template <typename R> inline PlasmaParams<R> plasma_params_as(const PlasmaParams<double>& d) {
  PlasmaParams<R> r;
  r.nc = d.nc;
  r.ns = d.ns;
  r.kdep = d.kdep;
  r.ereal = d.ereal;
  r.powerlaw = d.powerlaw;
  r.rate_n = d.rate_n;
  for (int i = 0; i < 4; ++i) {
    r.pidx[i] = d.pidx[i];
    r.b[i] = (R)d.b[i];
    for (int j = 0; j < 4; ++j) r.a[i][j] = (R)d.a[i][j];
  }
  r.dt = (R)d.dt;
  r.rho0 = (R)d.rho0;
  for (int c = 0; c < FIL_MAXCOMP; ++c) {
    r.rho_nt[c] = (R)d.rho_nt[c];
    r.rava_nt[c] = (R)d.rava_nt[c];
    r.kfix[c] = (R)d.kfix[c];
    for (int q = 0; q < FIL_MAXRATE; ++q) {
      r.lx[c][q] = d.lx[c][q];
      r.ly[c][q] = d.ly[c][q];
      r.sl[c][q] = d.sl[c][q];
    }
  }
  r.avalanche = d.avalanche;
  r.maxit = d.maxit;
  r.tol = (R)d.tol;
  r.skip = (R)d.skip;
  for (int c = 0; c < FIL_MAXCOMP; ++c) {
    r.ipow[c] = d.ipow[c];
    r.wscale[c] = (R)d.wscale[c];
  }
  r.skip_rel = (R)d.skip_rel;
  r.ychan_coef = (R)d.ychan_coef;
  r.rhont_sum = (R)d.rhont_sum;
  r.rava_sum = (R)d.rava_sum;
  return r;
}

template <typename R> struct PlasmaSmem {
  R lx[FIL_MAXCOMP][FIL_MAXRATE], ly[FIL_MAXCOMP][FIL_MAXRATE], sl[FIL_MAXCOMP][FIL_MAXRATE];
};

template <typename R, int NC> struct Aff {
  R L[NC][NC];
  R B[NC];
};

template <typename R, int NC> FIL_DEV Aff<R, NC> aff_identity() {
  Aff<R, NC> m;
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    m.B[i] = 0;
#pragma unroll
    for (int l = 0; l < NC; ++l) m.L[i][l] = 0;
  }
  return m;
}

// second o first : u -> (I-L2)((I-L1)u + B1) + B2
template <typename R, int NC> FIL_DEV Aff<R, NC> aff_compose(const Aff<R, NC>& m2, const Aff<R, NC>& m1) {
  Aff<R, NC> r;
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    R b = m1.B[i] + m2.B[i];
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      R p = 0;
#pragma unroll
      for (int m = 0; m < NC; ++m) p += m2.L[i][m] * m1.L[m][l];
      r.L[i][l] = m1.L[i][l] + m2.L[i][l] - p;
      b -= m2.L[i][l] * m1.B[l];
    }
    r.B[i] = b;
  }
  return r;
}

template <typename R, int NC> FIL_DEV void aff_apply(const Aff<R, NC>& m, const R* u, R* out) {
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    R v = u[i] + m.B[i];
#pragma unroll
    for (int l = 0; l < NC; ++l) v -= m.L[i][l] * u[l];
    out[i] = v;
  }
}

template <typename R, int NC> FIL_DEV Aff<R, NC> aff_shfl_up(const Aff<R, NC>& m, int off) {
  Aff<R, NC> r;
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    r.B[i] = __shfl_up_sync(0xffffffffu, m.B[i], off);
#pragma unroll
    for (int l = 0; l < NC; ++l) r.L[i][l] = __shfl_up_sync(0xffffffffu, m.L[i][l], off);
  }
  return r;
}

// Exclusive block scan: returns G_{t-1} o ... o G_0 for thread t (identity
// for t = 0).  scratch holds blockDim/32 maps.
template <typename R, int NC> FIL_DEV Aff<R, NC> aff_block_exclusive_scan(Aff<R, NC> g, Aff<R, NC>* scratch) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  Aff<R, NC> inc = g;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    Aff<R, NC> o = aff_shfl_up<R, NC>(inc, off);
    if (lane >= off) inc = aff_compose<R, NC>(inc, o);
  }
  Aff<R, NC> exc = aff_shfl_up<R, NC>(inc, 1);
  if (lane == 0) exc = aff_identity<R, NC>();
  __syncthreads();
  if (lane == 31) scratch[w] = inc;
  __syncthreads();
  if (w > 0) {
    Aff<R, NC> pre = scratch[0];
    for (int k = 1; k < w; ++k) pre = aff_compose<R, NC>(scratch[k], pre);
    exc = aff_compose<R, NC>(exc, pre);
  }
  (void)nw;
  __syncthreads();
  return exc;
}

// W(I) and its log-log slope (TabulatedFunctions restatement: linear
// interpolation of ln W over ln I, end segments extended, W(I<=0) = 0).
template <typename R> FIL_DEV R rate_eval(const PlasmaParams<R>& P, const PlasmaSmem<R>& T, int c, R I, R* slope) {
  int n = P.rate_n;
  if (!(I > (R)0)) {
    *slope = T.sl[c][0];
    return (R)0;
  }
  if (P.ipow[c] > 0) {
    // exp(ly + (ln I - lx) m) = (exp((ly - m lx)/m) I)^m
    *slope = T.sl[c][0];
    R b = I * P.wscale[c], r = (R)1;
    int m = P.ipow[c];
#pragma unroll 1
    while (m) {
      if (m & 1) r *= b;
      m >>= 1;
      if (m) b *= b;
    }
    return r;
  }
  R l = log(I);
  int i = 0;
  if (!P.powerlaw) {
    int lo = 0, hi = n - 2;
    while (lo < hi) {   // largest i in [0, n-2] with lx[i] <= l
      int mid = (lo + hi + 1) >> 1;
      if (T.lx[c][mid] <= l) lo = mid; else hi = mid - 1;
    }
    i = lo;
  }
  *slope = T.sl[c][i];
  return exp(T.ly[c][i] + (l - T.lx[c][i]) * T.sl[c][i]);
}

// W_c(I) in FP64 from the FP64 tables of the parameter block (one
// evaluation per row: the activity test of the surrogate).
template <typename R> FIL_DEV double rate_direct(const PlasmaParams<R>& P, int c, double I) {
  if (!(I > 0)) return 0;
  if (P.ipow[c] > 0) {
    double b = I * (double)P.wscale[c], r = 1;
    for (int m = P.ipow[c]; m; m >>= 1) {
      if (m & 1) r *= b;
      b *= b;
    }
    return r;
  }
  const double l = log(I);
  int i = 0;
  if (!P.powerlaw) {
    int lo = 0, hi = P.rate_n - 2;
    while (lo < hi) {
      int mid = (lo + hi + 1) >> 1;
      if (P.lx[c][mid] <= l) lo = mid; else hi = mid - 1;
    }
    i = lo;
  }
  return exp(P.ly[c][i] + (l - P.lx[c][i]) * P.sl[c][i]);
}

// The negligible-row test of the plasma solve (plasma_row) from the row's
// largest intensity and E^2 (the rates grow with I, so max W = W(max I)).
template <typename R> FIL_DEV bool plasma_row_negligible(const PlasmaParams<R>& P, double imax, double e2max,
                                                         double window, double rho_prev) {
  double wmax = 0;
  for (int c = 0; c < P.nc; ++c) wmax = fmax(wmax, rate_direct<R>(P, c, imax));
  bool skip = wmax * window < (double)P.skip;
  if (!skip && (double)P.skip_rel > 0 && rho_prev > 0) {
    const double g = (double)P.rava_sum * e2max * window;
    if (g < 40)
      skip = (wmax * window * (double)P.rhont_sum + P.nc * (double)P.rho0 * g) * exp(g) <
             (double)P.skip_rel * rho_prev;
  }
  return skip;
}

// One RK step u -> Phi(u) of the full (aval = true) or photoionisation-only
// equation, linearised at u: returns the affine map (L, B) with
// Phi(v) ~= (I - L) v + B exact for the affine case.
template <typename R, int NC>
FIL_DEV Aff<R, NC> step_map(const PlasmaParams<R>& P, const R* u, const R (&W)[3][NC], const R (&ava)[3],
                            bool aval) {
  R k[4][NC], dk[4][NC][NC];
  const R dt = (R)P.dt;
#pragma unroll
  for (int s = 0; s < 4; ++s) {
    if (s >= P.ns) break;
    R U[NC], dU[NC][NC];
#pragma unroll
    for (int i = 0; i < NC; ++i) {
      U[i] = u[i];
#pragma unroll
      for (int l = 0; l < NC; ++l) dU[i][l] = (i == l) ? (R)1 : (R)0;
    }
#pragma unroll
    for (int l = 0; l < s; ++l) {
      R al = (R)P.a[s][l];
      if (al != (R)0) {
#pragma unroll
        for (int i = 0; i < NC; ++i) {
          U[i] += dt * al * k[l][i];
#pragma unroll
          for (int m = 0; m < NC; ++m) dU[i][m] += dt * al * dk[l][i][m];
        }
      }
    }
    const int p = P.pidx[s];
    R S = 0;
#pragma unroll
    for (int i = 0; i < NC; ++i) S += U[i];
#pragma unroll
    for (int i = 0; i < NC; ++i) {
      const R rn = (R)P.rho_nt[i];
      const R ai = aval ? (R)P.rava_nt[i] * ava[p] : (R)0;
      const R g = W[p][i] + ai * S;
      k[s][i] = (rn - U[i]) * g;
      // Df_im = -delta_im g + (rn - U_i) a_i
#pragma unroll
      for (int m = 0; m < NC; ++m) {
        R d = 0;
#pragma unroll
        for (int q = 0; q < NC; ++q) {
          R Df = ((i == q) ? -g : (R)0) + (rn - U[i]) * ai;
          d += Df * dU[q][m];
        }
        dk[s][i][m] = d;
      }
    }
  }
  Aff<R, NC> M;
#pragma unroll
  for (int i = 0; i < NC; ++i) {
    R inc = 0;
    R Lrow[NC];
#pragma unroll
    for (int l = 0; l < NC; ++l) Lrow[l] = 0;
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      if (s >= P.ns) break;
      R bs = (R)P.b[s];
      inc += bs * k[s][i];
#pragma unroll
      for (int l = 0; l < NC; ++l) Lrow[l] += bs * dk[s][i][l];
    }
    R B = dt * inc;
#pragma unroll
    for (int l = 0; l < NC; ++l) {
      M.L[i][l] = -dt * Lrow[l];
      B += M.L[i][l] * u[l];
    }
    M.B[i] = B;
  }
  return M;
}
