// rowkernels.cuh -- kernels that own one transverse point (one time row) per
// thread block: the fused z-step row kernel, the reduction kernel, field
// in/out conversions.  Included once by rowkernels.cu.
//
// Data layout in HBM: the field lives in the frequency domain as the
// analytic half spectrum S[p][k], p = transverse point (Nr for RT, Nx*Ny for
// XYT), k = 0 .. Nt/2-1 (FFTW order, non-negative frequencies), contiguous in
// k.  The time-domain field E(t) = guard * fft(S, zero-padded) exists only in
// shared memory.
#pragma once
#include <cuda_bf16.h>
#include "common.cuh"
#include "fft.cuh"
#include "plasma.cuh"
#include "surrogate_consts.h"
#include "nn_tc.h"
#include "tsit5.h"

// Device control block: written by the controller kernel, read by the step
// kernels (fil_run) or set by the host (fil_step).
struct DevCtl {
  double z, dz, zmax;
  long long steps, nmax, run_steps;
  int done, status, flags, guard_pending, first, clamp_last, nonlinearity, newton_max;
  unsigned long long imax_acc, rhomax_acc;  // bit patterns of non-negative doubles
  double imax, rhomax, energy;
  double dz0, phimax, phik, phip, istop;
  // learned plasma surrogate (surrogate.cuh).  Armed (nn_on) it supplies the
  // density of the rows the reduction flags; every nn_every-th step is a
  // check step on which the ODE solves every row and the largest
  // |rho_net - rho_ode| / max rho_ode is measured.  The network is used on
  // the following steps only while that error is at most nn_tol (nn_use).
  int nn_on, nn_use, nn_check, nn_every;
  int nn_count;               // rows flagged by this step's reduction (atomic)
  int nn_rows;                // rows the network runs on in this step
  long long nn_steps, nn_used, nn_checked, nn_rejected;
  unsigned long long nn_diff_acc;   // check step: max |rho_net - rho_ode| (bits)
  double nn_tol, nn_err, nn_err_max;
  double nn_rows_sum;         // sum of nn_rows over the steps that used the network
  int nn_tiles;               // 128-point tiles the network runs on, of the flagged rows (atomic)
  int nn_tiles_run;           // entries of the tile list the network runs in this step
  double nn_tiles_sum;        // sum of nn_tiles over the steps that used the network
  // adaptive nonlinear step (FIL_ALG_ATSIT5): substep attempts and
  // rejections, summed over the transverse points and steps
  unsigned long long ode_attempts, ode_rejects;
};

#define FIL_FLAG_NAN 1
#define FIL_FLAG_ISTOP 2
#define FIL_FLAG_NEWTON 4
#define FIL_FLAG_ODE 8

template <typename R> struct RowParams {
  typedef typename C2T<R>::type C;
  int nrows, n2, geom, ld;
  const C* tw;                  // twiddles exp(-2 pi i m/N), m < N
  const R* g1;                  // field guard per transverse point (n1) or x
  const R* g2;                  // y guard (XYT) or NULL
  const R* gt;                  // t guard [N]
  int gt_bug;                   // XYT: t guard indexed by iy (Guards.jl:314)
  R dt;
  // nonlinear step
  int nonlin, has_cubic, has_free, has_losses, cubic_thg, losses_ereal;
  const C* Cc;                  // i QZ Rnl_cubic * (k ? 2 : 1), [nh]
  const C* Cf;
  const C* Cl;
  const C* Cr;                  // Raman
  R sc, sf, sl, sr;             // channel pre-scales (C tables are divided by them)
  int has_raman, raman_thg;
  const C* ramh;                // Raman response H(w) [N] (raman.jl:21-31)
  int ns;                       // RK stages
  R A0[4], A1[4], B[4];         // stage input U_s = S0 + dz (A0 k1 + A1 kprev)
  // Tsitouras 5(4) (tsit5.h): 1 one step of dz, 2 adaptive substeps.  The
  // stage derivatives live in tk [row][7][N/2]; ta[s][j], tb = ta[6],
  // tbt = b - bhat; babs = sum |b_s| (1 for RK2/3/4)
  int tsit;
  R ta[7][6], tbt[7];
  R babs;
  C* tk;
  double atol, rtol;
  // plasma
  int plasma;
  PlasmaParams<R> pp;
  R* rho_g;                     // optional full rho / Kdrho rows
  R* kdrho_g;
  int store_plasma;
  double* rho_end;              // rho(t_end) per row
  // state
  const C* S_in;
  C* S_out;
  int out_T;                    // 1: write s_row * S transposed, [2k + re/im][ldT]
  const R* out_scale;           // s_row (out_T), or NULL
  int ldT;
  DevCtl* ctl;
  // learned plasma surrogate: network inputs of the flagged rows
  // [slot][2][N] (BF16), slot of each row (-1: not flagged), network output
  // g(t), the log-amplification of the avalanche term of nn_density: [slot][N],
  // or with nn_part its layer-3 partial sums [slot][9][N] (nn_out_at) and the
  // output bias at nn_b3
  __nv_bfloat16* nn_feat;
  int* nn_slot;
  const float* nn_out;
  int nn_part;
  const float* nn_b3;
  // [slot][N/128] tile flags of the surrogate's rows (nn_features): bit 0 the
  // network's g enters the density in the tile, bit 1 the network runs on
  // it (bit 0 of the tile or of a neighbour); NULL: every tile both
  uint8_t* nn_tflag;
  // [slots x N/128] list of the tiles with bit 1 (slot * N/128 + tile), each
  // row's tiles at a range reserved with the nn_tiles count (or NULL)
  int* nn_tlist;
  // linear-only rows (FP32 form): max_k |i QZ Rnl_cubic (k ? 2 : 1)| (the
  // Kerr coefficient before the channel pre-scale); < 0 disables the test
  R cc_max;
  // Upper half of the spectrum: bins N/2 .. N-1 (the Nyquist bin and the
  // negative frequencies) that the time-domain field guard creates.  The
  // reference keeps them in its full-length spectrum: every analytic
  // response leaves them unchanged (rsig2aspec! zeroes them), the linear
  // step multiplies them by exp(i KZ dz) Kguard Wguard in r-space (its
  // Hankel transform covers the first N/2 columns only,
  // linear_propagators/spectral.jl:16-26, Fields.jl:108-110), and they
  // enter the time-domain field of every plasma solve and RK stage.
  // [row][N/2] complex (row stride ld); NULL = dropped (the analytic
  // projection).  U_in is read at load; U_out receives the t->w transform
  // of the guarded field (re-read by the stages) and then its propagated
  // value; the two may alias (each block touches its own row only).
  const C* U_in;
  C* U_out;
  const double* u_kzr;          // [row][N/2] Re KZ (zu units) in FP64: the phase KZ dz is reduced exactly
  const C* u_kg;                // [row][N/2] (Im KZ, Kguard Wguard)
  // [row][N/2] (row stride ld): the guarded spectrum S0 of a step parked
  // across the plasma solve (load_time_row_split)
  C* s0_park;
  // T geometry (no transverse transform): the lower half's linear step
  // exp(i KZ dz) Wguard applied by the row kernel on its output, tables as
  // u_kzr, u_kg; the kernel then marks the field guard pending
  const double* l_kzr;
  const C* l_kg;
  // [row][NC - 2][N]: the iterates of species 2, 3 in the plasma scan (NC > 2)
  R* spec_g;
  // non-paraxial prefactor (k_rowstep modes 2, 3; k_np_combine): [row][N/2]
  // complex, row stride ld; rho_g, kdrho_g hold the step's density rows
  C* np_S0;                     // t -> w transform of the guarded field
  const C* np_K1;               // stage 0's transformed right-hand side
  const C* np_KS;               // the last stage's transformed right-hand side
  C* np_ACC;                    // sum of B[l] k_l over the stages before
  int np_stage;                 // k_rowstage: the stage
};

template <typename R> FIL_DEV R row_guard(const RowParams<R>& P, int row, int* iy) {
  if (P.g2) {
    int ix = row / P.n2;
    *iy = row - ix * P.n2;
    return P.g1[ix] * P.g2[*iy];
  }
  *iy = 0;
  return P.g1[row];
}

// ---------------------------------------------------------------------------
// Load S_in[row] into X (zero upper half), fft to time, apply the pending
// field guard.  Afterwards X holds E(t).
template <typename R, int N>
FIL_DEV void load_time_row(const RowParams<R>& P, typename C2T<R>::type* X, int row, bool guard) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2, EW = NH / T;
  const int tid = threadIdx.x;
  const C* src = P.S_in + (size_t)row * P.ld;
  const C* up = P.U_in ? P.U_in + (size_t)row * P.ld : nullptr;
#pragma unroll
  for (int m = 0; m < EW; ++m) {
    int k = tid + m * T;
    X[pad16(k)] = src[k];
    X[pad16(k + NH)] = up ? up[k] : mk<R>(0, 0);
  }
  filfft::block_fft<C, N, -1>(X, P.tw);
  if (guard) {
    int iy;
    R gs = row_guard(P, row, &iy);
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      int j = tid + m * T;
      R g = gs * P.gt[P.gt_bug ? iy : j];
      X[pad16(j)] = g * X[pad16(j)];
    }
    __syncthreads();
  }
}

// ---------------------------------------------------------------------------
// The pending field guard of a step without the transform round trip.  The
// state [S, U] is the exact spectrum of E(t) = fft(S, U); the guarded
// spectrum is ifft(g E) = [S, U] - ifft((1 - g) E), so only the guard's
// correction (1 - g) E, small wherever the guard is 1, goes through the
// transforms and their rounding.  Afterwards X holds g E(t) (for the
// plasma solve); the guarded lower half is in s0_park, the upper half (when
// kept) in U_out.  Y is scratch and free again on return.
template <typename R, int N>
FIL_DEV void split_guard_row(const RowParams<R>& P, typename C2T<R>::type* X, typename C2T<R>::type* Y, int row);
template <typename R, int N>
FIL_DEV void load_time_row_split(const RowParams<R>& P, typename C2T<R>::type* X, typename C2T<R>::type* Y,
                                 int row) {
  load_time_row<R, N>(P, X, row, false);
  split_guard_row<R, N>(P, X, Y, row);
}
// The second half of load_time_row_split, on X = E(t) loaded without the
// guard (k_rowstep calls the two halves itself so that its row load, and
// the transform in it, is inlined once).
template <typename R, int N>
FIL_DEV void split_guard_row(const RowParams<R>& P, typename C2T<R>::type* X, typename C2T<R>::type* Y, int row) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2, EW = NH / T;
  const int tid = threadIdx.x;
  int iy;
  const R gs = row_guard(P, row, &iy);
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    const int j = tid + m * T;
    const R g = gs * P.gt[P.gt_bug ? iy : j];
    const C e = X[pad16(j)];
    Y[pad16(j)] = ((R)1 - g) * e;
    X[pad16(j)] = g * e;
  }
  filfft::block_fft<C, N, +1>(Y, P.tw);
  const R invN = (R)1 / (R)N;
  const size_t rb = (size_t)row * P.ld;
#pragma unroll
  for (int m = 0; m < EW; ++m) {
    const int k = tid + m * T;
    P.s0_park[rb + k] = P.S_in[rb + k] - invN * Y[pad16(k)];
    if (P.U_out) P.U_out[rb + k] = P.U_in[rb + k] - invN * Y[pad16(k + NH)];
  }
  __syncthreads();
}

// ---------------------------------------------------------------------------
// Plasma solve on the row in X.  Writes rho[] and kdrho[] (shared, indexed
// with pad16), Y is scratch (2*(N + N/16) reals).  Returns max rho
// (block-uniform).
//
// Work split: thread t owns the 16 consecutive time steps j = 16t .. 16t+15.
// Single-species power-law rates (the common case) are evaluated once per
// time point and midpoint into Y; otherwise they are re-evaluated per use.
// A row whose largest rate times the window length is below `skip` keeps
// rho = rho0 exactly to the working precision and needs no scan.
template <typename R, int N, int NC>
FIL_DEV R plasma_row(const RowParams<R>& P, const PlasmaSmem<R>& tabs, const typename C2T<R>::type* X,
                     R* rho, R* kdrho, R* Y, Aff<R, NC>* ascratch, R* rscratch, int* newton_flag, R rho_prev,
                     R dz, bool* ychan) {
  typedef typename C2T<R>::type C;
  constexpr int NP = N + N / 16;
  const PlasmaParams<R>& pp = P.pp;
  const int tid = threadIdx.x;
  const int j0 = tid * 16;
  const bool ereal = pp.ereal;
  const bool cached = (NC == 1) && pp.powerlaw;
  // iterate storage: species c at ub[c*NP + pad16(j)] (Y holds two rows of
  // reals); rho itself for NC = 1; species 2 and 3 of NC > 2 in the row's
  // slice of spec_g (only the thread that owns j reads and writes it)
  R* ub = (NC == 1) ? rho : Y;
  auto UB = [&](int c, int j) -> R& {
    if constexpr (NC > 2) {
      if (c >= 2) return P.spec_g[((size_t)blockIdx.x * (NC - 2) + (c - 2)) * N + j];
    }
    return ub[c * NP + pad16(j)];
  };
  R* Wp = Y;          // cached W(I_j)      (NC = 1, power law)
  R* Wm = Y + NP;     // cached W(I_{j+1/2})
  R u0[NC];
#pragma unroll
  for (int c = 0; c < NC; ++c) u0[c] = (R)pp.rho0;

  auto intens = [&](C e) -> R { return ereal ? e.x * e.x : e.x * e.x + e.y * e.y; };
  auto rates = [&](R I, R (&W)[NC], R (&S)[NC]) {
#pragma unroll
    for (int c = 0; c < NC; ++c) W[c] = rate_eval<R>(pp, tabs, c, I, &S[c]);
  };
  // W and E^2 at the three stage points of step j, slope at t_j in S0
  auto point_data = [&](int j, R (&W)[3][NC], R (&ava)[3], R (&S0)[NC]) {
    C e0 = X[pad16(j)], e1 = X[pad16(j + 1)];
    C em = (R)0.5 * (e0 + e1);
    if (cached) {
      W[0][0] = Wp[pad16(j)];
      W[1][0] = Wm[pad16(j)];
      W[2][0] = Wp[pad16(j + 1)];
      S0[0] = tabs.sl[0][0];
    } else {
      R Sd[NC];
      rates(intens(e0), W[0], S0);
      rates(intens(em), W[1], Sd);
      rates(intens(e1), W[2], Sd);
    }
    ava[0] = e0.x * e0.x;
    ava[1] = em.x * em.x;
    ava[2] = e1.x * e1.x;
  };

  // ---------------- rate cache and the negligible-row test
  R wmax = 0, e2max = 0, i2max = 0;
  *ychan = true;
  if (cached) {
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
      R sl;
      const C e = X[pad16(j)];
      R w0 = rate_eval<R>(pp, tabs, 0, intens(e), &sl);
      Wp[pad16(j)] = w0;
      wmax = max(wmax, w0);
      e2max = max(e2max, e.x * e.x);
      i2max = max(i2max, e.x * e.x + e.y * e.y);
      if (j < N - 1) {
        C em = (R)0.5 * (e + X[pad16(j + 1)]);
        R wm = rate_eval<R>(pp, tabs, 0, intens(em), &sl);
        Wm[pad16(j)] = wm;
        wmax = max(wmax, wm);
      }
    }
  } else {
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
      R W[NC], S[NC];
      const C e = X[pad16(j)];
      rates(intens(e), W, S);
      e2max = max(e2max, e.x * e.x);
      i2max = max(i2max, e.x * e.x + e.y * e.y);
#pragma unroll
      for (int c = 0; c < NC; ++c) wmax = max(wmax, W[c]);
    }
  }
  wmax = block_max<R>(wmax, rscratch);
  const R window = pp.dt * (R)(N - 1);
  bool skip = wmax * window < pp.skip;
  if (!skip && pp.skip_rel > (R)0 && rho_prev > (R)0) {
    // the midpoint intensities do not exceed the larger end-point one, so
    // e2max over the points bounds E^2 at every stage time
    e2max = block_max<R>(e2max, rscratch);
    const R g = pp.rava_sum * e2max * window;
    if (g < (R)40)
      skip = (wmax * window * pp.rhont_sum + (R)NC * pp.rho0 * g) * exp(g) < pp.skip_rel * rho_prev;
  }
  if (skip && pp.ychan_coef > (R)0) {
    i2max = block_max<R>(i2max, rscratch);
    *ychan = !(dz * pp.ychan_coef * wmax <= (R)9.313225746154785e-10 * i2max);   // 2^-30
  }
  if (skip) {
    // rho stays rho0; Kdrho = sum K W (rho_nt - rho0) to the same precision
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
      R kd = 0;
      if (j < N - 1) {
        R W[NC], S[NC];
        if (cached) { W[0] = Wp[pad16(j)]; S[0] = tabs.sl[0][0]; }
        else rates(intens(X[pad16(j)]), W, S);
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          R K = pp.kdep ? S[c] : (R)pp.kfix[c];
          kd += K * W[c] * ((R)pp.rho_nt[c] - u0[c]);
        }
      }
      kdrho[pad16(j)] = kd;
      R r = 0;
#pragma unroll
      for (int c = 0; c < NC; ++c) r += u0[c];
      rho[pad16(j)] = r;
    }
    __syncthreads();
    R r0 = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) r0 += u0[c];
    return r0;
  }

  // ---------------- iteration 0: photoionisation only (exact affine scan)
  if constexpr (NC == 1) {
    // one pass: the 16 local prefix maps stay in registers
    Aff<R, 1> Pq[16];
    R W[3][1], ava[3], S0[1], uz[1] = {0};
    Aff<R, 1> G = aff_identity<R, 1>();
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
      if (j < N - 1) {
        point_data(j, W, ava, S0);
        G = aff_compose<R, 1>(step_map<R, 1>(pp, uz, W, ava, false), G);
      }
      Pq[q] = G;
    }
    Aff<R, 1> Pin = aff_block_exclusive_scan<R, 1>(G, ascratch);
    R v[1];
    aff_apply<R, 1>(Pin, u0, v);
    const R K = pp.kdep ? tabs.sl[0][0] : (R)pp.kfix[0];
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
      R un[1];
      if (q == 0) ub[pad16(j)] = v[0];
      aff_apply<R, 1>(Pq[q], v, un);
      if (j < N - 1) {
        if (q < 15) ub[pad16(j + 1)] = un[0];
        R w0, sl0;
        if (cached) { w0 = Wp[pad16(j)]; sl0 = tabs.sl[0][0]; }
        else w0 = rate_eval<R>(pp, tabs, 0, intens(X[pad16(j)]), &sl0);
        kdrho[pad16(j)] = (pp.kdep ? sl0 : K) * w0 * ((R)pp.rho_nt[0] - un[0]);
      } else {
        kdrho[pad16(j)] = 0;   // never written by the reference (plasma_equations.jl:63-70)
      }
    }
  } else {
    Aff<R, NC> G = aff_identity<R, NC>();
    R W[3][NC], ava[3], S0[NC];
    R uz[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) uz[c] = 0;
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
      if (j >= N - 1) break;
      point_data(j, W, ava, S0);
      Aff<R, NC> M = step_map<R, NC>(pp, uz, W, ava, false);
      G = aff_compose<R, NC>(M, G);
    }
    Aff<R, NC> Pin = aff_block_exclusive_scan<R, NC>(G, ascratch);
    R u[NC];
    aff_apply<R, NC>(Pin, u0, u);
    for (int q = 0; q < 16; ++q) {
      int j = j0 + q;
#pragma unroll
      for (int c = 0; c < NC; ++c) UB(c, j) = u[c];
      if (j < N - 1) {
        point_data(j, W, ava, S0);
        Aff<R, NC> M = step_map<R, NC>(pp, uz, W, ava, false);
        R un[NC];
        aff_apply<R, NC>(M, u, un);
        R kd = 0;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          R K = pp.kdep ? S0[c] : (R)pp.kfix[c];
          kd += K * W[0][c] * ((R)pp.rho_nt[c] - un[c]);
          u[c] = un[c];
        }
        kdrho[pad16(j)] = kd;
      } else {
        kdrho[pad16(j)] = 0;   // never written by the reference (plasma_equations.jl:63-70)
      }
    }
  }
  __syncthreads();

  // ---------------- Newton iterations with avalanche.  The update d of
  // iteration m estimates the error of iteration m-1; Newton's quadratic
  // convergence leaves an error ~ d^2/|u| after it, so iteration stops when
  // d^2 <= tol |u|^2.
  if (pp.avalanche) {
    int it = 0;
    bool conv = false;
    for (; it < pp.maxit; ++it) {
      R dmax = 0, umax = 0;
      if constexpr (NC == 1) {
        Aff<R, 1> Pq[16];
        R ul[16];
        R W[3][1], ava[3], S0[1];
        Aff<R, 1> G = aff_identity<R, 1>();
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          int j = j0 + q;
          ul[q] = ub[pad16(j)];
          if (j < N - 1) {
            point_data(j, W, ava, S0);
            G = aff_compose<R, 1>(step_map<R, 1>(pp, &ul[q], W, ava, true), G);
          }
          Pq[q] = G;
        }
        Aff<R, 1> Pin = aff_block_exclusive_scan<R, 1>(G, ascratch);  // syncs: old values all read
        R v[1];
        aff_apply<R, 1>(Pin, u0, v);
#pragma unroll
        for (int q = 0; q < 16; ++q) {
          int j = j0 + q;
          R un;
          if (q == 0) {
            un = v[0];
          } else {
            R t[1];
            aff_apply<R, 1>(Pq[q - 1], v, t);
            un = t[0];
          }
          dmax = max(dmax, fabs(un - ul[q]));
          umax = max(umax, fabs(un));
          ub[pad16(j)] = un;
        }
      } else {
        R W[3][NC], ava[3], S0[NC];
        Aff<R, NC> G = aff_identity<R, NC>();
        for (int q = 0; q < 16; ++q) {
          int j = j0 + q;
          if (j >= N - 1) break;
          R ul[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) ul[c] = UB(c, j);
          point_data(j, W, ava, S0);
          Aff<R, NC> M = step_map<R, NC>(pp, ul, W, ava, true);
          G = aff_compose<R, NC>(M, G);
        }
        Aff<R, NC> Pin = aff_block_exclusive_scan<R, NC>(G, ascratch);
        R u[NC];
        aff_apply<R, NC>(Pin, u0, u);
        for (int q = 0; q < 16; ++q) {
          int j = j0 + q;
          R ul[NC];
#pragma unroll
          for (int c = 0; c < NC; ++c) {
            ul[c] = UB(c, j);
            dmax = max(dmax, fabs(u[c] - ul[c]));
            umax = max(umax, fabs(u[c]));
            UB(c, j) = u[c];
          }
          if (j < N - 1) {
            point_data(j, W, ava, S0);
            Aff<R, NC> M = step_map<R, NC>(pp, ul, W, ava, true);
            R un[NC];
            aff_apply<R, NC>(M, u, un);
#pragma unroll
            for (int c = 0; c < NC; ++c) u[c] = un[c];
          }
        }
      }
      dmax = block_max<R>(dmax, rscratch);
      umax = block_max<R>(umax, rscratch);
      if (dmax * dmax <= (R)pp.tol * umax * umax) { conv = true; break; }
    }
    if (!conv && tid == 0) *newton_flag = 1;
    if (tid == 0) atomicMax(&P.ctl->newton_max, it + 1);
  }
  // ---------------- rho = sum of species
  R rmax = 0;
  for (int q = 0; q < 16; ++q) {
    int j = j0 + q;
    R sm = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) sm += UB(c, j);
    if (NC > 1) rho[pad16(j)] = sm;
    rmax = max(rmax, sm);
  }
  __syncthreads();
  return block_max<R>(rmax, rscratch);
}

// ---------------------------------------------------------------------------
// Density of the row in X from the surrogate output g[j] (surrogate.cuh).
// Effective rate of the step t_j -> t_{j+1}:
//   w_j = Wb_j + kappa A_j (1 - e^{-S_j}) e^{g_j},
// with Wb_j = sum_s b_s W(I at the stage point of s) the quadrature of the
// time integrator of plasma_equations.jl:46-72 (stage points t_j, the
// midpoint of the linearly interpolated field, t_{j+1}) applied to
// W = sum_c W_c rho_nt,c / rho_nt; A_j the same quadrature of E^2 (the
// avalanche drive); kappa = sum_c Rava_c; S_j = dt sum_{i<j} Wb_i the base
// rate's ionised fraction exponent, so that the second term is the avalanche
// rate of the photoionised density and e^{g} its learned correction (the
// avalanche's own amplification; g is held to [NN_G_LO, NN_G_HI]).  Then S'_j = dt sum_{i<j} w_i (block scans),
// rho_j = rho_a + (rho_nt - rho_a)(1 - e^{-S'_j}) with rho_a = nc rho0, and the
// loss term Kdrho_j = sum_c K_c W_c(I_j) (rho_nt,c - rho_{j+1} rho_nt,c / rho_nt),
// 0 at the last point (the photoionisation-only density of
// plasma_equations.jl:63-70 approximated by rho).  Thread t owns
// j = 16t .. 16t+15 as in plasma_row.  check_step: compare with the density in
// rho[] instead of writing it; returns max |difference|.  Otherwise writes
// rho[], kdrho[] and returns max rho.
template <typename R, int N, int NC>
FIL_DEV R nn_density(const RowParams<R>& P, const PlasmaSmem<R>& tabs, const typename C2T<R>::type* X,
                     const float* __restrict__ g, R* rho, R* kdrho, Aff<R, 1>* ascratch, R* rscratch, bool check_step,
                     int slot) {
  typedef typename C2T<R>::type C;
  const PlasmaParams<R>& pp = P.pp;
  const int j0 = threadIdx.x * 16;
  const R rnt = pp.rhont_sum, ra = (R)NC * pp.rho0, dt = pp.dt;
  R kappa = 0;
#pragma unroll
  for (int c = 0; c < NC; ++c) kappa += pp.rava_nt[c] * pp.rho_nt[c];
  const float b3 = P.nn_part ? __ldg(P.nn_b3) : 0.f;
  // the thread's 16 points lie in one 128-point tile: g there, or g = 0 where
  // the tile flag says it cannot matter (nn_features)
  const bool use_g = !P.nn_tflag || (P.nn_tflag[(size_t)slot * (N / 128) + j0 / 128] & 1);
  // quadrature weights of the stage points t_j, t_j + dt/2, t_{j+1}
  R qw[3] = {0, 0, 0};
  for (int st = 0; st < pp.ns; ++st) qw[pp.pidx[st]] += pp.b[st];
  auto wsum = [&](C e) -> R {
    const R I = pp.ereal ? e.x * e.x : e.x * e.x + e.y * e.y;
    R w = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      R sl;
      w += rate_eval<R>(pp, tabs, c, I, &sl) * pp.rho_nt[c];
    }
    return w;
  };
  // base rate of step j times dt (0 for the last point)
  auto base = [&](int j) -> R {
    if (j >= N - 1) return (R)0;
    const C e0 = X[pad16(j)], e1 = X[pad16(j + 1)];
    return (qw[0] * wsum(e0) + qw[1] * wsum((R)0.5 * (e0 + e1)) + qw[2] * wsum(e1)) * (dt / rnt);
  };
  // pass 1: S_j
  R tsum = 0;
#pragma unroll 4
  for (int q = 0; q < 16; ++q) tsum += base(j0 + q);
  Aff<R, 1> G;
  G.L[0][0] = 0;
  G.B[0] = tsum;
  R S = aff_block_exclusive_scan<R, 1>(G, ascratch).B[0];
  // pass 2: effective rates
  R wl[16];
  tsum = 0;
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = j0 + q;
    const R wb = base(j);
    R w = wb;
    if (j < N - 1 && kappa != (R)0) {
      const C e0 = X[pad16(j)], e1 = X[pad16(j + 1)];
      const C em = (R)0.5 * (e0 + e1);
      const R A = qw[0] * e0.x * e0.x + qw[1] * em.x * em.x + qw[2] * e1.x * e1.x;
      float gj = 0.f;
      if (use_g) {
        const float gr = P.nn_part ? nn_out_at(g, b3, j, N) : __ldg(&g[j]);
        gj = fminf(fmaxf(gr, NN_G_LO), NN_G_HI);
      }
      w += kappa * A * dt * -expm1(-S) * exp((R)gj);
    }
    S += wb;
    wl[q] = w;
    tsum += w;
  }
  G.B[0] = tsum;
  S = aff_block_exclusive_scan<R, 1>(G, ascratch).B[0];
  R out = 0;
  R rcur = ra + (rnt - ra) * -expm1(-S);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = j0 + q;
    S += wl[q];
    const R rnext = ra + (rnt - ra) * -expm1(-S);
    if (check_step) {
      out = max(out, fabs(rcur - rho[pad16(j)]));
    } else {
      rho[pad16(j)] = rcur;
      R kd = 0;
      if (j < N - 1) {
        const C e = X[pad16(j)];
        const R I = pp.ereal ? e.x * e.x : e.x * e.x + e.y * e.y;
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          R sl;
          const R W = rate_eval<R>(pp, tabs, c, I, &sl);
          const R K = pp.kdep ? sl : (R)pp.kfix[c];
          kd += K * W * (pp.rho_nt[c] - rnext * pp.rho_nt[c] / rnt);
        }
      }
      kdrho[pad16(j)] = kd;
      out = max(out, rcur);
    }
    rcur = rnext;
  }
  __syncthreads();
  return block_max<R>(out, rscratch);
}

// ---------------------------------------------------------------------------
// One evaluation of func! (nonlinear_propagators.jl:38-67) on the row's stage
// input u(m) (analytic half, k = tid + m N/16 < N/2, EW = 8 per thread; d(m,
// value) receives the result at the same k) with the upper half of the
// spectrum from uo (NULL = zero): w -> t, the responses in the time domain
// (medium_responses/*.jl) times the field filter, their analytic spectra
// (rsig2aspec!) times Rnl and the paraxial i QZ (the C_ch tables), summed
// into d.  Channels are packed two per complex FFT by scale: X holds the
// Kerr response (real part) and the Raman response (imaginary part), Y the
// two plasma responses (free current in the real part, losses in the
// imaginary part); each channel is pre-scaled by |C_ch| at the carrier so
// packed partners have comparable size.  ych = false leaves the plasma
// channels out (their response is below the row's resolution).
template <typename R, int N, int NC, bool RAM, typename In, typename Out>
FIL_DEV void stage_rhs(const RowParams<R>& P, typename C2T<R>::type* X, typename C2T<R>::type* Y,
                       const R* rho, const R* kdrho, R gs, int iy, bool ych,
                       const typename C2T<R>::type* uo, In u, Out d) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2, EW = NH / T;
  static_assert(EW == 8, "eight half-spectrum points per thread");
  const int tid = threadIdx.x;
  const R invN = (R)1 / (R)N;
  __syncthreads();   // X and Y free
#pragma unroll
  for (int m = 0; m < EW; ++m) {
    int k = tid + m * T;
    X[pad16(k)] = u(m);
    X[pad16(k + NH)] = uo ? uo[k] : mk<R>(0, 0);
  }
  filfft::block_fft<C, N, -1>(X, P.tw);            // inverse_transform_time!
  if (RAM) {
    // raman.jl:80-98: conv = fft(H * ifft(x)), x = Re(E)^2 or 3/4 |E|^2,
    // in Y (free until the responses below are written)
#pragma unroll 4
    for (int m = 0; m < 16; ++m) {
      int j = tid + m * T;
      C e = X[pad16(j)];
      R x = P.raman_thg ? e.x * e.x : (R)0.75 * (e.x * e.x + e.y * e.y);
      Y[pad16(j)] = mk<R>(x, 0);
    }
    filfft::block_fft<C, N, +1>(Y, P.tw);
#pragma unroll 4
    for (int m = 0; m < 16; ++m) {
      int j = tid + m * T;
      Y[pad16(j)] = invN * cmul(Y[pad16(j)], __ldg(&P.ramh[j]));
    }
    filfft::block_fft<C, N, -1>(Y, P.tw);
  }
#pragma unroll 4
  for (int m = 0; m < 16; ++m) {
    int j = tid + m * T;
    C e = X[pad16(j)];
    R re = e.x;
    R I = e.x * e.x + e.y * e.y;
    R g = gs * P.gt[P.gt_bug ? iy : j];
    R fc = 0, ff = 0, fl = 0, fr = 0;
    if (P.has_cubic) fc = P.cubic_thg ? re * re * re : (R)0.75 * I * re;
    if (RAM) fr = Y[pad16(j)].x * re;
    if (NC > 0 && P.has_free) ff = rho[pad16(j)] * re;
    if (NC > 0 && P.has_losses) {
      R Il = P.losses_ereal ? re * re : I;
      R inv = (Il >= (R)1e-30) ? (R)1 / Il : (R)0;
      fl = kdrho[pad16(j)] * inv * re;
    }
    X[pad16(j)] = mk<R>(g * (R)P.sc * fc, RAM ? g * P.sr * fr : (R)0);
    Y[pad16(j)] = mk<R>(g * (R)P.sf * ff, g * (R)P.sl * fl);
  }
  const bool plas = NC > 0 && (P.has_free || P.has_losses) && ych;
  // rsig2aspec! of both buffers through one inlined transform (a second
  // copy of its code would only compete for the instruction cache)
#pragma unroll 1
  for (int f = 0; f < 2; ++f) {
    const bool on = f ? plas : (P.has_cubic || RAM);   // block-uniform
    if (on) filfft::block_fft<C, N, +1>(f ? Y : X, P.tw);
  }
  __syncthreads();
#pragma unroll
  for (int m = 0; m < EW; ++m) {
    int k = tid + m * T;
    const int km = (N - k) & (N - 1);
    C dd = mk<R>(0, 0);
    if (P.has_cubic || RAM) {
      C z = X[pad16(k)], zm = cconj(X[pad16(km)]);
      if (P.has_cubic) dd = cmul(__ldg(&P.Cc[k]), ((R)0.5 * invN) * (z + zm));
      if (RAM) {
        C dl = z - zm;
        dd = dd + cmul(__ldg(&P.Cr[k]), mk<R>(dl.y * (R)0.5 * invN, -dl.x * (R)0.5 * invN));
      }
    }
    if (plas) {
      C z = Y[pad16(k)], zm = cconj(Y[pad16(km)]);
      C ffr = ((R)0.5 * invN) * (z + zm);                 // (z + conj z_-k)/2
      C dl = z - zm;
      C flr = mk<R>(dl.y * (R)0.5 * invN, -dl.x * (R)0.5 * invN);  // (z - conj z_-k)/(2i)
      if (P.has_free) dd = dd + cmul(__ldg(&P.Cf[k]), ffr);
      if (P.has_losses) dd = dd + cmul(__ldg(&P.Cl[k]), flr);
    }
    d(m, dd);
  }
}

// One value of a row's output (of a step, or of a non-paraxial stage): the
// half-spectrum point k in the Hankel GEMM's operand layout (real column
// 2k + c, transverse index contiguous, scaled by s_row) or in the row layout.
template <typename R>
FIL_DEV void write_out(const RowParams<R>& P, int row, int k, typename C2T<R>::type v) {
  if (P.out_T) {
    R* base = reinterpret_cast<R*>(P.S_out);
    const R sc = P.out_scale ? P.out_scale[row] : (R)1;
    base[(size_t)(2 * k) * P.ldT + row] = sc * v.x;
    base[(size_t)(2 * k + 1) * P.ldT + row] = sc * v.y;
  } else {
    P.S_out[(size_t)row * P.ld + k] = v;
  }
}

// Linear step of the upper half of the spectrum at (row, k): u exp(i KZ dz)
// Kguard Wguard in r-space.  |Re KZ dz| reaches ~1e5 rad at the negative
// frequencies (moving frame), so the phase is formed in FP64 in units of pi
// and reduced there to [-1, 1] (exact: 2 rint(t/2) is representable), and
// sin/cos of pi x need no further argument reduction.
template <typename R>
FIL_DEV typename C2T<R>::type table_prop(const double* kzr, const typename C2T<R>::type* kgt, size_t idx,
                                         typename C2T<R>::type u, double dzd) {
  const double t = __ldg(&kzr[idx]) * dzd * 0.3183098861837907;   // phase / pi
  const R x = (R)(t - 2.0 * rint(0.5 * t));
  const typename C2T<R>::type kg = kgt[idx];
  const R amp = kg.y * exp(-kg.x * (R)dzd);
  R sn, cs;
  sincospi(x, &sn, &cs);
  return cmul(u, mk<R>(amp * cs, amp * sn));
}
template <typename R>
FIL_DEV typename C2T<R>::type upper_prop(const RowParams<R>& P, size_t idx, typename C2T<R>::type u, double dzd) {
  return table_prop<R>(P.u_kzr, P.u_kg, idx, u, dzd);
}

// ---------------------------------------------------------------------------
// Fused z-step of one row (blockIdx.x = row):
//   E(t) = guard * fft(S_in)   (guard from the previous step, Models.jl:116-118)
//   plasma solve on E(t)       (Models.jl:84-89)
//   S0 = ifft(E)[0:N/2]        (Models.jl:91-96)
//   RK step of func!            (Models.jl:98-103, nonlinear_propagators.jl:38-74)
//   S_out = S0 + dz sum b_s k_s
// mode 1: plasma only (initialisation), no S_out.  mode 4: the plasma solve
// of a step only (with the surrogate when armed), rho and Kdrho rows to
// rho_g, kdrho_g: the first launch of a non-paraxial step (k_rowstage).
// RAM: the Raman channel (compiled only where used, it costs registers).
// TS: the Tsitouras methods (FIL_ALG_TSIT5/ATSIT5, P.tsit), in kernels of
// their own so that the RK2/3/4 kernels keep their registers.
// Blocks are held to 128 registers so that two (4096-point rows) to sixteen
// (512-point rows, the XYT geometry) share an SM.
template <typename R, int N, int NC, bool RAM, bool TS>
__global__ void __launch_bounds__(N / 16, N <= 1024 ? 8192 / N : 2) k_rowstep(RowParams<R> P, int mode) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2, EW = NH / T, NP = N + N / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* X = reinterpret_cast<C*>(smem_raw);
  C* Y = X + NP;
  R* rho = reinterpret_cast<R*>(Y + NP);                 // [NP], pad16 index
  R* kdrho = rho + NP;
  R* rscratch = kdrho + NP;                              // 32
  Aff<R, (NC > 0 ? NC : 1)>* ascratch = reinterpret_cast<Aff<R, (NC > 0 ? NC : 1)>*>(rscratch + 32);
  PlasmaSmem<R>* tabs = reinterpret_cast<PlasmaSmem<R>*>(ascratch + 32);
  __shared__ int s_flag;
  __shared__ double s_dred[32];
  __shared__ struct {
    OdeStep o;
    int k1s, rej, ok, fin;
  } s_ode;   // FIL_ALG_ATSIT5 controller of the row
  bool ych = true;   // the plasma channels (Y) carry a response for this row

  DevCtl* ctl = P.ctl;
  if (ctl->done) return;
  const int row = blockIdx.x;
  const int tid = threadIdx.x;
  const R dz = (R)ctl->dz;
  const bool guard = ctl->guard_pending != 0;
  if (tid == 0) s_flag = 0;
  C* uo = P.U_out ? P.U_out + (size_t)row * P.ld : nullptr;

  if constexpr (NC > 0) {
    if (P.plasma) {
      for (int i = tid; i < FIL_MAXCOMP * FIL_MAXRATE; i += T) {
        int c = i / FIL_MAXRATE, q = i % FIL_MAXRATE;
        tabs->lx[c][q] = (R)P.pp.lx[c][q];
        tabs->ly[c][q] = (R)P.pp.ly[c][q];
        tabs->sl[c][q] = (R)P.pp.sl[c][q];
      }
    }
  }
  // a step's pending guard without the transform round trip (the guarded
  // spectrum to s0_park and U_out); the initial solve and the plasma-only
  // launch of a non-paraxial step only need g E(t)
  const bool split = mode == 0 && guard;
  load_time_row<R, N>(P, X, row, guard && !split);
  if (split) split_guard_row<R, N>(P, X, Y, row);
  // largest |E|^2 of the row (the linear-only test below)
  R e2row = 0;
  if (!RAM && mode == 0 && P.nonlin && P.cc_max >= (R)0) {
#pragma unroll
    for (int m = 0; m < 16; ++m) {
      const C e = X[pad16(tid + m * T)];
      e2row = max(e2row, e.x * e.x + e.y * e.y);
    }
    e2row = block_max<R>(e2row, rscratch);
  }

  // ---- plasma: the ODE solve, or the surrogate's density for the rows the
  // reduction flagged.  On a check step every row is solved and the flagged
  // rows also measure the surrogate against the solution.
  if constexpr (NC > 0) {
    if (P.plasma) {
      const bool stepping = mode == 0 || mode == 4;
      const int slot = (P.nn_out && stepping) ? P.nn_slot[row] : -1;
      const bool nn_row = slot >= 0 && slot < ctl->nn_rows;
      const bool check_step = P.nn_out && stepping && ctl->nn_check;
      Aff<R, 1>* sc1 = reinterpret_cast<Aff<R, 1>*>(ascratch);
      R rmax;
      const float* gslot = P.nn_out + (size_t)slot * N * (P.nn_part ? NN_K : 1);
      if (nn_row && !check_step) {
        rmax = nn_density<R, N, NC>(P, *tabs, X, gslot, rho, kdrho, sc1, rscratch, false, slot);
      } else {
        rmax = plasma_row<R, N, NC>(P, *tabs, X, rho, kdrho, reinterpret_cast<R*>(Y), ascratch, rscratch, &s_flag,
                                    stepping ? (R)ctl->rhomax : (R)0, dz, &ych);
        if (check_step) {
          // rows not flagged carry rho0 in the surrogate form
          const R diff = nn_row ? nn_density<R, N, NC>(P, *tabs, X, gslot, rho, kdrho, sc1, rscratch, true, slot)
                                : max(rmax - (R)NC * P.pp.rho0, (R)0);
          if (tid == 0) atomic_max_nonneg(&ctl->nn_diff_acc, (double)diff);
        }
      }
      if (tid == 0) {
        atomic_max_nonneg(&ctl->rhomax_acc, (double)rmax);
        P.rho_end[row] = (double)rho[pad16(N - 1)];
        if (s_flag) atomicOr(&ctl->flags, FIL_FLAG_NEWTON);
      }
      if (P.store_plasma || mode == 4) {
        for (int m = 0; m < 16; ++m) {
          int j = tid + m * T;
          P.rho_g[(size_t)row * N + j] = rho[pad16(j)];
          P.kdrho_g[(size_t)row * N + j] = kdrho[pad16(j)];
        }
      }
    }
  }
  if (mode == 1 || mode == 4) return;

  // ---- the guarded spectrum: the analytic half in registers (from the
  // parked values, or the state itself when no guard is pending); the upper
  // half (when kept) is in U_out, where the stages read it
  C S0[EW], k1[EW], kp[EW], acc[EW];
  {
    const C* s0 = (split ? P.s0_park : P.S_in) + (size_t)row * P.ld;
#pragma unroll
    for (int m = 0; m < EW; ++m) {
      int k = tid + m * T;
      S0[m] = s0[k];
      if (!split && uo && uo != P.U_in + (size_t)row * P.ld) uo[k] = P.U_in[(size_t)row * P.ld + k];
      acc[m] = mk<R>(0, 0);
    }
  }
  // Linear-only row: with the plasma channels off for this row (no plasma,
  // or a row left at rho0 = 0 whose losses response is below 2^-30 of its
  // spectrum, ych false) every stage's Kerr increment is bounded by
  // |d(k)| <= max|C_cubic| max_t|E_s(t)|^3 (|F| <= |E|^3, guards <= 1, the
  // transform pair normalised by 1/N), and the step adds dz sum_s b_s d_s.
  // When dz max|C_cubic| max|E|^3 <= 2^-31 max_k |S0(k)| (a factor 2 over
  // 2^-30 covers the stage fields' departure from E, itself of that order)
  // the step changes no spectral component by more than 2^-30 of the row's
  // largest, below FP32 resolution of the row, and the stages are skipped.
  bool lin_only = false;
  if (!RAM && P.nonlin && P.cc_max >= (R)0) {
    const bool plas_row = NC > 0 && (P.has_free || P.has_losses) && ych;
    R s2 = 0;
#pragma unroll
    for (int m = 0; m < EW; ++m) s2 = max(s2, S0[m].x * S0[m].x + S0[m].y * S0[m].y);
    s2 = block_max<R>(s2, rscratch);
    const R emax = sqrt(e2row);
    lin_only = !plas_row &&
               dz * P.babs * (P.has_cubic ? P.cc_max : (R)0) * emax * e2row <= (R)4.656612873077393e-10 * sqrt(s2);
  }
  if (P.nonlin && !lin_only) {
    int iy;
    const R gs = row_guard(P, row, &iy);
    // One call site of stage_rhs for every method (it inlines the row's
    // transforms).  RK2/3/4: U_s = S0 + dz (A0 k1 + A1 k_prev), k1 and
    // k_prev in registers.  Tsitouras: U_s = S0 + h sum_j a_sj k_j with the
    // k_j in this row's slots of tk (each thread reads back only the points
    // it wrote); the first and the seventh stage swap slots on acceptance
    // (first same as last).
    const int tsit = TS ? P.tsit : 0;   // compiled out of the RK2/3/4 kernels
    const int ns = tsit ? (tsit == 2 ? 7 : 6) : P.ns;
    C* tk = tsit ? P.tk + (size_t)row * 7 * NH : nullptr;
    // the adaptive controller lives in shared memory (thread 0 updates it
    // between two barriers): no FP64 state is held in registers across the
    // stages
    if (tsit == 2) {
      if (tid == 0) {
        ode_begin(s_ode.o, ctl->dz);
        s_ode.k1s = 0;
        s_ode.rej = 0;
      }
      __syncthreads();
    }
    int s = 0;
    for (;;) {
      const R h = tsit == 2 ? (R)s_ode.o.h : dz;
      const int k1s = tsit == 2 ? s_ode.k1s : 0;   // slot of k_1 (0 or 6)
      auto slot = [&](int j) -> C* { return tk + (size_t)(j == 0 ? k1s : (j == 6 ? 6 - k1s : j)) * NH; };
      auto u = [&](int m) -> C {
        if (!tsit) return s > 0 ? S0[m] + (dz * (R)P.A0[s]) * k1[m] + (dz * (R)P.A1[s]) * kp[m] : S0[m];
        const int k = tid + m * T;
        C v = S0[m];
        if (s == 6) return v + h * acc[m];
        for (int j = 0; j < s; ++j) v = v + (h * P.ta[s][j]) * slot(j)[k];
        return v;
      };
      auto d = [&](int m, C v) {
        if (!tsit) {
          if (s == 0) k1[m] = v;
          kp[m] = v;
          acc[m] = acc[m] + (R)P.B[s] * v;
          return;
        }
        slot(s)[tid + m * T] = v;
        if (s < 6) acc[m] = acc[m] + P.ta[6][s] * v;
      };
      stage_rhs<R, N, NC, RAM>(P, X, Y, rho, kdrho, gs, iy, ych, uo, u, d);
      if (++s < ns) continue;
      if (tsit != 2) break;
      // the attempt's error norm over the row (FP64 sum in a fixed order)
      double q = 0;
#pragma unroll
      for (int m = 0; m < EW; ++m) {
        const int k = tid + m * T;
        C e = mk<R>(0, 0);
#pragma unroll
        for (int j = 0; j < 7; ++j) e = e + P.tbt[j] * slot(j)[k];
        e = h * e;
        const C y1 = S0[m] + h * acc[m];
        const double sc = P.atol + P.rtol * fmax(sqrt((double)cabs2(S0[m])), sqrt((double)cabs2(y1)));
        const double r = sqrt((double)cabs2(e)) / sc;
        q += r * r;
      }
      q = block_sum<double>(q, s_dred);   // ends with a barrier
      if (tid == 0) {
        int fin;
        const int ok = ode_after(s_ode.o, sqrt(q / (double)NH), ctl->dz, &fin);
        if (ok) s_ode.k1s = 6 - s_ode.k1s;
        else s_ode.rej += 1;
        s_ode.ok = ok;
        s_ode.fin = fin;
        if (fin) {
          atomicAdd(&ctl->ode_attempts, (unsigned long long)s_ode.o.attempts);
          atomicAdd(&ctl->ode_rejects, (unsigned long long)s_ode.rej);
          if (fin == 2) atomicOr(&ctl->flags, FIL_FLAG_ODE);
        }
      }
      __syncthreads();
      const int ok = s_ode.ok, fin = s_ode.fin, k1n = s_ode.k1s;
      // the next attempt starts at stage 2: its sum of b_s k_s holds k_1
      // (after the last one S0 is the result: the sum is cleared).  Thread 0
      // writes s_ode again only after the next attempt's block_sum barrier.
#pragma unroll
      for (int m = 0; m < EW; ++m) {
        const int k = tid + m * T;
        if (ok) S0[m] = S0[m] + h * acc[m];
        acc[m] = fin ? mk<R>(0, 0) : P.ta[6][0] * tk[(size_t)k1n * NH + k];
      }
      if (fin) break;
      s = 1;
    }
  }
#pragma unroll
  for (int m = 0; m < EW; ++m) {
    const int k = tid + m * T;
    C v = S0[m] + dz * acc[m];
    if (P.l_kzr) v = table_prop<R>(P.l_kzr, P.l_kg, (size_t)row * P.ld + k, v, (double)ctl->dz);   // T geometry
    write_out<R>(P, row, k, v);
  }
  if (uo && P.u_kzr) {
    // linear step of the upper half in r-space (RT; the lower half's
    // follows in the Hankel transforms; XYT transforms both halves)
    const double dzd = ctl->dz;
    const size_t base = (size_t)row * P.ld;
#pragma unroll 2
    for (int m = 0; m < EW; ++m) {
      const int k = tid + m * T;
      uo[k] = upper_prop<R>(P, base + k, uo[k], dzd);
    }
  }
  // T geometry: the step's linear part is done; the field guard follows at
  // the next load (one block)
  if (P.l_kzr && tid == 0) ctl->guard_pending = 1;
}

// One RK stage of a non-paraxial step (QPARAXIAL = false).  func! then
// transforms its sum along r before the prefactor
// (nonlinear_propagators.jl:58-63), so every stage is one launch with the
// Hankel pair and i QZ(kt, w) in between (api.cu); the density rows come
// from the step's plasma launch (k_rowstep mode 4) in rho_g, kdrho_g.
// Stage 0 (np_stage = 0): E(t) = guard * fft(S_in), t -> w; S0 to np_S0,
//   the upper half to U_out; stage 0's paraxial right-hand side to S_out.
// Stage s >= 1: the stage input S0 + dz (A0 k1 + A1 k_prev) from np_S0,
//   np_K1 and np_KS (the transformed right-hand sides of stages 0 and
//   s - 1), the running sum np_ACC += B[s-1] k_{s-1}; this stage's paraxial
//   right-hand side to S_out.
template <typename R, int N, int NC, bool RAM>
__global__ void __launch_bounds__(N / 16) k_rowstage(RowParams<R> P) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2, EW = NH / T, NP = N + N / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* X = reinterpret_cast<C*>(smem_raw);
  C* Y = X + NP;
  R* rho = reinterpret_cast<R*>(Y + NP);                 // [NP], pad16 index
  R* kdrho = rho + NP;
  const DevCtl* ctl = P.ctl;
  if (ctl->done) return;
  const int row = blockIdx.x;
  const int tid = threadIdx.x;
  const R dz = (R)ctl->dz;
  const int s = P.np_stage;
  const size_t rb = (size_t)row * P.ld;
  C* uo = P.U_out ? P.U_out + rb : nullptr;
  if constexpr (NC > 0) {
    if (P.plasma) {
#pragma unroll 4
      for (int m = 0; m < 16; ++m) {
        int j = tid + m * T;
        rho[pad16(j)] = P.rho_g[(size_t)row * N + j];
        kdrho[pad16(j)] = P.kdrho_g[(size_t)row * N + j];
      }
    }
  }
  int iy;
  const R gs = row_guard(P, row, &iy);
  auto d = [&](int m, C v) { write_out<R>(P, row, tid + m * T, v); };
  if (s == 0) {
    // the guarded spectrum without the transform round trip
    // (load_time_row_split parks it in s0_park), kept in np_S0
    C S0[EW];
    if (ctl->guard_pending) {
      load_time_row_split<R, N>(P, X, Y, row);
#pragma unroll
      for (int m = 0; m < EW; ++m) {
        const int k = tid + m * T;
        S0[m] = P.s0_park[rb + k];
        P.np_S0[rb + k] = S0[m];
      }
    } else {
#pragma unroll
      for (int m = 0; m < EW; ++m) {
        const int k = tid + m * T;
        S0[m] = P.S_in[rb + k];
        P.np_S0[rb + k] = S0[m];
        if (uo && uo != P.U_in + rb) uo[k] = P.U_in[rb + k];
      }
    }
    auto u = [&](int m) -> C { return S0[m]; };
    stage_rhs<R, N, NC, RAM>(P, X, Y, rho, kdrho, gs, iy, true, uo, u, d);
  } else {
    const R a0 = (R)P.A0[s], a1 = (R)P.A1[s], bp = (R)P.B[s - 1];
    auto u = [&](int m) -> C {
      const int k = tid + m * T;
      const C k1 = P.np_K1[rb + k];
      const C kp = (s == 1) ? k1 : P.np_KS[rb + k];
      P.np_ACC[rb + k] = (s == 1) ? bp * k1 : P.np_ACC[rb + k] + bp * kp;
      return P.np_S0[rb + k] + (dz * a0) * k1 + (dz * a1) * kp;
    };
    stage_rhs<R, N, NC, RAM>(P, X, Y, rho, kdrho, gs, iy, true, uo, u, d);
  }
}

// Non-paraxial step, after the last stage's Hankel pair: S_out (operand or
// row layout) = S0 + dz (ACC + B_last k_last), and the upper half's linear
// step.  One block per row.
template <typename R>
__global__ void __launch_bounds__(256) k_np_combine(RowParams<R> P, int nh) {
  typedef typename C2T<R>::type C;
  const DevCtl* ctl = P.ctl;
  if (ctl->done) return;
  const int row = blockIdx.x;
  const R dz = (R)ctl->dz;
  const double dzd = ctl->dz;
  const R bl = (R)P.B[P.ns - 1];
  const size_t rb = (size_t)row * P.ld;
  const R sc = (P.out_T && P.out_scale) ? P.out_scale[row] : (R)1;
  for (int k = threadIdx.x; k < nh; k += blockDim.x) {
    const C v = P.np_S0[rb + k] + dz * (P.np_ACC[rb + k] + bl * P.np_KS[rb + k]);
    if (P.out_T) {
      R* base = reinterpret_cast<R*>(P.S_out);
      base[(size_t)(2 * k) * P.ldT + row] = sc * v.x;
      base[(size_t)(2 * k + 1) * P.ldT + row] = sc * v.y;
    } else {
      P.S_out[rb + k] = v;
    }
    if (P.U_out && P.u_kzr) P.U_out[rb + k] = upper_prop<R>(P, rb + k, P.U_out[rb + k], dzd);
  }
}

// ---------------------------------------------------------------------------
// Inputs of the learned surrogate for the row in X (surrogate.cuh):
// f0 = ln(max(I, 1e-30)) / 16, f1 = Re(E)^2 / max(I, 1e-30) and
// f2 = ln(max(S_j, 1e-30)) / 16 with S_j = dt sum_{i<j} Wb_i, Wb_i the base rate
// of step i (the integrator's quadrature of W = sum_c W_c rho_nt,c / rho_nt
// over t_i, the midpoint of the interpolated field and t_{i+1}, as in
// nn_density).  Thread t owns j = 16t .. 16t+15; f is [3][N] (BF16).
template <typename R, int N>
FIL_DEV void nn_features(const RowParams<R>& P, const typename C2T<R>::type* X, __nv_bfloat16* f, int slot) {
  typedef typename C2T<R>::type C;
  __shared__ PlasmaSmem<R> tabs;
  __shared__ Aff<R, 1> sc[32];
  const PlasmaParams<R>& pp = P.pp;
  for (int i = threadIdx.x; i < FIL_MAXCOMP * FIL_MAXRATE; i += blockDim.x) {
    const int c = i / FIL_MAXRATE, q = i % FIL_MAXRATE;
    tabs.lx[c][q] = (R)pp.lx[c][q];
    tabs.ly[c][q] = (R)pp.ly[c][q];
    tabs.sl[c][q] = (R)pp.sl[c][q];
  }
  __syncthreads();
  R qw[3] = {0, 0, 0};
  for (int st = 0; st < pp.ns; ++st) qw[pp.pidx[st]] += pp.b[st];
  auto wsum = [&](C e) -> R {
    const R I = pp.ereal ? e.x * e.x : e.x * e.x + e.y * e.y;
    R w = 0;
    for (int c = 0; c < pp.nc; ++c) {
      R sl;
      w += rate_eval<R>(pp, tabs, c, I, &sl) * pp.rho_nt[c];
    }
    return w;
  };
  const int j0 = threadIdx.x * 16;
  const R scale = pp.dt / pp.rhont_sum;
  R wl[16];
  R tsum = 0;
  R wcur = wsum(X[pad16(j0)]);
#pragma unroll
  for (int q = 0; q < 16; ++q) {
    const int j = j0 + q;
    R w = 0;
    if (j < N - 1) {
      const C e0 = X[pad16(j)], e1 = X[pad16(j + 1)];
      const R wnext = wsum(e1);
      w = (qw[0] * wcur + qw[1] * wsum((R)0.5 * (e0 + e1)) + qw[2] * wnext) * scale;
      wcur = wnext;
    }
    wl[q] = w;
    tsum += w;
  }
  Aff<R, 1> G;
  G.L[0][0] = 0;
  G.B[0] = tsum;
  R S = aff_block_exclusive_scan<R, 1>(G, sc).B[0];
  if (P.nn_tflag) {
    // Tile flags.  g enters the density only through the avalanche term
    // kappa A_j dt (1 - e^{-S_j}) e^{g_j} (nn_density), at most e^{NN_G_HI}
    // times its g = 0 value.  A 128-point tile whose sum of that bound is at
    // most 2^-30 of the row's base exponent S_total changes the density by
    // less than 2^-30 of its scale with any g: there the density uses g = 0
    // (bit 0 clear).  The network runs on the tiles with bit 0 and on their
    // neighbours (bit 1), so that the receptive field (+-16 points over the
    // four layers) of every tile that uses g is computed.
    __shared__ R s_tot;
    __shared__ uint8_t s_act[N / 128];
    R kappa = 0;
    for (int c = 0; c < pp.nc; ++c) kappa += pp.rava_nt[c] * pp.rho_nt[c];
    R av = 0, Sj = S;
#pragma unroll
    for (int q = 0; q < 16; ++q) {
      const int j = j0 + q;
      if (j < N - 1) {
        const C e0 = X[pad16(j)], e1 = X[pad16(j + 1)];
        const C em = (R)0.5 * (e0 + e1);
        const R A = qw[0] * e0.x * e0.x + qw[1] * em.x * em.x + qw[2] * e1.x * e1.x;
        av += kappa * A * pp.dt * -expm1(-Sj);
      }
      Sj += wl[q];
    }
    // the tile's 8 threads (16 points each) are consecutive lanes
    av += __shfl_xor_sync(0xffffffffu, av, 1);
    av += __shfl_xor_sync(0xffffffffu, av, 2);
    av += __shfl_xor_sync(0xffffffffu, av, 4);
    if (threadIdx.x == blockDim.x - 1) s_tot = S + tsum;
    __syncthreads();
    const int tile = j0 / 128;
    if ((threadIdx.x & 7) == 0) s_act[tile] = av * exp((R)NN_G_HI) > ldexp(s_tot, -30) ? 1 : 0;
    __syncthreads();
    if ((threadIdx.x & 7) == 0) {
      constexpr int NT = N / 128;
      const uint8_t a = s_act[tile];
      const uint8_t d = a | (tile > 0 ? s_act[tile - 1] : 0) | (tile + 1 < NT ? s_act[tile + 1] : 0);
      P.nn_tflag[(size_t)slot * NT + tile] = (uint8_t)(a | (d << 1));
    }
    if (threadIdx.x == 0) {
      // the row's tiles that the network runs on, appended to the tile list
      // at a range reserved by the count (the list's order does not matter:
      // every tile is computed on its own)
      constexpr int NT = N / 128;
      auto runs = [&](int t) { return s_act[t] | (t > 0 ? s_act[t - 1] : 0) | (t + 1 < NT ? s_act[t + 1] : 0); };
      int run = 0;
      for (int t = 0; t < NT; ++t) run += runs(t);
      int at = atomicAdd(&P.ctl->nn_tiles, run);
      if (P.nn_tlist)
        for (int t = 0; t < NT; ++t)
          if (runs(t)) P.nn_tlist[at++] = slot * NT + t;
    }
  }
  // the thread's 16 consecutive points of each channel, packed and written
  // as two 16-byte stores per channel (one channel at a time, the scanned
  // channel first so that its per-step rates are released early)
#pragma unroll
  for (int cc = 0; cc < 3; ++cc) {
    const int ch = (cc + 2) % 3;
    uint32_t pk[8];
#pragma unroll
    for (int q = 0; q < 16; q += 2) {
      float v[2];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const C e = X[pad16(j0 + q + u)];
        const float I = fmaxf((float)(e.x * e.x + e.y * e.y), 1e-30f);
        if (ch == 0) v[u] = __logf(I) * 0.0625f;
        else if (ch == 1) v[u] = (float)(e.x * e.x) / I;
        else {
          v[u] = __logf(fmaxf((float)S, 1e-30f)) * 0.0625f;
          S += wl[q + u];
        }
      }
      const __nv_bfloat162 h = __floats2bfloat162_rn(v[0], v[1]);
      pk[q / 2] = *reinterpret_cast<const uint32_t*>(&h);
    }
    uint4* d = reinterpret_cast<uint4*>(f + ch * N + j0);
    d[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    d[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
  }
}

// ---------------------------------------------------------------------------
// Reductions over the current field (FieldAnalyzers.jl:166-215): Imax,
// fluence per row F = sum_t |E|^2 dt, optionally |E|^2 itself into
// Iout[row][t] (for the power P[t] = sum_row w_row |E|^2, k_colsum).  Flags
// non-finite values.  The per-thread and
// per-warp sums run in the working precision (a pairwise sum of 4096
// positive terms: relative error below 1e-6 in FP32), the eight warp
// partials are joined in FP64.
template <typename R, int N>
__global__ void __launch_bounds__(N / 16) k_rowreduce(RowParams<R> P, double* fluence, R* Iout, int check_done) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NP = N + N / 16, NW = T / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* X = reinterpret_cast<C*>(smem_raw);
  R* rs = reinterpret_cast<R*>(X + NP);   // [3 * NW]
  DevCtl* ctl = P.ctl;
  if (check_done && ctl->done) return;
  const int row = blockIdx.x, tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
  load_time_row<R, N>(P, X, row, ctl->guard_pending != 0);
  R s[4] = {0, 0, 0, 0};
  R mx = 0, mr = 0;
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    int j = tid + m * T;
    C e = X[pad16(j)];
    R I = e.x * e.x + e.y * e.y;
    s[m & 3] += I;
    mx = max(mx, I);
    mr = max(mr, e.x * e.x);
    if (Iout) Iout[(size_t)row * N + j] = I;
  }
  R ts = warp_sum<R>((s[0] + s[1]) + (s[2] + s[3]));
  R tm = warp_max<R>(mx);
  R tr = warp_max<R>(mr);
  if (lane == 0) {
    rs[w] = ts;
    rs[NW + w] = tm;
    rs[2 * NW + w] = tr;
  }
  __syncthreads();
  __shared__ int s_slot;
  if (tid == 0) {
    double tot = 0, bm = 0, br = 0;
#pragma unroll
    for (int i = 0; i < NW; ++i) {
      tot += (double)rs[i];
      bm = fmax(bm, (double)rs[NW + i]);
      br = fmax(br, (double)rs[2 * NW + i]);
    }
    fluence[row] = tot * (double)P.dt;
    if (!isfinite(tot)) atomicOr(&ctl->flags, FIL_FLAG_NAN);
    else atomic_max_nonneg(&ctl->imax_acc, bm);
    // learned surrogate: the coming step needs the network (it is in use,
    // or the step is a check step) and the plasma solve would not skip the
    // row -> take a slot for its features
    int slot = -1;
    if (P.nn_feat && ctl->nn_on && (ctl->nn_use || ctl->nn_steps % ctl->nn_every == 0) && isfinite(tot)) {
      const double rho_prev = __longlong_as_double((long long)ctl->rhomax_acc);
      const double imax = P.pp.ereal ? br : bm;
      if (!plasma_row_negligible<R>(P.pp, imax, br, (double)P.pp.dt * (N - 1), rho_prev))
        slot = atomicAdd(&ctl->nn_count, 1);
    }
    if (P.nn_slot) P.nn_slot[row] = slot;
    s_slot = slot;
  }
  if (P.nn_feat) {
    __syncthreads();
    const int slot = s_slot;
    if (slot >= 0) nn_features<R, N>(P, X, P.nn_feat + (size_t)slot * 3 * N, slot);
  }
}

// Integral power spectrum (FieldAnalyzers.jl:180-197, 320-336), per row:
// the field as the analyzer sees it (E(t), the pending field guard applied,
// as k_rowreduce), its spectrum Sa = ifft(E) (FFTW's ifft, 1/N), the real
// spectrum Sr = aspec2rspec(Sa) on the nw = N/2 + 1 bins of rfftfreq, and
// out[row][k] = |2 Sr_k N dt|^2: with Sr_0 = Sa_0, Sr_k = Sa_k / 2 (0 < k <
// N/2) and the Nyquist bin Sr_{N/2} = Sa_{N/2} as the state holds it,
// 2 Sr_k N = c_k X_k, X = the unscaled +1 transform, c = 2, 1, ..., 1, 2.
// k_colsum then forms S[k] = sum_row w_row out[row][k].
template <typename R, int N>
__global__ void __launch_bounds__(N / 16) k_rowspec(RowParams<R> P, R* out) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* X = reinterpret_cast<C*>(smem_raw);
  const int row = blockIdx.x, tid = threadIdx.x;
  load_time_row<R, N>(P, X, row, P.ctl->guard_pending != 0);
  filfft::block_fft<C, N, +1>(X, P.tw);
  const R dt = P.dt;
  for (int k = tid; k <= NH; k += T) {
    const C x = X[pad16(k)];
    const R c = (k == 0 || k == NH) ? (R)2 : (R)1;
    const R a = c * dt;
    out[(size_t)row * (NH + 1) + k] = a * a * (x.x * x.x + x.y * x.y);
  }
}

// Power P[t] = sum_row w_row I[row][t] (FieldAnalyzers.jl:166-215): one
// thread per column t and block of 64 rows, a working-precision partial sum
// per block, FP64 atomics across the row blocks (16-way for 1000 rows).
template <typename R>
__global__ void __launch_bounds__(256) k_colsum(const R* __restrict__ I, const double* __restrict__ w,
                                                double* power, int nrows, int nt) {
  const int t = blockIdx.x * 256 + threadIdx.x;
  const int r0 = blockIdx.y * 64, r1 = min(r0 + 64, nrows);
  if (t >= nt) return;
  R a0 = 0, a1 = 0;
  int r = r0;
  for (; r + 1 < r1; r += 2) {
    a0 += (R)w[r] * I[(size_t)r * nt + t];
    a1 += (R)w[r + 1] * I[(size_t)(r + 1) * nt + t];
  }
  if (r < r1) a0 += (R)w[r] * I[(size_t)r * nt + t];
  atomicAdd(&power[t], (double)a0 + (double)a1);
}

// ---------------------------------------------------------------------------
// Field in: rows of E(t) (R complex, row-major) -> S = c_k ifft(E)[k], k < N/2
// with c_0 = 1, c_k = 2 (rsig2asig!, Fields.jl:115) or c_k = 1 (analytic).
template <typename R, int N>
__global__ void __launch_bounds__(N / 16) k_field_in(const typename C2T<R>::type* E, typename C2T<R>::type* S,
                                                     typename C2T<R>::type* U, int ld,
                                                     const typename C2T<R>::type* tw, int analytic) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16, NH = N / 2, EW = NH / T, NP = N + N / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* X = reinterpret_cast<C*>(smem_raw);
  (void)NP;
  const int row = blockIdx.x, tid = threadIdx.x;
  const C* src = E + (size_t)row * N;
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    int j = tid + m * T;
    X[pad16(j)] = src[j];
  }
  filfft::block_fft<C, N, +1>(X, tw);
  const R invN = (R)1 / (R)N;
#pragma unroll
  for (int m = 0; m < EW; ++m) {
    int k = tid + m * T;
    R c = (analytic || k == 0) ? invN : (R)2 * invN;
    S[(size_t)row * ld + k] = c * X[pad16(k)];
    // upper half: kept as given for an analytic field, zero after rsig2asig!
    if (U) U[(size_t)row * ld + k] = analytic ? invN * X[pad16(k + N / 2)] : mk<R>(0, 0);
  }
}

// Field out: E(t) = guard * fft(S), rows row-major.
template <typename R, int N>
__global__ void __launch_bounds__(N / 16) k_field_out(RowParams<R> P, typename C2T<R>::type* E) {
  typedef typename C2T<R>::type C;
  constexpr int T = N / 16;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  C* X = reinterpret_cast<C*>(smem_raw);
  const int row = blockIdx.x, tid = threadIdx.x;
  load_time_row<R, N>(P, X, row, P.ctl->guard_pending != 0);
  C* dst = E + (size_t)row * N;
#pragma unroll
  for (int m = 0; m < 16; ++m) {
    int j = tid + m * T;
    dst[j] = X[pad16(j)];
  }
}
