/*
 * filament_gb.h -- C ABI of the GB300-native per-z-step propagation loop.
 *
 * This library replaces the hot loop of Filament.jl:
 *
 *   src/Filament.jl:123-172   main_loop: dz = dzadaptive(analyzer); zstep; analyze!
 *   src/modules/Models.jl:75-121   Models.zstep(z, dz, grid, field, guard, model)
 *   src/modules/AdaptiveSteps.jl:91-107   the dz controller
 *   src/modules/FieldAnalyzers.jl:166-215  the reductions the controller needs
 *
 * A handle owns all device state of one problem (one field on one grid).  The
 * caller computes the physics set-up once on the host in FP64 (units, grids,
 * medium, guards, propagator and response tables: src/modules/Units.jl,
 * Grids.jl, Media.jl, Guards.jl, linear_propagators/spectral.jl,
 * nonlinear_propagators.jl, the medium_responses files,
 * plasma_equations/photoionization_avalanche.jl) and passes 1-D tables plus
 * the Hankel matrix; large 2-D tables (KZ, QZ, Kguard) are regenerated on the
 * device from them and never stored.
 *
 * Conventions
 *  - Return codes: FIL_OK (0) or a positive stop reason on success, negative
 *    on error; fil_last_error() gives the message.
 *  - Host pointers are borrowed for the duration of the call only.
 *  - One handle = one CUDA stream; a handle is not thread-safe, distinct
 *    handles are independent.
 *  - Units are the reference's dimensionless units (src/modules/Units.jl):
 *    z in zu, t in tu, |E|^2 in Iu, rho in rhou.  Transverse wave numbers and
 *    propagation constants are passed pre-multiplied by zu.
 *  - Field arrays crossing the boundary use the reference layout
 *    (column-major E[Nr, Nt] / E[Nx, Ny, Nt], FIL_LAYOUT_COLMAJOR) or the
 *    library's row layout (time fastest, FIL_LAYOUT_ROWMAJOR).
 */
#ifndef FILAMENT_GB_H
#define FILAMENT_GB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FIL_ABI_VERSION 1

/* ---- return codes --------------------------------------------------------*/
#define FIL_OK 0
#define FIL_STOP_ZMAX 1        /* fil_run: z reached zmax (Filament.jl:123)   */
#define FIL_STOP_ISTOP 2       /* fil_run: Imax > Istop (Filament.jl:160-164) */
#define FIL_STOP_NMAX 3        /* fil_run: step budget exhausted              */
#define FIL_ERR_ARG (-1)       /* bad argument / configuration                */
#define FIL_ERR_CUDA (-2)      /* CUDA runtime error                          */
#define FIL_ERR_NAN (-3)       /* non-finite value detected in the field      */
#define FIL_ERR_TIMEOUT (-4)   /* a bounded device wait gave up               */
#define FIL_ERR_UNSUPPORTED (-5) /* valid reference option not built here     */
#define FIL_ERR_STATE (-6)     /* call order (e.g. step before set_field)     */
#define FIL_ERR_NOMEM (-7)     /* device allocation failed                    */

/* ---- geometry (src/modules/Grids.jl:10-27) --------------------------------*/
#define FIL_GEOM_R 0
#define FIL_GEOM_T 1
#define FIL_GEOM_RT 2
#define FIL_GEOM_XY 3
#define FIL_GEOM_XYT 4

/* ---- precision forms ------------------------------------------------------*/
#define FIL_PREC_MIXED 0  /* complex FP32 field, FFTs and nonlinear terms;
                             FP64 controller, energy/fluence reductions     */
#define FIL_PREC_FP64 1   /* plain method: FP64 everywhere                  */

/* ---- explicit Runge-Kutta methods (ODEIntegrators RK2/RK3/RK4) ----------- */
#define FIL_ALG_RK2 2     /* midpoint                                       */
#define FIL_ALG_RK3 3     /* Kutta third order                              */
#define FIL_ALG_RK4 4     /* classic fourth order                           */
/* Tsitouras 5(4) pair (Ch. Tsitouras, Comput. Math. Appl. 62 (2011) 770-775),
 * nonlinear step only (input ALG), paraxial prefactor (QPARAXIAL = true):   */
#define FIL_ALG_TSIT5 5   /* fifth order, one step of dz: six evaluations   */
#define FIL_ALG_ATSIT5 6  /* the same pair with the embedded error estimate:
                             substeps of [z, z + dz] chosen per transverse
                             point (rows are independent ODE systems in the
                             paraxial step), err = RMS over the point's
                             spectrum of |e| / (atol + rtol max(|y0|, |y1|)),
                             accept err <= 1, h <- h min(fmax, max(0.2,
                             0.9 err^-1/5)), fmax 10 (1 after a rejection),
                             first-same-as-last; see FIL_OPT_ODE_RTOL/ATOL */

/* ---- nonlinear response channels (src/modules/medium_responses) --------- */
#define FIL_RESP_CUBIC 1u   /* cubic.jl: F = Re(E)^3 or 3/4|E|^2 Re(E)       */
#define FIL_RESP_FREE 2u    /* current_free.jl: F = rho Re(E)                */
#define FIL_RESP_LOSSES 4u  /* current_losses.jl: F = Kdrho Re(E)/|E|^2      */
#define FIL_RESP_RAMAN 8u   /* raman.jl: F = (H * Re(E)^2) Re(E)             */

/* ---- field dtypes and layouts ---------------------------------------------*/
#define FIL_DTYPE_C64 0     /* interleaved complex float                     */
#define FIL_DTYPE_C128 1    /* interleaved complex double                    */
#define FIL_DTYPE_F32 2
#define FIL_DTYPE_F64 3
#define FIL_LAYOUT_COLMAJOR 0 /* reference layout: transverse index fastest  */
#define FIL_LAYOUT_ROWMAJOR 1 /* time fastest                                */

/* ---- options (fil_set_option) --------------------------------------------*/
#define FIL_OPT_STORE_PLASMA 1 /* keep rho(t), Kdrho(t) of the last plasma
                                  solve for fil_get_rho (extra HBM writes) */
#define FIL_OPT_XYT_GUARD_BUGCOMPAT 2 /* reproduce Guards.jl:314 (t window
                                  indexed by the y index) in XYT           */
#define FIL_OPT_CLAMP_LAST_DZ 3 /* fil_run shortens the last step so that z
                                  lands on zmax exactly (off = reference)  */
#define FIL_OPT_TIMING 4       /* benchmark mode (value m >= 1, 0 = off):
                                  fil_run runs steps one at a time and times
                                  every m-th (the first included): a buffer
                                  larger than L2 is written before it and
                                  its per-kernel device times are recorded
                                  (fil_kernel_times)                       */
#define FIL_OPT_DHT_SIMT 6      /* mixed form: run the Hankel transforms as
                                  FP32 CUDA-core GEMMs instead of the
                                  tcgen05 tensor-core GEMMs on exact FP16
                                  slices (the default)                    */
#define FIL_OPT_ANALYTIC_PROJECTION 5 /* 1: drop the upper half of the
                                  spectrum (bins Nt/2..Nt-1, the negative
                                  frequencies the time guard creates) after
                                  every t->w transform, i.e. keep only the
                                  analytic half.  0 (default): keep it as the
                                  reference does -- it enters the time-domain
                                  field and receives the linear step's
                                  exp(i KZ dz) Kguard Wguard in r-space
                                  (spectral.jl:16-26; its Hankel transform
                                  covers the first Nt/2 columns).  RT only;
                                  XYT always projects.                     */
#define FIL_OPT_ODE_RTOL 7     /* FIL_ALG_ATSIT5 relative tolerance, value =
                                  rtol x 1e12 (default 1e9: rtol = 1e-3)   */
#define FIL_OPT_ODE_ATOL 8     /* FIL_ALG_ATSIT5 absolute tolerance in the
                                  units of the state (spectral amplitude in
                                  T, RT, XYT; field in R, XY), value = atol x
                                  1e12 (default 1e6: atol = 1e-6)          */

typedef struct fil_config {
  int32_t abi_version;   /* FIL_ABI_VERSION                                  */
  int32_t geometry;      /* FIL_GEOM_*                                       */
  int32_t precision;     /* FIL_PREC_*                                       */
  int32_t alg;           /* FIL_ALG_*: nonlinear step (input ALG)            */
  int32_t n1;            /* Nr (R, RT) or Nx (XY, XYT); 1 for T              */
  int32_t n2;            /* Ny (XY, XYT); 1 otherwise                        */
  int32_t nt;            /* Nt (T, RT, XYT); 1 for R, XY                     */
  int32_t nonlinearity;  /* NONLINEARITY                                     */
  int32_t plasma;        /* PLASMA                                           */
  int32_t kparaxial;     /* KPARAXIAL (linear propagator)                    */
  int32_t qparaxial;     /* QPARAXIAL (nonlinear prefactor)                  */
  uint32_t resp_mask;    /* OR of FIL_RESP_* channels present                */
  int32_t cubic_thg;     /* 1: F=Re(E)^3, 0: F=3/4|E|^2 Re(E)  (cubic.jl)     */
  int32_t losses_ereal;  /* current_losses EREAL: 1 Re(E)^2, 0 |E|^2         */
  int32_t raman_thg;     /* raman.jl THG switch                              */
  int32_t plasma_alg;    /* FIL_ALG_* of the plasma ODE (plasma dict "ALG")  */
  int32_t plasma_ereal;  /* plasma dict "EREAL"                              */
  int32_t plasma_kdep;   /* plasma dict "KDEP"                               */
  int32_t plasma_ncomp;  /* number of ionising species (<= 4)                */
  int32_t rate_n;        /* points in each tabulated ionisation rate         */
  int32_t reserved_i[8];
  double dt;             /* time step t[2]-t[1] (tu)                         */
  double dz0;            /* AdaptiveSteps dz0 (dz_initial)                   */
  double phimax;         /* dzphimax                                         */
  double phik;           /* phi_kerr  (AdaptiveSteps.jl:46-58)               */
  double phip;           /* phi_plasma (AdaptiveSteps.jl:60-72); 0: no plasma */
  double istop;          /* Istop (Iu)                                       */
  double rho0;           /* initial density of each species (rhou)           */
  double dxdy;           /* XY/XYT: dx*dy (area element)                     */
  double reserved_d[8];
} fil_config;

/* Host FP64 tables.  "complex" tables are interleaved (re, im) pairs.
 * Frequencies are in FFTW order (fftfreq), length nt.                       */
typedef struct fil_tables {
  /* transverse axes */
  const double* kt1;     /* [n1] R/RT: k_i*unit.k*zu; XY/XYT: kx*unit.kx*zu */
  const double* kt2;     /* [n2] XY/XYT: ky*unit.ky*zu; else NULL            */
  const double* guard1;  /* [n1] field guard Rguard / Xguard                 */
  const double* guard2;  /* [n2] field guard Yguard; else NULL               */
  const double* guardt;  /* [nt] field guard Tguard; NULL for R, XY          */
  const double* sguard1; /* [n1] XY/XYT spectral guard KXguard; else NULL    */
  const double* sguard2; /* [n2] XY/XYT spectral guard KYguard; else NULL    */
  const double* kmax;    /* [nt] R/RT: k(w)*sind(kguard)*zu for Kguard      */
  const double* wguard;  /* [nt] Wguard(w); NULL = 1                         */
  /* propagation constants (linear_propagators/spectral.jl:160-184)        */
  const double* beta;    /* complex [nt] beta(w)*zu                          */
  const double* dfr;     /* complex [nt] (beta(w) - w/vf)*zu                 */
  /* nonlinear prefactor, paraxial (nonlinear_propagators.jl:220-229)       */
  const double* qz;      /* complex [nt] QZ(w)                               */
  /* per-channel Rnl(w), summed over responses of that channel              */
  const double* rnl_cubic;  /* complex [nt]                                  */
  const double* rnl_free;   /* complex [nt]                                  */
  const double* rnl_losses; /* complex [nt]                                  */
  const double* rnl_raman;  /* complex [nt]                                  */
  const double* raman_h;    /* complex [nt] H(w) (raman.jl:21-31)            */
  /* Hankel transform (R, RT): E <- diag(1/s) T D T diag(s) E               */
  const double* dht;     /* [n1*n1] row-major T_ij                           */
  const double* dht_s;   /* [n1] s_i = R/|J1(j_i)|                           */
  const double* rdr;     /* [n1] r_i*dr_i (FieldAnalyzers.jl:160)            */
  /* plasma (photoionization_avalanche.jl:1-116)                            */
  const double* rho_nt;  /* [ncomp] fraction*rho_nt/rhou                     */
  const double* rava;    /* [ncomp] avalanche coefficient Rava              */
  const double* kfix;    /* [ncomp] ceil(Ui/(hbar w0)) (KDEP = false)        */
  const double* rate_lx; /* [ncomp*rate_n] ln(I) knots of W(I), Iu units    */
  const double* rate_ly; /* [ncomp*rate_n] ln(W) at the knots, 1/tu units    */
} fil_tables;

typedef struct fil_stats {
  double z;         /* current z (zu)                                        */
  double dz;        /* last dz                                               */
  double imax;      /* max |E|^2 of the current field                        */
  double rhomax;    /* max rho of the last plasma solve                      */
  double energy;    /* W = 2 pi sum F(r) r dr (RT) or sum F dx dy (XYT)      */
  int64_t steps;    /* z-steps taken on this handle                          */
  int32_t status;   /* last stop reason / error code                         */
  int32_t flags;    /* device status bits: 1 NaN seen, 2 Istop, 4 Newton
                       iteration cap hit in the plasma scan, 8 an adaptive
                       nonlinear step (FIL_ALG_ATSIT5) gave up after 256
                       attempts at one point; bits 8-15: the largest
                       Newton iteration count of any plasma solve          */
} fil_stats;

typedef struct fil_handle fil_handle;

/* ---- lifecycle ------------------------------------------------------------*/
/* Builds the device state of one problem.  Replaces the device part of
 * Filament.run's construction of Field, Guard and Model
 * (src/Filament.jl:72-79, src/modules/Fields.jl:96-160,
 * src/modules/Models.jl:33-72).  Tables are copied; the caller may free them. */
int fil_create(const fil_config* cfg, const fil_tables* tab, fil_handle** out);

/* Frees all device memory of the handle. */
int fil_destroy(fil_handle* h);

/* Last error message of the handle (h may be NULL for create errors). */
const char* fil_last_error(const fil_handle* h);

/* Sets an FIL_OPT_* option. */
int fil_set_option(fil_handle* h, int option, int64_t value);

/* ---- field in / out -------------------------------------------------------*/
/* Uploads the initial field.  analytic = 0 converts the real signal to an
 * analytic signal first (AnalyticSignals.rsig2asig!, Fields.jl:115,152);
 * analytic = 1 takes E as an analytic signal (restart from a saved field,
 * examples/RT/gauss_restart.jl).  With PLASMA on, the plasma equation is
 * solved once on the new field (Models.jl:66) so that rhomax is defined.   */
int fil_set_field(fil_handle* h, const void* E, int dtype, int layout,
                  int analytic);

/* Downloads the current field E(t) (after the last step's field guard,
 * Models.jl:116-118). */
int fil_get_field(fil_handle* h, void* E, int dtype, int layout);

/* Downloads rho(t) (which=0) or Kdrho(t) (which=1) of the last plasma solve
 * (needs FIL_OPT_STORE_PLASMA). */
int fil_get_plasma(fil_handle* h, int which, void* out, int dtype, int layout);

/* ---- stepping -------------------------------------------------------------*/
/* One Lie-split z-step with the given dz: Models.zstep (Models.jl:75-121):
 * plasma -> t->w -> nonlinear RK step -> linear propagator -> w->t -> field
 * guard.  z is the position after the step (the reference passes z+dz).   */
int fil_step(fil_handle* h, double z, double dz);

/* The main loop on the device (Filament.jl:123-172): per step the adaptive
 * dz (AdaptiveSteps.jl:96-107) from the Imax/rhomax of the previous field,
 * the z-step, the Imax > Istop stop test.  Runs until z >= zmax, Istop, or
 * nmax steps.  Returns FIL_STOP_* or an error; fills *stats (may be NULL). */
int fil_run(fil_handle* h, double z0, double zmax, int64_t nmax,
            fil_stats* stats);

/* ---- diagnostics (FieldAnalyzers.jl:166-215, 272-353) ----------------------*/
/* Reductions over the current field, FP64: Imax, rhomax, energy W in *st;
 * fluence F[n1*n2] = sum_t |E|^2 dt; power P[nt] = 2 pi sum_r |E|^2 r dr
 * (RT) or sum_xy |E|^2 dx dy (XYT); rho_end[n1*n2] = rho(t_end).  Any array
 * pointer may be NULL.                                                      */
int fil_analyze(fil_handle* h, fil_stats* st, double* fluence, double* power,
                double* rho_end);

/* Integral power spectrum of the current field (FieldAnalyzers.jl:180-197
 * RT, :320-336 XYT): S[k] = sum over the transverse points of
 * w |2 Sr_k Nt dt|^2, Sr = aspec2rspec(ifft(E)) on the nw = Nt/2 + 1 bins of
 * rfftfreq(Nt), w = 2 pi r dr (RT), dx dy (XYT), 1 (T).  Bin 0 and the
 * Nyquist bin count twice (Sr_0 = Sa_0; the Nyquist bin as the state holds
 * it), the others once (Sr_k = Sa_k / 2).  T, RT, XYT; nw = Nt/2 + 1. */
int fil_analyze_spectrum(fil_handle* h, double* S, int nw);

/* Current controller state without launching work beyond a copy. */
int fil_get_stats(fil_handle* h, fil_stats* st);

/* Average device time per step of each kernel family over the timed steps
 * since FIL_OPT_TIMING was set, in ms: 0 row kernel (plasma + nonlinear
 * step, with the surrogate network when armed), 1 forward transverse
 * transform + propagator, 2 inverse transform, 3 reductions + controller,
 * 4 whole step; ms[5] = number of timed steps; ms[6] = the surrogate
 * network's part of ms[0].                                                  */
int fil_kernel_times(fil_handle* h, double* ms, int n);

/* Adaptive nonlinear step (FIL_ALG_ATSIT5): counts since fil_create, summed
 * over the transverse points and steps: out[0] substep attempts, out[1]
 * rejected attempts.  Zero for the fixed-step methods.                     */
int fil_get_ode_stats(fil_handle* h, int64_t out[2]);

/* ---- linear propagator without device allocation ----------------------------
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory where they need the step (inside a region where cudaMalloc is not
 * allowed, or a host that hands out fixed device pools): applies the linear
 * propagator of an RT z-step, out = M2 P M1 in, to caller-owned FP32 device
 * buffers, where M1 = T diag(s) and M2 = diag(1/s) T are the Hankel pair
 * ([mpad][mpad], row-major, zero padded), `in`/`out` are the half spectrum
 * [mpad][nh] complex (interleaved), and P = exp(i KZ dz) * guard is built from
 * kt2[mpad] (kt^2, zu units), beta[2*nh], dfr[2*nh] (interleaved complex),
 * kmax2[nh] and wg[nh] (NULL = no guard), with KPARAXIAL as kparaxial.
 * mpad and 2*nh must be multiples of 128 and mpad*2*nh <= 4194304.
 * The one intermediate lives in a fixed 16 MiB __device__ array that every
 * GPU loading this library holds until exit; the call allocates and frees
 * nothing.  The first call on a device looks up that array's device address
 * (do it before any stream capture); the lookup is redone when the device's
 * current context has changed since (a cudaDeviceReset in between, for
 * example).  All calls share the array: calls that
 * overlap on the GPU (different streams or threads) race.  Runs on `stream`
 * (NULL = default stream) and returns without synchronising; errors go to
 * fil_last_error(NULL).                                                     */
int fil_hankel_propagate_noalloc(const float* m1, const float* m2, const float* kt2,
                                 const float* beta, const float* dfr, const float* kmax2,
                                 const float* wg, int kparaxial, const float* in, float* out,
                                 int mpad, int nh, double dz, void* stream);

/* ---- learned plasma surrogate (no counterpart in the reference, which
 * always solves the plasma ODE, plasma_equations.jl:46-72).  A 1-D
 * convolutional network (3 -> 64 -> 64 -> 64 -> 1 channels, kernel 9, tanh,
 * BF16 weights and activations, FP32 accumulation and output) maps three
 * inputs of every point of a time row,
 *   f0 = ln(max(I, 1e-30)) / 16, f1 = Re(E)^2 / max(I, 1e-30),
 *   f2 = ln(max(S_j, 1e-30)) / 16, S_j = dt sum_{i<j} Wb_i,
 * to g_j in the effective ionisation rate of the step t_j -> t_{j+1},
 *   w_j = Wb_j + kappa A_j (1 - e^{-S_j}) e^{g_j},
 * (Wb_j, A_j: the medium's rate and E^2 averaged with the time integrator's
 * quadrature over the step; kappa: the summed avalanche coefficient); the
 * density is rho_j = rho0 + (rho_nt - rho0)(1 - exp(-dt sum_{i<j} w_i)).
 * Feature arrays are [rows][3][nt], targets and weights [rows][nt] (FP32,
 * host memory).                                                             */
typedef struct fil_nn fil_nn;
int fil_nn_nparams(void);
const char* fil_nn_last_error(const fil_nn* n);
int fil_nn_create(int nt, uint64_t seed, fil_nn** out);
int fil_nn_destroy(fil_nn* n);
int fil_nn_get_params(fil_nn* n, float* params);        /* fil_nn_nparams() FP32 */
int fil_nn_set_params(fil_nn* n, const float* params);
int fil_nn_forward(fil_nn* n, const float* feat, int rows, float* out);   /* out [rows][nt] */
/* the same network through the inference kernels the simulation runs (the
 * 64 -> 64 layers as tcgen05 implicit GEMMs); nt a multiple of 128          */
int fil_nn_infer(fil_nn* n, const float* feat, int rows, float* out);
/* loss = sum m (out - target)^2 / sum m (m: the point weights) and its
 * gradient                                                                 */
int fil_nn_grad(fil_nn* n, const float* feat, const float* target, const float* mask, int rows,
                float* grad, float* loss);
/* Adam training, `iters` batches of `batch` rows drawn with `seed`;
 * loss_hist[iters] (may be NULL) receives the batch losses             */
int fil_nn_train(fil_nn* n, const float* feat, const float* target, const float* mask, int rows,
                 int batch, int iters, float lr, uint64_t seed, float* loss_hist);

/* Arm the surrogate on a handle (T, RT or XYT geometry with a plasma
 * equation; the network's nt must match): inside fil_run the density of
 * every row whose plasma solve would not be skipped comes from the network.
 * Every `every`-th step the ODE solves all rows and the largest
 * |rho_net - rho_ode| / max rho_ode is measured; the network is used on the
 * following steps only while that error is at most `tol` (the ODE takes
 * over otherwise, until a later check passes).  fil_step always solves the
 * ODE; fil_set_field keeps the handle armed with fresh counters.  nn = NULL
 * disarms.  The network must stay alive while armed.                      */
int fil_set_surrogate(fil_handle* h, const fil_nn* nn, int every, double tol);
/* out[0..n): armed, in use, steps since armed, steps that used the network,
 * checks, failed checks, last error, largest error, mean rows per step
 * that used the network, mean 128-point tiles per such step that the
 * network ran on (tiles whose output cannot reach the density are skipped) */
int fil_get_surrogate_stats(fil_handle* h, double* out, int n);

/* ---- batched parameter sweep ------------------------------------------------
 * Many RT problems with uneven (Nr, Nt) grids stepped together.  The
 * reference runs one problem per Filament.run call (src/Filament.jl:
 * 100-172); a sweep there is a host loop over decks.  Here the members'
 * z-steps (src/Filament.jl:123-172 with Models.zstep, Models.jl:75-121, and
 * the adaptive step, AdaptiveSteps.jl:96-107, each member with its own
 * controller) are one CUDA graph per z-step whose branches run the members
 * concurrently.
 * fil_create_batch: n members from cfg[n] and tab[n] (RT only); the members
 *   are handles owned by the batch (fil_batch_member), used with
 *   fil_set_field, fil_get_field, fil_analyze and fil_set_option as usual;
 *   do not destroy them.  A member may not have the surrogate armed.
 * fil_batch_tune: the autotuner.  For every member it times one z-step with
 *   each Hankel transform kernel the member can run (tensor-core 128 x 128
 *   FP16-slice tiles, or CUDA-core 128 x 128 FP32 tiles) and keeps the
 *   faster; then it assigns the members to 1, 2, 4, ... max_branches
 *   concurrent branches (longest measured step first, to the least loaded
 *   branch) and keeps the branch count whose graph runs fastest.
 *   ms_per_branches[j] (j < n_out, may be NULL) receives the batch step
 *   time with 2^j branches (0 where not tried).  Field states and
 *   controllers are restored after the trials.
 * fil_batch_run: every member i from z0[i] to zmax[i] (or nmax steps, or
 *   Istop), stats[i] as fil_run's.  Returns FIL_OK, or the negative status
 *   of the first member that failed.
 * fil_batch_plan: branch, Hankel kernel (1 = CUDA core) and step cost (ms,
 *   measured by the tuner, else a size model) of each member; returns the
 *   branch count.                                                          */
typedef struct fil_batch fil_batch;
int fil_create_batch(int n, const fil_config* cfg, const fil_tables* tab, fil_batch** out);
int fil_batch_destroy(fil_batch* b);
const char* fil_batch_last_error(const fil_batch* b);
int fil_batch_size(const fil_batch* b);
fil_handle* fil_batch_member(fil_batch* b, int i);
int fil_batch_tune(fil_batch* b, int max_branches, double* ms_per_branches, int n_out);
int fil_batch_plan(const fil_batch* b, int* branch, int* dht_simt, double* cost_ms);
int fil_batch_run(fil_batch* b, const double* z0, const double* zmax, int64_t nmax,
                  fil_stats* stats);

#ifdef __cplusplus
}
#endif

#endif /* FILAMENT_GB_H */
