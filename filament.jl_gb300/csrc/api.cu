// api.cu -- the C ABI of include/filament_gb.h.
//
// One handle = one problem on the current device, one CUDA stream.  The
// field state lives in HBM as the analytic half spectrum S[Mpad][Nt/2]
// (transverse points padded to a multiple of 128 with zero rows for the
// Hankel GEMMs).  A z-step is four kernels:
//   k_rowreduce (fil_run only)  Imax / fluence of the current field
//   k_control   (fil_run only)  adaptive dz, stop tests, z update
//   k_rowstep                    plasma + t<->w + nonlinear RK step, per row
//   k_dht (x2)                   Hankel transform, propagator, inverse
// fil_run captures a few steps into a CUDA graph and replays it until the
// on-device controller raises its done flag.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/filament_gb.h"
#include "launch.h"
#include "nn_tc.h"
#include "rowkernels.cuh"
#include "dht_simt.cuh"
#include "tc_params.h"
#include <cuda_fp16.h>
#include "tc_host.h"
#include "xyfft.h"

namespace {
thread_local std::string g_err;
const int kGraphSteps = 8;
const int kGraphsPerCheck = 4;
}

struct fil_handle {
  fil_config cfg;
  std::string err;
  int geom, n1, n2, nt, nh, nrows, mpad, nc;
  int ld;                   // row stride of S, W1, W2 (complex): nh, or nt for XYT (both halves of the spectrum)
  bool fp64;
  cudaStream_t st = nullptr;
  // device buffers (void* to serve both precisions)
  void* S = nullptr;      // state [mpad][nh] complex
  void* W1 = nullptr;     // row-kernel output
  void* W2 = nullptr;     // DHT intermediate
  void* M1 = nullptr;     // [mpad][mpad]
  void* M2 = nullptr;
  void* tw = nullptr;     // [nt] complex, per-pass twiddle layout of fft.cuh
  void* g1 = nullptr; void* g2 = nullptr; void* gt = nullptr;
  void* Cc = nullptr; void* Cf = nullptr; void* Cl = nullptr; void* Cr = nullptr; void* ramh = nullptr;
  void* kt2 = nullptr; void* beta = nullptr; void* dfr = nullptr; void* kmax2 = nullptr; void* wg = nullptr;
  void* rho_g = nullptr; void* kdrho_g = nullptr;
  double* l_kzr = nullptr; void* l_kg = nullptr;   // T: the lower half's linear step (as u_kzr, u_kg)
  void* spec_g = nullptr;   // plasma scan iterates of species 2, 3 (more than two species)
  void* stage = nullptr;  // field staging [nrows][nt] complex
  // upper half of the spectrum (RT; the reference keeps it, rowkernels.cuh):
  // state [nrows][nh] complex, Re KZ [nrows][nh] FP64, (Im KZ, guard) [nrows][nh]
  void* SU = nullptr;
  double* u_kzr = nullptr;
  void* u_kg = nullptr;
  bool full_spec = false;   // SU carried (FIL_OPT_ANALYTIC_PROJECTION off)
  void* park = nullptr;     // [nrows][nh] complex: a step's guarded spectrum across its plasma solve
  // non-paraxial prefactor (QPARAXIAL = false, RT): per-stage buffers
  // [mpad][nh] complex (S0, k1, k of the last stage, running sum) and the
  // tensor-core path's factor QZ(kt, w) / QZ(w) * Kguard Wguard, [nh][mpad]
  bool np = false;
  void* np_S0 = nullptr; void* np_K1 = nullptr; void* np_KS = nullptr; void* np_ACC = nullptr;
  void* qrt = nullptr;
  double* fluence = nullptr;   // [nrows]
  double* power = nullptr;     // [nt]
  double* pw = nullptr;        // [nrows] transverse weights
  double* rho_end = nullptr;   // [nrows]
  DevCtl* ctl = nullptr;
  DevCtl* ctl_host = nullptr;  // pinned
  double* an_host = nullptr;   // pinned: fluence[nrows], power[nt], rho_end[nrows], w[nrows]
  PlasmaParams<double> pp;
  int ns;
  double A0[4], A1[4], B[4];
  double sc = 1, sf = 1, sl = 1, sr = 1;   // response channel pre-scales
  // Tsitouras 5(4) (tsit5.h): stage derivatives [nrows][7][nh] of the row
  // kernel (T, RT, XYT); tolerances of the adaptive form
  void* tk = nullptr;
  double ode_atol = 1e-6, ode_rtol = 1e-3;
  double cc_max = -1;                      // linear-only row test (FP32 form), < 0: off
  std::complex<double> c0 = 0.0;           // XY: i QZ(w0) Rnl_cubic(w0)
  bool field_set = false, store_plasma = false;
  int bugcompat = 0, clamp_last = 0;
  int timing = 0;                      // FIL_OPT_TIMING: time one step in every `timing` (0: off)
  int gen = 0;                         // bumped by every option change (batch graphs rebuild)
  cudaGraphExec_t graph = nullptr;
  cudaEvent_t ev[8];
  double tsum[6] = {0, 0, 0, 0, 0, 0};   // row (with the surrogate), dht fwd, dht inv, reduce+control,
                                         // whole step, surrogate network
  long tcount = 0;
  void* flushbuf = nullptr;            // > L2, benchmark timing only
  size_t flushbytes = 0;
  // XYT transverse transform (xyfft.cu)
  void* kx2 = nullptr; void* ky2 = nullptr; void* sg1 = nullptr; void* sg2 = nullptr;
  void* twx = nullptr; void* twy = nullptr;
  double* kcol = nullptr;   // XY/XYT: [nt] Re C(w) of KZ = C(w) + D(kt, w), FP64 (propagator_cd)
  // tensor-core Hankel path (mixed form)
  bool use_tc = false;
  void* MA1[3] = {nullptr, nullptr, nullptr};  // M1 = T diag(s): FP16 slices a0, a1, a2
  void* MA2[3] = {nullptr, nullptr, nullptr};  // M2 = diag(1/s) T
  void* qa1 = nullptr; void* qa2 = nullptr;    // [mpad] row scales of M1, M2
  void* BS[3] = {nullptr, nullptr, nullptr};   // FP16 slices of the GEMM operand W1 or W2, [2 nh][mpad]
  void* qb = nullptr;                          // [mpad/64][2 nh] chunk scales of the operand
  void* kzt = nullptr; void* gdt = nullptr;    // [nh][mpad] KZ (float2), guard (float)
  int* tc_err = nullptr;
  CUtensorMap tm_a1[3], tm_a2[3], tm_b[3];
  // learned plasma surrogate (fil_set_surrogate): the network (caller-owned)
  // and its per-step buffers
  const fil_nn* nn = nullptr;
  void* nn_feat = nullptr;     // [nrows][3][nt] BF16
  void* nn_a1 = nullptr;       // [nrows][64][nt] BF16
  void* nn_a2 = nullptr;
  float* nn_out = nullptr;     // [nrows][nt] network output, or [nrows][9][nt] layer-3 partial sums
  int* nn_slot = nullptr;      // [nrows]
  int* nn_err = nullptr;       // tensor-core inference: a wait timed out
  uint8_t* nn_tflag = nullptr; // [nrows][nt/128] tile flags of the surrogate rows (nn_features)
  int* nn_tlist = nullptr;     // [nrows * nt/128] list of the tiles the network runs (nn_features)
  NnRowsPlan nn_plan;          // tensor-core inference over the buffers above
  bool nn_tc = false;          // nt is a multiple of 128: tensor-core path
  int nn_every = 1;
  double nn_tol = 0;
};

void fil_set_global_error(const std::string& m) { g_err = m; }

static int fail(fil_handle* h, int code, const std::string& m) {
  if (h) h->err = m; else g_err = m;
  return code;
}
#define CK(call)                                                                  \
  do {                                                                            \
    cudaError_t e_ = (call);                                                      \
    if (e_ != cudaSuccess)                                                        \
      return fail(h, FIL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static bool is_pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }

// ----------------------------------------------------------------- tables --
template <typename R> static std::vector<R> cvt(const std::vector<double>& v) {
  return std::vector<R>(v.begin(), v.end());
}

template <typename R>
static int upload(fil_handle* h, void** dst, const std::vector<double>& v) {
  std::vector<R> t = cvt<R>(v);
  CK(cudaMalloc(dst, t.size() * sizeof(R)));
  CK(cudaMemcpy(*dst, t.data(), t.size() * sizeof(R), cudaMemcpyHostToDevice));
  return 0;
}

static void rk_tableau(int alg, int* s, double a[4][4], double b[4], double c[4]) {
  std::memset(a, 0, sizeof(double) * 16);
  std::memset(b, 0, sizeof(double) * 4);
  std::memset(c, 0, sizeof(double) * 4);
  if (alg == FIL_ALG_RK2) {
    *s = 2; a[1][0] = 0.5; b[1] = 1.0; c[1] = 0.5;
  } else if (alg == FIL_ALG_RK3) {
    *s = 3; a[1][0] = 0.5; a[2][0] = -1.0; a[2][1] = 2.0;
    b[0] = 1.0 / 6.0; b[1] = 4.0 / 6.0; b[2] = 1.0 / 6.0; c[1] = 0.5; c[2] = 1.0;
  } else {
    *s = 4; a[1][0] = 0.5; a[2][1] = 0.5; a[3][2] = 1.0;
    b[0] = 1.0 / 6.0; b[1] = 1.0 / 3.0; b[2] = 1.0 / 3.0; b[3] = 1.0 / 6.0;
    c[1] = 0.5; c[2] = 0.5; c[3] = 1.0;
  }
}

// Twiddles of the block FFT of length n (fft.cuh), laid out per pass: for
// each radix-16 pass of stride NS > 1, entries (r - 1) NS + k = w^(k r n /
// (16 NS)), r = 1..15, k < NS, with w^m = exp(-2 pi i m / n).  In single
// precision each value is the pair of FP32 neighbours of (cos, sin) whose
// magnitude is closest to 1, so that the table carries no systematic gain.
static std::vector<double> fft_twiddles(int n, bool fp32) {
  std::vector<double> v(2 * n);
  for (int m = 0; m < n; ++m) {
    double a = -2.0 * M_PI * (double)m / (double)n;
    double c = std::cos(a), sn = std::sin(a);
    v[2 * m] = c;
    v[2 * m + 1] = sn;
    if (fp32) {
      float cf = (float)c, sf = (float)sn, bc = cf, bs = sf;
      double best = 1e300;
      for (int dc = -1; dc <= 1; ++dc)
        for (int ds = -1; ds <= 1; ++ds) {
          float cc = cf, ss = sf;
          if (dc) cc = std::nextafter(cf, dc > 0 ? 2.0f : -2.0f);
          if (ds) ss = std::nextafter(sf, ds > 0 ? 2.0f : -2.0f);
          double err = std::fabs((double)cc * cc + (double)ss * ss - 1.0);
          if (err < best) { best = err; bc = cc; bs = ss; }
        }
      v[2 * m] = bc;
      v[2 * m + 1] = bs;
    }
  }
  std::vector<double> p(2 * n, 0.0);
  int lg = 0;
  while ((1 << lg) < n) ++lg;
  size_t o = 0;
  for (int ns = 1 << (lg % 4); ns < n; ns *= 16) {
    if (ns == 1) continue;
    for (int r = 1; r < 16; ++r)
      for (int k = 0; k < ns; ++k) {
        const size_t m = (size_t)k * r * (n / (16 * ns));
        p[2 * o] = v[2 * m];
        p[2 * o + 1] = v[2 * m + 1];
        ++o;
      }
  }
  return p;
}

template <typename R>
static int create_tables(fil_handle* h, const fil_tables* t) {
  const fil_config& c = h->cfg;
  const int n1 = h->n1, nt = h->nt, nh = h->nh, mp = h->mpad, nr = h->nrows;
  typedef std::complex<double> cd;
  if (upload<R>(h, &h->tw, fft_twiddles(nt, sizeof(R) == 4))) return FIL_ERR_CUDA;
  // guards
  {
    std::vector<double> g(n1, 1.0), gtt(nt, 1.0);
    if (t->guard1) g.assign(t->guard1, t->guard1 + n1);
    if (t->guardt) gtt.assign(t->guardt, t->guardt + nt);
    if (upload<R>(h, &h->g1, g) || upload<R>(h, &h->gt, gtt)) return FIL_ERR_CUDA;
    if (h->geom == FIL_GEOM_XYT || h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R) {
      std::vector<double> g2(h->n2, 1.0);
      if (t->guard2) g2.assign(t->guard2, t->guard2 + h->n2);
      if (upload<R>(h, &h->g2, g2)) return FIL_ERR_CUDA;
    }
  }
  // nonlinear coefficients C_ch[k] = i QZ Rnl_ch (k ? 2 : 1) / s_ch, k < nh.
  // The row kernel multiplies response ch by s_ch, the median of |C_ch| over
  // the band, so that channels sharing a complex FFT have comparable size
  // (any positive constant gives the same result in exact arithmetic).
  {
    auto coef = [&](const double* rnl, int k) {
      cd q(t->qz[2 * k], t->qz[2 * k + 1]), r(rnl[2 * k], rnl[2 * k + 1]);
      return cd(0, 1) * q * r * (k ? 2.0 : 1.0);
    };
    auto scale = [&](const double* rnl) {
      if (!rnl || !t->qz || nh < 2) return 1.0;
      std::vector<double> a;
      for (int k = 1; k < nh; ++k) {
        double v = std::abs(coef(rnl, k));
        if (v > 0 && std::isfinite(v)) a.push_back(v);
      }
      if (a.empty()) return 1.0;
      std::nth_element(a.begin(), a.begin() + a.size() / 2, a.end());
      return a[a.size() / 2];
    };
    h->sc = scale(t->rnl_cubic);
    if (!h->fp64) {
      // the FP32 form skips the stages of rows whose nonlinear step is below
      // its resolution (k_rowstep); the FP64 form computes every row
      h->cc_max = 0;
      if (t->rnl_cubic && t->qz && (c.resp_mask & FIL_RESP_CUBIC))
        for (int k = 0; k < nh; ++k) h->cc_max = std::max(h->cc_max, std::abs(coef(t->rnl_cubic, k)));
      if (!std::isfinite(h->cc_max)) h->cc_max = -1;
    }
    h->sf = scale(t->rnl_free);
    h->sl = scale(t->rnl_losses);
    h->sr = scale(t->rnl_raman);
    if ((h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R) && t->qz && t->rnl_cubic && (c.resp_mask & FIL_RESP_CUBIC))
      h->c0 = coef(t->rnl_cubic, 0);
    auto comb = [&](const double* rnl, double sch, void** dst) -> int {
      std::vector<double> v(2 * nh, 0.0);
      if (rnl && t->qz)
        for (int k = 0; k < nh; ++k) {
          cd x = coef(rnl, k) / sch;
          v[2 * k] = x.real();
          v[2 * k + 1] = x.imag();
        }
      return upload<R>(h, dst, v);
    };
    if (comb(t->rnl_cubic, h->sc, &h->Cc) || comb(t->rnl_free, h->sf, &h->Cf) ||
        comb(t->rnl_losses, h->sl, &h->Cl) || comb(t->rnl_raman, h->sr, &h->Cr))
      return FIL_ERR_CUDA;
    if (t->raman_h) {
      std::vector<double> v(t->raman_h, t->raman_h + 2 * nt);
      if (upload<R>(h, &h->ramh, v)) return FIL_ERR_CUDA;
    }
  }
  // propagator tables
  {
    // full-length frequency tables (the XYT transverse passes also
    // propagate the upper half of the spectrum)
    std::vector<double> kt2(mp, 0.0), be(2 * nt), df(2 * nt);
    for (int i = 0; i < n1; ++i) kt2[i] = t->kt1[i] * t->kt1[i];
    for (int k = 0; k < 2 * nt; ++k) { be[k] = t->beta[k]; df[k] = t->dfr[k]; }
    if (upload<R>(h, &h->kt2, kt2) || upload<R>(h, &h->beta, be) || upload<R>(h, &h->dfr, df)) return FIL_ERR_CUDA;
    if (t->kmax) {
      std::vector<double> km(nt);
      for (int k = 0; k < nt; ++k) km[k] = t->kmax[k] * t->kmax[k];
      if (upload<R>(h, &h->kmax2, km)) return FIL_ERR_CUDA;
    }
    if (t->wguard) {
      std::vector<double> w(t->wguard, t->wguard + nt);
      if (upload<R>(h, &h->wg, w)) return FIL_ERR_CUDA;
    }
  }
  // KZ(k_i, w_j) + frame (spectral.jl:78-101,160-184) and the spectral
  // guard Kguard(k_i, w_j) Wguard(w_j) (Guards.jl:72-126) of columns
  // j0 .. j0 + nh - 1 for every row, as the pointwise tables of table_prop:
  // Re KZ in FP64, (Im KZ, guard) in the working precision
  auto kz_tables = [&](int j0, double** kzr, void** kgp) -> int {
    std::vector<double> kr((size_t)nr * nh);
    std::vector<double> kg((size_t)nr * nh * 2);
    for (int i = 0; i < nr; ++i) {
      const double kt2 = t->kt1[i] * t->kt1[i];
      for (int k = 0; k < nh; ++k) {
        const int j = j0 + k;
        const cd b(t->beta[2 * j], t->beta[2 * j + 1]), d(t->dfr[2 * j], t->dfr[2 * j + 1]);
        cd K;
        if (c.kparaxial) K = (b != cd(0, 0)) ? b - kt2 / (2.0 * b) : cd(0, 0);
        else K = std::sqrt(b * b - kt2 + cd(0.0, 0.0));
        K += d - b;
        double g = 1.0;
        if (t->kmax) {
          const double km = t->kmax[j];
          g = (km == 0.0) ? 0.0 : std::exp(-std::pow(kt2 / (km * km), 20));
        }
        if (t->wguard) g *= t->wguard[j];
        kr[(size_t)i * nh + k] = K.real();
        kg[2 * ((size_t)i * nh + k)] = K.imag();
        kg[2 * ((size_t)i * nh + k) + 1] = g;
      }
    }
    CK(cudaMalloc((void**)kzr, kr.size() * sizeof(double)));
    CK(cudaMemcpy(*kzr, kr.data(), kr.size() * sizeof(double), cudaMemcpyHostToDevice));
    return upload<R>(h, kgp, kg);
  };
  if (h->geom == FIL_GEOM_T) {
    // no transverse transform: the whole linear step is pointwise in w
    // (spectral.jl:54-75), the lower half's done by the row kernel
    if (kz_tables(0, &h->l_kzr, &h->l_kg)) return FIL_ERR_CUDA;
  }
  if (h->geom == FIL_GEOM_RT || h->geom == FIL_GEOM_T) {
    // upper half of the spectrum, columns j = nh + k (FFTW order, w < 0 and
    // the Nyquist bin), propagated in r-space as the reference's broadcast
    // does (its Hankel transform covers the first nh columns)
    if (kz_tables(nh, &h->u_kzr, &h->u_kg)) return FIL_ERR_CUDA;
    CK(cudaMalloc(&h->SU, (size_t)nr * nh * 2 * sizeof(R)));
    CK(cudaMemset(h->SU, 0, (size_t)nr * nh * 2 * sizeof(R)));
    h->full_spec = true;
  }
  if (h->geom == FIL_GEOM_XYT || h->geom == FIL_GEOM_XY) {
    // transverse 2-D transform tables (xyfft.cu)
    const int nx = h->n1, ny = h->n2;
    std::vector<double> kx2(nx), ky2(ny), s1(nx, 1.0), s2(ny, 1.0);
    for (int i = 0; i < nx; ++i) kx2[i] = t->kt1[i] * t->kt1[i];
    for (int i = 0; i < ny; ++i) ky2[i] = t->kt2[i] * t->kt2[i];
    if (t->sguard1) s1.assign(t->sguard1, t->sguard1 + nx);
    if (t->sguard2) s2.assign(t->sguard2, t->sguard2 + ny);
    // the column term of KZ in FP64 (its phase is reduced in FP64)
    std::vector<double> kc(nt);
    for (int j = 0; j < nt; ++j) {
      const cd b(t->beta[2 * j], t->beta[2 * j + 1]), d(t->dfr[2 * j], t->dfr[2 * j + 1]);
      kc[j] = (c.kparaxial || b.real() >= 0.0) ? d.real() : (d - 2.0 * b).real();
    }
    CK(cudaMalloc((void**)&h->kcol, nt * sizeof(double)));
    CK(cudaMemcpy(h->kcol, kc.data(), nt * sizeof(double), cudaMemcpyHostToDevice));
    if (upload<R>(h, &h->kx2, kx2) || upload<R>(h, &h->ky2, ky2) || upload<R>(h, &h->sg1, s1) ||
        upload<R>(h, &h->sg2, s2) || upload<R>(h, &h->twx, fft_twiddles(nx, sizeof(R) == 4)) ||
        upload<R>(h, &h->twy, fft_twiddles(ny, sizeof(R) == 4)))
      return FIL_ERR_CUDA;
  }
  // Hankel matrices M1 = T diag(s), M2 = diag(1/s) T, zero padded
  if (h->geom == FIL_GEOM_RT || h->geom == FIL_GEOM_R) {
    std::vector<double> m1((size_t)mp * mp, 0.0), m2((size_t)mp * mp, 0.0);
    for (int i = 0; i < n1; ++i)
      for (int k = 0; k < n1; ++k) {
        double T = t->dht[(size_t)i * n1 + k];
        m1[(size_t)i * mp + k] = T * t->dht_s[k];
        m2[(size_t)i * mp + k] = T / t->dht_s[i];
      }
    if (upload<R>(h, &h->M1, m1) || upload<R>(h, &h->M2, m2)) return FIL_ERR_CUDA;
  }
  // transverse weights 2 pi r dr
  {
    std::vector<double> w(nr);
    for (int i = 0; i < nr; ++i)
      w[i] = (h->geom == FIL_GEOM_XYT || h->geom == FIL_GEOM_XY) ? c.dxdy
             : (h->geom == FIL_GEOM_T) ? 1.0 : 2.0 * M_PI * (t->rdr ? t->rdr[i] : 0.0);
    CK(cudaMalloc(&h->pw, nr * sizeof(double)));
    CK(cudaMemcpy(h->pw, w.data(), nr * sizeof(double), cudaMemcpyHostToDevice));
  }
  // plasma
  if (c.plasma && c.plasma_ncomp > 2) {
    const size_t bytes = (size_t)nr * (c.plasma_ncomp - 2) * nt * sizeof(R);
    CK(cudaMalloc(&h->spec_g, bytes));
    CK(cudaMemset(h->spec_g, 0, bytes));
  }
  if (c.plasma) {
    PlasmaParams<double>& P = h->pp;
    std::memset(&P, 0, sizeof P);
    int nc = c.plasma_ncomp, n = c.rate_n;
    P.nc = nc;
    double a[4][4], b[4], cc[4];
    rk_tableau(c.plasma_alg, &P.ns, a, b, cc);
    for (int s = 0; s < 4; ++s) {
      P.b[s] = b[s];
      for (int l = 0; l < 4; ++l) P.a[s][l] = a[s][l];
      P.pidx[s] = cc[s] == 0.0 ? 0 : (cc[s] == 1.0 ? 2 : 1);
    }
    P.kdep = c.plasma_kdep;
    P.ereal = c.plasma_ereal;
    P.rate_n = n;
    P.dt = c.dt;
    P.rho0 = c.rho0;
    P.maxit = 8;
    P.tol = h->fp64 ? 1e-26 : 1e-8;
    P.skip = h->fp64 ? 1e-250 : 1e-30;
    // single precision: rows whose density rise stays below 2^-30 of the
    // previous maximum are left at rho0 (their free-current contribution is
    // far below the FP32 resolution of the step); FP64 solves every row
    P.skip_rel = h->fp64 ? 0.0 : std::ldexp(1.0, -30);
    bool pl = true;
    for (int i = 0; i < nc; ++i) {
      P.rho_nt[i] = t->rho_nt[i];
      P.rava_nt[i] = t->rava[i] / t->rho_nt[i];
      P.kfix[i] = t->kfix[i];
      if (t->rava[i] != 0.0) P.avalanche = 1;
      P.rhont_sum += t->rho_nt[i];
      P.rava_sum += std::fabs(t->rava[i]);
      double s0 = 0;
      for (int q = 0; q < n; ++q) {
        P.lx[i][q] = t->rate_lx[i * n + q];
        P.ly[i][q] = t->rate_ly[i * n + q];
      }
      for (int q = 0; q < n - 1; ++q) {
        double s = (P.ly[i][q + 1] - P.ly[i][q]) / (P.lx[i][q + 1] - P.lx[i][q]);
        P.sl[i][q] = s;
        if (q == 0) s0 = s;
        else if (std::fabs(s - s0) > 1e-12 * std::fabs(s0)) pl = false;
      }
      P.sl[i][n - 1] = P.sl[i][n - 2];
    }
    P.powerlaw = pl ? 1 : 0;
    {
      // plasma-channel skip bound (plasma.cuh): power-law rates of order
      // >= 1/2, |E|^2 losses, rho0 = 0, single precision
      bool ok = !h->fp64 && pl && !c.losses_ereal && c.rho0 == 0.0;
      double kmax = 0;
      for (int i = 0; i < nc && ok; ++i) {
        if (P.sl[i][0] < 0.5) ok = false;
        kmax = std::max(kmax, c.plasma_kdep ? P.sl[i][0] : std::fabs(t->kfix[i]));
      }
      double clmax = 0;
      if (ok && t->rnl_losses && t->qz)
        for (int k = 0; k < nh; ++k) {
          cd q(t->qz[2 * k], t->qz[2 * k + 1]), r(t->rnl_losses[2 * k], t->rnl_losses[2 * k + 1]);
          clmax = std::max(clmax, std::abs(q * r) * (k ? 2.0 : 1.0));
        }
      double rnt = 0;
      for (int i = 0; i < nc; ++i) rnt += t->rho_nt[i];
      P.ychan_coef = ok ? std::max(clmax * kmax * rnt * nh, 1e-300) : 0.0;
    }
    for (int i = 0; i < nc && pl; ++i) {
      // an integer multiphoton order: rate by repeated squaring
      const double s0 = P.sl[i][0], m = std::nearbyint(s0);
      if (m >= 1 && m <= 32 && std::fabs(s0 - m) <= 1e-9 * m) {
        P.ipow[i] = (int)m;
        P.wscale[i] = std::exp((P.ly[i][0] - m * P.lx[i][0]) / m);
      }
    }
  }
  return 0;
}

// Slices of a fixed Hankel matrix for the tensor-core GEMM: per row i a
// power-of-two scale q_i = 2^(E_i - 9), 2^E_i <= max_k |x_ik| < 2^(E_i + 1),
// and x_ik = q_i (a0 + a1 + a2) with a0 = round(x/q_i) (|a0| <= 1024) and
// a1, a2 the FP16 roundings of the remainders: 32 significant bits relative
// to the row maximum.
static void slice_rows(const std::vector<double>& x, int n, int mp, std::vector<__half> (&a)[3],
                       std::vector<float>& q) {
  for (int k = 0; k < 3; ++k) a[k].assign((size_t)mp * mp, __float2half_rn(0.f));
  q.assign(mp, 0.f);
  for (int i = 0; i < n; ++i) {
    double m = 0;
    for (int k = 0; k < n; ++k) m = std::max(m, std::fabs(x[(size_t)i * n + k]));
    if (m == 0) continue;
    int e;
    std::frexp(m, &e);                      // m = f 2^e, f in [1/2, 1)
    const double qi = std::ldexp(1.0, e - 1 - 9);
    q[i] = (float)qi;
    for (int k = 0; k < n; ++k) {
      const double y = x[(size_t)i * n + k] / qi;
      const double a0 = std::nearbyint(y);
      const double r = y - a0;
      const __half a1 = __float2half_rn((float)r);
      const double r2 = r - (double)__half2float(a1);
      a[0][(size_t)i * mp + k] = __float2half_rn((float)a0);
      a[1][(size_t)i * mp + k] = a1;
      a[2][(size_t)i * mp + k] = __float2half_rn((float)r2);
    }
  }
}

// Tables of the tensor-core Hankel path: the slices of M1 = T diag(s) and
// M2 = diag(1/s) T with their row scales, the propagator's KZ and guard per
// (r, w), the slice buffers of the field operand and the TMA maps.
static int create_tc(fil_handle* h, const fil_tables* t) {
  typedef std::complex<double> cd;
  const int n1 = h->n1, nh = h->nh, mp = h->mpad;
  std::vector<double> m1((size_t)n1 * n1), m2((size_t)n1 * n1);
  for (int i = 0; i < n1; ++i)
    for (int k = 0; k < n1; ++k) {
      const double T = t->dht[(size_t)i * n1 + k];
      m1[(size_t)i * n1 + k] = T * t->dht_s[k];
      m2[(size_t)i * n1 + k] = T / t->dht_s[i];
    }
  std::vector<__half> a1[3], a2[3];
  std::vector<float> q1, q2;
  slice_rows(m1, n1, mp, a1, q1);
  slice_rows(m2, n1, mp, a2, q2);
  std::vector<float> kz((size_t)mp * nh * 2, 0.f), gd((size_t)mp * nh, 0.f);
  for (int i = 0; i < n1; ++i) {
    double kt2 = t->kt1[i] * t->kt1[i];
    for (int j = 0; j < nh; ++j) {
      cd b(t->beta[2 * j], t->beta[2 * j + 1]), d(t->dfr[2 * j], t->dfr[2 * j + 1]);
      cd K = d;
      if (h->cfg.kparaxial) {
        if (b != cd(0, 0)) K = d - kt2 / (2.0 * b);
      } else {
        cd den = b + std::sqrt(b * b - kt2 + cd(0.0, 0.0));
        if (den != cd(0, 0)) K = d - kt2 / den;
      }
      double g = 1.0;
      if (t->kmax) {
        double km = t->kmax[j];
        g = (km == 0.0) ? 0.0 : std::exp(-std::pow(kt2 / (km * km), 20));
      }
      if (t->wguard) g *= t->wguard[j];
      kz[((size_t)j * mp + i) * 2] = (float)K.real();
      kz[((size_t)j * mp + i) * 2 + 1] = (float)K.imag();
      gd[(size_t)j * mp + i] = (float)g;
    }
  }
  auto up = [&](void** dst, const void* src, size_t bytes) -> int {
    CK(cudaMalloc(dst, bytes));
    CK(cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice));
    return 0;
  };
  const size_t sb = (size_t)mp * mp * sizeof(__half);
  for (int k = 0; k < 3; ++k)
    if (up(&h->MA1[k], a1[k].data(), sb) || up(&h->MA2[k], a2[k].data(), sb)) return FIL_ERR_CUDA;
  if (up(&h->qa1, q1.data(), mp * sizeof(float)) || up(&h->qa2, q2.data(), mp * sizeof(float)) ||
      up(&h->kzt, kz.data(), kz.size() * sizeof(float)) || up(&h->gdt, gd.data(), gd.size() * sizeof(float)))
    return FIL_ERR_CUDA;
  for (int k = 0; k < 3; ++k) {
    CK(cudaMalloc(&h->BS[k], sb / mp * 2 * nh));
    CK(cudaMemset(h->BS[k], 0, sb / mp * 2 * nh));
  }
  CK(cudaMalloc(&h->qb, (size_t)(mp / 64) * 2 * nh * sizeof(float)));
  CK(cudaMalloc(&h->tc_err, sizeof(int)));
  CK(cudaMemset(h->tc_err, 0, sizeof(int)));
  for (int k = 0; k < 3; ++k)
    if (tc_make_map(&h->tm_a1[k], h->MA1[k], 2, mp, mp, 32, 128) ||
        tc_make_map(&h->tm_a2[k], h->MA2[k], 2, mp, mp, 32, 128) ||
        tc_make_map(&h->tm_b[k], h->BS[k], 2, mp, 2 * nh, 32, 128))
      return fail(h, FIL_ERR_CUDA, "cuTensorMapEncodeTiled failed");
  return 0;
}

// Buffers of the non-paraxial prefactor (QPARAXIAL = false, RT): the
// per-stage state, the density rows of the step's plasma solve, and for the
// tensor-core path the factor QZ(kt_i, w_j) / QZ(w_j) * Kguard Wguard =
// beta / sqrt(beta^2 - kt^2) * guard (Qfunc_nonparaxial,
// nonlinear_propagators.jl:232-241; 0 where the root is 0), [nh][mpad].
static int create_np(fil_handle* h, const fil_tables* t) {
  typedef std::complex<double> cd;
  const int n1 = h->n1, nh = h->nh, mp = h->mpad;
  const size_t es = h->fp64 ? sizeof(double2) : sizeof(float2);
  const size_t sz = (size_t)mp * nh * es;
  for (void** b : {&h->np_S0, &h->np_K1, &h->np_KS, &h->np_ACC}) {
    CK(cudaMalloc(b, sz));
    CK(cudaMemset(*b, 0, sz));
  }
  if (h->cfg.plasma && !h->rho_g) {
    const size_t rs = (size_t)h->nrows * h->nt * (h->fp64 ? sizeof(double) : sizeof(float));
    CK(cudaMalloc(&h->rho_g, rs));
    CK(cudaMalloc(&h->kdrho_g, rs));
    CK(cudaMemset(h->rho_g, 0, rs));
    CK(cudaMemset(h->kdrho_g, 0, rs));
  }
  if (h->use_tc) {
    std::vector<float> q((size_t)nh * mp * 2, 0.f);
    for (int i = 0; i < n1; ++i) {
      const double kt2 = t->kt1[i] * t->kt1[i];
      for (int j = 0; j < nh; ++j) {
        const cd b(t->beta[2 * j], t->beta[2 * j + 1]);
        const cd kz = std::sqrt(b * b - kt2 + cd(0.0, 0.0));
        cd r = (kz == cd(0, 0)) ? cd(0, 0) : b / kz;
        double g = 1.0;
        if (t->kmax) {
          const double km = t->kmax[j];
          g = (km == 0.0) ? 0.0 : std::exp(-std::pow(kt2 / (km * km), 20));
        }
        if (t->wguard) g *= t->wguard[j];
        r *= g;
        q[((size_t)j * mp + i) * 2] = (float)r.real();
        q[((size_t)j * mp + i) * 2 + 1] = (float)r.imag();
      }
    }
    CK(cudaMalloc(&h->qrt, q.size() * sizeof(float)));
    CK(cudaMemcpy(h->qrt, q.data(), q.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  h->np = true;
  return 0;
}

template <typename R> static RowParams<R> row_params(fil_handle* h) {
  typedef typename C2T<R>::type C;
  RowParams<R> P;
  std::memset(&P, 0, sizeof P);
  const fil_config& c = h->cfg;
  P.nrows = h->nrows;
  P.n2 = h->n2;
  P.geom = h->geom;
  P.ld = h->ld;
  P.tw = (const C*)h->tw;
  P.g1 = (const R*)h->g1;
  P.g2 = (const R*)h->g2;
  P.gt = (const R*)h->gt;
  P.gt_bug = (h->geom == FIL_GEOM_XYT) ? h->bugcompat : 0;
  P.dt = (R)c.dt;
  P.nonlin = c.nonlinearity;
  P.has_cubic = (c.resp_mask & FIL_RESP_CUBIC) ? 1 : 0;
  P.has_free = (c.resp_mask & FIL_RESP_FREE) && c.plasma ? 1 : 0;
  P.has_losses = (c.resp_mask & FIL_RESP_LOSSES) && c.plasma ? 1 : 0;
  P.cubic_thg = c.cubic_thg;
  P.losses_ereal = c.losses_ereal;
  P.Cc = (const C*)h->Cc;
  P.Cf = (const C*)h->Cf;
  P.Cl = (const C*)h->Cl;
  P.Cr = (const C*)h->Cr;
  P.sr = (R)h->sr;
  P.has_raman = (c.resp_mask & FIL_RESP_RAMAN) && h->ramh ? 1 : 0;
  P.raman_thg = c.raman_thg;
  P.ramh = (const C*)h->ramh;
  P.sc = (R)h->sc;
  P.cc_max = (R)h->cc_max;
  P.sf = (R)h->sf;
  P.sl = (R)h->sl;
  P.ns = h->ns;
  for (int s = 0; s < 4; ++s) {
    P.A0[s] = (R)h->A0[s];
    P.A1[s] = (R)h->A1[s];
    P.B[s] = (R)h->B[s];
  }
  P.tsit = c.alg == FIL_ALG_TSIT5 ? 1 : (c.alg == FIL_ALG_ATSIT5 ? 2 : 0);
  P.babs = (R)1;
  if (P.tsit) {
    double babs = 0;
    for (int i = 0; i < TSIT_STAGES; ++i) {
      for (int j = 0; j < TSIT_STAGES - 1; ++j) P.ta[i][j] = (R)kTsitA[i][j];
      P.tbt[i] = (R)kTsitBt[i];
    }
    for (int j = 0; j < TSIT_STAGES - 1; ++j) babs += std::fabs(kTsitA[TSIT_STAGES - 1][j]);
    P.babs = (R)babs;
  }
  P.tk = (C*)h->tk;
  P.atol = h->ode_atol;
  P.rtol = h->ode_rtol;
  P.plasma = c.plasma;
  P.pp = plasma_params_as<R>(h->pp);
  P.rho_g = (R*)h->rho_g;
  P.kdrho_g = (R*)h->kdrho_g;
  P.store_plasma = h->store_plasma ? 1 : 0;
  P.rho_end = h->rho_end;
  P.ctl = h->ctl;
  P.out_T = 0;
  P.ldT = h->mpad;
  if (h->full_spec && h->geom == FIL_GEOM_XYT) {
    // both halves in one row of S (input) and of W1 (output); the upper
    // half's linear step is the transverse passes' (xyfft.cu)
    P.U_in = (const C*)h->S + h->nh;
    P.U_out = (C*)h->W1 + h->nh;
  } else if (h->full_spec) {
    P.U_in = (const C*)h->SU;
    P.U_out = (C*)h->SU;
    P.u_kzr = h->u_kzr;
    P.u_kg = (const C*)h->u_kg;
  }
  P.s0_park = (C*)h->park;
  P.l_kzr = h->l_kzr;
  P.spec_g = (R*)h->spec_g;
  P.l_kg = (const C*)h->l_kg;
  P.np_S0 = (C*)h->np_S0;
  P.np_K1 = (const C*)h->np_K1;
  P.np_KS = (const C*)h->np_KS;
  P.np_ACC = (C*)h->np_ACC;
  return P;
}

template <typename R> static PropParams<R> prop_params(fil_handle* h) {
  typedef typename C2T<R>::type C;
  PropParams<R> p;
  p.kt2 = (const R*)h->kt2;
  p.beta = (const C*)h->beta;
  p.dfr = (const C*)h->dfr;
  p.kmax2 = (const R*)h->kmax2;
  p.wg = (const R*)h->wg;
  p.kparaxial = h->cfg.kparaxial;
  return p;
}

// Learned plasma surrogate: the network over the rows flagged by this step's
// reduction (a device count; nothing runs when the controller set it to 0),
// and the row kernel's view of its output.
template <typename R> static cudaError_t enqueue_surrogate(fil_handle* h, RowParams<R>& P) {
  if (!h->nn) return cudaSuccess;
  P.nn_slot = h->nn_slot;
  P.nn_out = h->nn_out;
  P.nn_tflag = h->nn_tflag;
  if (h->nn_tc) {
    P.nn_part = 1;
    P.nn_b3 = nn_out_bias(h->nn);
    return nn_infer(h->nn, h->nn_plan, h->st);
  }
  return nn_forward_rows(h->nn, h->nn_feat, h->nn_a1, h->nn_a2, h->nn_out, h->nt, h->nrows, &h->ctl->nn_rows,
                         &h->ctl->done, h->st);
}

// one z-step: row kernel (W1 <- S), DHT forward + propagator (W2 <- W1),
// inverse (S <- W2)
// XYT: row kernel (W1 <- S, row-major), fft along y, fft along x with the
// propagator and the inverse along x, inverse along y (S <- W1)
template <typename R> static int enqueue_zstep_xyt(fil_handle* h, bool timed) {
  typedef typename C2T<R>::type C;
  RowParams<R> P = row_params<R>(h);
  P.S_in = (const C*)h->S;
  P.S_out = (C*)h->W1;
  if (timed) CK(cudaEventRecord(h->ev[1], h->st));
  CK(enqueue_surrogate<R>(h, P));
  if (timed) CK(cudaEventRecord(h->ev[5], h->st));
  CK(launch_rowstep<R>(P, h->nt, h->cfg.plasma ? h->nc : 0, 0, h->st));
  if (timed) CK(cudaEventRecord(h->ev[2], h->st));
  const int nx = h->n1, ny = h->n2, ld = h->ld;
  const int ncols = h->full_spec ? h->nt : h->nh;   // frequency columns transformed
  XyParams<R> q;
  std::memset(&q, 0, sizeof q);
  q.in = (const C*)h->W1;
  q.out = (C*)h->W1;
  q.ctl = h->ctl;
  // along y: lines p = ix*ny + iy
  q.line_stride = ld;
  q.outer_stride = (size_t)ny * ld;
  q.tw = (const C*)h->twy;
  q.scale = (R)1;
  CK(launch_xylines<R>(q, ny, 0, ncols, nx, h->st));
  // along x, propagator, back along x
  XyParams<R> qx = q;
  qx.line_stride = (size_t)ny * ld;
  qx.outer_stride = ld;
  qx.tw = (const C*)h->twx;
  qx.scale = (R)1 / (R)nx;
  qx.pp = prop_params<R>(h);
  qx.pp.kmax2 = nullptr;
  qx.wg = (const R*)h->wg;
  qx.wg_bug = h->bugcompat;
  qx.kt2_line = (const R*)h->kx2;
  qx.kcol = h->kcol;
  qx.kt2_outer = (const R*)h->ky2;
  qx.sg_line = (const R*)h->sg1;
  qx.sg_outer = (const R*)h->sg2;
  CK(launch_xylines<R>(qx, nx, 1, ncols, ny, h->st));
  if (timed) CK(cudaEventRecord(h->ev[3], h->st));
  XyParams<R> qi = q;
  qi.out = (C*)h->S;
  qi.scale = (R)1 / (R)ny;
  CK(launch_xylines<R>(qi, ny, 2, ncols, nx, h->st));
  if (timed) CK(cudaEventRecord(h->ev[4], h->st));
  return 0;
}

// Tableau of the pointwise nonlinear step (XY, R): RK2/3/4 or Tsitouras.
template <typename R> static void xy_tableau(const fil_handle* h, XyNlParams<R>& q) {
  const int alg = h->cfg.alg;
  if (alg == FIL_ALG_TSIT5 || alg == FIL_ALG_ATSIT5) {
    q.ns = TSIT_STAGES - 1;
    q.tsit = alg == FIL_ALG_TSIT5 ? 1 : 2;
    for (int i = 0; i < TSIT_STAGES; ++i) {
      for (int j = 0; j < TSIT_STAGES - 1; ++j) q.a[i][j] = (R)kTsitA[i][j];
      q.bt[i] = (R)kTsitBt[i];
    }
    for (int j = 0; j < TSIT_STAGES - 1; ++j) q.b[j] = (R)kTsitA[TSIT_STAGES - 1][j];
    q.b[TSIT_STAGES - 1] = (R)0;
  } else {
    double a[4][4], b[4], cc[4];
    rk_tableau(alg, &q.ns, a, b, cc);
    for (int i = 0; i < 4; ++i) {
      q.b[i] = (R)b[i];
      for (int j = 0; j < 4; ++j) q.a[i][j] = (R)a[i][j];
    }
  }
  q.atol = h->ode_atol;
  q.rtol = h->ode_rtol;
}

// XY (no time axis): pointwise nonlinear RK step (W1 <- S), fft along y,
// fft along x with the propagator and the inverse along x, inverse along y
// times the field guard (S <- W1)
template <typename R> static int enqueue_zstep_xy(fil_handle* h, bool timed) {
  typedef typename C2T<R>::type C;
  const int nx = h->n1, ny = h->n2;
  const C* src = (const C*)h->S;
  if (timed) CK(cudaEventRecord(h->ev[1], h->st));
  if (h->cfg.nonlinearity) {
    XyNlParams<R> q;
    std::memset(&q, 0, sizeof q);
    q.n = (long)nx * ny;
    q.ny = ny;
    xy_tableau<R>(h, q);
    q.c0 = mk<R>((R)h->c0.real(), (R)h->c0.imag());
    q.g1 = (const R*)h->g1;
    q.g2 = (const R*)h->g2;
    q.ctl = h->ctl;
    CK(launch_xy_nonlinear<R>(src, (C*)h->W1, q, h->st));
    src = (const C*)h->W1;
  }
  if (timed) CK(cudaEventRecord(h->ev[2], h->st));
  XyParams<R> q;
  std::memset(&q, 0, sizeof q);
  q.in = src;
  q.out = (C*)h->W1;
  q.ctl = h->ctl;
  q.line_stride = 1;
  q.outer_stride = (size_t)ny;
  q.tw = (const C*)h->twy;
  q.scale = (R)1;
  CK(launch_xylines<R>(q, ny, 0, 1, nx, h->st));
  XyParams<R> qx = q;
  qx.in = (const C*)h->W1;
  qx.line_stride = (size_t)ny;
  qx.outer_stride = 1;
  qx.tw = (const C*)h->twx;
  qx.scale = (R)1 / (R)nx;
  qx.pp = prop_params<R>(h);
  qx.pp.kmax2 = nullptr;
  qx.wg = (const R*)h->wg;
  qx.kt2_line = (const R*)h->kx2;
  qx.kcol = h->kcol;
  qx.kt2_outer = (const R*)h->ky2;
  qx.sg_line = (const R*)h->sg1;
  qx.sg_outer = (const R*)h->sg2;
  CK(launch_xylines<R>(qx, nx, 1, 1, ny, h->st));
  if (timed) CK(cudaEventRecord(h->ev[3], h->st));
  XyParams<R> qi = q;
  qi.in = (const C*)h->W1;
  qi.out = (C*)h->S;
  qi.scale = (R)1 / (R)ny;
  qi.g_outer = (const R*)h->g1;
  qi.g_line = (const R*)h->g2;
  CK(launch_xylines<R>(qi, ny, 3, 1, nx, h->st));
  if (timed) CK(cudaEventRecord(h->ev[4], h->st));
  return 0;
}

// Hankel pair of a non-paraxial stage: k = M2 (QZ(kt, w)/QZ(w) Kguard Wguard)
// (M1 W1), out = the stage's transformed right-hand side (row layout)
template <typename R> static int enqueue_np_transverse(fil_handle* h, void* out) {
  const int Nc = 2 * h->nh;
  if (h->use_tc && sizeof(R) == 4) {
    TcGemmParams p1;
    std::memset(&p1, 0, sizeof p1);
    p1.out = (float*)h->W2;
    p1.ldo = h->mpad;
    p1.K = h->mpad;
    p1.mode = 1;
    p1.qa = (const float*)h->qa1;
    p1.qb = (const float*)h->qb;
    p1.ldqb = Nc;
    p1.ctl = h->ctl;
    p1.err = h->tc_err;
    CK(launch_slice((const float*)h->W1, h->BS, (float*)h->qb, Nc, h->mpad, h->ctl, h->st));
    CK(launch_dht_tc(h->tm_a1, h->tm_b, p1, h->mpad, Nc, h->st));
    TcGemmParams p2 = p1;
    p2.out = (float*)out;
    p2.ldo = Nc;
    p2.mode = 3;
    p2.qa = (const float*)h->qa2;
    CK(launch_slice_mul((const float*)h->W2, (const float2*)h->qrt, h->BS, (float*)h->qb, h->nh, h->mpad, h->ctl,
                        h->st));
    CK(launch_dht_tc(h->tm_a2, h->tm_b, p2, h->mpad, Nc, h->st));
  } else {
    PropParams<R> pp = prop_params<R>(h);
    CK(launch_dht_simt<R>((const R*)h->M1, (const R*)h->W1, (R*)h->W2, h->mpad, Nc, h->mpad, pp, h->ctl, 3, h->st));
    CK(launch_dht_simt<R>((const R*)h->M2, (const R*)h->W2, (R*)out, h->mpad, Nc, h->mpad, pp, h->ctl, 4, h->st));
  }
  return 0;
}

// The nonlinear part of a z-step with the non-paraxial prefactor
// (QPARAXIAL = false, nonlinear_propagators.jl:56-63): the plasma solve,
// then per RK stage the row kernel's paraxial right-hand side, the Hankel
// pair with QZ(kt, w) in between, and finally the RK combination into W1,
// the linear step's operand.
template <typename R> static int enqueue_nonlinear_np(fil_handle* h, RowParams<R>& P) {
  typedef typename C2T<R>::type C;
  if (h->cfg.plasma) CK(launch_rowstep<R>(P, h->nt, h->nc, 4, h->st));
  P.S_out = (C*)h->W1;
  for (int s = 0; s < h->ns; ++s) {
    P.np_stage = s;
    CK(launch_rowstage<R>(P, h->nt, h->cfg.plasma ? h->nc : 0, h->st));
    int rc = enqueue_np_transverse<R>(h, s == 0 ? h->np_K1 : h->np_KS);
    if (rc) return rc;
  }
  CK(launch_np_combine<R>(P, h->nh, h->st));
  return 0;
}

// R (no time axis): pointwise nonlinear RK step (W1 <- S, the spatial
// cubic response, cubic.jl:49-54), then the Hankel pair as matrix-vector
// products with the propagator and, on the inverse's store, the field guard
// (S <- W2 <- W1).
template <typename R> static int enqueue_zstep_r(fil_handle* h, bool timed) {
  typedef typename C2T<R>::type C;
  const C* src = (const C*)h->S;
  if (timed) CK(cudaEventRecord(h->ev[1], h->st));
  if (h->cfg.nonlinearity) {
    XyNlParams<R> q;
    std::memset(&q, 0, sizeof q);
    q.n = h->nrows;
    q.ny = 1;
    xy_tableau<R>(h, q);
    q.c0 = mk<R>((R)h->c0.real(), (R)h->c0.imag());
    q.g1 = (const R*)h->g1;
    q.g2 = (const R*)h->g2;
    q.ctl = h->ctl;
    CK(launch_xy_nonlinear<R>(src, (C*)h->W1, q, h->st));
    src = (const C*)h->W1;
  }
  if (timed) CK(cudaEventRecord(h->ev[5], h->st));
  if (timed) CK(cudaEventRecord(h->ev[2], h->st));
  PropParams<R> pp = prop_params<R>(h);
  CK(launch_dht_vec<R>((const R*)h->M1, src, (C*)h->W2, h->nrows, h->mpad, pp, nullptr, h->ctl, 1, h->st));
  if (timed) CK(cudaEventRecord(h->ev[3], h->st));
  CK(launch_dht_vec<R>((const R*)h->M2, (const C*)h->W2, (C*)h->S, h->nrows, h->mpad, pp, (const R*)h->g1, h->ctl,
                       2, h->st));
  if (timed) CK(cudaEventRecord(h->ev[4], h->st));
  return 0;
}

// T: the row kernel does the whole step in place, its linear part pointwise
// in w on both halves of the spectrum (l_kzr, u_kzr).
template <typename R> static int enqueue_zstep_t(fil_handle* h, bool timed) {
  typedef typename C2T<R>::type C;
  RowParams<R> P = row_params<R>(h);
  P.S_in = (const C*)h->S;
  P.S_out = (C*)h->S;
  if (timed) CK(cudaEventRecord(h->ev[1], h->st));
  CK(enqueue_surrogate<R>(h, P));
  if (timed) CK(cudaEventRecord(h->ev[5], h->st));
  CK(launch_rowstep<R>(P, h->nt, h->cfg.plasma ? h->nc : 0, 0, h->st));
  if (timed) {
    CK(cudaEventRecord(h->ev[2], h->st));
    CK(cudaEventRecord(h->ev[3], h->st));
    CK(cudaEventRecord(h->ev[4], h->st));
  }
  return 0;
}

template <typename R> static int enqueue_zstep(fil_handle* h, bool timed) {
  if (h->geom == FIL_GEOM_XYT) return enqueue_zstep_xyt<R>(h, timed);
  if (h->geom == FIL_GEOM_XY) return enqueue_zstep_xy<R>(h, timed);
  if (h->geom == FIL_GEOM_R) return enqueue_zstep_r<R>(h, timed);
  if (h->geom == FIL_GEOM_T) return enqueue_zstep_t<R>(h, timed);
  RowParams<R> P = row_params<R>(h);
  P.S_in = (const typename C2T<R>::type*)h->S;
  P.S_out = (typename C2T<R>::type*)h->W1;
  PropParams<R> pp = prop_params<R>(h);
  const int Nc = 2 * h->nh;
  const bool tcp = h->use_tc && sizeof(R) == 4;
  if (tcp) {
    P.out_T = 1;
    P.out_scale = nullptr;   // the scalings live in M1, M2
  }
  if (timed) CK(cudaEventRecord(h->ev[1], h->st));
  CK(enqueue_surrogate<R>(h, P));
  if (timed) CK(cudaEventRecord(h->ev[5], h->st));
  if (h->np) {
    int rc = enqueue_nonlinear_np<R>(h, P);
    if (rc) return rc;
  } else {
    CK(launch_rowstep<R>(P, h->nt, h->cfg.plasma ? h->nc : 0, 0, h->st));
  }
  if (timed) CK(cudaEventRecord(h->ev[2], h->st));
  if (tcp) {
    TcGemmParams p1;
    std::memset(&p1, 0, sizeof p1);
    p1.out = (float*)h->W2;
    p1.ldo = h->mpad;
    p1.K = h->mpad;
    p1.mode = 1;
    p1.qa = (const float*)h->qa1;
    p1.qb = (const float*)h->qb;
    p1.ldqb = Nc;
    p1.ctl = h->ctl;
    p1.err = h->tc_err;
    CK(launch_slice((const float*)h->W1, h->BS, (float*)h->qb, Nc, h->mpad, h->ctl, h->st));
    CK(launch_dht_tc(h->tm_a1, h->tm_b, p1, h->mpad, Nc, h->st));
    if (timed) CK(cudaEventRecord(h->ev[3], h->st));
    TcGemmParams p2 = p1;
    p2.out = (float*)h->S;
    p2.ldo = Nc;
    p2.mode = 2;
    p2.qa = (const float*)h->qa2;
    CK(launch_slice_prop((const float*)h->W2, (const float2*)h->kzt, (const float*)h->gdt, h->BS, (float*)h->qb,
                         h->nh, h->mpad, h->ctl, h->st));
    CK(launch_dht_tc(h->tm_a2, h->tm_b, p2, h->mpad, Nc, h->st));
  } else {
    CK(launch_dht_simt<R>((const R*)h->M1, (const R*)h->W1, (R*)h->W2, h->mpad, Nc, h->mpad, pp, h->ctl, 1, h->st));
    if (timed) CK(cudaEventRecord(h->ev[3], h->st));
    CK(launch_dht_simt<R>((const R*)h->M2, (const R*)h->W2, (R*)h->S, h->mpad, Nc, h->mpad, pp, h->ctl, 2, h->st));
  }
  if (timed) CK(cudaEventRecord(h->ev[4], h->st));
  return 0;
}

// Imax and fluence of the current field; with `power`, also
// power[t] = sum_row w_row |E|^2 (the intensities pass through the staging
// buffer)
template <typename R> static int enqueue_reduce(fil_handle* h, double* power, int check_done) {
  if (h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R) {   // power = sum F w, formed on the host (fil_analyze)
    CK(launch_xy_reduce<R>((const typename C2T<R>::type*)h->S, h->fluence, h->ctl, h->nrows, check_done, h->st));
    return 0;
  }
  RowParams<R> P = row_params<R>(h);
  P.S_in = (const typename C2T<R>::type*)h->S;
  if (h->nn && check_done) {   // the stepping loop: flag the rows (and their tiles) for the surrogate
    P.nn_feat = (__nv_bfloat16*)h->nn_feat;
    P.nn_slot = h->nn_slot;
    P.nn_tflag = h->nn_tflag;
    P.nn_tlist = h->nn_tc ? h->nn_tlist : nullptr;
  }
  R* I = power ? (R*)h->stage : nullptr;
  CK(launch_rowreduce<R>(P, h->nt, h->fluence, I, check_done, h->st));
  if (power) CK(launch_colsum<R>(I, h->pw, power, h->nrows, h->nt, h->st));
  return 0;
}

// integral power spectrum (fil_analyze_spectrum): per-row |2 Sr N dt|^2,
// then the weighted column sum
template <typename R> static int enqueue_spectrum(fil_handle* h, double* S) {
  RowParams<R> P = row_params<R>(h);
  P.S_in = (const typename C2T<R>::type*)h->S;
  const int nw = h->nt / 2 + 1;
  R* tmp = (R*)h->stage;   // [nrows][nw] of the [nrows][nt] staging buffer
  CK(launch_rowspec<R>(P, h->nt, tmp, h->st));
  CK(launch_colsum<R>(tmp, h->pw, S, h->nrows, nw, h->st));
  return 0;
}

static int zstep(fil_handle* h, bool timed) {
  return h->fp64 ? enqueue_zstep<double>(h, timed) : enqueue_zstep<float>(h, timed);
}
static int reduce(fil_handle* h, double* power, int check_done) {
  return h->fp64 ? enqueue_reduce<double>(h, power, check_done) : enqueue_reduce<float>(h, power, check_done);
}

// surrogate fields of a control block: armed (with fresh counters) when the
// handle holds a network
static void arm_surrogate(const fil_handle* h, DevCtl& c) {
  c.nn_on = h->nn ? 1 : 0;
  c.nn_use = 1;
  c.nn_check = 0;
  c.nn_every = h->nn ? h->nn_every : 1;
  c.nn_tol = h->nn ? h->nn_tol : 0;
  c.nn_count = c.nn_rows = c.nn_tiles = c.nn_tiles_run = 0;
  c.nn_steps = c.nn_used = c.nn_checked = c.nn_rejected = 0;
  c.nn_diff_acc = 0;
  c.nn_err = c.nn_err_max = c.nn_rows_sum = c.nn_tiles_sum = 0;
}

static int check_tc(fil_handle* h) {
  for (int* flag : {h->tc_err, h->nn_err}) {
    if (!flag) continue;
    int e = 0;
    CK(cudaMemcpyAsync(&e, flag, sizeof(int), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    if (e) return fail(h, FIL_ERR_TIMEOUT, "a tensor-core pipeline wait timed out");
  }
  return 0;
}

// zeroes the Hankel-step work buffers W1, W2 (their padding rows and
// columns are read by the next step but written by neither path)
static int clear_work(fil_handle* h) {
  const size_t sz = (size_t)h->mpad * h->ld * (h->fp64 ? sizeof(double2) : sizeof(float2));
  CK(cudaMemsetAsync(h->W1, 0, sz, h->st));
  CK(cudaMemsetAsync(h->W2, 0, sz, h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

static int read_ctl(fil_handle* h) {
  CK(cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

static void free_all(fil_handle* h) {
  void* bufs[] = {h->S, h->W1, h->W2, h->M1, h->M2, h->tw, h->g1, h->g2, h->gt, h->Cc, h->Cf, h->Cl, h->Cr, h->ramh,
                  h->kt2, h->beta, h->dfr, h->kmax2, h->wg, h->rho_g, h->kdrho_g, h->stage,
                  h->fluence, h->power, h->pw, h->rho_end, h->ctl, h->flushbuf,
                  h->qa1, h->qa2, h->BS[0], h->BS[1], h->BS[2], h->qb, h->kzt, h->gdt, h->tc_err,
                  h->kx2, h->ky2, h->sg1, h->sg2, h->twx, h->twy,
                  h->MA1[0], h->MA1[1], h->MA1[2], h->MA2[0], h->MA2[1], h->MA2[2],
                  h->nn_feat, h->nn_a1, h->nn_a2, h->nn_out, h->nn_slot, h->nn_err, h->nn_tflag, h->nn_tlist,
                  h->SU, h->u_kzr, h->u_kg, h->np_S0, h->np_K1, h->np_KS, h->np_ACC, h->qrt, h->park,
                  h->kcol, h->l_kzr, h->l_kg, h->spec_g, h->tk};
  for (void* p : bufs)
    if (p) cudaFree(p);
  if (h->ctl_host) cudaFreeHost(h->ctl_host);
  if (h->an_host) cudaFreeHost(h->an_host);
  if (h->graph) cudaGraphExecDestroy(h->graph);
  for (int i = 0; i < 8; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  if (h->st) cudaStreamDestroy(h->st);
}

// host layout conversion: user array -> row-major complex R staging
template <typename R>
static void to_rows(const fil_handle* h, const void* src, int dtype, int layout, std::vector<R>& out) {
  const long nr = h->nrows, nt = h->nt;
  out.assign((size_t)nr * nt * 2, (R)0);
  for (long p = 0; p < nr; ++p)
    for (long j = 0; j < nt; ++j) {
      long s = layout == FIL_LAYOUT_ROWMAJOR ? p * nt + j
                                             : j * nr + (h->n2 > 1 ? (p % h->n2) * h->n1 + p / h->n2 : p);
      double re, im;
      if (dtype == FIL_DTYPE_C128) { re = ((const double*)src)[2 * s]; im = ((const double*)src)[2 * s + 1]; }
      else { re = ((const float*)src)[2 * s]; im = ((const float*)src)[2 * s + 1]; }
      out[2 * (p * nt + j)] = (R)re;
      out[2 * (p * nt + j) + 1] = (R)im;
    }
}
template <typename R>
static void from_rows(const fil_handle* h, const std::vector<R>& in, void* dst, int dtype, int layout, int ncomp) {
  const long nr = h->nrows, nt = h->nt;
  for (long p = 0; p < nr; ++p)
    for (long j = 0; j < nt; ++j) {
      long s = layout == FIL_LAYOUT_ROWMAJOR ? p * nt + j
                                             : j * nr + (h->n2 > 1 ? (p % h->n2) * h->n1 + p / h->n2 : p);
      if (ncomp == 2) {
        double re = in[2 * (p * nt + j)], im = in[2 * (p * nt + j) + 1];
        if (dtype == FIL_DTYPE_C128) { ((double*)dst)[2 * s] = re; ((double*)dst)[2 * s + 1] = im; }
        else { ((float*)dst)[2 * s] = (float)re; ((float*)dst)[2 * s + 1] = (float)im; }
      } else {
        double v = in[p * nt + j];
        if (dtype == FIL_DTYPE_F64) ((double*)dst)[s] = v;
        else ((float*)dst)[s] = (float)v;
      }
    }
}

template <typename R> static int set_field_t(fil_handle* h, const void* E, int dtype, int layout, int analytic) {
  typedef typename C2T<R>::type C;
  std::vector<R> rows;
  to_rows<R>(h, E, dtype, layout, rows);
  if (h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R) {   // no time axis: the state is the field
    CK(cudaMemcpyAsync(h->S, rows.data(), rows.size() * sizeof(R), cudaMemcpyHostToDevice, h->st));
    DevCtl c;
    std::memset(&c, 0, sizeof c);
    c.first = 1;
    CK(cudaMemcpyAsync(h->ctl, &c, sizeof c, cudaMemcpyHostToDevice, h->st));
    CK(cudaStreamSynchronize(h->st));
    return 0;
  }
  CK(cudaMemcpyAsync(h->stage, rows.data(), rows.size() * sizeof(R), cudaMemcpyHostToDevice, h->st));
  C* up = nullptr;
  if (h->full_spec) up = (h->geom == FIL_GEOM_XYT) ? (C*)h->S + h->nh : (C*)h->SU;
  CK(launch_field_in<R>((const C*)h->stage, (C*)h->S, up, h->ld, (const C*)h->tw, analytic, h->nrows, h->nt,
                        h->st));
  // control block: fresh simulation, no pending guard; an armed surrogate
  // stays armed with fresh counters
  DevCtl c;
  std::memset(&c, 0, sizeof c);
  c.first = 1;
  arm_surrogate(h, c);
  CK(cudaMemcpyAsync(h->ctl, &c, sizeof c, cudaMemcpyHostToDevice, h->st));
  CK(cudaMemsetAsync(h->rho_end, 0, h->nrows * sizeof(double), h->st));
  if (h->cfg.plasma) {   // Models.jl:66: plasma solved on the initial field
    RowParams<R> P = row_params<R>(h);
    P.S_in = (const C*)h->S;
    CK(launch_rowstep<R>(P, h->nt, h->nc, 1, h->st));
  }
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

template <typename R> static int get_field_t(fil_handle* h, void* E, int dtype, int layout) {
  typedef typename C2T<R>::type C;
  if (h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R) {
    std::vector<R> rows((size_t)h->nrows * 2);
    CK(cudaMemcpyAsync(rows.data(), h->S, rows.size() * sizeof(R), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    from_rows<R>(h, rows, E, dtype, layout, 2);
    return 0;
  }
  RowParams<R> P = row_params<R>(h);
  P.S_in = (const C*)h->S;
  CK(launch_field_out<R>(P, h->nt, (C*)h->stage, h->st));
  std::vector<R> rows((size_t)h->nrows * h->nt * 2);
  CK(cudaMemcpyAsync(rows.data(), h->stage, rows.size() * sizeof(R), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  from_rows<R>(h, rows, E, dtype, layout, 2);
  return 0;
}

// =================================================================== ABI ==
extern "C" {

const char* fil_last_error(const fil_handle* h) { return h ? h->err.c_str() : g_err.c_str(); }

int fil_destroy(fil_handle* h) {
  if (!h) return FIL_OK;
  free_all(h);
  delete h;
  return FIL_OK;
}

int fil_create(const fil_config* cfg, const fil_tables* t, fil_handle** out) {
  fil_handle* h = nullptr;
  if (!cfg || !t || !out) return fail(h, FIL_ERR_ARG, "null argument");
  *out = nullptr;
  if (cfg->abi_version != FIL_ABI_VERSION) return fail(h, FIL_ERR_ARG, "ABI version mismatch");
  if (cfg->geometry < FIL_GEOM_R || cfg->geometry > FIL_GEOM_XYT) return fail(h, FIL_ERR_ARG, "unknown geometry");
  if (cfg->geometry == FIL_GEOM_R && (cfg->nt != 1 || cfg->n2 != 1 || cfg->plasma))
    return fail(h, FIL_ERR_ARG, "R: nt and n2 must be 1 and the plasma off");
  if (cfg->geometry == FIL_GEOM_T && (cfg->n1 != 1 || cfg->n2 != 1))
    return fail(h, FIL_ERR_ARG, "T: n1 and n2 must be 1");
  if (cfg->geometry == FIL_GEOM_XY &&
      (!is_pow2(cfg->n1) || !is_pow2(cfg->n2) || cfg->n1 < 64 || cfg->n1 > 4096 || cfg->n2 < 64 || cfg->n2 > 4096))
    return fail(h, FIL_ERR_UNSUPPORTED, "XY: nx and ny must be powers of two in [64, 4096]");
  if (cfg->geometry == FIL_GEOM_XY && (cfg->nt != 1 || cfg->plasma))
    return fail(h, FIL_ERR_ARG, "XY: nt must be 1 and the plasma off");
  if (cfg->geometry == FIL_GEOM_XYT &&
      (!is_pow2(cfg->n1) || !is_pow2(cfg->n2) || cfg->n1 < 64 || cfg->n1 > 1024 || cfg->n2 < 64 || cfg->n2 > 1024))
    return fail(h, FIL_ERR_UNSUPPORTED, "XYT: nx and ny must be powers of two in [64, 1024]");
  if (cfg->geometry != FIL_GEOM_XY && cfg->geometry != FIL_GEOM_R &&
      (!is_pow2(cfg->nt) || cfg->nt < 512 || cfg->nt > 4096))
    return fail(h, FIL_ERR_UNSUPPORTED, "nt must be a power of two in [512, 4096]");
  if (cfg->n1 < 1 || cfg->n1 > 65536) return fail(h, FIL_ERR_ARG, "bad n1");
  if (cfg->nonlinearity && !cfg->qparaxial && cfg->geometry != FIL_GEOM_RT)
    return fail(h, FIL_ERR_UNSUPPORTED, "QPARAXIAL=false is built for the RT geometry");
  if (cfg->alg < FIL_ALG_RK2 || cfg->alg > FIL_ALG_ATSIT5) return fail(h, FIL_ERR_ARG, "unknown ALG");
  if (cfg->nonlinearity && cfg->alg > FIL_ALG_RK4 && (!cfg->qparaxial || (cfg->plasma && cfg->plasma_ncomp > 2)))
    return fail(h, FIL_ERR_UNSUPPORTED, "Tsit5/ATsit5 with QPARAXIAL=false or more than two species");
  if (cfg->plasma && (cfg->plasma_alg < FIL_ALG_RK2 || cfg->plasma_alg > FIL_ALG_RK4))
    return fail(h, cfg->plasma_alg > FIL_ALG_RK4 && cfg->plasma_alg <= FIL_ALG_ATSIT5 ? FIL_ERR_UNSUPPORTED : FIL_ERR_ARG,
                "plasma ALG must be RK2, RK3 or RK4");
  if (cfg->nonlinearity && (cfg->resp_mask & FIL_RESP_RAMAN) && !t->raman_h)
    return fail(h, FIL_ERR_ARG, "missing Raman response table");
  if (cfg->plasma && (cfg->plasma_ncomp < 1 || cfg->plasma_ncomp > FIL_MAXCOMP))
    return fail(h, FIL_ERR_ARG, "plasma_ncomp must be 1 .. 4");
  if (cfg->plasma && cfg->plasma_ncomp > 2 && cfg->nonlinearity &&
      ((cfg->resp_mask & FIL_RESP_RAMAN) || !cfg->qparaxial))
    return fail(h, FIL_ERR_UNSUPPORTED, "more than two species with the Raman channel or QPARAXIAL=false");
  if (cfg->plasma && (cfg->rate_n < 2 || cfg->rate_n > FIL_MAXRATE))
    return fail(h, FIL_ERR_ARG, "rate_n must be in [2, 32]");
  if (!t->kt1 || !t->beta || !t->dfr) return fail(h, FIL_ERR_ARG, "missing propagator tables");
  if ((cfg->geometry == FIL_GEOM_RT || cfg->geometry == FIL_GEOM_R) && (!t->dht || !t->dht_s))
    return fail(h, FIL_ERR_ARG, "missing DHT tables");
  if ((cfg->geometry == FIL_GEOM_XYT || cfg->geometry == FIL_GEOM_XY) && !t->kt2)
    return fail(h, FIL_ERR_ARG, "missing ky table");
  if (cfg->nonlinearity && !t->qz) return fail(h, FIL_ERR_ARG, "missing QZ table");
  if (cfg->plasma && (!t->rho_nt || !t->rava || !t->kfix || !t->rate_lx || !t->rate_ly))
    return fail(h, FIL_ERR_ARG, "missing plasma tables");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return fail(h, FIL_ERR_CUDA, "no CUDA device");
  h = new fil_handle();
  std::memset(h->ev, 0, sizeof h->ev);
  h->cfg = *cfg;
  h->geom = cfg->geometry;
  h->n1 = cfg->n1;
  h->n2 = cfg->n2;
  h->nt = cfg->nt;
  // XY, R: the field itself, one column
  h->nh = (cfg->geometry == FIL_GEOM_XY || cfg->geometry == FIL_GEOM_R) ? 1 : cfg->nt / 2;
  h->ld = cfg->geometry == FIL_GEOM_XYT ? cfg->nt : h->nh;
  h->nrows = cfg->n1 * cfg->n2;
  h->mpad = (h->nrows + 127) / 128 * 128;
  h->nc = cfg->plasma ? cfg->plasma_ncomp : 0;
  h->fp64 = cfg->precision == FIL_PREC_FP64;
  {
    double a[4][4], b[4], c[4];
    rk_tableau(cfg->alg, &h->ns, a, b, c);
    for (int s = 0; s < 4; ++s) {
      h->B[s] = b[s];
      h->A0[s] = s >= 1 ? a[s][0] : 0.0;
      h->A1[s] = s >= 2 ? a[s][s - 1] : 0.0;
    }
  }
  int rc = 0;
  const size_t es = h->fp64 ? sizeof(double2) : sizeof(float2);
  const size_t sz = (size_t)h->mpad * h->ld * es;
#define CKC(call)                                                                    \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess) {                                                         \
      g_err = std::string(#call) + ": " + cudaGetErrorString(e_);                   \
      free_all(h); delete h;                                                         \
      return FIL_ERR_CUDA;                                                           \
    }                                                                                \
  } while (0)
  CKC(cudaStreamCreateWithFlags(&h->st, cudaStreamNonBlocking));
  for (int i = 0; i < 8; ++i) CKC(cudaEventCreate(&h->ev[i]));
  CKC(cudaMalloc(&h->S, sz));
  CKC(cudaMalloc(&h->W1, sz));
  CKC(cudaMalloc(&h->W2, sz));
  CKC(cudaMemset(h->S, 0, sz));
  CKC(cudaMemset(h->W1, 0, sz));
  CKC(cudaMemset(h->W2, 0, sz));
  CKC(cudaMalloc(&h->stage, (size_t)h->nrows * h->nt * es));
  if (h->geom != FIL_GEOM_XY && h->geom != FIL_GEOM_R) {
    CKC(cudaMalloc(&h->park, (size_t)h->nrows * h->ld * es));
    CKC(cudaMemset(h->park, 0, (size_t)h->nrows * h->ld * es));
    if (cfg->nonlinearity && cfg->alg > FIL_ALG_RK4) {
      CKC(cudaMalloc(&h->tk, (size_t)h->nrows * TSIT_STAGES * h->nh * es));
      CKC(cudaMemset(h->tk, 0, (size_t)h->nrows * TSIT_STAGES * h->nh * es));
    }
  }
  if (h->geom == FIL_GEOM_XYT) {
    h->full_spec = true;      // the upper half lives in columns nh .. nt - 1 of S
  }
  CKC(cudaMalloc(&h->fluence, h->nrows * sizeof(double)));
  CKC(cudaMalloc(&h->power, h->nt * sizeof(double)));
  CKC(cudaMalloc(&h->rho_end, h->nrows * sizeof(double)));
  CKC(cudaMemset(h->rho_end, 0, h->nrows * sizeof(double)));
  CKC(cudaMalloc(&h->ctl, sizeof(DevCtl)));
  CKC(cudaMemset(h->ctl, 0, sizeof(DevCtl)));
  CKC(cudaMallocHost(&h->ctl_host, sizeof(DevCtl)));
  CKC(cudaMallocHost(&h->an_host, (3 * (size_t)h->nrows + h->nt) * sizeof(double)));
  rc = h->fp64 ? create_tables<double>(h, t) : create_tables<float>(h, t);
  if (!rc && !h->fp64 && h->geom == FIL_GEOM_RT && h->nh * 2 % 128 == 0) {
    rc = create_tc(h, t);
    h->use_tc = (rc == 0);
  }
  if (!rc && h->geom == FIL_GEOM_RT && cfg->nonlinearity && !cfg->qparaxial) rc = create_np(h, t);
  if (rc) {
    g_err = h->err;
    free_all(h);
    delete h;
    return rc;
  }
  *out = h;
  return FIL_OK;
}

int fil_set_option(fil_handle* h, int option, int64_t value) {
  if (!h) return fail(h, FIL_ERR_ARG, "null handle");
  if (option == FIL_OPT_STORE_PLASMA) {
    bool on = value != 0;
    if (on && !h->rho_g) {
      size_t es = h->fp64 ? sizeof(double) : sizeof(float);
      CK(cudaMalloc(&h->rho_g, (size_t)h->nrows * h->nt * es));
      CK(cudaMalloc(&h->kdrho_g, (size_t)h->nrows * h->nt * es));
      CK(cudaMemset(h->rho_g, 0, (size_t)h->nrows * h->nt * es));
      CK(cudaMemset(h->kdrho_g, 0, (size_t)h->nrows * h->nt * es));
    }
    h->store_plasma = on;
  } else if (option == FIL_OPT_XYT_GUARD_BUGCOMPAT) {
    h->bugcompat = value != 0;
  } else if (option == FIL_OPT_CLAMP_LAST_DZ) {
    h->clamp_last = value != 0;
  } else if (option == FIL_OPT_TIMING) {
    if (value < 0 || value > (1 << 30)) return fail(h, FIL_ERR_ARG, "timing stride out of range");
    h->timing = (int)value;
    for (int i = 0; i < 6; ++i) h->tsum[i] = 0;
    h->tcount = 0;
  } else if (option == FIL_OPT_DHT_SIMT) {
    const bool tc = !h->fp64 && (value == 0) && h->MA1[0] != nullptr;
    if (!h->fp64 && tc != h->use_tc) {
      // the two paths lay out W1 and W2 differently ([2 nh][mpad] vs
      // [mpad][2 nh]); padding the new path never writes must read zero
      h->use_tc = tc;
      int rc = clear_work(h);
      if (rc) return rc;
    }
  } else if (option == FIL_OPT_ANALYTIC_PROJECTION) {
    // on: the state is the analytic half spectrum (the upper half dropped
    // after every t->w transform); off (RT default): the upper half is kept
    // as the reference keeps it.  XYT always projects.
    const bool full = (value == 0) && (h->SU != nullptr || h->geom == FIL_GEOM_XYT);
    if (full != h->full_spec) {
      if (full) {   // the upper half restarts from zero
        const size_t es = h->fp64 ? sizeof(double2) : sizeof(float2);
        if (h->geom == FIL_GEOM_XYT)
          CK(cudaMemset2DAsync((char*)h->S + h->nh * es, h->ld * es, 0, h->nh * es, h->nrows, h->st));
        else
          CK(cudaMemsetAsync(h->SU, 0, (size_t)h->nrows * h->nh * es, h->st));
        CK(cudaStreamSynchronize(h->st));
      }
      h->full_spec = full;
    }
  }
  else if (option == FIL_OPT_ODE_RTOL || option == FIL_OPT_ODE_ATOL) {
    if (value <= 0) return fail(h, FIL_ERR_ARG, "tolerance must be positive");
    (option == FIL_OPT_ODE_RTOL ? h->ode_rtol : h->ode_atol) = (double)value * 1e-12;
  }
  else {
    return fail(h, FIL_ERR_ARG, "unknown option");
  }
  h->gen += 1;
  if (h->graph) {           // parameters baked into the graph changed
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return FIL_OK;
}

int fil_set_field(fil_handle* h, const void* E, int dtype, int layout, int analytic) {
  if (!h || !E) return fail(h, FIL_ERR_ARG, "null argument");
  if (dtype != FIL_DTYPE_C64 && dtype != FIL_DTYPE_C128) return fail(h, FIL_ERR_ARG, "field dtype must be complex");
  int rc = h->fp64 ? set_field_t<double>(h, E, dtype, layout, analytic) : set_field_t<float>(h, E, dtype, layout, analytic);
  if (rc) return rc;
  h->field_set = true;
  return FIL_OK;
}

int fil_get_field(fil_handle* h, void* E, int dtype, int layout) {
  if (!h || !E) return fail(h, FIL_ERR_ARG, "null argument");
  if (!h->field_set) return fail(h, FIL_ERR_STATE, "field not set");
  if (dtype != FIL_DTYPE_C64 && dtype != FIL_DTYPE_C128) return fail(h, FIL_ERR_ARG, "field dtype must be complex");
  return h->fp64 ? get_field_t<double>(h, E, dtype, layout) : get_field_t<float>(h, E, dtype, layout);
}

int fil_get_plasma(fil_handle* h, int which, void* out, int dtype, int layout) {
  if (!h || !out) return fail(h, FIL_ERR_ARG, "null argument");
  if (!h->store_plasma || !h->rho_g) return fail(h, FIL_ERR_STATE, "FIL_OPT_STORE_PLASMA is off");
  if (dtype != FIL_DTYPE_F32 && dtype != FIL_DTYPE_F64) return fail(h, FIL_ERR_ARG, "dtype must be real");
  size_t n = (size_t)h->nrows * h->nt;
  void* src = which == 0 ? h->rho_g : h->kdrho_g;
  if (h->fp64) {
    std::vector<double> v(n);
    CK(cudaMemcpyAsync(v.data(), src, n * sizeof(double), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    from_rows<double>(h, v, out, dtype, layout, 1);
  } else {
    std::vector<float> v(n);
    CK(cudaMemcpyAsync(v.data(), src, n * sizeof(float), cudaMemcpyDeviceToHost, h->st));
    CK(cudaStreamSynchronize(h->st));
    from_rows<float>(h, v, out, dtype, layout, 1);
  }
  return FIL_OK;
}

int fil_step(fil_handle* h, double z, double dz) {
  if (!h) return fail(h, FIL_ERR_ARG, "null handle");
  if (!h->field_set) return fail(h, FIL_ERR_STATE, "field not set");
  CK(launch_setdz(h->ctl, z, dz, h->st));
  int rc = zstep(h, false);
  if (rc) return rc;
  CK(cudaStreamSynchronize(h->st));
  rc = check_tc(h);
  if (rc) return rc;
  return FIL_OK;
}

static int build_graph(fil_handle* h) {
  cudaGraph_t g;
  CK(cudaStreamBeginCapture(h->st, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  for (int s = 0; s < kGraphSteps && !rc; ++s) {
    rc = reduce(h, nullptr, 1);
    if (!rc) {
      cudaError_t e = launch_control(h->ctl, h->fluence, h->pw, h->nrows, h->st);
      if (e != cudaSuccess) rc = fail(h, FIL_ERR_CUDA, cudaGetErrorString(e));
    }
    if (!rc) rc = zstep(h, false);
  }
  cudaError_t e = cudaStreamEndCapture(h->st, &g);
  if (rc) return rc;
  if (e != cudaSuccess) return fail(h, FIL_ERR_CUDA, std::string("capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&h->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(h, FIL_ERR_CUDA, std::string("instantiate: ") + cudaGetErrorString(e));
  return 0;
}

// arms the device controller of a run from z0 to zmax (at most nmax steps)
static int arm_run(fil_handle* h, double z0, double zmax, int64_t nmax) {
  CK(cudaMemcpyAsync(h->ctl_host, h->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  DevCtl c = *h->ctl_host;
  c.z = z0;
  c.zmax = zmax;
  c.nmax = nmax;
  c.run_steps = 0;
  c.done = 0;
  c.status = 0;
  c.flags &= ~(FIL_FLAG_ISTOP);
  c.dz0 = h->cfg.dz0;
  c.phimax = h->cfg.phimax;
  c.phik = h->cfg.phik;
  c.phip = h->cfg.phip;
  c.istop = h->cfg.istop;
  c.nonlinearity = h->cfg.nonlinearity;
  c.clamp_last = h->clamp_last;
  c.imax_acc = 0;
  c.nn_count = 0;
  c.nn_tiles = 0;
  CK(cudaMemcpyAsync(h->ctl, &c, sizeof c, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  return 0;
}

int fil_run(fil_handle* h, double z0, double zmax, int64_t nmax, fil_stats* stats) {
  if (!h) return fail(h, FIL_ERR_ARG, "null handle");
  if (!h->field_set) return fail(h, FIL_ERR_STATE, "field not set");
  {
    int rc = arm_run(h, z0, zmax, nmax);
    if (rc) return rc;
  }
  if (h->timing) {
    // benchmark path: one step at a time; every `timing`-th step (the first
    // included) is timed: L2 flushed before it (outside the timed events),
    // device time of each kernel accumulated
    if (!h->flushbuf) {
      h->flushbytes = (size_t)512 << 20;
      CK(cudaMalloc(&h->flushbuf, h->flushbytes));
    }
    for (long n = 0;; ++n) {
      const bool timed = (n % h->timing) == 0;
      if (timed) {
        CK(launch_flush(h->flushbuf, h->flushbytes, h->st));
        CK(cudaEventRecord(h->ev[0], h->st));
      }
      int rc = reduce(h, nullptr, 1);
      if (rc) return rc;
      CK(launch_control(h->ctl, h->fluence, h->pw, h->nrows, h->st));
      rc = zstep(h, timed);
      if (rc) return rc;
      rc = read_ctl(h);
      if (rc) return rc;
      if (h->ctl_host->done) break;
      if (!timed) continue;
      float t[4], tot;
      for (int i = 0; i < 4; ++i) CK(cudaEventElapsedTime(&t[i], h->ev[i], h->ev[i + 1]));
      CK(cudaEventElapsedTime(&tot, h->ev[0], h->ev[4]));
      h->tsum[0] += t[1];
      h->tsum[1] += t[2];
      h->tsum[2] += t[3];
      h->tsum[3] += t[0];
      h->tsum[4] += tot;
      if (h->geom == FIL_GEOM_RT || h->geom == FIL_GEOM_T || h->geom == FIL_GEOM_XYT) {
        float tn;
        CK(cudaEventElapsedTime(&tn, h->ev[1], h->ev[5]));
        h->tsum[5] += tn;
      }
      h->tcount += 1;
    }
  } else {
  if (!h->graph) {
    int rc = build_graph(h);
    if (rc) return rc;
  }
  for (;;) {
    for (int i = 0; i < kGraphsPerCheck; ++i) CK(cudaGraphLaunch(h->graph, h->st));
    int rc = read_ctl(h);
    if (rc) return rc;
    if (h->ctl_host->done) break;
  }
  }
  {
    int rc = check_tc(h);
    if (rc) return rc;
  }
  const DevCtl& r = *h->ctl_host;
  if (stats) {
    stats->z = r.z;
    stats->dz = r.dz;
    stats->imax = r.imax;
    stats->rhomax = r.rhomax;
    stats->energy = r.energy;
    stats->steps = r.steps;
    stats->status = r.status;
    stats->flags = r.flags | (std::min(r.newton_max, 255) << 8);
  }
  if (r.status < 0) return fail(h, r.status, "non-finite field during fil_run");
  return r.status;
}

int fil_analyze(fil_handle* h, fil_stats* st, double* fluence, double* power, double* rho_end) {
  if (!h) return fail(h, FIL_ERR_ARG, "null handle");
  if (!h->field_set) return fail(h, FIL_ERR_STATE, "field not set");
  CK(cudaMemsetAsync(h->power, 0, h->nt * sizeof(double), h->st));
  // fresh Imax accumulator
  CK(cudaMemsetAsync((char*)h->ctl + offsetof(DevCtl, imax_acc), 0, sizeof(unsigned long long), h->st));
  int rc = reduce(h, h->power, 0);
  if (rc) return rc;
  const int nr = h->nrows;
  double* F = h->an_host;
  double* P = F + nr;
  double* re = P + h->nt;
  double* w = re + nr;
  CK(cudaMemcpyAsync(F, h->fluence, nr * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(P, h->power, h->nt * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(re, h->rho_end, nr * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaMemcpyAsync(w, h->pw, nr * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  rc = read_ctl(h);
  if (rc) return rc;
  rc = check_tc(h);
  if (rc) return rc;
  const DevCtl& c = *h->ctl_host;
  if (h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R) {   // FieldAnalyzers.jl:240-255: P = sum |E|^2 dA
    double sp = 0;
    for (int i = 0; i < nr; ++i) sp += F[i] * w[i];
    P[0] = sp;
  }
  if (fluence) std::memcpy(fluence, F, nr * sizeof(double));
  if (power) std::memcpy(power, P, h->nt * sizeof(double));
  if (rho_end) std::memcpy(rho_end, re, nr * sizeof(double));
  if (st) {
    double e = 0;
    for (int i = 0; i < nr; ++i) e += F[i] * w[i];
    st->z = c.z;
    st->dz = c.dz;
    double im, rm;
    std::memcpy(&im, &c.imax_acc, sizeof im);
    std::memcpy(&rm, &c.rhomax_acc, sizeof rm);
    st->imax = im;
    st->rhomax = rm;   // maximum of the last plasma solve
    st->energy = e;
    st->steps = c.steps;
    st->status = c.status;
    st->flags = c.flags;
  }
  if (c.flags & FIL_FLAG_NAN) return fail(h, FIL_ERR_NAN, "non-finite field");
  return FIL_OK;
}

int fil_analyze_spectrum(fil_handle* h, double* S, int nw) {
  if (!h || !S) return fail(h, FIL_ERR_ARG, "null argument");
  if (!h->field_set) return fail(h, FIL_ERR_STATE, "field not set");
  if (h->geom != FIL_GEOM_RT && h->geom != FIL_GEOM_XYT && h->geom != FIL_GEOM_T)
    return fail(h, FIL_ERR_UNSUPPORTED, "the integral spectrum needs a time axis");
  if (nw != h->nt / 2 + 1) return fail(h, FIL_ERR_ARG, "nw must be nt/2 + 1");
  double* d = h->power;   // [nt] >= nw doubles, recomputed by the next fil_analyze
  CK(cudaMemsetAsync(d, 0, nw * sizeof(double), h->st));
  int rc = h->fp64 ? enqueue_spectrum<double>(h, d) : enqueue_spectrum<float>(h, d);
  if (rc) return rc;
  CK(cudaMemcpyAsync(h->an_host, d, nw * sizeof(double), cudaMemcpyDeviceToHost, h->st));
  CK(cudaStreamSynchronize(h->st));
  std::memcpy(S, h->an_host, nw * sizeof(double));
  return FIL_OK;
}

int fil_get_stats(fil_handle* h, fil_stats* st) {
  if (!h || !st) return fail(h, FIL_ERR_ARG, "null argument");
  int rc = read_ctl(h);
  if (rc) return rc;
  const DevCtl& c = *h->ctl_host;
  st->z = c.z;
  st->dz = c.dz;
  st->imax = c.imax;
  st->rhomax = c.rhomax;
  st->energy = c.energy;
  st->steps = c.steps;
  st->status = c.status;
  st->flags = c.flags | (std::min(c.newton_max, 255) << 8);
  return FIL_OK;
}

int fil_get_ode_stats(fil_handle* h, int64_t out[2]) {
  if (!h || !out) return fail(h, FIL_ERR_ARG, "null argument");
  int rc = read_ctl(h);
  if (rc) return rc;
  out[0] = (int64_t)h->ctl_host->ode_attempts;
  out[1] = (int64_t)h->ctl_host->ode_rejects;
  return FIL_OK;
}

int fil_set_surrogate(fil_handle* h, const fil_nn* nn, int every, double tol) {
  if (!h) return fail(h, FIL_ERR_ARG, "null handle");
  if (nn) {
    if (!h->cfg.plasma || h->nc < 1 || h->geom == FIL_GEOM_XY || h->geom == FIL_GEOM_R)
      return fail(h, FIL_ERR_UNSUPPORTED, "the surrogate needs a time axis and a plasma equation");
    if (nn_time_points(nn) != h->nt) return fail(h, FIL_ERR_ARG, "network built for another Nt");
    if (every < 1 || !(tol > 0)) return fail(h, FIL_ERR_ARG, "every >= 1 and tol > 0 required");
    if (!h->nn_feat) {
      const size_t rt = (size_t)h->nrows * h->nt;
      CK(cudaMalloc(&h->nn_feat, rt * 3 * 2));
      CK(cudaMalloc(&h->nn_a1, rt * 64 * 2));
      CK(cudaMalloc(&h->nn_a2, rt * 64 * 2));
      CK(cudaMalloc((void**)&h->nn_out, rt * NN_K * sizeof(float)));
      CK(cudaMalloc((void**)&h->nn_slot, (size_t)h->nrows * sizeof(int)));
      CK(cudaMemset(h->nn_slot, 0xff, (size_t)h->nrows * sizeof(int)));
      CK(cudaMalloc((void**)&h->nn_err, sizeof(int)));
      CK(cudaMemset(h->nn_err, 0, sizeof(int)));
      CK(cudaMalloc((void**)&h->nn_tflag, (size_t)h->nrows * (h->nt / 128)));
      CK(cudaMemset(h->nn_tflag, 3, (size_t)h->nrows * (h->nt / 128)));
      CK(cudaMalloc((void**)&h->nn_tlist, (size_t)h->nrows * (h->nt / 128) * sizeof(int)));
      CK(cudaMemset(h->nn_tlist, 0, (size_t)h->nrows * (h->nt / 128) * sizeof(int)));
      NnRowsPlan& pl = h->nn_plan;
      std::memset(&pl, 0, sizeof pl);
      pl.x0 = (const __nv_bfloat16*)h->nn_feat;
      pl.a1 = (__nv_bfloat16*)h->nn_a1;
      pl.a2 = (__nv_bfloat16*)h->nn_a2;
      pl.part = h->nn_out;
      pl.T = h->nt;
      pl.maxrows = h->nrows;
      pl.count = &h->ctl->nn_rows;
      pl.stop = &h->ctl->done;
      pl.err = h->nn_err;
      pl.tlist = h->nn_tlist;
      pl.tcount = &h->ctl->nn_tiles_run;
      h->nn_tc = nn_plan_init(&pl) == 0;
    }
  }
  int rc = read_ctl(h);
  if (rc) return rc;
  h->nn = nn;
  h->nn_every = every;
  h->nn_tol = tol;
  DevCtl c = *h->ctl_host;
  arm_surrogate(h, c);
  CK(cudaMemcpyAsync(h->ctl, &c, sizeof c, cudaMemcpyHostToDevice, h->st));
  CK(cudaStreamSynchronize(h->st));
  h->gen += 1;   // a batch holding this handle rebuilds its graph
  if (h->graph) {
    cudaGraphExecDestroy(h->graph);
    h->graph = nullptr;
  }
  return FIL_OK;
}

int fil_get_surrogate_stats(fil_handle* h, double* out, int n) {
  if (!h || !out) return fail(h, FIL_ERR_ARG, "null argument");
  int rc = read_ctl(h);
  if (rc) return rc;
  const DevCtl& c = *h->ctl_host;
  const double v[10] = {(double)c.nn_on, (double)c.nn_use, (double)c.nn_steps, (double)c.nn_used,
                        (double)c.nn_checked, (double)c.nn_rejected, c.nn_err, c.nn_err_max,
                        c.nn_used ? c.nn_rows_sum / (double)c.nn_used : 0.0,
                        c.nn_used ? c.nn_tiles_sum / (double)c.nn_used : 0.0};
  for (int i = 0; i < n; ++i) out[i] = i < 10 ? v[i] : 0.0;
  return FIL_OK;
}

int fil_kernel_times(fil_handle* h, double* ms, int n) {
  if (!h || !ms) return fail(h, FIL_ERR_ARG, "null argument");
  for (int i = 0; i < n; ++i) ms[i] = (i < 5 && h->tcount) ? h->tsum[i] / h->tcount : 0.0;
  if (n > 6) ms[6] = h->tcount ? h->tsum[5] / h->tcount : 0.0;
  if (n > 5) ms[5] = (double)h->tcount;
  return FIL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batched parameter sweep: many RT problems of uneven (Nr, Nt) stepped
// together.  One CUDA graph holds one z-step of every member: a fork to
// `nbranch` streams, each running the reduce + controller + row kernel +
// Hankel step of its members in sequence (every member keeps its own
// device controller and adaptive dz, and a member whose controller is done
// turns its kernels into no-ops), then a join and one block counting the
// members still live.  The host replays the graph and reads that count
// every kBatchCheck steps.  fil_batch_tune measures each member's step with
// each Hankel transform kernel it can run (tcgen05 128 x 128 FP16-slice
// tiles or the CUDA-core 128 x 128 FP32 tiles), keeps the faster, then
// spreads the members over 1, 2, 4, ... branches by longest-step-first
// assignment on the measured times and keeps the branch count whose graph
// replays fastest.  Member states are saved before and restored after
// every trial.
namespace {
const int kBatchCheck = 32;
const int kBatchMaxBranches = 32;
}

struct fil_batch {
  std::vector<fil_handle*> m;
  std::vector<int> branch;     // branch of each member
  std::vector<double> cost;    // ms per step of each member (measured by the tuner, else a size model)
  std::vector<double> tune_ms; // ms per batch step for 1, 2, 4, ... branches (tuner)
  int nbranch = 0;
  bool tuned = false;
  int gen = -1;                // sum of the members' option generations baked into the graph
  cudaStream_t st = nullptr;   // the graph's launch stream
  std::vector<cudaStream_t> bst;
  std::vector<cudaEvent_t> ev; // fork, joins, timing
  cudaGraphExec_t graph = nullptr;
  DevCtl** ctls = nullptr;     // device array of the members' control blocks
  int* live = nullptr;         // device
  int* live_host = nullptr;    // pinned
  std::string err;
};

static int bfail(fil_batch* b, int code, const std::string& m) {
  if (b) b->err = m;
  g_err = m;
  return code;
}
#define CKB(call)                                                                        \
  do {                                                                                   \
    cudaError_t e_ = (call);                                                             \
    if (e_ != cudaSuccess)                                                               \
      return bfail(b, FIL_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

static int batch_gen(const fil_batch* b) {
  int g = 0;
  for (fil_handle* h : b->m) g += h->gen;
  return g;
}

// size model used before tuning: Hankel GEMMs (Mpad^2 Nt) + row work (Mpad Nt log Nt)
static double batch_model_cost(const fil_handle* h) {
  const double lg = std::log2((double)h->nt);
  return 1e-9 * ((double)h->mpad * h->mpad * h->nt * (h->use_tc ? 0.1 : 1.0) + 40.0 * h->mpad * h->nt * lg);
}

// longest-step-first assignment of the members to k branches
static void batch_assign(fil_batch* b, int k) {
  const int n = (int)b->m.size();
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->cost[x] > b->cost[y]; });
  std::vector<double> load(k, 0.0);
  b->branch.assign(n, 0);
  for (int i : order) {
    int best = 0;
    for (int j = 1; j < k; ++j)
      if (load[j] < load[best]) best = j;
    b->branch[i] = best;
    load[best] += b->cost[i];
  }
  b->nbranch = k;
}

static int batch_build_graph(fil_batch* b) {
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  const int n = (int)b->m.size();
  std::vector<int> order(n);
  for (int i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return b->cost[x] > b->cost[y]; });
  cudaGraph_t g;
  CKB(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
  int rc = 0;
  cudaError_t e = cudaEventRecord(b->ev[0], b->st);
  for (int k = 0; k < b->nbranch && e == cudaSuccess; ++k) e = cudaStreamWaitEvent(b->bst[k], b->ev[0], 0);
  if (e != cudaSuccess) rc = bfail(b, FIL_ERR_CUDA, std::string("batch fork: ") + cudaGetErrorString(e));
  for (int k = 0; k < b->nbranch && !rc; ++k) {
    for (int i : order) {
      if (b->branch[i] != k) continue;
      fil_handle* h = b->m[i];
      cudaStream_t own = h->st;
      h->st = b->bst[k];
      rc = reduce(h, nullptr, 1);
      if (!rc) {
        cudaError_t e2 = launch_control(h->ctl, h->fluence, h->pw, h->nrows, h->st);
        if (e2 != cudaSuccess) rc = fail(h, FIL_ERR_CUDA, cudaGetErrorString(e2));
      }
      if (!rc) rc = zstep(h, false);
      h->st = own;
      if (rc) {
        rc = bfail(b, rc, "member " + std::to_string(i) + ": " + h->err);
        break;
      }
    }
  }
  for (int k = 0; k < b->nbranch && !rc; ++k) {
    e = cudaEventRecord(b->ev[1 + k], b->bst[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(b->st, b->ev[1 + k], 0);
    if (e != cudaSuccess) rc = bfail(b, FIL_ERR_CUDA, std::string("batch join: ") + cudaGetErrorString(e));
  }
  if (!rc) {
    e = launch_batch_live(b->ctls, n, b->live, b->st);
    if (e != cudaSuccess) rc = bfail(b, FIL_ERR_CUDA, cudaGetErrorString(e));
  }
  e = cudaStreamEndCapture(b->st, &g);
  if (rc) {
    if (e == cudaSuccess) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return bfail(b, FIL_ERR_CUDA, std::string("batch capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&b->graph, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return bfail(b, FIL_ERR_CUDA, std::string("batch instantiate: ") + cudaGetErrorString(e));
  b->gen = batch_gen(b);
  return 0;
}

// Members may arm the learned surrogate: its tensor-core network kernels and
// k_dht_tc both allocate tensor memory and the branches run concurrently,
// but a CTA of either kernel takes more than half of an SM's shared memory,
// so no two of them are resident on one SM together.
static int batch_check_members(fil_batch* b) {
  for (size_t i = 0; i < b->m.size(); ++i) {
    fil_handle* h = b->m[i];
    if (!h->field_set) return bfail(b, FIL_ERR_STATE, "member " + std::to_string(i) + ": field not set");
  }
  return 0;
}

// saved field state and controller of every member (tuner trials)
struct BatchSaved {
  std::vector<void*> S;
  std::vector<void*> U;        // the upper half of the spectrum (RT keeps it)
  std::vector<DevCtl> ctl;
};
static size_t upper_bytes(const fil_handle* h) {
  return (size_t)h->nrows * h->nh * (h->fp64 ? sizeof(double2) : sizeof(float2));
}
static size_t state_bytes(const fil_handle* h) {
  return (size_t)h->mpad * h->nh * (h->fp64 ? sizeof(double2) : sizeof(float2));
}
static int batch_save(fil_batch* b, BatchSaved& sv) {
  const size_t n = b->m.size();
  sv.S.assign(n, nullptr);
  sv.U.assign(n, nullptr);
  sv.ctl.resize(n);
  for (size_t i = 0; i < n; ++i) {
    fil_handle* h = b->m[i];
    CKB(cudaMalloc(&sv.S[i], state_bytes(h)));
    CKB(cudaMemcpyAsync(sv.S[i], h->S, state_bytes(h), cudaMemcpyDeviceToDevice, h->st));
    if (h->SU) {
      CKB(cudaMalloc(&sv.U[i], upper_bytes(h)));
      CKB(cudaMemcpyAsync(sv.U[i], h->SU, upper_bytes(h), cudaMemcpyDeviceToDevice, h->st));
    }
    CKB(cudaMemcpyAsync(&sv.ctl[i], h->ctl, sizeof(DevCtl), cudaMemcpyDeviceToHost, h->st));
    CKB(cudaStreamSynchronize(h->st));
  }
  return 0;
}
static int member_restore(fil_batch* b, const BatchSaved& sv, int i) {
  fil_handle* h = b->m[i];
  CKB(cudaMemcpyAsync(h->S, sv.S[i], state_bytes(h), cudaMemcpyDeviceToDevice, h->st));
  if (sv.U[i]) CKB(cudaMemcpyAsync(h->SU, sv.U[i], upper_bytes(h), cudaMemcpyDeviceToDevice, h->st));
  CKB(cudaMemcpyAsync(h->ctl, &sv.ctl[i], sizeof(DevCtl), cudaMemcpyHostToDevice, h->st));
  CKB(cudaStreamSynchronize(h->st));
  // a trial with the other Hankel kernel left its layout in W1, W2
  if (clear_work(h)) return bfail(b, FIL_ERR_CUDA, h->err);
  return 0;
}
static int batch_restore(fil_batch* b, const BatchSaved& sv) {
  CKB(cudaStreamSynchronize(b->st));
  for (size_t i = 0; i < b->m.size(); ++i) {
    int rc = member_restore(b, sv, (int)i);
    if (rc) return rc;
  }
  return 0;
}
static void batch_free_saved(BatchSaved& sv) {
  for (void* p : sv.S)
    if (p) cudaFree(p);
  for (void* p : sv.U)
    if (p) cudaFree(p);
  sv.S.clear();
  sv.U.clear();
}

// controller armed for trial steps that never stop on z or the step count
static int batch_arm_trial(fil_batch* b, const BatchSaved& sv) {
  for (size_t i = 0; i < b->m.size(); ++i) {
    int rc = arm_run(b->m[i], sv.ctl[i].z, 1e300, (int64_t)1 << 60);
    if (rc) return bfail(b, rc, "member " + std::to_string(i) + ": " + b->m[i]->err);
  }
  return 0;
}

// ms per step of member h alone on its own stream: one warm-up step, then
// `reps` timed steps
static int batch_time_member(fil_batch* b, fil_handle* h, int reps, double* ms) {
  for (int s = 0; s < 1 + reps; ++s) {
    if (s == 1) CKB(cudaEventRecord(b->ev[kBatchMaxBranches + 1], h->st));
    int rc = reduce(h, nullptr, 1);
    if (!rc) {
      cudaError_t e = launch_control(h->ctl, h->fluence, h->pw, h->nrows, h->st);
      if (e != cudaSuccess) rc = fail(h, FIL_ERR_CUDA, cudaGetErrorString(e));
    }
    if (!rc) rc = zstep(h, false);
    if (rc) return bfail(b, rc, h->err);
  }
  CKB(cudaEventRecord(b->ev[kBatchMaxBranches + 2], h->st));
  CKB(cudaEventSynchronize(b->ev[kBatchMaxBranches + 2]));
  float t = 0;
  CKB(cudaEventElapsedTime(&t, b->ev[kBatchMaxBranches + 1], b->ev[kBatchMaxBranches + 2]));
  *ms = t / reps;
  return 0;
}

static void batch_free(fil_batch* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (cudaStream_t s : b->bst)
    if (s) cudaStreamDestroy(s);
  for (cudaEvent_t e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->st) cudaStreamDestroy(b->st);
  if (b->ctls) cudaFree(b->ctls);
  if (b->live) cudaFree(b->live);
  if (b->live_host) cudaFreeHost(b->live_host);
  for (fil_handle* h : b->m) fil_destroy(h);
  b->m.clear();
}

extern "C" {

const char* fil_batch_last_error(const fil_batch* b) { return b ? b->err.c_str() : g_err.c_str(); }

int fil_create_batch(int n, const fil_config* cfg, const fil_tables* tab, fil_batch** out) {
  fil_batch* b = nullptr;
  if (!cfg || !tab || !out || n < 1) return bfail(b, FIL_ERR_ARG, "fil_create_batch: bad argument");
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (cfg[i].geometry != FIL_GEOM_RT)
      return bfail(b, FIL_ERR_UNSUPPORTED, "fil_create_batch: members must use the RT geometry");
  b = new fil_batch();
  for (int i = 0; i < n; ++i) {
    fil_handle* h = nullptr;
    int rc = fil_create(&cfg[i], &tab[i], &h);
    if (rc) {
      std::string m = "member " + std::to_string(i) + ": " + g_err;
      batch_free(b);
      delete b;
      return bfail(nullptr, rc, m);
    }
    b->m.push_back(h);
  }
  b->cost.resize(n);
  for (int i = 0; i < n; ++i) b->cost[i] = batch_model_cost(b->m[i]);
#define CKBC(call)                                                              \
  do {                                                                          \
    cudaError_t e_ = (call);                                                    \
    if (e_ != cudaSuccess) {                                                    \
      std::string m_ = std::string(#call) + ": " + cudaGetErrorString(e_);      \
      batch_free(b);                                                            \
      delete b;                                                                 \
      return bfail(nullptr, FIL_ERR_CUDA, m_);                                  \
    }                                                                           \
  } while (0)
  CKBC(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
  b->bst.assign(kBatchMaxBranches, nullptr);
  for (int k = 0; k < kBatchMaxBranches; ++k) CKBC(cudaStreamCreateWithFlags(&b->bst[k], cudaStreamNonBlocking));
  b->ev.assign(kBatchMaxBranches + 3, nullptr);
  for (int k = 0; k < kBatchMaxBranches + 1; ++k) CKBC(cudaEventCreateWithFlags(&b->ev[k], cudaEventDisableTiming));
  CKBC(cudaEventCreate(&b->ev[kBatchMaxBranches + 1]));
  CKBC(cudaEventCreate(&b->ev[kBatchMaxBranches + 2]));
  std::vector<DevCtl*> c(n);
  for (int i = 0; i < n; ++i) c[i] = b->m[i]->ctl;
  CKBC(cudaMalloc((void**)&b->ctls, n * sizeof(DevCtl*)));
  CKBC(cudaMemcpy(b->ctls, c.data(), n * sizeof(DevCtl*), cudaMemcpyHostToDevice));
  CKBC(cudaMalloc((void**)&b->live, sizeof(int)));
  CKBC(cudaMallocHost((void**)&b->live_host, sizeof(int)));
#undef CKBC
  batch_assign(b, std::min(n, 8));
  *out = b;
  return FIL_OK;
}

int fil_batch_destroy(fil_batch* b) {
  if (!b) return FIL_OK;
  batch_free(b);
  delete b;
  return FIL_OK;
}

int fil_batch_size(const fil_batch* b) { return b ? (int)b->m.size() : 0; }

fil_handle* fil_batch_member(fil_batch* b, int i) {
  if (!b || i < 0 || i >= (int)b->m.size()) return nullptr;
  return b->m[i];
}

int fil_batch_tune(fil_batch* b, int max_branches, double* ms_per_branches, int n_out) {
  if (!b) return bfail(b, FIL_ERR_ARG, "null batch");
  int rc = batch_check_members(b);
  if (rc) return rc;
  const int n = (int)b->m.size();
  max_branches = std::max(1, std::min(std::min(max_branches, kBatchMaxBranches), n));
  BatchSaved sv;
  rc = batch_save(b, sv);
  const bool saved = rc == 0;   // every member's state copied
  if (!rc) rc = batch_arm_trial(b, sv);
  // 1. the Hankel transform kernel of each member
  for (int i = 0; i < n && !rc; ++i) {
    fil_handle* h = b->m[i];
    const bool can_tc = !h->fp64 && h->MA1[0] != nullptr;
    double best = 0;
    bool best_tc = h->use_tc;
    for (int path = 0; path < (can_tc ? 2 : 1) && !rc; ++path) {
      if (can_tc) h->use_tc = (path == 0);
      double ms = 0;
      rc = batch_time_member(b, h, 3, &ms);
      if (!rc) rc = member_restore(b, sv, i);
      if (!rc) rc = arm_run(h, sv.ctl[i].z, 1e300, (int64_t)1 << 60);
      if (!rc && (path == 0 || ms < best)) {
        best = ms;
        best_tc = h->use_tc;
      }
    }
    h->use_tc = best_tc;
    b->cost[i] = best;
    if (h->graph) {   // the member's own fil_run graph may hold the other kernel
      cudaGraphExecDestroy(h->graph);
      h->graph = nullptr;
    }
  }
  // 2. the branch count
  b->tune_ms.clear();
  int best_k = 1;
  double best_ms = 0;
  // errors end the trials through rc, so that the states are still restored
  // and the saved copies freed below
  auto ck = [&](cudaError_t e, const char* what) {
    if (e != cudaSuccess && !rc) rc = bfail(b, FIL_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
  };
  for (int k = 1; k <= max_branches && !rc; k *= 2) {
    batch_assign(b, k);
    rc = batch_build_graph(b);
    if (rc) break;
    const int reps = 5;
    for (int s = 0; s < 1 + reps && !rc; ++s) {
      if (s == 1) ck(cudaEventRecord(b->ev[kBatchMaxBranches + 1], b->st), "batch timing");
      if (!rc) ck(cudaGraphLaunch(b->graph, b->st), "batch replay");
    }
    float t = 0;
    if (!rc) ck(cudaEventRecord(b->ev[kBatchMaxBranches + 2], b->st), "batch timing");
    if (!rc) ck(cudaEventSynchronize(b->ev[kBatchMaxBranches + 2]), "batch timing");
    if (!rc) ck(cudaEventElapsedTime(&t, b->ev[kBatchMaxBranches + 1], b->ev[kBatchMaxBranches + 2]), "batch timing");
    if (rc) break;
    const double ms = t / reps;
    b->tune_ms.push_back(ms);
    if (k == 1 || ms < best_ms) {
      best_ms = ms;
      best_k = k;
    }
    rc = batch_restore(b, sv);
    if (!rc) rc = batch_arm_trial(b, sv);
  }
  // the members' states as they were before tuning (also after a failed trial)
  if (saved) {
    const int rr = batch_restore(b, sv);
    if (!rc) rc = rr;
  }
  batch_free_saved(sv);
  for (int i = 0; i < n && !rc; ++i) rc = check_tc(b->m[i]) ? bfail(b, FIL_ERR_TIMEOUT, b->m[i]->err) : 0;
  if (rc) return rc;
  batch_assign(b, best_k);
  rc = batch_build_graph(b);
  if (rc) return rc;
  b->tuned = true;
  if (ms_per_branches)
    for (int j = 0; j < n_out; ++j) ms_per_branches[j] = j < (int)b->tune_ms.size() ? b->tune_ms[j] : 0.0;
  return FIL_OK;
}

int fil_batch_plan(const fil_batch* b, int* branch, int* dht_simt, double* cost_ms) {
  if (!b) return bfail(nullptr, FIL_ERR_ARG, "null batch");
  for (size_t i = 0; i < b->m.size(); ++i) {
    if (branch) branch[i] = b->branch[i];
    if (dht_simt) dht_simt[i] = b->m[i]->use_tc ? 0 : 1;
    if (cost_ms) cost_ms[i] = b->cost[i];
  }
  return b->nbranch;
}

int fil_batch_run(fil_batch* b, const double* z0, const double* zmax, int64_t nmax, fil_stats* stats) {
  if (!b || !z0 || !zmax) return bfail(b, FIL_ERR_ARG, "null argument");
  int rc = batch_check_members(b);
  if (rc) return rc;
  const int n = (int)b->m.size();
  for (int i = 0; i < n; ++i) {
    rc = arm_run(b->m[i], z0[i], zmax[i], nmax);
    if (rc) return bfail(b, rc, "member " + std::to_string(i) + ": " + b->m[i]->err);
  }
  if (!b->graph || b->gen != batch_gen(b)) {
    rc = batch_build_graph(b);
    if (rc) return rc;
  }
  for (;;) {
    for (int i = 0; i < kBatchCheck; ++i) CKB(cudaGraphLaunch(b->graph, b->st));
    CKB(cudaMemcpyAsync(b->live_host, b->live, sizeof(int), cudaMemcpyDeviceToHost, b->st));
    CKB(cudaStreamSynchronize(b->st));
    if (*b->live_host == 0) break;
  }
  int worst = FIL_OK;
  for (int i = 0; i < n; ++i) {
    fil_handle* h = b->m[i];
    rc = read_ctl(h);
    if (!rc) rc = check_tc(h);
    if (rc) return bfail(b, rc, "member " + std::to_string(i) + ": " + h->err);
    const DevCtl& r = *h->ctl_host;
    if (stats) {
      fil_stats& s = stats[i];
      s.z = r.z;
      s.dz = r.dz;
      s.imax = r.imax;
      s.rhomax = r.rhomax;
      s.energy = r.energy;
      s.steps = r.steps;
      s.status = r.status;
      s.flags = r.flags | (std::min(r.newton_max, 255) << 8);
    }
    if (r.status < 0 && worst >= 0) {
      worst = r.status;
      b->err = "member " + std::to_string(i) + ": non-finite field during fil_batch_run";
    }
  }
  return worst;
}

}  // extern "C"
