// tsit5.h -- the Tsitouras 5(4) Runge-Kutta pair (FIL_ALG_TSIT5, FIL_ALG_ATSIT5)
// and the step-size controller of its adaptive form.
//
// Reference: the nonlinear step's ALG (examples/RT/input.jl:46 accepts Tsit5
// and ATsit5), integrated by ODEIntegrators.step! (nonlinear_propagators.jl:
// 70-74).  ODEIntegrators is not vendored; the pair is the published one
// (Ch. Tsitouras, "Runge-Kutta pairs of order 5(4) satisfying only the first
// column simplifying assumption", Comput. Math. Appl. 62 (2011) 770-775),
// seven stages, first same as last: b = a[6][.], the seventh stage is the
// derivative at the new point and the first stage of the next substep.
// The controller is the textbook one (Hairer, Norsett, Wanner, Solving ODEs
// I, II.4): the error norm is the RMS over one transverse point's spectrum
// of |e| / (atol + rtol max(|y0|, |y1|)), e = h sum_j btilde_j k_j.
#pragma once
#include <cmath>

#define TSIT_STAGES 7
#define TSIT_MAX_ATTEMPTS 256

// a[s][j], s = 1..6 (row 6 = b), btilde = b - bhat (the fifth-order minus
// the embedded fourth-order weights; btilde[6] weighs the seventh stage)
static const double kTsitA[TSIT_STAGES][TSIT_STAGES - 1] = {
    {0, 0, 0, 0, 0, 0},
    {0.161, 0, 0, 0, 0, 0},
    {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
    {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
    {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
    {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0},
    {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
static const double kTsitBt[TSIT_STAGES] = {-0.00178001105222577714, -0.0008164344596567469, 0.007880878010261995,
                                            -0.1447110071732629,     0.5823571654525552,    -0.45808210592918697,
                                            0.015151515151515152};

// Substep controller of one transverse point over [z, z + dz].
struct OdeStep {
  double h;       // substep of the next attempt
  double zdone;   // distance integrated so far
  int last;       // the next attempt ends at z + dz
  int rejected;   // the previous attempt was rejected
  int attempts;
};

#ifdef __CUDACC__
#define TSIT_HD __host__ __device__ __forceinline__
#else
#define TSIT_HD inline
#endif

TSIT_HD void ode_begin(OdeStep& o, double dz) {
  o.h = dz;
  o.zdone = 0.0;
  o.last = 1;
  o.rejected = 0;
  o.attempts = 0;
}

// After an attempt with error norm err: returns 1 if it is accepted.  *fin
// becomes 1 when the step is complete (the last substep accepted, or a
// non-finite error: the attempt is then taken so that the NaN reaches the
// field and its checks) and 2 when the point gave up after
// TSIT_MAX_ATTEMPTS attempts (it keeps the accepted part of the step).
TSIT_HD int ode_after(OdeStep& o, double err, double dz, int* fin) {
  ++o.attempts;
  *fin = 0;
  if (!(err == err)) {
    *fin = 1;
    return 1;
  }
  const int ok = err <= 1.0;
  double fac;
  if (ok) {
    o.zdone += o.h;
    if (o.last) {
      *fin = 1;
      return 1;
    }
    fac = err > 0.0 ? 0.9 * pow(err, -0.2) : 10.0;
    fac = fmax(fmin(fac, o.rejected ? 1.0 : 10.0), 0.2);
    o.rejected = 0;
  } else {
    fac = fmax(0.9 * pow(err, -0.2), 0.2);
    o.rejected = 1;
  }
  o.h *= fac;
  const double rem = dz - o.zdone;
  o.last = o.h >= rem;
  if (o.last) o.h = rem;
  if (o.attempts >= TSIT_MAX_ATTEMPTS) *fin = 2;
  return ok;
}
