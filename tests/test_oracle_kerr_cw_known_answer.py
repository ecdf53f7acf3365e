"""Known answers of the oracle's nonlinear step on continuous waves: the
Kerr (cubic) and Raman responses, without and with third-harmonic
generation, and the multiphoton losses.

A field that is one frequency bin k0 of the time window, E(t) = a e(t) with
|e(t)| = 1, has constant |E|^2 = |a|^2.  Without the time guard (tguard = 0
makes the window 1 everywhere, Guards.jl:322-375) the sources stay on that
bin:
  cubic, calc_cubic_nothg (cubic.jl:41-46): F = 3/4 |E|^2 Re(E), analytic
    spectrum 3/4 |a|^2 a;
  Raman, calc_raman_nothg (raman.jl:57-77): the circular convolution of the
    constant 3/4 |E|^2 with H is 3/4 |a|^2 H(w = 0), then times Re(E).
So every RK stage of func! (nonlinear_propagators.jl:38-67) is a multiple
of the same bin and the step is the RK step of the scalar equation
  da/dz = i (QZ Rnl_cubic + QZ Rnl_raman H(0)) 3/4 |a|^2 a,
followed by the linear step exp(i KZ dz) Wguard (Models.jl:75-121).  With
QZ = mu0 w^2 / (2 beta) zu / Eu and Rnl = eps0 chi3 Eu^3, chi3 = 4/3 n0^2
eps0 c n2 (cubic.jl:4-13), the coefficient is the textbook self-phase rate
w n0 n2 Iu zu / (n(w) c) per unit |a|^2, and H(0), the integral of the
response, is 1 for the air response of Mlejnek et al.  The step's phase
(0.5 rad) puts the RK steps 2e-4 (Tsitouras 5(4)), 3e-3 (RK4) to 5e-2
(RK2) from the exact solution a e^{i gamma |a|^2 dz}; the Tsitouras
coefficients are read from the library's own table (csrc/tsit5.h).
"""
import numpy as np
import pytest
import scipy.constants as sc

from gpu_helpers import t_input

N2 = 1e-23
DZ = 1e-3
AMP2 = 640.0          # |a|^2 in Iu = 1e16 W/m^2


def _complex(v):
    return np.ascontiguousarray(v, dtype=np.float64).view(np.complex128)


def _tsitouras():
    """The Tsitouras 5(4) tableau as the library states it (csrc/tsit5.h):
    a[s][j] for the seven stages, b = a[6]."""
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "filament.jl_gb300", "csrc", "tsit5.h")).read()
    body = src.split("kTsitA[TSIT_STAGES][TSIT_STAGES - 1] = {", 1)[1].split("};", 1)[0]
    rows = re.findall(r"\{([^{}]*)\}", body)
    return [[float(v) for v in r.split(",")] for r in rows]


def _rk(alg, f, y, h):
    """Midpoint RK2, Kutta's RK3, the classical RK4 and the Tsitouras 5(4)
    step (the nonlinear step's integrators)."""
    if alg == "Tsit5":
        a = _tsitouras()
        k = []
        for s_ in range(6):
            k.append(f(y + h * sum(a[s_][j] * k[j] for j in range(s_))))
        return y + h * sum(a[6][j] * k[j] for j in range(6))
    k1 = f(y)
    if alg == "RK2":
        return y + h * f(y + h / 2 * k1)
    k2 = f(y + h / 2 * k1)
    if alg == "RK3":
        k3 = f(y - h * k1 + 2 * h * k2)
        return y + h / 6 * (k1 + 4 * k2 + k3)
    k3 = f(y + h / 2 * k2)
    k4 = f(y + h * k3)
    return y + h / 6 * (k1 + 2 * k2 + 2 * k3 + k4)


@pytest.mark.parametrize("raman", [False, True], ids=["kerr", "kerr+raman"])
@pytest.mark.parametrize("alg", ["RK2", "RK3", "RK4", "Tsit5"])
def test_cw_step_is_the_rk_step_of_self_phase_modulation(oracle_binding, alg, raman):
    import filament_gb as fg
    from filament_gb.responses import init_raman, raman_response_air
    # a window of 2 ps holds the Raman response (decay time 77 fs) to 3e-5
    inp = t_input(Nt=4096, tmin=-1000.0, tmax=1000.0, ALG=alg, tguard=0.0)
    responses, pe, keys = inp["p_model"]
    cubic = [dict(r, THG=False, n2=N2 / 2 if raman else N2) for r in responses if "n2" in r]
    assert len(cubic) == 1
    if raman:
        cubic.append({"init": init_raman, "THG": False, "n2": N2 / 2, "raman_response": raman_response_air})
    inp["p_model"] = (cubic, pe, dict(keys, PLASMA=False, ALG=alg))
    sim = fg.Simulation(inp, binding=oracle_binding)
    prob, h = sim.problem, sim.handle
    a = prob._arrays
    nt, dt = prob.config.nt, prob.config.dt
    tu, zu, Iu = 1e-15, 1.0, 1e16               # the deck's units
    assert np.all(np.asarray(a["guardt"]) == 1.0)

    w = 2 * np.pi * np.fft.fftfreq(nt, dt * tu)
    k0 = int(round(2 * np.pi * sc.c / 800e-9 / w[1]))   # the bin of the carrier
    S0 = np.zeros(nt, complex)
    S0[k0] = np.sqrt(AMP2)
    h.set_field(np.fft.fft(S0), analytic=True)
    h.step(DZ, DZ)
    E1 = h.get_field()

    qz = _complex(a["qz"])[k0]
    coef = qz * _complex(a["rnl_cubic"])[k0] * 0.75
    if raman:
        H0 = _complex(a["raman_h"])[0]
        assert abs(H0 - 1.0) < 1e-3                # the response integrates to one
        coef += qz * _complex(a["rnl_raman"])[k0] * 0.75 * H0
    # the self-phase rate from the constants and the medium's beta(w) * zu
    gamma = w[k0] ** 2 * zu * N2 * Iu / (_complex(a["beta"])[k0].real / zu * sc.c ** 2)
    gamma *= (_complex(a["beta"])[k0].real * sc.c / w[k0])   # n0 ~ n(w_k0)
    assert coef.imag == pytest.approx(0.0, abs=1e-12 * abs(coef))
    assert coef.real == pytest.approx(gamma, rel=1e-3 if raman else 1e-7)
    assert 0.4 < coef.real * AMP2 * DZ < 0.6

    lin = np.asarray(a["wguard"])[k0] * np.exp(1j * _complex(a["dfr"])[k0] * DZ)

    def field(y1):
        S1 = np.zeros(nt, complex)
        S1[k0] = lin * y1
        return np.fft.fft(S1)

    def err(E):
        return np.linalg.norm(E - E1) / np.linalg.norm(E1)

    f = lambda y: 1j * coef * abs(y) ** 2 * y
    y0 = np.sqrt(AMP2) + 0j
    assert err(field(_rk(alg, f, y0, DZ))) < 1e-12
    # the answer tells the integrators apart, and from the exact solution
    others = [_rk(o, f, y0, DZ) for o in ("RK2", "RK3", "RK4", "Tsit5") if o != alg]
    others.append(y0 * np.exp(1j * coef * AMP2 * DZ))
    assert min(err(field(y)) for y in others) > 1e-4
    sim.close()


@pytest.mark.parametrize("alg", ["RK2", "RK3", "RK4"])
def test_cw_step_with_multiphoton_losses(oracle_binding, alg):
    """The losses response (current_losses.jl:4-46) on the same continuous
    wave: the plasma solve sees the constant I = |a|^2, so Kdrho is a
    constant kappa at every point but the last, where it is 0
    (plasma_equations.jl:45-69).  The wave's phase is chosen so that Re(E)
    vanishes at that last point; then F = Kdrho Re(E) / |E|^2 is
    kappa Re(E) / |a|^2 at every point, with analytic spectrum kappa a / |a|^2
    on the bin, and the step is the RK step of da/dz = c kappa a / |a|^2,
    c = i QZ Rnl_losses = -hbar w0 rhou zu n0 / (4 n(w) tu Iu).  A rate
    table that is small at this intensity keeps Kdrho constant to 2e-12
    over the window; a neutral density scaled up by 1e12 makes the losses
    change the field by 1e-3 in the step."""
    import filament_gb as fg
    from filament_gb.plasma import power_law_rate
    inp = t_input(Nt=4096, tmin=-1000.0, tmax=1000.0, ALG=alg, tguard=0.0)
    responses, pe, keys = inp["p_model"]
    losses = [dict(r, EREAL=False) for r in responses if "EREAL" in r]
    assert len(losses) == 1
    tu, zu, Iu, rhou = 1e-15, 1.0, 1e16, 2.5e25      # the deck's units
    pe = dict(pe, nuc=0.0, rho_nt=5.4e24 * 1e12, KDEP=True,
              components=[{"fraction": 1.0, "ionization_energy": 12.06,
                           "ionization_rate": power_law_rate(8.0, AMP2 * Iu, 2.5)}])
    inp["p_model"] = (losses, pe, dict(keys, PLASMA=True, ALG=alg))
    sim = fg.Simulation(inp, binding=oracle_binding)
    prob, h = sim.problem, sim.handle
    a = prob._arrays
    nt, dt = prob.config.nt, prob.config.dt
    w = 2 * np.pi * np.fft.fftfreq(nt, dt * tu)
    k0 = int(round(2 * np.pi * sc.c / 800e-9 / w[1]))
    a0 = np.sqrt(AMP2) * 1j * np.exp(2j * np.pi * k0 * (nt - 1) / nt)   # Re(E) = 0 at the last point
    S0 = np.zeros(nt, complex)
    S0[k0] = a0
    h.set_field(np.fft.fft(S0), analytic=True)
    h.step(DZ, DZ)
    E1 = h.get_field()
    kd = h.get_plasma(1)
    kappa = kd[0]
    assert kd[-1] == 0.0 and np.max(np.abs(kd[:-1] - kappa)) <= 1e-11 * kappa

    c = 1j * _complex(a["qz"])[k0] * _complex(a["rnl_losses"])[k0]
    w0 = 2 * np.pi * sc.c / 800e-9
    assert c.imag == pytest.approx(0.0, abs=1e-12 * abs(c))
    assert c.real == pytest.approx(-sc.hbar * w0 * rhou * zu / (4 * tu * Iu), rel=1e-6)

    lin = np.asarray(a["wguard"])[k0] * np.exp(1j * _complex(a["dfr"])[k0] * DZ)

    def err(y1):
        S1 = np.zeros(nt, complex)
        S1[k0] = lin * y1
        return np.linalg.norm(np.fft.fft(S1) - E1) / np.linalg.norm(E1)

    f = lambda y: c * kappa * y / abs(y) ** 2
    assert 5e-4 < abs(c * kappa * DZ) / AMP2 < 5e-3
    assert err(_rk(alg, f, a0, DZ)) < 1e-13
    assert err(a0) > 1e-4                       # the losses act
    sim.close()


def _re(A):
    """Real part of the analytic field sum_m A_m e^{-i m th} as the
    coefficients R_f of e^{-i f th}, f of either sign."""
    R = {}
    for m, c in A.items():
        R[m] = R.get(m, 0) + c / 2
        R[-m] = R.get(-m, 0) + np.conj(c) / 2
    return R


def _mul(P, Q):
    out = {}
    for f, p in P.items():
        for g, q in Q.items():
            out[f + g] = out.get(f + g, 0) + p * q
    return out


def _axpy(A, h, B):
    out = dict(A)
    for m, c in B.items():
        out[m] = out.get(m, 0) + h * c
    return out


@pytest.mark.parametrize("raman", [False, True], ids=["kerr-thg", "kerr-thg+raman-thg"])
def test_third_harmonic_forms_by_harmonic_algebra(oracle_binding, raman):
    """The third-harmonic forms, calc_cubic (F = Re(E)^3, cubic.jl:33-38) and
    calc_raman (F = (H * Re(E)^2) Re(E), raman.jl:46-55), on a wave at a low
    bin k0 = 3: a field that is a sum of odd harmonics m k0 stays one, its
    sources are finite trigonometric polynomials, and the RK4 step of
    func! follows exactly in the harmonic coefficients (no harmonic of the
    four stages, up to 81 k0, reaches Nyquist, so the grid's transforms
    are exact).  The analytic spectrum doubles the positive harmonics and
    drops the negative ones; the Raman convolution multiplies harmonic f of
    Re(E)^2 by H at bin f k0 (mod Nt)."""
    import filament_gb as fg
    from filament_gb.responses import init_raman, raman_response_air
    k0, nt, amp2 = 3, 1024, 1.6e3       # self-phase 0.05 rad at k0
    inp = t_input(Nt=nt, ALG="RK4", tguard=0.0)
    responses, pe, keys = inp["p_model"]
    cubic = [dict(r, THG=True, n2=N2 / 2 if raman else N2) for r in responses if "n2" in r]
    if raman:
        cubic.append({"init": init_raman, "THG": True, "n2": N2 / 2, "raman_response": raman_response_air})
    inp["p_model"] = (cubic, pe, dict(keys, PLASMA=False, ALG="RK4"))
    sim = fg.Simulation(inp, binding=oracle_binding)
    prob, h = sim.problem, sim.handle
    a = prob._arrays
    assert np.all(np.asarray(a["guardt"]) == 1.0)
    S0 = np.zeros(nt, complex)
    S0[k0] = np.sqrt(amp2)
    h.set_field(np.fft.fft(S0), analytic=True)
    h.step(DZ, DZ)
    S1 = np.fft.ifft(h.get_field())

    qz = _complex(a["qz"])
    rc = _complex(a["rnl_cubic"])
    rr = _complex(a["rnl_raman"]) if raman else None
    H = _complex(a["raman_h"]) if raman else None
    assert 81 * k0 < nt // 2

    def rhs(A):
        Re = _re(A)
        R2 = _mul(Re, Re)
        F = {f: rc[(f * k0) % nt] * c for f, c in _mul(R2, Re).items()}
        if raman:
            R2h = {f: c * H[(f * k0) % nt] for f, c in R2.items()}
            for f, c in _mul(R2h, Re).items():
                F[f] = F.get(f, 0) + rr[(f * k0) % nt] * c
        # analytic spectrum (positive harmonics doubled), then i QZ
        return {f: 1j * qz[f * k0] * 2 * c for f, c in F.items() if f > 0}

    A0 = {1: np.sqrt(amp2) + 0j}
    k1 = rhs(A0)
    k2 = rhs(_axpy(A0, DZ / 2, k1))
    k3 = rhs(_axpy(A0, DZ / 2, k2))
    k4 = rhs(_axpy(A0, DZ, k3))
    A1 = A0
    for kk, wgt in ((k1, 1), (k2, 2), (k3, 2), (k4, 1)):
        A1 = _axpy(A1, DZ * wgt / 6, kk)
    want = np.zeros(nt, complex)
    lin = np.asarray(a["wguard"]) * np.exp(1j * _complex(a["dfr"]) * DZ)
    for m, c in A1.items():
        want[m * k0] = lin[m * k0] * c
    assert abs(A1[3]) > 1e-3 * abs(A1[1])        # the third harmonic is generated
    assert np.linalg.norm(S1 - want) <= 1e-12 * np.linalg.norm(want)
    sim.close()


def _tsitouras_bt():
    import os
    import re
    src = open(os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "filament.jl_gb300", "csrc", "tsit5.h")).read()
    body = src.split("kTsitBt[TSIT_STAGES] = {", 1)[1].split("};", 1)[0]
    return [float(v) for v in re.findall(r"-?\d+\.\d+(?:e-?\d+)?", body)]


def _atsit5(f, y, dz, rtol, atol, nh):
    """The adaptive Tsitouras step as the library states it (csrc/tsit5.h,
    ode_after): FSAL stages, error e = h sum btilde_j k_j, RMS norm over the
    point's nh analytic bins (one of them non-zero here), factor
    0.9 err^-1/5 clamped to [0.2, 10] (1 after a rejection)."""
    a, bt = _tsitouras(), _tsitouras_bt()
    h, zdone, last, rejected, attempts, rejects = dz, 0.0, True, False, 0, 0
    k0 = f(y)
    while True:
        k = [k0]
        for s_ in range(1, 6):
            k.append(f(y + h * sum(a[s_][j] * k[j] for j in range(s_))))
        y1 = y + h * sum(a[6][j] * k[j] for j in range(6))
        k.append(f(y1))
        e = h * sum(bt[j] * k[j] for j in range(7))
        err = abs(e) / (atol + rtol * max(abs(y), abs(y1))) / np.sqrt(nh)
        attempts += 1
        if err <= 1.0:
            zdone += h
            y, k0 = y1, k[6]
            if last:
                return y, attempts, rejects
            fac = 0.9 * err ** -0.2 if err > 0 else 10.0
            fac = max(min(fac, 1.0 if rejected else 10.0), 0.2)
            rejected = False
        else:
            fac = max(0.9 * err ** -0.2, 0.2)
            rejected, rejects = True, rejects + 1
        h *= fac
        last = h >= dz - zdone
        if last:
            h = dz - zdone


def test_cw_adaptive_tsitouras_step(oracle_binding):
    """ATsit5 on the continuous wave: the substeps, their number and the
    rejections follow the stated controller exactly."""
    import filament_gb as fg
    from filament_gb import _abi
    inp = t_input(Nt=1024, ALG="ATsit5", tguard=0.0)
    responses, pe, keys = inp["p_model"]
    cubic = [dict(r, THG=False, n2=N2) for r in responses if "n2" in r]
    inp["p_model"] = (cubic, pe, dict(keys, PLASMA=False, ALG="ATsit5"))
    sim = fg.Simulation(inp, binding=oracle_binding)
    prob, h = sim.problem, sim.handle
    a = prob._arrays
    rtol, atol = 1e-7, 1e-9
    h.set_option(_abi.OPT_ODE_RTOL, int(round(rtol * 1e12)))
    h.set_option(_abi.OPT_ODE_ATOL, int(round(atol * 1e12)))
    nt, dt = prob.config.nt, prob.config.dt
    w = 2 * np.pi * np.fft.fftfreq(nt, dt * 1e-15)
    k0 = int(round(2 * np.pi * sc.c / 800e-9 / w[1]))
    S0 = np.zeros(nt, complex)
    S0[k0] = np.sqrt(AMP2)
    h.set_field(np.fft.fft(S0), analytic=True)
    h.step(DZ, DZ)
    E1 = h.get_field()
    attempts, rejects = h.ode_stats()
    coef = _complex(a["qz"])[k0] * _complex(a["rnl_cubic"])[k0] * 0.75
    y1, n_att, n_rej = _atsit5(lambda y: 1j * coef * abs(y) ** 2 * y, np.sqrt(AMP2) + 0j, DZ, rtol, atol, nt // 2)
    assert n_att > 3                                   # the tolerance forces substeps
    S1 = np.zeros(nt, complex)
    S1[k0] = np.asarray(a["wguard"])[k0] * np.exp(1j * _complex(a["dfr"])[k0] * DZ) * y1
    assert np.linalg.norm(np.fft.fft(S1) - E1) <= 1e-12 * np.linalg.norm(E1)
    assert (attempts, rejects) == (n_att, n_rej)
    print("ATsit5 on the wave: %d attempts, %d rejected" % (n_att, n_rej))
    sim.close()
