"""Known answer of the oracle's nonlinear step: the free-current response
alone on a plasma of constant density.

With the collision frequency of the plasma equation at zero (Rava = 0,
photoionization_avalanche.jl:41-47) and a photoionisation rate that
vanishes at the pulse's intensities, the density stays rho0 at every t.
The free-current source F = rho Re(E) (current_free.jl:31-37) then has the
analytic spectrum rho0 E(w), and func! (nonlinear_propagators.jl:38-67)
reduces to the diagonal linear equation dE(w)/dz = lambda(w) E(w) with
    lambda = i QZ(w) Rnl(w) rho0
           = -mu0 w zu e^2 rho0 / (2 beta(w) m_r (nu_c - i w))
(QZ = mu0 w^2 / (2 beta) zu / Eu, nonlinear_propagators.jl:130-135, 220-229; Rnl =
i / w e^2 / m_r / (nu_c - i w) rhou Eu, current_free.jl:4-28; Eu cancels).
One z-step (Models.jl:75-121: RK step, linear step of spectral.jl:16-26, 56-74, field guard) is
    E1(w) = Wguard(w) exp(i KZ(w) dz) P(lambda dz) E0(w),  E1(t) <- G(t) E1(t)
with P the stability polynomial of the explicit RK tableau.  This pins the
response's form, the paraxial prefactor, the RK2/RK3/RK4 tableaus of the
nonlinear step and the order of the split in the oracle -- parts no
reference test covers.  The step size puts lambda dz at the carrier near
0.56, where P differs from exp by 5e-4 (RK4) to 3e-2 (RK2).
"""
import numpy as np
import pytest
import scipy.constants as sc

from gpu_helpers import rt_input, t_input

RHO0 = 2.5e24      # m^-3
NUC = 5e12         # collision frequency of the free-current response (1/s)
DZ = 1e-4          # zu = 1 m
P = {"RK2": lambda x: 1 + x + x ** 2 / 2,
     "RK3": lambda x: 1 + x + x ** 2 / 2 + x ** 3 / 6,
     "RK4": lambda x: 1 + x + x ** 2 / 2 + x ** 3 / 6 + x ** 4 / 24}


def _complex(v):
    return np.ascontiguousarray(v, dtype=np.float64).view(np.complex128)


@pytest.mark.parametrize("alg", ["RK2", "RK3", "RK4"])
def test_free_current_step_is_the_rk_polynomial_of_the_plasma_dispersion(oracle_binding, alg):
    import filament_gb as fg
    from filament_gb.plasma import power_law_rate
    inp = t_input(Nt=2048, tmin=-250.0, tmax=250.0, ALG=alg)
    responses, pe, keys = inp["p_model"]
    free = [dict(r, nuc=NUC) for r in responses if "nuc" in r and "mr" in r]
    assert len(free) == 1
    pe = dict(pe, nuc=0.0, rho0=RHO0,
              components=[{"fraction": 1.0, "ionization_energy": 12.06,
                           "ionization_rate": power_law_rate(8.0, 1e18, 1e-200)}])
    inp["p_model"] = (free, pe, dict(keys, ALG=alg))
    sim = fg.Simulation(inp, binding=oracle_binding)
    prob, h = sim.problem, sim.handle
    a = prob._arrays
    nt, dt = prob.config.nt, prob.config.dt
    tu, zu, rhou = 1e-15, 1.0, 2.5e25          # the deck's units
    E0 = h.get_field()
    h.step(DZ, DZ)
    E1 = h.get_field()
    rho = h.get_plasma(0)
    assert np.all(prob.pe.rava == 0.0) and np.allclose(rho, RHO0 / rhou, rtol=1e-14)

    # lambda from the physical constants and the medium's beta(w) * zu
    w = 2 * np.pi * np.fft.fftfreq(nt, dt * tu)
    beta = _complex(a["beta"]) / zu
    k = np.arange(1, nt // 2)
    lam = np.zeros(nt, complex)
    lam[k] = -sc.mu_0 * w[k] * zu * sc.e ** 2 * RHO0 / (2 * beta[k] * sc.m_e * (NUC - 1j * w[k]))
    # the library's tables give the same product (to the CODATA differences
    # of the constants)
    lam_tab = np.zeros(nt, complex)
    lam_tab[k] = 1j * _complex(a["qz"])[k] * _complex(a["rnl_free"])[k] * RHO0 / rhou
    assert np.max(np.abs(lam_tab - lam)) <= 1e-8 * np.max(np.abs(lam))

    S0 = np.fft.ifft(E0)                       # the spectrum, FFTW order
    kc = int(np.argmax(np.abs(S0[: nt // 2])))
    assert 0.4 < abs(lam[kc] * DZ) < 0.7

    def one_step(lmb, poly):
        S1 = np.asarray(a["wguard"]) * np.exp(1j * _complex(a["dfr"]) * DZ) * poly(lmb * DZ) * S0
        return np.asarray(a["guardt"]) * np.fft.fft(S1)

    def err(E):
        return np.linalg.norm(E - E1) / np.linalg.norm(E1)

    assert err(one_step(lam_tab, P[alg])) < 1e-9
    assert err(one_step(lam, P[alg])) < 1e-8
    # the answer tells the tableaus apart, and from the exact exponential
    others = [P[o] for o in P if o != alg] + [np.exp]
    assert min(err(one_step(lam_tab, f)) for f in others) > 1e-4
    sim.close()


@pytest.mark.parametrize("qparaxial", [True, False], ids=["RT paraxial", "RT non-paraxial"])
def test_rt_free_current_step_and_the_nonparaxial_prefactor(oracle_binding, qparaxial):
    """The same plasma in RT, on a 50 um beam whose transverse spectrum
    reaches kt ~ 0.3% of beta.  In the Hankel domain (E^ = T diag(s) E,
    E = diag(1/s) T E^, Fields.jl:105-111) the step is diagonal:
      E^1 = D(kt, w) P(lambda(kt, w) dz) E^0,
      D = exp(i KZ dz) Kguard Wguard, KZ = sqrt(beta^2 - kt^2) - w / vf
      (KPARAXIAL = false, spectral.jl:16-26, 160-184; Guards.jl:95-126),
    with lambda = i QZ Rnl rho0 for the paraxial prefactor, and
    lambda = i QZ beta / sqrt(beta^2 - kt^2) Rnl rho0 Kguard Wguard for
    the non-paraxial one (func!'s transform, prefactor and spectral guard,
    nonlinear_propagators.jl:56-63, 232-242).  The tolerance covers the
    Hankel matrix's departure from an involution (T T = I to 2.4e-10); the
    two prefactors differ by 3e-6 on this beam."""
    import filament_gb as fg
    from filament_gb.plasma import power_law_rate
    inp = rt_input(Nr=128, rmax=0.5, rguard=0.1, beam_a0=50e-6, Nt=2048, tmin=-250.0, tmax=250.0,
                   ALG="RK4", QPARAXIAL=qparaxial)
    responses, pe, keys = inp["p_model"]
    free = [dict(r, nuc=NUC) for r in responses if "nuc" in r and "mr" in r]
    pe = dict(pe, nuc=0.0, rho0=RHO0,
              components=[{"fraction": 1.0, "ionization_energy": 12.06,
                           "ionization_rate": power_law_rate(8.0, 1e18, 1e-200)}])
    inp["p_model"] = (free, pe, dict(keys, ALG="RK4", QPARAXIAL=qparaxial))
    sim = fg.Simulation(inp, binding=oracle_binding)
    prob, h = sim.problem, sim.handle
    a = prob._arrays
    nr, nt = prob.config.n1, prob.config.nt
    rhou = inp["p_unit"][-1]
    E0 = h.get_field()
    h.step(DZ, DZ)
    E1 = h.get_field()

    beta, dfr = _complex(a["beta"]), _complex(a["dfr"])
    qz, rnl = _complex(a["qz"]), _complex(a["rnl_free"])
    kt, kmax, wg = np.asarray(a["kt1"]), np.asarray(a["kmax"]), np.asarray(a["wguard"])
    T, s = np.asarray(a["dht"]), np.asarray(a["dht_s"])
    G = np.asarray(a["guard1"])[:, None] * np.asarray(a["guardt"])[None, :]
    j = np.arange(1, nt // 2)
    Kg = np.zeros((nr, nt))
    Kg[:, j] = np.exp(-((kt[:, None] ** 2 / kmax[None, j] ** 2)) ** 20)
    kz = np.sqrt(beta[None, :] ** 2 - kt[:, None] ** 2 + 0j)
    D = np.exp(1j * (kz - (beta - dfr)[None, :]) * DZ) * Kg * wg[None, :]

    def lam(nonparaxial):
        out = np.zeros((nr, nt), complex)
        base = 1j * qz[None, j] * rnl[None, j] * RHO0 / rhou
        if nonparaxial:
            out[:, j] = base * beta[None, j] / kz[:, j] * Kg[:, j] * wg[None, j]
        else:
            out[:, j] = np.broadcast_to(base, (nr, len(j)))
        return out

    def one_step(nonparaxial):
        S0 = np.fft.ifft(E0, axis=1)
        P = P_RK4(lam(nonparaxial) * DZ)
        if nonparaxial:
            Eh = P * (T @ (s[:, None] * S0))
        else:
            Eh = T @ (s[:, None] * (P * S0))
        return G * np.fft.fft((1.0 / s)[:, None] * (T @ (D * Eh)), axis=1)

    def err(E):
        return np.linalg.norm(E - E1) / np.linalg.norm(E1)

    assert err(one_step(not qparaxial)) < 1e-8
    assert err(one_step(qparaxial)) > 1e-6        # the prefactors are told apart
    sim.close()


def P_RK4(x):
    return P["RK4"](x)
