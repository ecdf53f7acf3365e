"""Known answers of the oracle's plasma solve with the reference's own rate
tables (examples/RT/multiphoton_N2.tf and multiphoton_O2.tf, copied to
tests/golden).

For a field of constant intensity I and no avalanche (collision frequency
zero, so Rava = 0 in photoionization_avalanche.jl:41-47), every species
obeys the linear equation drho_c/dt = W_c(I) (rho_nt,c - rho_c), and the
explicit RK step of plasma_equations.jl:46-72 multiplies the deficit
rho_nt,c - rho_c by the stability polynomial of the tableau,
R(h) = 1 + h + h^2/2 + h^3/6 for the third-order method (h = -W_c dt).  So
  rho_j   = sum_c rho_nt,c (1 - R(-W_c dt)^j)
  Kdrho_j = sum_c K_c W_c rho_nt,c R(-W_c dt)^(j+1),  Kdrho_{Nt-1} = 0,
with W_c the tables' log-log interpolation (a power law between the knots
for these tables) and K_c = tfpower = the tables' local order (KDEP).
This pins the table reader, the interpolation, tfpower, the RK3 tableau and
the species sum of the oracle, the parts of the reference path no reference
test covers.
"""
import numpy as np
import pytest

from gpu_helpers import GOLDEN, reference_air_components, rt_input


def _table(name):
    d = np.loadtxt(GOLDEN + "/" + name)
    return d[:, 0], d[:, 1]


def test_reference_rate_tables_are_read_as_tabulated():
    from filament_gb.plasma import TFunction
    for name, order in (("multiphoton_N2.tf", 7.5), ("multiphoton_O2.tf", 6.5)):
        I, W = _table(name)
        assert len(I) == 10
        tf = TFunction.from_file(GOLDEN + "/" + name)
        for x, y in zip(I, W):
            assert tf(x) == pytest.approx(y, rel=1e-12)
        # between knots: the power law of the segment; tfpower its order
        xm = np.sqrt(I[3] * I[4])
        assert tf(xm) == pytest.approx(np.sqrt(W[3] * W[4]), rel=1e-12)
        assert tf.power(xm) == pytest.approx(order, rel=1e-9)


PHASE = 0.6   # rad: Re(E)^2 = cos^2(0.6) |E|^2 for the EREAL cases


@pytest.mark.parametrize("ereal", [False, True], ids=["I=|E|^2", "EREAL: I=Re(E)^2"])
@pytest.mark.parametrize("i_iu", [3.0, 20.0, 60.0])
def test_oracle_plasma_matches_closed_form_with_reference_tables(oracle_binding, i_iu, ereal):
    """The field is constant in t with phase 0.6 rad, so the rate's argument
    (photoionization_avalanche.jl:1-17: |E|^2, or Re(E)^2 with EREAL) is the
    constant I = A^2 or A^2 cos^2(0.6)."""
    import filament_gb as fg
    from filament_gb import _abi
    inp = rt_input(Nr=4, Nt=512, PPcr=1.0)
    pe = inp["p_model"][1]
    pe["components"] = reference_air_components()
    pe["KDEP"] = True
    pe["EREAL"] = ereal
    pe["rho_nt"] = 2.5e25
    pe["nuc"] = 0.0                      # no avalanche: Rava = 0
    pe["ALG"] = "RK3"
    sim = fg.Simulation(inp, binding=oracle_binding, make_handle=False)
    prob = sim.problem
    assert np.all(prob.pe.rava == 0.0)
    h = fg.Handle(prob, oracle_binding)
    nr, nt = prob.config.n1, prob.config.nt
    amp = np.sqrt(i_iu * np.array([1.0, 0.5, 0.25, 0.0])) * np.exp(1j * PHASE)
    E = np.repeat(amp[:, None], nt, axis=1).astype(np.complex128)   # |E|^2 constant in t
    h.set_field(E, analytic=True)
    rho = h.get_plasma(0)
    kd = h.get_plasma(1)
    dt = prob.config.dt
    j = np.arange(nt)
    for r in range(nr):
        I = amp[r].real ** 2 if ereal else abs(amp[r]) ** 2
        rho_ref = np.zeros(nt)
        kd_ref = np.zeros(nt)
        for c, tf in enumerate(prob.pe.tfs):
            W = tf(I)
            K = tf.power(I) if I > 0 else tf.power(1e-300)
            x = -W * dt
            lnR = np.log1p(x + x * x / 2 + x ** 3 / 6)   # R - 1 without cancellation
            rnt = prob.pe.rho_nt[c]
            rho_ref += rnt * -np.expm1(j * lnR)
            kd_ref += K * W * rnt * np.exp((j + 1) * lnR)
        kd_ref[-1] = 0.0
        scale = max(np.max(np.abs(rho_ref)), 1e-300)
        assert np.max(np.abs(rho[r] - rho_ref)) <= 1e-12 * scale + 1e-300
        kscale = max(np.max(np.abs(kd_ref)), 1e-300)
        assert np.max(np.abs(kd[r] - kd_ref)) <= 1e-12 * kscale + 1e-300
    assert np.max(rho) > 0 or i_iu < 10
    h.close()


def _kutta3(f, y, h):
    k1 = f(y)
    k2 = f(y + h / 2 * k1)
    k3 = f(y - h * k1 + 2 * h * k2)
    return y + h / 6 * (k1 + 4 * k2 + k3)


@pytest.mark.parametrize("i_iu", [1.0, 10.0])
def test_oracle_avalanche_matches_the_rk3_recursion(oracle_binding, i_iu):
    """With avalanche (photoionization_avalanche.jl:119-148): for a real
    field of constant amplitude A, so that I = |E|^2 = Re(E)^2 = A^2 at
    every stage point, the species obey the autonomous system
      drho_c/dt = W_c(I) (rho_nt,c - rho_c)
                  + Rava_c A^2 (rho_nt,c - rho_c) / rho_nt,c sum_c' rho_c',
    and the plasma solve is the RK3 (Kutta) recursion of that system from
    rho = rho0.  Kdrho comes from a second recursion of the photoionisation
    terms alone (plasma_equations.jl:45-69 steps func_photoionization for
    it): Kdrho_j = sum_c K_c W_c (rho_nt,c - rho'_c,j+1) (kdrho_func,
    photoionization_avalanche.jl:176-204; 0 at the last point).
    Rava_c = e^2 / m_r nu_c / (nu_c^2 + w0^2) / Ui_c tu Eu^2
    (photoionization_avalanche.jl:41-47) is checked from the constants.  A
    collision frequency near w0 makes the avalanche dominate the density."""
    import scipy.constants as sc
    import filament_gb as fg
    inp = rt_input(Nr=4, Nt=512, PPcr=1.0)
    pe = inp["p_model"][1]
    pe["components"] = reference_air_components()
    pe["KDEP"] = True
    pe["rho_nt"] = 2.5e25
    pe["nuc"] = 2e15
    pe["ALG"] = "RK3"
    sim = fg.Simulation(inp, binding=oracle_binding, make_handle=False)
    prob = sim.problem
    h = fg.Handle(prob, oracle_binding)
    nr, nt, dt = prob.config.n1, prob.config.nt, prob.config.dt
    tu, Iu = inp["p_unit"][2], inp["p_unit"][3]

    # Rava from the constants; n0 from the medium's beta at the carrier bin
    w0 = 2 * np.pi * sc.c / inp["lam0"]
    w = 2 * np.pi * np.fft.fftfreq(nt, dt * tu)
    kc = int(round(w0 / w[1]))
    beta = np.ascontiguousarray(prob._arrays["beta"], dtype=np.float64).view(np.complex128)
    n0 = beta[kc].real / inp["p_unit"][1] * sc.c / w[kc]
    Eu2 = Iu / (n0 * sc.epsilon_0 * sc.c / 2)
    for c, comp in enumerate(reference_air_components()):
        sigma = sc.e ** 2 / sc.m_e * pe["nuc"] / (pe["nuc"] ** 2 + w0 ** 2)
        rava = sigma / (comp["ionization_energy"] * sc.e) * tu * Eu2
        assert prob.pe.rava[c] == pytest.approx(rava, rel=1e-6)

    amp = np.sqrt(i_iu * np.array([1.0, 0.7, 0.5, 0.35]))
    E = np.repeat(amp[:, None], nt, axis=1).astype(np.complex128)
    h.set_field(E, analytic=True)
    rho = h.get_plasma(0)
    kd = h.get_plasma(1)
    rnt = np.asarray(prob.pe.rho_nt, dtype=np.float64)
    rava = np.asarray(prob.pe.rava, dtype=np.float64)
    for r in range(nr):
        I = amp[r] ** 2
        W = np.array([tf(I) for tf in prob.pe.tfs])
        K = np.array([tf.power(I) for tf in prob.pe.tfs])
        f_ava = lambda y: W * (rnt - y) + rava * I * (rnt - y) / rnt * np.sum(y)
        f_photo = lambda y: W * (rnt - y)
        y = np.full(len(rnt), float(prob.pe.rho0))
        yp = y.copy()
        rho_ref, rho_photo, kd_ref = np.zeros(nt), np.zeros(nt), np.zeros(nt)
        rho_ref[0] = rho_photo[0] = np.sum(y)
        for j in range(nt - 1):
            y = _kutta3(f_ava, y, dt)
            yp = _kutta3(f_photo, yp, dt)
            rho_ref[j + 1], rho_photo[j + 1] = np.sum(y), np.sum(yp)
            kd_ref[j] = np.sum(K * W * (rnt - yp))
        scale = np.max(np.abs(rho_ref))
        assert np.max(np.abs(rho[r] - rho_ref)) <= 1e-12 * scale
        assert np.max(np.abs(kd[r] - kd_ref)) <= 1e-12 * np.max(np.abs(kd_ref))
        # the avalanche term carries most of the density
        assert rho_ref[-1] > 2 * rho_photo[-1]
    h.close()
