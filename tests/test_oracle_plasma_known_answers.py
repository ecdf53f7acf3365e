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


@pytest.mark.parametrize("i_iu", [3.0, 20.0, 60.0])
def test_oracle_plasma_matches_closed_form_with_reference_tables(oracle_binding, i_iu):
    import filament_gb as fg
    from filament_gb import _abi
    inp = rt_input(Nr=4, Nt=512, PPcr=1.0)
    pe = inp["p_model"][1]
    pe["components"] = reference_air_components()
    pe["KDEP"] = True
    pe["rho_nt"] = 2.5e25
    pe["nuc"] = 0.0                      # no avalanche: Rava = 0
    pe["ALG"] = "RK3"
    sim = fg.Simulation(inp, binding=oracle_binding, make_handle=False)
    prob = sim.problem
    assert np.all(prob.pe.rava == 0.0)
    h = fg.Handle(prob, oracle_binding)
    nr, nt = prob.config.n1, prob.config.nt
    amp = np.sqrt(i_iu * np.array([1.0, 0.5, 0.25, 0.0]))
    E = np.repeat(amp[:, None], nt, axis=1).astype(np.complex128)   # |E|^2 constant in t
    h.set_field(E, analytic=True)
    rho = h.get_plasma(0)
    kd = h.get_plasma(1)
    dt = prob.config.dt
    j = np.arange(nt)
    for r in range(nr):
        I = abs(amp[r]) ** 2
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
