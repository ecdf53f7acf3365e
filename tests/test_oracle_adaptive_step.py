"""Known answers of the adaptive z-step (AdaptiveSteps.jl:20-107) in the
oracle's device loop.

The phase rates are the textbook ones:
  phi_kerr = QZ0 |Rnl0| (AdaptiveSteps.jl:46-58) = w0 n2 Iu zu / c, the Kerr
    phase per zu at the unit intensity (n0 cancels);
  phi_plasma = QZ0 |Re Rnl0| (AdaptiveSteps.jl:60-72)
    = mu0 w0^2 zu e^2 rhou / (2 k0 m_r (nu_c^2 + w0^2)), k0 = n0 w0 / c, the
    plasma phase per zu at the unit density.
Each step of the loop takes dz = min(dz0, phimax / (phi_kerr Imax),
phimax / (phi_plasma rhomax)) (AdaptiveSteps.jl:96-107) with Imax of the
current field and rhomax of the last plasma solve (Filament.jl:123-172):
a 1 mm beam at 60 critical powers is held by the Kerr bound, a 0.4 mm one
forms enough plasma that the plasma bound decides its steps."""
import numpy as np
import pytest
import scipy.constants as sc

from gpu_helpers import rt_input


def _setup(oracle_binding, **kw):
    import filament_gb as fg
    inp = rt_input(PPcr=60.0, ALG="RK4", dzphimax=0.1, dz_initial=1e-2, zmax=0.03, **kw)
    return inp, fg.Simulation(inp, binding=oracle_binding)


def test_phase_rates(oracle_binding):
    inp, sim = _setup(oracle_binding)
    cfg = sim.problem.config
    ru, zu, tu, Iu, rhou = inp["p_unit"]
    dz0, phimax, mr, nuc, _ = inp["p_dzadaptive"]
    n2 = inp["p_medium"][2]
    w0 = 2 * np.pi * sc.c / inp["lam0"]
    w = 2 * np.pi * np.fft.fftfreq(cfg.nt, cfg.dt * tu)
    kc = int(round(w0 / w[1]))
    beta = np.ascontiguousarray(sim.problem._arrays["beta"], dtype=np.float64).view(np.complex128)
    n0 = beta[kc].real / zu * sc.c / w[kc]         # n(w) at the carrier's bin
    assert cfg.phik == pytest.approx(w0 * n2 * Iu * zu / sc.c, rel=1e-9)
    k0 = n0 * w0 / sc.c
    phip = sc.mu_0 * w0 ** 2 * zu * sc.e ** 2 * rhou / (2 * k0 * mr * sc.m_e * (nuc ** 2 + w0 ** 2))
    assert cfg.phip == pytest.approx(phip, rel=1e-6)
    assert cfg.dz0 == dz0 and cfg.phimax == phimax
    sim.close()


@pytest.mark.parametrize("beam_a0, nsteps, bound", [(1e-3, 40, 1), (0.4e-3, 6, 2)],
                         ids=["kerr-bound to zmax", "plasma-bound"])
def test_step_sizes(oracle_binding, beam_a0, nsteps, bound):
    """The 1 mm beam's steps are set by the Kerr bound up to zmax (the last
    step may pass it, as the reference's loop does); the 0.4 mm beam's first
    steps by the plasma bound."""
    inp, sim = _setup(oracle_binding, beam_a0=beam_a0)
    cfg, h = sim.problem.config, sim.handle
    st = h.analyze()
    imax, rhomax = st["imax"], st["rhomax"]
    z, kinds, n = 0.0, set(), 0
    while n < nsteps:
        code, st = h.run(z, inp["zmax"], 1)
        if st["z"] == z:
            break
        bounds = [cfg.dz0, cfg.phimax / (cfg.phik * imax),
                  cfg.phimax / (cfg.phip * rhomax) if rhomax > 0 else np.inf]
        assert st["dz"] == pytest.approx(min(bounds), rel=1e-12)
        kinds.add(int(np.argmin(bounds)))
        z, imax, rhomax, n = st["z"], st["imax"], st["rhomax"], n + 1
    assert n >= 5 and kinds == {bound}
    if bound == 1:
        assert z >= inp["zmax"]
    sim.close()
