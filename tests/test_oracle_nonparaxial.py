"""The oracle's non-paraxial nonlinear prefactor (func!'s else branch,
nonlinear_propagators.jl:58-63, with Qfunc_nonparaxial, :232-241).

QZ(kt, w) / QZ(w) = beta / sqrt(beta^2 - kt^2) = 1 + kt^2 / (2 beta^2) + ...,
so for a beam whose transverse spectrum lies at kt << beta the non-paraxial
step differs from the paraxial one by that relative amount, while the
Hankel transform pair around the factor must not add an error of its own.
"""
import numpy as np

from gpu_helpers import rel_l2, rt_input


def _run(oracle_binding, qparaxial, steps=3, dz=2e-3, **kw):
    import filament_gb as fg
    inp = rt_input(PLASMA=False, PPcr=30.0, QPARAXIAL=qparaxial, **kw)
    sim = fg.Simulation(inp, binding=oracle_binding)
    z = 0.0
    for _ in range(steps):
        z += dz
        sim.handle.step(z, dz)
    E = sim.handle.get_field()
    kt = sim.grid.k * sim.unit.k
    sim.close()
    return E, kt


def test_nonparaxial_prefactor_approaches_the_paraxial_one(oracle_binding):
    import filament_gb as fg
    from filament_gb import media
    Ep, kt = _run(oracle_binding, True)
    En, _ = _run(oracle_binding, False)
    d = rel_l2(En, Ep)
    # bound: the largest kt^2 / (2 beta^2) on the grid times the nonlinear
    # share of the step (the step's change of the field is far below 1)
    inp = rt_input(PLASMA=False, PPcr=30.0)
    sim = fg.Simulation(inp, make_handle=False)
    beta = media.k_func(sim.medium, sim.field.w0)
    bound = float(np.max(kt) ** 2 / (2 * beta ** 2))
    assert 0.0 < d < bound
    # the effect grows with the beam's transverse spectrum: a narrower beam
    # (wider spectrum) sees a larger difference
    Epn, _ = _run(oracle_binding, True, beam_a0=0.25e-3)
    Enn, _ = _run(oracle_binding, False, beam_a0=0.25e-3)
    assert rel_l2(Enn, Epn) > 3 * d
