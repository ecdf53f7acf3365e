"""Shared set-up for the GPU parity tests: the same input drives the CUDA
library and the FP64 oracle through the same C ABI."""
import os

import numpy as np

from conftest import PKG_DECKS

FIL_DECK = os.path.join(PKG_DECKS, "filament_RT", "input.py")
XYT_DECK = os.path.join(PKG_DECKS, "filament_XYT", "input.py")


def rt_input(**kw):
    import filament_gb as fg
    base = dict(Nr=64, Nt=512, rmax=2.0, tmin=-100.0, tmax=100.0, zmax=0.02, ALG="RK3")
    base.update(kw)
    return fg.prepare(FIL_DECK, **base)


def xyt_input(**kw):
    """The XYT multifilamentation deck on a small grid (64 x 64 x 512)."""
    import filament_gb as fg
    base = dict(Nx=64, Ny=64, Nt=512, zmax=0.02)
    base.update(kw)
    return fg.prepare(XYT_DECK, **base)


def two_species_rates():
    """N2 and O2 power laws with the multiphoton orders and magnitudes of
    the reference's examples (K = 7.5 and 6.5 log-log slopes)."""
    from filament_gb.plasma import power_law_rate
    n2 = {"fraction": 0.79, "ionization_energy": 15.576,
          "ionization_rate": power_law_rate(7.5, 1e18, 1.0e11)}
    o2 = {"fraction": 0.21, "ionization_energy": 12.063,
          "ionization_rate": power_law_rate(6.5, 1e18, 8.85e12)}
    return [n2, o2]


def pair(inp, precision="mixed", store_plasma=False, project=True):
    """(CUDA simulation, oracle simulation) on the same input.  With
    project=True the oracle drops negative frequencies after each t->w
    transform, as the library's half-spectrum state does, so that the two
    differ by arithmetic only."""
    import filament_gb as fg
    import oracle
    from filament_gb import _abi
    g = fg.Simulation(inp, precision=precision)
    r = fg.Simulation(inp, binding=oracle.binding())
    if project:
        r.handle.set_option(_abi.OPT_ANALYTIC_PROJECTION, 1)
    if store_plasma:
        from filament_gb import _abi
        g.handle.set_option(_abi.OPT_STORE_PLASMA, 1)
        g.handle.set_field(g.field.E0, analytic=False)
    return g, r


def rel_l2(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b)))


def step_both(g, r, n, dz):
    z = 0.0
    for _ in range(n):
        z += dz
        g.handle.step(z, dz)
        r.handle.step(z, dz)
    return z
