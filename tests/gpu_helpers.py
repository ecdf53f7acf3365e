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


def t_input(**kw):
    """A T-geometry deck: the RT filament deck's pulse and air on one time
    row (the beam factor taken at r = 0)."""
    import filament_gb as fg
    from conftest import DECKS
    base = dict(Nt=1024, tmin=-100.0, tmax=100.0, zmax=0.02)
    base.update(kw)
    return fg.prepare(os.path.join(DECKS, "nonlinear_T", "input.py"), **base)


def r_input(**kw):
    """An R-geometry deck: a Gaussian beam with Kerr self-focusing."""
    import filament_gb as fg
    from conftest import DECKS
    base = dict(Nr=256, rmax=4.0, zmax=0.02)
    base.update(kw)
    return fg.prepare(os.path.join(DECKS, "nonlinear_R", "input.py"), **base)


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


def many_species_rates(n):
    """n ionising species (3 or 4): N2 and O2 as two_species_rates, then an
    argon-like (K = 10.5) and a water-like (K = 7) trace species, power laws
    of the form of the reference's .tf tables."""
    from filament_gb.plasma import power_law_rate
    comps = two_species_rates()
    comps[0]["fraction"] = 0.78
    comps.append({"fraction": 0.01, "ionization_energy": 15.76,
                  "ionization_rate": power_law_rate(10.5, 1e18, 2.0e10)})
    comps.append({"fraction": 0.01, "ionization_energy": 12.62,
                  "ionization_rate": power_law_rate(7.0, 1e18, 3.0e12)})
    return comps[:n]


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def reference_air_components():
    """The reference's two-species air (examples/RT/air.jl:96-108): N2 and
    O2 with the multiphoton rates of its examples/RT/multiphoton_N2.tf and
    multiphoton_O2.tf (copied to tests/golden), loaded by file name through
    TFunction.from_file as init_photoionization_avalanche does."""
    n2 = {"fraction": 0.79, "ionization_energy": 15.576,
          "ionization_rate": os.path.join(GOLDEN, "multiphoton_N2.tf")}
    o2 = {"fraction": 0.21, "ionization_energy": 12.063,
          "ionization_rate": os.path.join(GOLDEN, "multiphoton_O2.tf")}
    return [n2, o2]


def saturating_rate(n=14):
    """A tabulated rate that is not a power law: W = W8(I) / (1 + (I/Is)^5),
    W8 the sigma_8 I^8 multiphoton rate of the decks, Is = 5e17 W/m^2, so
    the local order d ln W / d ln I falls from 8 to 3 across the table (the
    general interpolation branch and tfpower on distinct segments)."""
    I = np.logspace(9.0, 20.0, n)
    W = 8.85e12 * (I / 1e18) ** 8 / (1.0 + (I / 5e17) ** 5)
    return I, W


def pair(inp, precision="mixed", store_plasma=False, project=None):
    """(CUDA simulation, oracle simulation) on the same input, both with the
    same treatment of the upper half of the spectrum: kept as the reference
    keeps it (project=False, the default) or dropped after each t->w
    transform (project=True), so that the two differ by arithmetic only."""
    import filament_gb as fg
    import oracle
    from filament_gb import _abi
    if project is None:
        project = False
    g = fg.Simulation(inp, precision=precision)
    r = fg.Simulation(inp, binding=oracle.binding())
    if project:
        r.handle.set_option(_abi.OPT_ANALYTIC_PROJECTION, 1)
        g.handle.set_option(_abi.OPT_ANALYTIC_PROJECTION, 1)
        g.handle.set_field(g.field.E0, analytic=False)
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
