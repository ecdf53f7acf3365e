"""Known answer of the oracle's nonlinear step in the geometries without a
time axis (R and XY): the spatial Kerr form F = 3/4 |E|^2 E
(calc_cubic_nothg_spatial, cubic.jl:49-54) times the field guard G
(nonlinear_propagators.jl:38-67 filters F before Rnl and i QZ) acts point by
point, so the RK step is the scalar RK step of
    dy/dz = i QZ Rnl G 3/4 |y|^2 y
at every transverse point, with QZ Rnl 3/4 = w0 n2 Iu zu / c.  The z-step
(Models.jl:75-121) then applies the linear step and the field guard; the
test applies them by stepping a linear-only handle of the same grid from
the pointwise result, so the linear operator (pinned by the reference's
diffraction tests) is the same on both sides."""
import os

import numpy as np
import pytest
import scipy.constants as sc

from conftest import DECKS
from gpu_helpers import r_input


def _complex(v):
    return np.ascontiguousarray(v, dtype=np.float64).view(np.complex128)


def _rk(alg, f, y, h):
    """Midpoint RK2, Kutta's RK3, the classical RK4 and the Tsitouras 5(4)
    step (its coefficients as the library states them, csrc/tsit5.h)."""
    if alg == "Tsit5":
        from test_oracle_kerr_cw_known_answer import _rk as rk_cw
        return rk_cw(alg, f, y, h)
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


def _xy_input(**kw):
    import filament_gb as fg
    base = dict(Nx=256, Ny=128, xguard=1.0, yguard=1.0)
    base.update(kw)
    return fg.prepare(os.path.join(DECKS, "diffraction_XY", "input.py"), **base)


@pytest.mark.parametrize("geom, alg", [("R", "RK2"), ("R", "RK3"), ("R", "RK4"), ("R", "Tsit5"), ("XY", "RK4")])
def test_spatial_kerr_step_is_the_pointwise_rk_step(oracle_binding, geom, alg):
    import filament_gb as fg
    make = r_input if geom == "R" else _xy_input
    inp = make(NONLINEARITY=True, ALG=alg)
    sim = fg.Simulation(inp, binding=oracle_binding)
    a = sim.problem._arrays
    E0 = sim.handle.get_field()
    c = _complex(a["qz"])[0] * _complex(a["rnl_cubic"])[0] * 0.75
    n2, Iu, zu = inp["p_medium"][2], inp["p_unit"][-1], inp["p_unit"][-2]
    w0 = 2 * np.pi * sc.c / inp["lam0"]
    assert c.imag == 0.0 and c.real == pytest.approx(w0 * n2 * Iu * zu / sc.c, rel=1e-9)
    G = np.asarray(a["guard1"])
    if geom == "XY":
        G = G[:, None] * np.asarray(a["guard2"])[None, :]
    dz = 0.3 / (c.real * np.max(np.abs(E0)) ** 2)      # 0.3 rad of self-phase at the peak
    N = _rk(alg, lambda y: 1j * c * G * np.abs(y) ** 2 * y, E0, dz)
    sim.handle.step(dz, dz)
    E1 = sim.handle.get_field()

    lin = fg.Simulation(make(NONLINEARITY=False, ALG=alg), binding=oracle_binding)
    lin.handle.set_field(N, analytic=True)
    lin.handle.step(dz, dz)
    assert np.linalg.norm(lin.handle.get_field() - E1) <= 1e-13 * np.linalg.norm(E1)
    # the nonlinear step matters, and the tableau is told apart
    lin.handle.set_field(E0, analytic=True)
    lin.handle.step(dz, dz)
    assert np.linalg.norm(lin.handle.get_field() - E1) > 1e-3 * np.linalg.norm(E1)
    for other in ("RK2", "RK3", "RK4", "Tsit5"):
        if other != alg:
            No = _rk(other, lambda y: 1j * c * G * np.abs(y) ** 2 * y, E0, dz)
            assert np.linalg.norm(No - N) > 1e-6 * np.linalg.norm(N)
    lin.close()
    sim.close()
