"""XY geometry (no time axis): the CUDA path (pointwise nonlinear RK step,
transverse 2-D transform with the propagator, field guard) against the FP64
oracle on the same input, through the C ABI.  Tolerances: 1e-5 relative L2
(mixed), 1e-10 (FP64)."""
import os

import pytest

from conftest import DECKS
from gpu_helpers import pair, rel_l2, step_both

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-5, "fp64": 1e-10}


def xy_input(**kw):
    import filament_gb as fg
    base = dict(Nx=256, Ny=128)
    base.update(kw)
    return fg.prepare(os.path.join(DECKS, "diffraction_XY", "input.py"), **base)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("kparaxial", [False, True])
def test_xy_linear_step(gpu_lib, precision, kparaxial):
    """Five 10 cm steps of free diffraction.  The oracle evaluates KZ as the
    reference writes it, sqrt(beta^2 - k^2) + (dfr - beta), which at
    beta = 7.9e6 carries an absolute error of ~8e-10 from cancellation
    (a numpy FFT propagation with the same formula reproduces the oracle);
    the device uses the equal, cancellation-free dfr - k^2/(beta + sqrt(beta^2 -
    k^2)).  Over 0.5 m that leaves ~2e-10 between the FP64 forms."""
    tol = {"mixed": 1e-5, "fp64": 1e-9}[precision]
    g, r = pair(xy_input(KPARAXIAL=kparaxial), precision, project=False)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision] / 10
    step_both(g, r, 5, 0.1)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < tol


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("alg", ["RK2", "RK3", "RK4"])
def test_xy_kerr_step(gpu_lib, precision, alg):
    """cubic.jl:49-54: F = 3/4 |E|^2 E on the spatial field, with guards."""
    inp = xy_input(NONLINEARITY=True, ALG=alg, xguard=1.0, yguard=1.0)
    g, r = pair(inp, precision, project=False)
    step_both(g, r, 3, 0.02)
    ag, ar = g.handle.analyze(), r.handle.analyze()
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]
    assert ag["imax"] == pytest.approx(ar["imax"], rel=10 * TOL[precision])
    assert ag["power"][0] == pytest.approx(ar["power"][0], rel=10 * TOL[precision])


def test_xy_device_loop(gpu_lib):
    inp = xy_input(NONLINEARITY=True)
    g, r = pair(inp, "mixed", project=False)
    cg, sg = g.handle.run(0.0, 1.0, 8)
    cr, sr = r.handle.run(0.0, 1.0, 8)
    assert (cg, sg["steps"]) == (cr, sr["steps"])
    assert sg["z"] == pytest.approx(sr["z"], rel=1e-5)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 1e-5
