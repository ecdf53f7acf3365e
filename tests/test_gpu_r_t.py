"""The R and T geometries on the GPU against the FP64 oracle through the C
ABI: R (no time axis) runs the pointwise nonlinear step of the spatial
cubic response (cubic.jl:49-54) and the Hankel pair as matrix-vector
products; T (one time row) runs the row kernel with the linear step
pointwise in w on both halves of the spectrum (spectral.jl:54-75).
Tolerances as in test_gpu_parity."""
import numpy as np
import pytest

from gpu_helpers import pair, r_input, rel_l2, step_both, t_input

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-5, "fp64": 1e-10}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_t_steps_with_plasma(gpu_lib, precision):
    g, r = pair(t_input(), precision, store_plasma=True)
    assert g.problem.config.geometry == 1
    step_both(g, r, 4, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]
    rho_r = r.handle.get_plasma(0)
    assert np.max(rho_r) > 1e-6
    assert rel_l2(g.handle.get_plasma(0), rho_r) < TOL[precision]
    ag, ar = g.handle.analyze(), r.handle.analyze()
    assert ag["energy"] == pytest.approx(ar["energy"], rel=TOL[precision])
    assert rel_l2(ag["power"], ar["power"]) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_t_device_loop(gpu_lib, precision):
    inp = t_input(dzphimax=0.1, dz_initial=1e-2, zmax=0.03, ALG="RK3")
    g, r = pair(inp, precision)
    code_g, st_g = g.handle.run(0.0, inp["zmax"], 10 ** 6)
    code_r, st_r = r.handle.run(0.0, inp["zmax"], 10 ** 6)
    assert code_g == code_r == 1 and st_g["steps"] == st_r["steps"]
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 10 * TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_r_kerr_steps(gpu_lib, precision):
    g, r = pair(r_input(), precision)
    assert g.problem.config.geometry == 0
    step_both(g, r, 5, 2e-3)
    Eg, Er = g.handle.get_field(), r.handle.get_field()
    assert rel_l2(Eg, Er) < TOL[precision]
    # the Kerr term acted: a linear run differs
    lin, rl = pair(r_input(NONLINEARITY=False), "fp64")
    step_both(lin, rl, 5, 2e-3)
    assert rel_l2(rl.handle.get_field(), Er) > 1e-4
    ag, ar = g.handle.analyze(), r.handle.analyze()
    assert ag["energy"] == pytest.approx(ar["energy"], rel=TOL[precision])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_r_device_loop(gpu_lib, precision):
    inp = r_input(dzphimax=0.05, dz_initial=1e-2, zmax=0.05)
    g, r = pair(inp, precision)
    code_g, st_g = g.handle.run(0.0, inp["zmax"], 10 ** 6)
    code_r, st_r = r.handle.run(0.0, inp["zmax"], 10 ** 6)
    assert code_g == code_r == 1 and st_g["steps"] == st_r["steps"]
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 10 * TOL[precision]
