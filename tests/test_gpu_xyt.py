"""XYT geometry: the CUDA path (row kernel over the (x, y) points, transverse
2-D transform with the propagator) against the FP64 oracle on the same
seeded multifilamentation input, through the C ABI.  Tolerances as in
test_gpu_parity: 1e-5 relative L2 for the mixed form, 1e-10 for FP64."""
import numpy as np
import pytest

from gpu_helpers import pair, rel_l2, step_both, xyt_input

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-5, "fp64": 1e-10}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_xyt_field_upload(gpu_lib, precision):
    inp = xyt_input(PLASMA=False)
    g, r = pair(inp, precision)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision] / 10


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("kparaxial", [False, True])
def test_xyt_linear_step(gpu_lib, precision, kparaxial):
    """Diffraction and dispersion through the transverse FFT pair and KZ."""
    inp = xyt_input(NONLINEARITY=False, PLASMA=False, KPARAXIAL=kparaxial)
    g, r = pair(inp, precision)
    step_both(g, r, 5, 2e-2)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_xyt_kerr_step(gpu_lib, precision):
    inp = xyt_input(PLASMA=False)
    g, r = pair(inp, precision)
    step_both(g, r, 3, 2e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_xyt_full_step_with_plasma(gpu_lib, precision):
    inp = xyt_input(PPcr=200.0)
    g, r = pair(inp, precision)
    step_both(g, r, 3, 1e-3)
    ag, ar = g.handle.analyze(), r.handle.analyze()
    assert ar["rhomax"] > 0
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]
    assert ag["rhomax"] == pytest.approx(ar["rhomax"], rel=1e-4 if precision == "mixed" else 1e-9)
    assert rel_l2(ag["fluence"], ar["fluence"]) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_xyt_guard_bug_compat(gpu_lib, precision):
    """Guards.jl:314 indexes the time guard by iy; both sides reproduce it."""
    from filament_gb import _abi
    inp = xyt_input(PLASMA=False)
    g, r = pair(inp, precision)
    for s in (g, r):
        s.handle.set_option(_abi.OPT_XYT_GUARD_BUGCOMPAT, 1)
    step_both(g, r, 3, 2e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


def test_xyt_device_loop(gpu_lib):
    inp = xyt_input(PPcr=100.0)
    g, r = pair(inp, "mixed")
    cg, sg = g.handle.run(0.0, 0.05, 6)
    cr, sr = r.handle.run(0.0, 0.05, 6)
    assert (cg, sg["steps"]) == (cr, sr["steps"])
    assert sg["z"] == pytest.approx(sr["z"], rel=1e-5)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 1e-5


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_xyt_upper_half_spectrum(gpu_lib, precision):
    """The upper half of the spectrum (negative frequencies from the time
    guard) goes through the transverse transform and KZ(kx, ky, w) with the
    rest, as in the reference's full-array plan (Fields.jl:150-160,
    spectral.jl:16-26): kept by default, dropped on both sides with
    FIL_OPT_ANALYTIC_PROJECTION.  A narrow time guard makes it visible."""
    inp = xyt_input(PLASMA=False, tguard=60.0, tmin=-100.0, tmax=100.0)
    out = {}
    for project in (False, True):
        g, r = pair(inp, precision, project=project)
        step_both(g, r, 4, 2e-3)
        assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]
        out[project] = r.handle.get_field()
    assert rel_l2(out[True], out[False]) > 100 * TOL["fp64"]
