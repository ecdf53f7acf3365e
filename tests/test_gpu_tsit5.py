"""The Tsitouras 5(4) methods (ALG = Tsit5, ATsit5) on the GPU against the
FP64 oracle, through the C ABI, in every geometry: the row kernel's
Tsitouras variant (T, RT, XYT: stage derivatives in HBM, per-row
substeps with a block-reduced error norm) and the pointwise kernel (R, XY:
per-point substeps).  Fixed steps: tolerances of the other parity tests.
Adaptive steps: in FP64 the substep decisions are the oracle's (equal
attempt and rejection counts) and so is the field; in the mixed form
decisions near err = 1 may differ, so counts agree to 5% and the field to
the tolerance's order.  Inputs are scaled (x2, x3) and tolerances tightened
where the unscaled decks need no substeps."""
import numpy as np
import pytest

from gpu_helpers import pair, r_input, rel_l2, rt_input, step_both, t_input, xyt_input

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-5, "fp64": 1e-10}


def _xy_input(**kw):
    from test_gpu_xy import xy_input
    return xy_input(NONLINEARITY=True, xguard=1.0, yguard=1.0, **kw)


INPUTS = {
    "RT": lambda **kw: rt_input(**kw),
    "T": lambda **kw: t_input(**kw),
    "XYT": lambda **kw: xyt_input(**kw),
    "R": lambda **kw: r_input(**kw),
    "XY": lambda **kw: _xy_input(**kw),
}
DZ = {"RT": 2e-3, "T": 1e-3, "XYT": 2e-3, "R": 2e-3, "XY": 0.02}


def _tolerances(sims, rtol, atol):
    from filament_gb import _abi
    for s in sims:
        s.handle.set_option(_abi.OPT_ODE_RTOL, int(round(rtol * 1e12)))
        s.handle.set_option(_abi.OPT_ODE_ATOL, int(round(atol * 1e12)))


def _scale(sims, sc):
    for s in sims:
        s.handle.set_field(s.field.E0 * sc, analytic=False)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("geom", ["RT", "T", "XYT", "R", "XY"])
def test_tsit5_steps(gpu_lib, geom, precision):
    g, r = pair(INPUTS[geom](ALG="Tsit5"), precision)
    step_both(g, r, 3, DZ[geom])
    Eg, Er = g.handle.get_field(), r.handle.get_field()
    e = rel_l2(Eg, Er)
    assert e < TOL[precision]
    assert g.handle.ode_stats() == (0, 0)
    if precision == "fp64" and geom in ("T", "R"):
        # the method is Tsitouras, not RK4: the FP64 field is far closer to
        # the oracle's Tsit5 step than to its RK4 step (T: the row kernel's
        # variant, the methods differ by 8e-6; R: the pointwise kernel,
        # 2e-10; in RT, XY and XYT the steps are too small to tell them apart
        # at FP64 resolution)
        import filament_gb as fg
        import oracle
        r4 = fg.Simulation(INPUTS[geom](ALG="RK4"), binding=oracle.binding())
        z = 0.0
        for _ in range(3):
            z += DZ[geom]
            r4.handle.step(z, DZ[geom])
        d4 = rel_l2(Eg, r4.handle.get_field())
        print("%s: Tsit5 GPU vs oracle Tsit5 %.2e, vs oracle RK4 %.2e" % (geom, e, d4))
        assert d4 > 10 * e


# (geometry, dz, steps, field scale, rtol = atol) per precision; the FP64
# cases reject and substep
ADAPTIVE = {
    "fp64": [("RT", 5e-3, 2, 2.0, 1e-12), ("T", 4e-3, 2, 1.0, 1e-6), ("R", 5e-3, 2, 1.0, 1e-12),
             ("XY", 0.1, 2, 1.0, 1e-12), ("XYT", 5e-3, 1, 2.0, 1e-12)],
    "mixed": [("RT", 5e-3, 2, 2.0, 1e-5), ("T", 4e-3, 2, 1.0, 1e-3), ("R", 5e-3, 2, 3.0, 1e-5),
              ("XY", 0.1, 2, 3.0, 1e-5)],
}


@pytest.mark.parametrize("case", [("fp64",) + c for c in ADAPTIVE["fp64"]] +
                         [("mixed",) + c for c in ADAPTIVE["mixed"]],
                         ids=lambda c: "%s-%s" % (c[0], c[1]))
def test_atsit5_steps(gpu_lib, case):
    precision, geom, dz, n, sc, tol = case
    g, r = pair(INPUTS[geom](ALG="ATsit5"), precision)
    _tolerances((g, r), tol, tol)
    if sc != 1.0:
        _scale((g, r), sc)
    step_both(g, r, n, dz)
    (ag, jg), (ar, jr) = g.handle.ode_stats(), r.handle.ode_stats()
    print("%s %s: attempts %d / %d, rejected %d / %d (GPU / oracle)" % (precision, geom, ag, ar, jg, jr))
    e = rel_l2(g.handle.get_field(), r.handle.get_field())
    if precision == "fp64":
        assert (ag, jg) == (ar, jr)
        assert e < TOL["fp64"]
    else:
        assert abs(ag - ar) <= 0.05 * ar and abs(jg - jr) <= 0.05 * max(jr, 20)
        assert e < 3 * TOL["mixed"]
    assert g.handle.stats()["flags"] & 8 == 0


def test_atsit5_substeps_happen(gpu_lib):
    """The FP64 adaptive cases above do take substeps (more attempts than
    points x steps) and reject some."""
    g, r = pair(rt_input(ALG="ATsit5"), "fp64")
    _tolerances((g, r), 1e-12, 1e-12)
    _scale((g, r), 2.0)
    step_both(g, r, 2, 5e-3)
    att, rej = g.handle.ode_stats()
    assert att > 2 * g.problem.config.n1 and rej > 0


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_tsit5_device_loop(gpu_lib, precision):
    """fil_run's device loop (adaptive dz, phimax) with the Tsitouras step."""
    inp = rt_input(ALG="Tsit5", zmax=0.05)
    g, r = pair(inp, precision)
    cg, sg = g.handle.run(0.0, inp["zmax"], 10 ** 6)
    cr, sr = r.handle.run(0.0, inp["zmax"], 10 ** 6)
    assert cg == cr == 1 and sg["steps"] == sr["steps"]
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 10 * TOL[precision]


def test_tsit5_refusals(gpu_lib):
    """Built for the paraxial prefactor and up to two species; the plasma
    equation's own ALG stays RK2/3/4."""
    import ctypes as C
    import filament_gb as fg
    from filament_gb import _abi
    from gpu_helpers import many_species_rates
    b = fg.load_library()
    three = rt_input(ALG="ATsit5")
    three["p_model"][1]["components"] = many_species_rates(3)
    for inp in (rt_input(ALG="Tsit5", QPARAXIAL=False), three):
        with pytest.raises(_abi.FilError) as ei:
            fg.Simulation(inp, precision="fp64")
        assert ei.value.code == _abi.FIL_ERR_UNSUPPORTED
    sim = fg.Simulation(rt_input(), precision="fp64")
    cfg = _abi.fil_config()
    C.memmove(C.byref(cfg), C.byref(sim.problem.config), C.sizeof(cfg))
    cfg.plasma_alg = _abi.ALG["Tsit5"]
    h = C.c_void_p()
    rc = b.create(C.byref(cfg), C.byref(sim.problem.tables), C.byref(h))
    sim.close()
    assert rc == _abi.FIL_ERR_UNSUPPORTED
