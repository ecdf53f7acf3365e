"""The Tsitouras 5(4) methods of the FP64 oracle (ALG = Tsit5, ATsit5 of the
reference's decks, examples/RT/input.jl:46): one z-step of the T deck
(Kerr, plasma, Drude current and losses on one time row) against an
accurate ATsit5 solution of the same step.  The local error of the fixed
step falls with the sixth power of dz (order five), RK4's with the fifth;
the adaptive form takes substeps where one step of dz is inaccurate, and
the tolerance options act.  These pin the oracle's tableau by its order;
the CUDA library's copy is held to the oracle by the -m gpu parity tests."""
import os

import numpy as np
import pytest

from conftest import DECKS


def _t_input(**kw):
    import filament_gb as fg
    base = dict(Nt=1024, tmin=-100.0, tmax=100.0, zmax=0.02)
    base.update(kw)
    return fg.prepare(os.path.join(DECKS, "nonlinear_T", "input.py"), **base)


def _one_step(binding, alg, dz, rtol=None, atol=None):
    import filament_gb as fg
    from filament_gb import _abi
    sim = fg.Simulation(_t_input(ALG=alg), binding=binding)
    if rtol is not None:
        sim.handle.set_option(_abi.OPT_ODE_RTOL, int(round(rtol * 1e12)))
    if atol is not None:
        sim.handle.set_option(_abi.OPT_ODE_ATOL, int(round(atol * 1e12)))
    sim.handle.step(dz, dz)
    E = sim.handle.get_field()
    stats = sim.handle.ode_stats()
    sim.close()
    return E, stats


def _accurate(binding, dz):
    return _one_step(binding, "ATsit5", dz, rtol=1e-13, atol=1e-10)


def _err(E, ref):
    return float(np.linalg.norm(E - ref) / np.linalg.norm(ref))


def test_local_error_orders(oracle_binding):
    e5, e4 = [], []
    for dz in (1e-3, 5e-4):
        ref, (att, _) = _accurate(oracle_binding, dz)
        assert att > 1                       # the reference took substeps
        e5.append(_err(_one_step(oracle_binding, "Tsit5", dz)[0], ref))
        e4.append(_err(_one_step(oracle_binding, "RK4", dz)[0], ref))
    r5, r4 = e5[0] / e5[1], e4[0] / e4[1]
    print("local error ratio over a halving of dz: Tsit5 %.1f (%.2e, %.2e), RK4 %.1f" % (r5, *e5, r4))
    assert 20.0 < r4 < 45.0                  # 2^5 = 32
    assert r5 > 50.0                         # 2^6 = 64 (pre-asymptotic: larger)
    assert e5[1] < 1e-2 * e4[1]


def test_fixed_step_counts_no_substeps(oracle_binding):
    _, stats = _one_step(oracle_binding, "Tsit5", 1e-3)
    assert stats == (0, 0)


@pytest.mark.parametrize("dz", [4e-3, 8e-3])
def test_adaptive_substeps(oracle_binding, dz):
    """At dz = 4e-3 and 8e-3 one Tsit5 step is inaccurate (the stiff part of
    the Kerr spectrum); the adaptive form rejects, substeps, and lands near
    the accurate solution, closer with the tighter tolerance."""
    ref, _ = _accurate(oracle_binding, dz)
    fixed = _err(_one_step(oracle_binding, "Tsit5", dz)[0], ref)
    E_def, (att, rej) = _one_step(oracle_binding, "ATsit5", dz)
    E_tight, (att_t, _) = _one_step(oracle_binding, "ATsit5", dz, rtol=1e-9, atol=1e-9)
    e_def, e_tight = _err(E_def, ref), _err(E_tight, ref)
    print("dz %.0e: Tsit5 %.2e, ATsit5 default %.2e (%d attempts, %d rejected), tight %.2e (%d attempts)"
          % (dz, fixed, e_def, att, rej, e_tight, att_t))
    assert att >= 3 and rej >= 1
    assert e_def < 1e-4 < fixed
    assert att_t > att and e_tight < 0.1 * e_def


def test_plasma_alg_tsit5_refused(oracle_binding):
    """The plasma equation's ALG stays RK2/3/4 (its scan is built on
    three stage points per time step): Tsit5 there is refused."""
    import ctypes as C
    import filament_gb as fg
    from filament_gb import _abi
    sim = fg.Simulation(_t_input(), binding=oracle_binding)
    cfg = _abi.fil_config()
    C.memmove(C.byref(cfg), C.byref(sim.problem.config), C.sizeof(cfg))
    cfg.plasma_alg = _abi.ALG["Tsit5"]
    h = C.c_void_p()
    rc = oracle_binding.create(C.byref(cfg), C.byref(sim.problem.tables), C.byref(h))
    sim.close()
    assert rc == _abi.FIL_ERR_UNSUPPORTED
