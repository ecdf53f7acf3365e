"""Host side of the batched sweep: the seeded parameter draw and the C ABI's
argument checks (which run before any device call)."""
import ctypes

import numpy as np


def test_draw_is_seeded_and_in_range():
    from filament_gb import sweep
    a = sweep.draw(64, 0)
    b = sweep.draw(64, 0)
    assert a == b
    assert a != sweep.draw(64, 1)
    assert len(a) == 64
    assert {p["Nr"] for p in a} == set(sweep.NR_CHOICES)
    assert {p["Nt"] for p in a} == set(sweep.NT_CHOICES)
    P = np.array([p["PPcr"] for p in a])
    ch = np.array([p["chirp_fs2"] for p in a])
    w0 = np.array([p["beam_a0"] for p in a])
    assert P.min() >= 2 and P.max() <= 10
    assert ch.min() >= -500 and ch.max() <= 500
    assert w0.min() >= 0.5e-3 and w0.max() <= 2e-3


def test_chirped_initial_condition_keeps_energy_and_stretches_the_pulse():
    """A spectral phase leaves the pulse energy unchanged and lowers its peak
    by (1 + (phi2 / t0^2)^2)^(-1/2) in intensity."""
    from filament_gb import sweep
    from filament_gb.filament import Simulation
    base = dict(Nr=32, Nt=2048, PPcr=3.0, beam_a0=1e-3)
    E0 = Simulation(sweep.member_input(dict(base, chirp_fs2=0.0)), make_handle=False).field.E0
    E1 = Simulation(sweep.member_input(dict(base, chirp_fs2=400.0)), make_handle=False).field.E0
    assert abs(np.sum(np.abs(E1[0]) ** 2) / np.sum(np.abs(E0[0]) ** 2) - 1) < 1e-3
    t0 = 35.0 / (2 * np.sqrt(np.log(2)))
    stretch = np.sqrt(1 + (400.0 / t0 ** 2) ** 2)
    # intensity envelope peak of the real field: max over t of the squared
    # field, close to the envelope maximum at this carrier sampling
    assert abs(np.max(np.abs(E1[0]) ** 2) / np.max(np.abs(E0[0]) ** 2) - 1 / stretch) < 0.02


def test_create_batch_rejects_bad_arguments_before_touching_the_device():
    import build as b
    import filament_gb._abi as abi
    from filament_gb.backend import _batch_fns
    lib = ctypes.CDLL(b.build())
    f = _batch_fns(lib)
    cfg = (abi.fil_config * 2)()
    tab = (abi.fil_tables * 2)()
    out = ctypes.c_void_p()
    assert f["create_batch"](0, cfg, tab, ctypes.byref(out)) == abi.FIL_ERR_ARG
    cfg[0].geometry = abi.GEOM["RT"]
    cfg[1].geometry = abi.GEOM["XYT"]
    assert f["create_batch"](2, cfg, tab, ctypes.byref(out)) == abi.FIL_ERR_UNSUPPORTED
    assert b"RT" in f["batch_last_error"](None)
    assert not out
