"""fil_create's argument checks (csrc/api.cu), which run before any device
call, so they are tested here without a GPU: each invalid configuration is
refused with the documented code and a message.  A configuration that is
invalid in itself is refused by the CUDA library and the oracle alike; one
beyond what the CUDA path is built for (Nt outside [512, 4096], the
Tsitouras step with the non-paraxial prefactor or more than two species) by
the library alone, while the oracle, like the reference, runs it.  A valid
configuration passes the checks (the library then stops at "no CUDA
device" on a machine without one, the oracle builds the handle)."""
import ctypes

import pytest

from gpu_helpers import rt_input


def _problem():
    import filament_gb as fg
    return fg.Simulation(rt_input(), make_handle=False).problem


def _copy(cfg):
    import filament_gb._abi as abi
    out = abi.fil_config()
    ctypes.memmove(ctypes.byref(out), ctypes.byref(cfg), ctypes.sizeof(cfg))
    return out


def _bindings(oracle_binding):
    import build as b
    import filament_gb._abi as abi
    return {"library": abi.Binding(b.build(), "fil_"), "oracle": oracle_binding}


CASES = [   # field, value, code, message, refused by the oracle too
    ("abi_version", 999, "ARG", b"version", True),
    ("geometry", 9, "ARG", b"geometry", True),
    ("nt", 1000, "UNSUPPORTED", b"power of two", True),
    ("nt", 256, "UNSUPPORTED", b"power of two", False),
    ("nt", 8192, "UNSUPPORTED", b"power of two", False),
    ("n1", 0, "ARG", b"n1", True),
    ("alg", 9, "ARG", b"ALG", True),
    ("plasma_alg", 5, "UNSUPPORTED", b"plasma ALG", True),
    ("plasma_alg", 0, "ARG", b"plasma ALG", True),
    ("plasma_ncomp", 5, "ARG", b"plasma_ncomp", True),
    ("rate_n", 1, "ARG", b"rate_n", True),
]


@pytest.mark.parametrize("field, value, code, text, both", CASES, ids=["%s=%s" % (c[0], c[1]) for c in CASES])
def test_invalid_configs_are_refused(oracle_binding, field, value, code, text, both):
    import filament_gb._abi as abi
    prob = _problem()
    cfg = _copy(prob.config)
    setattr(cfg, field, value)
    for name, bd in _bindings(oracle_binding).items():
        if name == "oracle" and not both:
            continue
        h = ctypes.c_void_p()
        rc = bd.create(ctypes.byref(cfg), ctypes.byref(prob.tables), ctypes.byref(h))
        assert rc == getattr(abi, "FIL_ERR_" + code), (name, rc)
        assert text.lower() in bd.last_error(None).lower(), (name, bd.last_error(None))
        assert not h.value


def test_tsitouras_refusals(oracle_binding):
    """The CUDA Tsitouras step is built for the paraxial prefactor and up to
    two species; the oracle refuses only the adaptive form with the
    non-paraxial prefactor (whose right-hand side couples the points)."""
    import filament_gb._abi as abi
    prob = _problem()
    b = _bindings(oracle_binding)
    for change, oracle_refuses in (({"alg": abi.ALG["Tsit5"], "qparaxial": 0}, False),
                                   ({"alg": abi.ALG["ATsit5"], "qparaxial": 0}, True),
                                   ({"alg": abi.ALG["ATsit5"], "plasma_ncomp": 3}, False)):
        cfg = _copy(prob.config)
        for k, v in change.items():
            setattr(cfg, k, v)
        h = ctypes.c_void_p()
        rc = b["library"].create(ctypes.byref(cfg), ctypes.byref(prob.tables), ctypes.byref(h))
        assert rc == abi.FIL_ERR_UNSUPPORTED, (change, rc)
        if oracle_refuses:
            rc = b["oracle"].create(ctypes.byref(cfg), ctypes.byref(prob.tables), ctypes.byref(h))
            assert rc == abi.FIL_ERR_UNSUPPORTED, (change, rc)


def test_valid_config_passes_the_checks(oracle_binding):
    import filament_gb._abi as abi
    prob = _problem()
    b = _bindings(oracle_binding)
    h = ctypes.c_void_p()
    rc = b["oracle"].create(ctypes.byref(prob.config), ctypes.byref(prob.tables), ctypes.byref(h))
    assert rc == abi.FIL_OK and h.value
    b["oracle"].destroy(h)
    rc = b["library"].create(ctypes.byref(prob.config), ctypes.byref(prob.tables), ctypes.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except ImportError:
        has_gpu = False
    if has_gpu:
        assert rc == abi.FIL_OK
        b["library"].destroy(h)
    else:
        assert rc == abi.FIL_ERR_CUDA and b"device" in b["library"].last_error(None)


@pytest.mark.parametrize("mpad, nh, text", [(4096, 1024, b"exceeds"), (128, 2 ** 30 + 64, b"exceeds"),
                                            (100, 64, b"mpad"), (128, 0, b"2*nh"), (128, 96, b"2*nh")])
def test_noalloc_entry_checks_its_sizes_first(mpad, nh, text):
    """fil_hankel_propagate_noalloc (csrc/noalloc.cu) refuses sizes that are
    malformed or beyond its fixed 16 MiB array before any device call; the
    pointers (non-null, never dereferenced) stand for device buffers."""
    import build as b
    lib = ctypes.CDLL(b.build())
    f = lib.fil_hankel_propagate_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 7 + [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_double, ctypes.c_void_p]
    err = lib.fil_last_error
    err.restype = ctypes.c_char_p
    err.argtypes = [ctypes.c_void_p]
    one = ctypes.c_void_p(16)
    rc = f(one, one, one, one, one, None, None, 0, one, one, mpad, nh, 1e-3, None)
    assert rc == -1 and text in err(None)
    rc = f(None, one, one, one, one, None, None, 0, one, one, 128, 64, 1e-3, None)
    assert rc == -1 and b"null" in err(None)


def test_null_handle_is_refused_by_every_entry_point(oracle_binding):
    """Every entry point taking a handle answers FIL_ERR_ARG to a null one
    (before touching anything else), in the library and the oracle."""
    import filament_gb._abi as abi
    import build as b
    for bd in (abi.Binding(b.build(), "fil_"), oracle_binding):
        st = abi.fil_stats()
        buf = (ctypes.c_double * 8)()
        i64 = (ctypes.c_int64 * 2)()
        calls = [lambda: bd.step(None, 0.0, 1e-3),
                 lambda: bd.run(None, 0.0, 1.0, 1, ctypes.byref(st)),
                 lambda: bd.analyze(None, ctypes.byref(st), buf, buf, buf),
                 lambda: bd.get_stats(None, ctypes.byref(st)),
                 lambda: bd.set_option(None, 0, 0),
                 lambda: bd.set_field(None, ctypes.cast(buf, ctypes.c_void_p), abi.DTYPE_C128, 0, 0),
                 lambda: bd.get_field(None, ctypes.cast(buf, ctypes.c_void_p), abi.DTYPE_C128, 0),
                 lambda: bd.get_plasma(None, 0, ctypes.cast(buf, ctypes.c_void_p), 0, 0),
                 lambda: bd.kernel_times(None, buf, 8),
                 lambda: bd.get_ode_stats(None, i64),
                 lambda: bd.analyze_spectrum(None, buf, 8)]
        for k, call in enumerate(calls):
            assert call() == abi.FIL_ERR_ARG, (bd.prefix, k)


def test_network_and_batch_entry_points_check_their_arguments():
    """The learned surrogate's and the batched sweep's entry points refuse
    null handles and bad sizes before any device work, and a failure to
    create a network states its cause."""
    import build as b
    L = ctypes.CDLL(b.build())
    vp = ctypes.c_void_p

    def f(name, res, args):
        g = getattr(L, name)
        g.restype, g.argtypes = res, args
        return g

    assert f("fil_nn_nparams", ctypes.c_int, [])() == 76225
    create = f("fil_nn_create", ctypes.c_int, [ctypes.c_int, ctypes.c_uint64, ctypes.POINTER(vp)])
    last = f("fil_nn_last_error", ctypes.c_char_p, [vp])
    assert create(512, 1, None) == -1
    assert create(8, 1, ctypes.byref(vp())) == -1 and b"argument" in last(None)
    for name, args, vals in [("fil_nn_get_params", [vp, vp], [None, None]),
                             ("fil_nn_set_params", [vp, vp], [None, None]),
                             ("fil_nn_forward", [vp, vp, ctypes.c_int, vp], [None, None, 1, None]),
                             ("fil_nn_infer", [vp, vp, ctypes.c_int, vp], [None, None, 1, None]),
                             ("fil_set_surrogate", [vp, vp, ctypes.c_int, ctypes.c_double], [None, None, 1, 1.0]),
                             ("fil_get_surrogate_stats", [vp, vp, ctypes.c_int], [None, None, 0]),
                             ("fil_batch_tune", [vp, ctypes.c_int, vp, ctypes.c_int], [None, 1, None, 0]),
                             ("fil_batch_plan", [vp, vp, vp, vp], [None, None, None, None]),
                             ("fil_create_batch", [ctypes.c_int, vp, vp, ctypes.POINTER(vp)],
                              [0, None, None, ctypes.byref(vp())])]:
        assert f(name, ctypes.c_int, args)(*vals) == -1, name
    assert f("fil_batch_member", vp, [vp, ctypes.c_int])(None, 0) is None
    assert f("fil_nn_destroy", ctypes.c_int, [vp])(None) == 0          # destroying nothing is fine
    assert f("fil_batch_destroy", ctypes.c_int, [vp])(None) == 0


@pytest.mark.parametrize("table, text", [("beta", b"propagator"), ("kt1", b"propagator"), ("dht", b"DHT"),
                                         ("qz", b"QZ"), ("rate_lx", b"plasma tables")])
def test_missing_tables_are_refused(table, text):
    """fil_create refuses a problem whose required table is missing
    (csrc/api.cu), before any device call."""
    import filament_gb._abi as abi
    import build as b
    prob = _problem()
    tab = abi.fil_tables()
    ctypes.memmove(ctypes.byref(tab), ctypes.byref(prob.tables), ctypes.sizeof(tab))
    setattr(tab, table, None)
    bd = abi.Binding(b.build(), "fil_")
    h = ctypes.c_void_p()
    assert bd.create(ctypes.byref(prob.config), ctypes.byref(tab), ctypes.byref(h)) == abi.FIL_ERR_ARG
    assert text in bd.last_error(None)
