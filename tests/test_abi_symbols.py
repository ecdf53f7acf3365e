"""The C-ABI library builds, loads without a GPU, exports every function
declared in include/filament_gb.h, and refuses work loudly without one."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "filament_gb.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(fil_[a-z_]+)\s*\(", src)))


def test_header_declares_the_abi():
    names = declared_functions()
    for n in ("fil_create", "fil_destroy", "fil_set_field", "fil_get_field", "fil_step",
              "fil_run", "fil_analyze", "fil_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol():
    import build as b
    lib = ctypes.CDLL(b.build())
    for n in declared_functions():
        assert hasattr(lib, n), n


def test_julia_binding_calls_declared_symbols():
    """Julia is absent here, so the ccall shim (julia/FilamentGB.jl) is not
    run; every symbol it binds must still be one the header declares, and
    the handle's core entry points must all be bound."""
    jl = open(os.path.join(ROOT, "filament.jl_gb300", "julia", "FilamentGB.jl")).read()
    called = set(re.findall(r"ccall\(\(:(fil_[a-z_0-9]+)\s*,", jl))
    names = set(declared_functions())
    assert called and called <= names, sorted(called - names)
    for n in ("fil_create", "fil_destroy", "fil_set_field", "fil_get_field", "fil_run", "fil_analyze",
              "fil_analyze_spectrum", "fil_get_surrogate_stats", "fil_create_batch", "fil_batch_run"):
        assert n in called, n


def _c_struct(name):
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct %s \{(.*?)\} %s;" % (name, name), src, flags=re.S).group(1)
    out = []
    for ty, field, n in re.findall(r"(int32_t|uint32_t|int64_t|double)\s+(\w+)(?:\[(\d+)\])?;", body):
        out.append((field, ty, int(n) if n else 1))
    return out


def _jl_struct(name):
    jl = open(os.path.join(ROOT, "filament.jl_gb300", "julia", "FilamentGB.jl")).read()
    body = re.search(r"struct %s\b(.*?)\nend" % name, jl, flags=re.S).group(1)
    types = {"Int32": "int32_t", "UInt32": "uint32_t", "Int64": "int64_t", "Float64": "double"}
    out = []
    for field, ty in re.findall(r"(\w+)::((?:NTuple\{\d+,\w+\})|\w+)", body):
        m = re.match(r"NTuple\{(\d+),(\w+)\}", ty)
        out.append((field, types[m.group(2)], int(m.group(1))) if m else (field, types[ty], 1))
    return out


@pytest.mark.parametrize("c_name, jl_name", [("fil_config", "FilConfig"), ("fil_stats", "FilStats")])
def test_julia_structs_mirror_the_header(c_name, jl_name):
    """The Julia mirrors of the ABI structs list the header's fields in its
    order with the same C types (a ccall passes them by layout)."""
    assert _jl_struct(jl_name) == _c_struct(c_name)


@pytest.mark.parametrize("c_name", ["fil_config", "fil_stats", "fil_tables"])
def test_python_structs_mirror_the_header(c_name):
    """The ctypes mirrors in filament_gb/_abi.py: the header's fields in
    its order with the same C types."""
    import ctypes as C
    import filament_gb._abi as abi
    types = {C.c_int32: "int32_t", C.c_uint32: "uint32_t", C.c_int64: "int64_t", C.c_double: "double"}
    got = []
    for field, ty in getattr(abi, c_name)._fields_:
        if issubclass(ty, C.Array):
            got.append((field, types[ty._type_], ty._length_))
        elif ty is C.POINTER(C.c_double):
            got.append((field, "const double*", 1))
        else:
            got.append((field, types[ty], 1))
    if c_name == "fil_tables":
        src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
        body = re.search(r"typedef struct fil_tables \{(.*?)\} fil_tables;", src, flags=re.S).group(1)
        want = [(f, "const double*", 1) for f in re.findall(r"const double\*\s+(\w+);", body)]
    else:
        want = _c_struct(c_name)
    assert got == want


def test_julia_tables_hold_every_pointer():
    src = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    body = re.search(r"typedef struct fil_tables \{(.*?)\} fil_tables;", src, flags=re.S).group(1)
    n = len(re.findall(r"const double\*\s+\w+;", body))
    jl = open(os.path.join(ROOT, "filament.jl_gb300", "julia", "FilamentGB.jl")).read()
    assert re.search(r"p::NTuple\{(\d+),Ptr\{Float64\}\}", jl).group(1) == str(n)


def test_oracle_exports_same_abi(oracle_binding):
    """The oracle mirrors the problem-handle ABI; the handle-free device
    buffer entry point, the learned surrogate (whose CPU reference is
    oracle/surrogate_ref.py) and the batched sweep (whose members are
    checked against single handles) have no C counterpart."""
    import oracle
    lib = ctypes.CDLL(oracle.LIB)
    for n in declared_functions():
        if (n == "fil_hankel_propagate_noalloc" or n.startswith("fil_nn_") or "surrogate" in n
                or "batch" in n):
            continue
        assert hasattr(lib, "filo_" + n[4:]), n


def test_create_rejects_bad_config_before_touching_the_device():
    import filament_gb._abi as abi
    import build as b
    bd = abi.Binding(b.build(), "fil_")
    cfg = abi.fil_config()
    cfg.abi_version = 999
    tab = abi.fil_tables()
    h = ctypes.c_void_p()
    rc = bd.create(ctypes.byref(cfg), ctypes.byref(tab), ctypes.byref(h))
    assert rc == abi.FIL_ERR_ARG
    assert b"version" in bd.last_error(None)


def test_product_has_no_cpu_fallback(monkeypatch):
    """Without the library the host package raises instead of computing."""
    import filament_gb.backend as be
    monkeypatch.setattr(be, "LIB_PATH", "/nonexistent/libfilament_gb.so")
    monkeypatch.setattr(be, "_binding", None)
    with pytest.raises(RuntimeError):
        be.load_library()
