"""Loads the CUDA library (libfilament_gb.so, built in-tree) and wraps one
problem handle.  There is no CPU fallback: if the library is missing or no
GPU is present the calls fail with an error."""
import ctypes as C
import os

import numpy as np

from . import _abi

HERE = os.path.dirname(os.path.abspath(__file__))
PKG_ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG_ROOT, "_build", "libfilament_gb.so")

_binding = None


def library_path():
    return LIB_PATH


def load_library():
    """The product binding.  Raises if the extension has not been built."""
    global _binding
    if _binding is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "libfilament_gb.so is not built (%s); run "
                "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        _binding = _abi.Binding(LIB_PATH, "fil_")
    return _binding


class Handle:
    """One problem on one device (or on any library exporting the ABI)."""

    def __init__(self, problem, binding=None):
        self.b = binding if binding is not None else load_library()
        self.problem = problem
        self.h = C.c_void_p()
        code = self.b.create(C.byref(problem.config), C.byref(problem.tables), C.byref(self.h))
        if code < 0:
            msg = self.b.last_error(None)
            raise _abi.FilError(code, "%screate failed: %s" % (self.b.prefix, msg.decode() if msg else "?"))
        self.shape = problem.field_shape

    @classmethod
    def borrow(cls, binding, problem, hptr):
        """A Handle object for a handle that something else owns (a batch
        member): closing it does not destroy the handle."""
        self = cls.__new__(cls)
        self.b = binding
        self.problem = problem
        self.h = C.c_void_p(hptr)
        self.shape = problem.field_shape
        self._owned = False
        return self

    def close(self):
        if self.h and getattr(self, "_owned", True):
            self.b.destroy(self.h)
        self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _chk(self, code, what):
        return self.b.check(self.h, code, what)

    def set_option(self, opt, value):
        self._chk(self.b.set_option(self.h, opt, int(value)), "set_option")

    def set_field(self, E, analytic=False):
        E = np.ascontiguousarray(np.asarray(E, dtype=np.complex128).reshape(self.shape))
        self._chk(self.b.set_field(self.h, E.ctypes.data_as(C.c_void_p), _abi.DTYPE_C128,
                                   _abi.LAYOUT_ROWMAJOR, int(bool(analytic))), "set_field")

    def get_field(self):
        E = np.empty(self.shape, dtype=np.complex128)
        self._chk(self.b.get_field(self.h, E.ctypes.data_as(C.c_void_p), _abi.DTYPE_C128,
                                   _abi.LAYOUT_ROWMAJOR), "get_field")
        return E

    def get_plasma(self, which=0):
        out = np.empty(self.shape, dtype=np.float64)
        self._chk(self.b.get_plasma(self.h, which, out.ctypes.data_as(C.c_void_p),
                                    _abi.DTYPE_F64, _abi.LAYOUT_ROWMAJOR), "get_plasma")
        return out

    def step(self, z, dz):
        self._chk(self.b.step(self.h, float(z), float(dz)), "step")

    def run(self, z0, zmax, nmax):
        st = _abi.fil_stats()
        code = self._chk(self.b.run(self.h, float(z0), float(zmax), int(nmax), C.byref(st)), "run")
        return code, st.as_dict()

    def analyze(self):
        c = self.problem.config
        ntr = c.n1 * c.n2
        has_t = self.problem.geometry in ("T", "RT", "XYT")
        F = np.zeros(ntr)
        P = np.zeros(c.nt if has_t else 1)
        rho_end = np.zeros(ntr)
        st = _abi.fil_stats()
        dp = C.POINTER(C.c_double)
        self._chk(self.b.analyze(self.h, C.byref(st), F.ctypes.data_as(dp), P.ctypes.data_as(dp),
                                 rho_end.ctypes.data_as(dp)), "analyze")
        d = st.as_dict()
        d["fluence"] = F
        d["power"] = P
        d["rho_end"] = rho_end
        return d

    def stats(self):
        st = _abi.fil_stats()
        self._chk(self.b.get_stats(self.h, C.byref(st)), "get_stats")
        return st.as_dict()

    def kernel_times(self, n=3):
        out = np.zeros(n)
        self._chk(self.b.kernel_times(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), n),
                  "kernel_times")
        return out

    def spectrum(self):
        """Integral power spectrum S over the nt/2 + 1 bins of rfftfreq
        (FieldAnalyzers.jl:180-197, 320-336)."""
        nw = self.problem.config.nt // 2 + 1
        out = np.zeros(nw)
        self._chk(self.b.analyze_spectrum(self.h, out.ctypes.data_as(C.POINTER(C.c_double)), nw), "analyze_spectrum")
        return out

    def ode_stats(self):
        """ATsit5: (substep attempts, rejected attempts), summed over the
        transverse points and steps."""
        out = np.zeros(2, np.int64)
        self._chk(self.b.get_ode_stats(self.h, out.ctypes.data_as(C.POINTER(C.c_int64))), "get_ode_stats")
        return int(out[0]), int(out[1])


def _batch_fns(lib):
    vp = C.c_void_p
    dp = C.POINTER(C.c_double)
    ip = C.POINTER(C.c_int)
    sigs = {
        "fil_create_batch": (C.c_int, [C.c_int, C.POINTER(_abi.fil_config), C.POINTER(_abi.fil_tables),
                                       C.POINTER(vp)]),
        "fil_batch_destroy": (C.c_int, [vp]),
        "fil_batch_last_error": (C.c_char_p, [vp]),
        "fil_batch_size": (C.c_int, [vp]),
        "fil_batch_member": (vp, [vp, C.c_int]),
        "fil_batch_tune": (C.c_int, [vp, C.c_int, dp, C.c_int]),
        "fil_batch_plan": (C.c_int, [vp, ip, ip, dp]),
        "fil_batch_run": (C.c_int, [vp, dp, dp, C.c_int64, C.POINTER(_abi.fil_stats)]),
    }
    out = {}
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
        out[name[4:]] = f
    return out


class Batch:
    """Many RT problems stepped together on one device (fil_create_batch):
    one CUDA graph per z-step runs every member's step, each member with
    its own adaptive-dz controller.  `members[i]` is a Handle for member i
    (set_field, get_field, analyze, set_option)."""

    def __init__(self, problems, binding=None):
        self.b = binding if binding is not None else load_library()
        self.f = _batch_fns(self.b.lib)
        self.problems = list(problems)
        n = len(self.problems)
        cfgs = (_abi.fil_config * n)(*[p.config for p in self.problems])
        tabs = (_abi.fil_tables * n)(*[p.tables for p in self.problems])
        self.ptr = C.c_void_p()
        code = self.f["create_batch"](n, cfgs, tabs, C.byref(self.ptr))
        if code < 0:
            msg = self.f["batch_last_error"](None)
            raise _abi.FilError(code, "fil_create_batch failed: %s" % (msg.decode() if msg else "?"))
        self.members = [Handle.borrow(self.b, p, self.f["batch_member"](self.ptr, i))
                        for i, p in enumerate(self.problems)]

    def __len__(self):
        return len(self.members)

    def _chk(self, code, what):
        if code < 0:
            msg = self.f["batch_last_error"](self.ptr)
            raise _abi.FilError(code, "fil_batch_%s failed: %s" % (what, msg.decode() if msg else "?"))
        return code

    def tune(self, max_branches=16):
        """Runs the autotuner; returns the batch step time (ms) per branch
        count tried (1, 2, 4, ...)."""
        ms = np.zeros(8)
        self._chk(self.f["batch_tune"](self.ptr, int(max_branches), ms.ctypes.data_as(C.POINTER(C.c_double)),
                                       len(ms)), "tune")
        return {1 << j: float(v) for j, v in enumerate(ms) if v > 0}

    def plan(self):
        n = len(self.members)
        br = np.zeros(n, dtype=np.int32)
        simt = np.zeros(n, dtype=np.int32)
        cost = np.zeros(n)
        ip = C.POINTER(C.c_int)
        k = self._chk(self.f["batch_plan"](self.ptr, br.ctypes.data_as(ip), simt.ctypes.data_as(ip),
                                           cost.ctypes.data_as(C.POINTER(C.c_double))), "plan")
        return {"branches": k, "branch": br.tolist(), "dht_simt": simt.tolist(), "cost_ms": cost.tolist()}

    def run(self, z0, zmax, nmax):
        """Every member i from z0[i] to zmax[i] (scalars broadcast), at most
        nmax steps; returns (code, [stats of each member])."""
        n = len(self.members)
        z0 = np.ascontiguousarray(np.broadcast_to(np.asarray(z0, dtype=np.float64), (n,)))
        zm = np.ascontiguousarray(np.broadcast_to(np.asarray(zmax, dtype=np.float64), (n,)))
        st = (_abi.fil_stats * n)()
        dp = C.POINTER(C.c_double)
        code = self._chk(self.f["batch_run"](self.ptr, z0.ctypes.data_as(dp), zm.ctypes.data_as(dp), int(nmax), st),
                         "run")
        return code, [st[i].as_dict() for i in range(n)]

    def close(self):
        if self.ptr:
            for m in self.members:
                m.h = C.c_void_p()
            self.f["batch_destroy"](self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
