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

    def close(self):
        if self.h:
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
