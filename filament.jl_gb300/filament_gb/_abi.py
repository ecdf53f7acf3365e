"""ctypes mirror of include/filament_gb.h and a binding class for any shared
library that exports that ABI under a symbol prefix."""
import ctypes as C

import numpy as np

FIL_ABI_VERSION = 1

FIL_OK = 0
FIL_STOP_ZMAX = 1
FIL_STOP_ISTOP = 2
FIL_STOP_NMAX = 3
FIL_ERR_ARG = -1
FIL_ERR_CUDA = -2
FIL_ERR_NAN = -3
FIL_ERR_TIMEOUT = -4
FIL_ERR_UNSUPPORTED = -5
FIL_ERR_STATE = -6
FIL_ERR_NOMEM = -7

GEOM = {"R": 0, "T": 1, "RT": 2, "XY": 3, "XYT": 4}
PREC = {"mixed": 0, "fp64": 1}
ALG = {"RK2": 2, "RK3": 3, "RK4": 4, "Tsit5": 5, "ATsit5": 6}

RESP_CUBIC = 1
RESP_FREE = 2
RESP_LOSSES = 4
RESP_RAMAN = 8

DTYPE_C64 = 0
DTYPE_C128 = 1
DTYPE_F32 = 2
DTYPE_F64 = 3
LAYOUT_COLMAJOR = 0
LAYOUT_ROWMAJOR = 1

OPT_STORE_PLASMA = 1
OPT_XYT_GUARD_BUGCOMPAT = 2
OPT_CLAMP_LAST_DZ = 3
OPT_TIMING = 4
OPT_ANALYTIC_PROJECTION = 5
OPT_DHT_SIMT = 6
OPT_ODE_RTOL = 7     # value = rtol x 1e12
OPT_ODE_ATOL = 8     # value = atol x 1e12

_dp = C.POINTER(C.c_double)


class fil_config(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("geometry", C.c_int32),
        ("precision", C.c_int32), ("alg", C.c_int32),
        ("n1", C.c_int32), ("n2", C.c_int32), ("nt", C.c_int32),
        ("nonlinearity", C.c_int32), ("plasma", C.c_int32),
        ("kparaxial", C.c_int32), ("qparaxial", C.c_int32),
        ("resp_mask", C.c_uint32), ("cubic_thg", C.c_int32),
        ("losses_ereal", C.c_int32), ("raman_thg", C.c_int32),
        ("plasma_alg", C.c_int32), ("plasma_ereal", C.c_int32),
        ("plasma_kdep", C.c_int32), ("plasma_ncomp", C.c_int32),
        ("rate_n", C.c_int32), ("reserved_i", C.c_int32 * 8),
        ("dt", C.c_double), ("dz0", C.c_double), ("phimax", C.c_double),
        ("phik", C.c_double), ("phip", C.c_double), ("istop", C.c_double),
        ("rho0", C.c_double), ("dxdy", C.c_double),
        ("reserved_d", C.c_double * 8),
    ]


class fil_tables(C.Structure):
    _fields_ = [(n, _dp) for n in (
        "kt1", "kt2", "guard1", "guard2", "guardt", "sguard1", "sguard2",
        "kmax", "wguard", "beta", "dfr", "qz", "rnl_cubic", "rnl_free",
        "rnl_losses", "rnl_raman", "raman_h", "dht", "dht_s", "rdr",
        "rho_nt", "rava", "kfix", "rate_lx", "rate_ly")]


class fil_stats(C.Structure):
    _fields_ = [
        ("z", C.c_double), ("dz", C.c_double), ("imax", C.c_double),
        ("rhomax", C.c_double), ("energy", C.c_double),
        ("steps", C.c_int64), ("status", C.c_int32), ("flags", C.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


def dptr(a):
    """Pointer to a contiguous float64 array (or NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


class FilError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class Binding:
    """Calls the C ABI of one shared library.  `prefix` is "fil_" for the
    CUDA library; the oracle exports the same ABI as "filo_"."""

    def __init__(self, path, prefix="fil_"):
        self.path = str(path)
        self.lib = C.CDLL(self.path)
        self.prefix = prefix
        L = self.lib
        vp = C.c_void_p

        def fn(name, res, args):
            f = getattr(L, prefix + name)
            f.restype = res
            f.argtypes = args
            return f

        self.create = fn("create", C.c_int, [C.POINTER(fil_config), C.POINTER(fil_tables), C.POINTER(vp)])
        self.destroy = fn("destroy", C.c_int, [vp])
        self.last_error = fn("last_error", C.c_char_p, [vp])
        self.set_option = fn("set_option", C.c_int, [vp, C.c_int, C.c_int64])
        self.set_field = fn("set_field", C.c_int, [vp, vp, C.c_int, C.c_int, C.c_int])
        self.get_field = fn("get_field", C.c_int, [vp, vp, C.c_int, C.c_int])
        self.get_plasma = fn("get_plasma", C.c_int, [vp, C.c_int, vp, C.c_int, C.c_int])
        self.step = fn("step", C.c_int, [vp, C.c_double, C.c_double])
        self.run = fn("run", C.c_int, [vp, C.c_double, C.c_double, C.c_int64, C.POINTER(fil_stats)])
        self.analyze = fn("analyze", C.c_int, [vp, C.POINTER(fil_stats), _dp, _dp, _dp])
        self.get_stats = fn("get_stats", C.c_int, [vp, C.POINTER(fil_stats)])
        self.kernel_times = fn("kernel_times", C.c_int, [vp, _dp, C.c_int])
        self.get_ode_stats = fn("get_ode_stats", C.c_int, [vp, C.POINTER(C.c_int64)])
        self.analyze_spectrum = fn("analyze_spectrum", C.c_int, [vp, _dp, C.c_int])

    def check(self, h, code, what):
        if code < 0:
            msg = self.last_error(h)
            raise FilError(code, "%s%s failed: %s" % (self.prefix, what, msg.decode() if msg else "?"))
        return code
