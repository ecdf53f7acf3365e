"""fil_hankel_propagate_noalloc: the linear propagator of an RT z-step for
callers that cannot allocate device memory where they need it.  Its output
is checked on two calls in a row against the library's ordinary entry point
(fil_step of a linear-only problem), with the same 1e-5 relative L2
tolerance as the other mixed-precision parity tests, and against the FP64
oracle's steps of the same problem (within the sum of that tolerance and
the mixed form's own 1e-5 bound against the oracle).  The caller (this
test) owns every input and output buffer; the entry point uses only its
fixed device array."""
import ctypes as C

import numpy as np
import pytest

from gpu_helpers import rel_l2, rt_input

pytestmark = pytest.mark.gpu

TOL = 1e-5


def _entry(lib_path):
    lib = C.CDLL(lib_path)
    f = lib.fil_hankel_propagate_noalloc
    f.restype = C.c_int
    f.argtypes = [C.c_void_p] * 7 + [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_double, C.c_void_p]
    err = lib.fil_last_error
    err.restype = C.c_char_p
    err.argtypes = [C.c_void_p]
    return f, err


def _half_spectrum(E, nh, mpad, analytic_doubling):
    """Row-wise ifft, the non-negative half, rows padded to mpad."""
    X = np.fft.ifft(E, axis=1)[:, :nh]
    if analytic_doubling:
        X[:, 1:] *= 2.0
    S = np.zeros((mpad, nh), dtype=np.complex128)
    S[: E.shape[0]] = X
    return S


def _to_time(S, nr, nt, G):
    X = np.zeros((nr, nt), dtype=np.complex128)
    X[:, : S.shape[1]] = S[:nr]
    return G * np.fft.fft(X, axis=1)


def test_noalloc_propagator_matches_fil_step(gpu_lib):
    torch = pytest.importorskip("torch")
    import build
    from filament_gb import Simulation
    inp = rt_input(NONLINEARITY=False, PLASMA=False)
    sim = Simulation(inp, precision="mixed")
    import oracle
    ref = Simulation(inp, binding=oracle.binding())
    p = sim.problem
    nr, nt = p.config.n1, p.config.nt
    nh, mpad = nt // 2, ((nr + 127) // 128) * 128
    a = p._arrays
    T, s = a["dht"], a["dht_s"]
    m1 = np.zeros((mpad, mpad), np.float32)
    m2 = np.zeros((mpad, mpad), np.float32)
    m1[:nr, :nr] = T * s[None, :]
    m2[:nr, :nr] = T / s[:, None]
    kt2 = np.zeros(mpad, np.float32)
    kt2[:nr] = a["kt1"] ** 2
    beta = a["beta"][: 2 * nh].astype(np.float32)
    dfr = a["dfr"][: 2 * nh].astype(np.float32)
    kmax2 = (a["kmax"][:nh] ** 2).astype(np.float32)
    wg = a["wguard"][:nh].astype(np.float32)
    G = a["guard1"][:, None] * a["guardt"][None, :]        # field guard after a step
    dev = lambda x: torch.from_numpy(np.ascontiguousarray(x)).cuda()
    d_m1, d_m2, d_kt2, d_beta, d_dfr, d_kmax2, d_wg = map(dev, (m1, m2, kt2, beta, dfr, kmax2, wg))
    prop, last_error = _entry(build.LIB)

    def call(S):
        d_in = dev(S.astype(np.complex64).view(np.float32))
        d_out = torch.empty_like(d_in)
        rc = prop(d_m1.data_ptr(), d_m2.data_ptr(), d_kt2.data_ptr(), d_beta.data_ptr(), d_dfr.data_ptr(),
                  d_kmax2.data_ptr(), d_wg.data_ptr(), int(p.config.kparaxial), d_in.data_ptr(),
                  d_out.data_ptr(), mpad, nh, dz, None)
        assert rc == 0, last_error(None)
        torch.cuda.synchronize()
        return d_out.cpu().numpy().view(np.complex64).astype(np.complex128)

    dz = 2e-3
    # call 1: from the uploaded field (no guard pending), against fil_step #1
    S = _half_spectrum(sim.field.E0, nh, mpad, analytic_doubling=True)
    S1 = call(S)
    sim.handle.step(dz, dz)
    E1 = sim.handle.get_field()
    ref.handle.step(dz, dz)
    assert rel_l2(_to_time(S1, nr, nt, G), E1) < TOL
    assert rel_l2(_to_time(S1, nr, nt, G), ref.handle.get_field()) < 2 * TOL
    # call 2 reuses the fixed array: guard the previous result, then propagate
    S = _half_spectrum(_to_time(S1, nr, nt, G), nh, mpad, analytic_doubling=False)
    S2 = call(S)
    sim.handle.step(2 * dz, dz)
    E2 = sim.handle.get_field()
    ref.handle.step(2 * dz, dz)
    assert rel_l2(_to_time(S2, nr, nt, G), E2) < TOL
    assert rel_l2(_to_time(S2, nr, nt, G), ref.handle.get_field()) < 2 * TOL
    sim.close()
    ref.close()


def test_noalloc_rejects_sizes_beyond_the_fixed_array(gpu_lib):
    import build
    prop, last_error = _entry(build.LIB)
    one = C.c_void_p(16)       # never dereferenced: the size check comes first
    rc = prop(one, one, one, one, one, None, None, 0, one, one, 4096, 1024, 1e-3, None)
    assert rc == -1
    assert b"exceeds" in last_error(None)
    # an nh whose 2 * nh would overflow an int is rejected as too large too
    rc = prop(one, one, one, one, one, None, None, 0, one, one, 128, 2 ** 30 + 64, 1e-3, None)
    assert rc == -1
    assert b"exceeds" in last_error(None)
