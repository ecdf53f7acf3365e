"""Host wrapper of the learned plasma surrogate (fil_nn_* of
include/filament_gb.h): a 1-D convolutional network trained on the GPU by
the library's own forward and backward kernels, and its training data.

The reference has no counterpart: it integrates the plasma rate equation
for every transverse point (src/modules/plasma_equations.jl:46-72,
src/modules/Models.jl:205-219).  The surrogate forms the density of a time
row in closed form from the effective rate of every step,
    w_j = Wb_j + kappa A_j (1 - e^{-S_j}) e^{g_j},
    rho_j = rho_a + (rho_nt - rho_a) (1 - exp(-dt sum_{i<j} w_i)),
where Wb_j and A_j are the medium's rate and E^2 averaged with the plasma
integrator's quadrature over the step, kappa the summed avalanche
coefficient, S_j = dt sum_{i<j} Wb_i, and g_j the network's output (the
avalanche's amplification of itself, learned from the ODE).
"""
import ctypes as C

import numpy as np

from . import _abi
from .backend import load_library

_fp = C.POINTER(C.c_float)
_bound = set()


def _bind(b):
    if id(b) in _bound:
        return b.lib
    L, vp = b.lib, C.c_void_p
    for name, res, args in (
            ("fil_nn_nparams", C.c_int, []),
            ("fil_nn_last_error", C.c_char_p, [vp]),
            ("fil_nn_create", C.c_int, [C.c_int, C.c_uint64, C.POINTER(vp)]),
            ("fil_nn_destroy", C.c_int, [vp]),
            ("fil_nn_get_params", C.c_int, [vp, _fp]),
            ("fil_nn_set_params", C.c_int, [vp, _fp]),
            ("fil_nn_forward", C.c_int, [vp, _fp, C.c_int, _fp]),
            ("fil_nn_infer", C.c_int, [vp, _fp, C.c_int, _fp]),
            ("fil_nn_grad", C.c_int, [vp, _fp, _fp, _fp, C.c_int, _fp, _fp]),
            ("fil_nn_train", C.c_int, [vp, _fp, _fp, _fp, C.c_int, C.c_int, C.c_int, C.c_float,
                                       C.c_uint64, _fp]),
            ("fil_set_surrogate", C.c_int, [vp, vp, C.c_int, C.c_double]),
            ("fil_get_surrogate_stats", C.c_int, [vp, C.POINTER(C.c_double), C.c_int])):
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    _bound.add(id(b))
    return L


def _f32(a, shape=None):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    if shape is not None:
        a = a.reshape(shape)
    return a


def _p(a):
    return a.ctypes.data_as(_fp)


def features(E, pe, dt):
    """Network inputs of time rows E [rows][nt] (complex analytic field,
    |E|^2 = I): f0 = ln(max(I, 1e-30)) / 16, f1 = Re(E)^2 / max(I, 1e-30),
    f2 = ln(max(S_j, 1e-30)) / 16 with S_j = dt sum_{i<j} Wb_i the ionised
    fraction exponent of the base rate (quad_rate).  Returns float32
    [rows][3][nt]."""
    E = np.atleast_2d(np.asarray(E))
    I = np.abs(E) ** 2
    Ic = np.maximum(I, 1e-30)
    S = np.zeros(E.shape)
    S[:, 1:] = np.cumsum(quad_rate(pe, E) * dt, axis=1)
    return np.stack([np.log(Ic) / 16.0, E.real ** 2 / Ic, np.log(np.maximum(S, 1e-30)) / 16.0],
                    axis=1).astype(np.float32)


def base_rate(pe, I):
    """Wb(I) = sum_c W_c(I) rho_nt,c / rho_nt, the instantaneous rate the
    network's output multiplies (log-log interpolation of the rate tables,
    W(I <= 0) = 0), vectorised over I."""
    I = np.asarray(I, dtype=np.float64)
    pos = I > 0
    lI = np.log(np.where(pos, I, 1.0))
    out = np.zeros_like(I)
    for tf, rn in zip(pe.tfs, pe.rho_nt):
        i = np.clip(np.searchsorted(tf.lx, lI, side="right") - 1, 0, len(tf.lx) - 2)
        sl = (tf.ly[i + 1] - tf.ly[i]) / (tf.lx[i + 1] - tf.lx[i])
        out += np.where(pos, np.exp(tf.ly[i] + (lI - tf.lx[i]) * sl), 0.0) * rn
    return out / float(np.sum(pe.rho_nt))


# weights of the stage points (t_j, midpoint, t_{j+1}) in the RK tableaus of
# the plasma equation's time integrator (plasma_equations.jl:46-72)
QUADRATURE = {"RK2": (0.0, 1.0, 0.0), "RK3": (1 / 6, 4 / 6, 1 / 6), "RK4": (1 / 6, 4 / 6, 1 / 6)}

# range of the network output the density uses (NN_G_LO, NN_G_HI of the kernels)
G_RANGE = (-2.0, 4.0)


def quad_rate(pe, E):
    """Base rate of every step t_j -> t_{j+1} of the time rows E [rows][nt]:
    Wb_j = sum_p q_p Wb(I_p) over the stage points of the integrator (the
    field linearly interpolated at the midpoint, as the ODE solve does).
    Returns [rows][nt - 1]."""
    E = np.atleast_2d(np.asarray(E))
    q0, qm, q1 = QUADRATURE[pe.alg]

    def inten(e):
        return e.real ** 2 if pe.EREAL else np.abs(e) ** 2

    e0, e1 = E[:, :-1], E[:, 1:]
    return (q0 * base_rate(pe, inten(e0)) + qm * base_rate(pe, inten(0.5 * (e0 + e1)))
            + q1 * base_rate(pe, inten(e1)))


def quad_ava(pe, E):
    """kappa A_j: the avalanche drive of every step, kappa = sum_c Rava_c
    times the integrator's quadrature of E^2 = Re(E)^2.  [rows][nt - 1]"""
    E = np.atleast_2d(np.asarray(E))
    q0, qm, q1 = QUADRATURE[pe.alg]
    e0, e1 = E[:, :-1], E[:, 1:]
    em = 0.5 * (e0 + e1)
    return float(np.sum(pe.rava)) * (q0 * e0.real ** 2 + qm * em.real ** 2 + q1 * e1.real ** 2)


def _base_exponent(pe, E, dt):
    """(Wb dt [rows][nt - 1], S_j = dt sum_{i<j} Wb_i for j < nt - 1)."""
    wb = quad_rate(pe, E) * dt
    S = np.concatenate([np.zeros((wb.shape[0], 1)), np.cumsum(wb, axis=1)[:, :-1]], axis=1)
    return wb, S


def closed_form_density(E, g, pe, dt):
    """The density the row kernel forms from the network output g [rows][nt]
    (FP64): w_j = Wb_j + kappa A_j (1 - e^{-S_j}) e^{g_j},
    rho_j = rho_a + (rho_nt - rho_a)(1 - exp(-dt sum_{i<j} w_i))."""
    E = np.atleast_2d(np.asarray(E))
    wb, S = _base_exponent(pe, E, dt)
    g = np.clip(np.asarray(g, dtype=np.float64)[:, :-1], *G_RANGE)
    w = wb + quad_ava(pe, E) * dt * -np.expm1(-S) * np.exp(g)
    St = np.concatenate([np.zeros((E.shape[0], 1)), np.cumsum(w, axis=1)], axis=1)
    ra = len(pe.rho_nt) * float(pe.rho0)
    rnt = float(np.sum(pe.rho_nt))
    return ra + (rnt - ra) * -np.expm1(-St)


def tile_flags(E, pe, dt, tile=128):
    """Tile flags of the rows E [rows][nt] (the rule nn_features in
    csrc/rowkernels.cuh applies in the row reduction, here in FP64).

    g enters the density only through the avalanche term
    kappa A_j dt (1 - e^{-S_j}) e^{g_j}, at most e^{G_RANGE[1]} times its
    g = 0 value.  Bit 0: the sum of that bound over the tile exceeds 2^-30
    of the row's base exponent S_total = dt sum_j Wb_j, so the density uses
    g there; elsewhere it uses g = 0.  Bit 1: the network runs on the tile
    (bit 0 of the tile or of a neighbour, which covers the four layers'
    receptive field of +-16 points).  Returns uint8 [rows][nt / tile]."""
    E = np.atleast_2d(np.asarray(E))
    rows, nt = E.shape
    wb, S = _base_exponent(pe, E, dt)
    av = np.zeros((rows, nt))
    av[:, :-1] = quad_ava(pe, E) * dt * -np.expm1(-S)
    per_tile = av.reshape(rows, nt // tile, tile).sum(axis=2)
    s_total = wb.sum(axis=1, keepdims=True)
    a = per_tile * np.exp(G_RANGE[1]) > np.ldexp(s_total, -30)
    d = a.copy()
    d[:, 1:] |= a[:, :-1]
    d[:, :-1] |= a[:, 1:]
    return a.astype(np.uint8) | (d.astype(np.uint8) << 1)


def training_pairs(E, rho, pe, dt, row_frac=1e-9, resolve=1e-6, floor=0.0):
    """Network inputs, targets and loss weights from time rows of the field
    E [rows][nt] (complex analytic signal) and the density rho [rows][nt]
    that the plasma equation gives on them.

    The effective rate of step j is w_j = -ln(1 - (rho_{j+1} - rho_j) / (rho_nt - rho_j)) / dt
    (the closed form then reproduces the solve exactly) and the target
    g_j = ln((w_j - Wb_j) / (kappa A_j (1 - e^{-S_j}))).  An error e in g_j
    moves the final density by about (rho_{j+1} - rho_j)(1 - Wb_j / w_j) e, so
    a point weighs that increment relative to the row's largest, at least
    `floor`; targets are clipped to G_RANGE.  Points where the avalanche
    part w_j - Wb_j is below `resolve`
    times w_j (not resolved by the solve, or absent) or whose increment is
    below 1e-10 of the density (not resolved in FP64) weigh 0.  Rows whose
    density rise is below `row_frac` of the largest rise are dropped."""
    E = np.atleast_2d(np.asarray(E))
    rho = np.atleast_2d(np.asarray(rho, dtype=np.float64))
    nt = E.shape[1]
    rnt = float(np.sum(pe.rho_nt))
    rise = rho[:, -1] - rho[:, 0]
    keep = rise > row_frac * max(float(rise.max()), 0.0)
    if not keep.any():
        return (np.zeros((0, 3, nt), np.float32), np.zeros((0, nt), np.float32), np.zeros((0, nt), np.float32))
    E, rho = E[keep], rho[keep]
    drho = np.diff(rho, axis=1)
    wb, S = _base_exponent(pe, E, dt)
    av = quad_ava(pe, E) * dt * -np.expm1(-S)
    with np.errstate(divide="ignore", invalid="ignore"):
        w = -np.log1p(-drho / (rnt - rho[:, :-1]))
        excess = w - wb
        # the increment must be resolved in FP64 (rounding of rho below 1e-6
        # of it) and carry an avalanche part
        good = (excess > resolve * w) & (av > 0) & (drho > 1e-10 * np.abs(rho[:, 1:]))
        g = np.where(good, np.log(np.where(good, excess, 1.0) / np.where(good, av, 1.0)), 0.0)
        contrib = np.where(good, drho * excess / np.where(good, w, 1.0), 0.0)
    rel = contrib / np.maximum(contrib.max(axis=1, keepdims=True), 1e-300)
    tgt = np.zeros(rho.shape, np.float32)
    mask = np.zeros(rho.shape, np.float32)
    tgt[:, :-1] = np.clip(g, *G_RANGE)
    mask[:, :-1] = np.where(good, np.maximum(rel, floor), 0.0)
    return features(E, pe, dt), tgt, mask


def solver_states(inp, snapshots, steps_between, precision="mixed", skip_steps=0):
    """States of the plain solver with their plasma density: propagates
    `inp` with the device loop (`precision` form), skips `skip_steps` steps,
    then at `snapshots` states `steps_between` steps apart solves the plasma
    equation of the current field in an FP64 handle.  Yields
    (z, E [rows][nt], rho [rows][nt]); stops early at zmax."""
    from . import _abi
    from .filament import Simulation
    sim = Simulation(inp, precision=precision)
    ref = Simulation(inp, precision="fp64")
    ref.handle.set_option(_abi.OPT_STORE_PLASMA, 1)
    z = sim.z
    try:
        if skip_steps:
            _, st = sim.handle.run(z, sim.zmax, skip_steps)
            z = st["z"]
        for k in range(snapshots):
            if k:
                _, st = sim.handle.run(z, sim.zmax, steps_between)
                z = st["z"]
            if z >= sim.zmax:
                break
            E = sim.handle.get_field()
            ref.handle.set_field(E, analytic=True)
            yield z, E, ref.handle.get_plasma(0)
    finally:
        sim.close()
        ref.close()


def solver_pairs(inp, snapshots, steps_between, precision="mixed", skip_steps=0, **kw):
    """Training data from the plain solver: training_pairs of every state
    of solver_states(...), concatenated."""
    from .filament import Simulation
    probe = Simulation(inp, precision=precision)
    pe, dt = probe.problem.pe, float(probe.grid.dt)
    probe.close()
    F, T, M = [], [], []
    for _, E, rho in solver_states(inp, snapshots, steps_between, precision, skip_steps):
        f, t, m = training_pairs(E, rho, pe, dt, **kw)
        F.append(f)
        T.append(t)
        M.append(m)
    return np.concatenate(F), np.concatenate(T), np.concatenate(M)


class Surrogate:
    """One network on the current device.  Parameters are FP32 masters;
    the kernels compute with their BF16 copies."""

    def __init__(self, nt, seed=1, binding=None):
        self.b = binding if binding is not None else load_library()
        self.L = _bind(self.b)
        self.nt = int(nt)
        self.h = C.c_void_p()
        self._chk(self.L.fil_nn_create(self.nt, int(seed), C.byref(self.h)), "create", None)

    @property
    def nparams(self):
        return self.L.fil_nn_nparams()

    def _chk(self, code, what, h="self"):
        if code < 0:
            msg = self.L.fil_nn_last_error(self.h if h == "self" else None)
            raise _abi.FilError(code, "fil_nn_%s failed: %s" % (what, msg.decode() if msg else "?"))
        return code

    def close(self):
        if self.h:
            self.L.fil_nn_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        out = np.empty(self.nparams, dtype=np.float32)
        self._chk(self.L.fil_nn_get_params(self.h, _p(out)), "get_params")
        return out

    def set_params(self, p):
        p = _f32(p, (self.nparams,))
        self._chk(self.L.fil_nn_set_params(self.h, _p(p)), "set_params")

    def forward(self, feat):
        feat = _f32(feat, (-1, 3, self.nt))
        out = np.empty((feat.shape[0], self.nt), dtype=np.float32)
        self._chk(self.L.fil_nn_forward(self.h, _p(feat), feat.shape[0], _p(out)), "forward")
        return out

    def infer(self, feat):
        """The simulation's inference path (tensor-core layers); nt a
        multiple of 128."""
        feat = _f32(feat, (-1, 3, self.nt))
        out = np.empty((feat.shape[0], self.nt), dtype=np.float32)
        self._chk(self.L.fil_nn_infer(self.h, _p(feat), feat.shape[0], _p(out)), "infer")
        return out

    def grad(self, feat, target, mask):
        feat = _f32(feat, (-1, 3, self.nt))
        rows = feat.shape[0]
        target, mask = _f32(target, (rows, self.nt)), _f32(mask, (rows, self.nt))
        g = np.empty(self.nparams, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        self._chk(self.L.fil_nn_grad(self.h, _p(feat), _p(target), _p(mask), rows, _p(g), _p(loss)), "grad")
        return float(loss[0]), g

    def train(self, feat, target, mask, iters, batch=64, lr=1e-3, seed=1):
        """Adam on the device; returns the per-iteration batch losses."""
        feat = _f32(feat, (-1, 3, self.nt))
        rows = feat.shape[0]
        target, mask = _f32(target, (rows, self.nt)), _f32(mask, (rows, self.nt))
        hist = np.zeros(max(int(iters), 1), dtype=np.float32)
        self._chk(self.L.fil_nn_train(self.h, _p(feat), _p(target), _p(mask), rows, int(batch), int(iters),
                                      float(lr), int(seed), _p(hist)), "train")
        return hist[:int(iters)]

    def arm(self, handle, every=20, tol=1e-3):
        """Use the network for the plasma density of `handle` (a backend
        Handle) inside its device loop, checked every `every` steps."""
        L = _bind(handle.b)
        handle.b.check(handle.h, L.fil_set_surrogate(handle.h, self.h, int(every), float(tol)), "set_surrogate")
        handle._surrogate = self


def disarm(handle):
    L = _bind(handle.b)
    handle.b.check(handle.h, L.fil_set_surrogate(handle.h, None, 1, 1.0), "set_surrogate")
    handle._surrogate = None


STAT_KEYS = ("armed", "in_use", "steps", "steps_used", "checks", "checks_failed", "err_last", "err_max",
             "rows_mean", "tiles_mean")


def stats(handle):
    """Surrogate counters of a handle (fil_get_surrogate_stats)."""
    L = _bind(handle.b)
    out = np.zeros(len(STAT_KEYS))
    code = L.fil_get_surrogate_stats(handle.h, out.ctypes.data_as(C.POINTER(C.c_double)), len(out))
    handle.b.check(handle.h, code, "get_surrogate_stats")
    return dict(zip(STAT_KEYS, out.tolist()))
