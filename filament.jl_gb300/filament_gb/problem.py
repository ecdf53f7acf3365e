"""Builds the C-ABI image (fil_config + fil_tables) of one problem from the
reference-style set-up objects.  This is the FP64 host set-up that the
reference performs in Filament.run (src/Filament.jl:72-79):
LinearPropagator KZ tables (linear_propagators/spectral.jl:78-184), QZ
(nonlinear_propagators.jl:139-229), response Rnl (medium_responses/*.jl),
guards (Guards.jl), the DHT plan (Fields.jl:105-111) and the plasma
parameters (photoionization_avalanche.jl:1-116).  Only 1-D tables and the
Hankel matrix are produced; the device regenerates the 2-D ones.
"""
import math

import numpy as np

from . import _abi
from . import media as Media
from . import units as Units
from .constants import EPS0, ME, MU0, QE
from .grids import dht_matrix


def _c(a):
    """complex array -> interleaved float64."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return np.ascontiguousarray(a.view(np.float64))


def _f(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64))


def qfunc_paraxial(medium, w):
    """Qfunc_paraxial (nonlinear_propagators.jl:220-229)."""
    mu = medium.permeability(w)
    beta = Media.beta_func(medium, w)
    if beta == 0:
        return 0.0
    return MU0 * mu * w ** 2 / (2 * beta)


def phi_kerr(unit, medium, w0):
    """AdaptiveSteps.jl:46-58."""
    mu = medium.permeability(w0)
    n0 = Media.refractive_index(medium, w0)
    k0 = Media.k_func(medium, w0)
    chi3 = Media.chi3_func(medium, w0)
    Eu = Units.E(unit, n0.real)
    QZ0 = MU0 * mu * w0 ** 2 / (2 * k0) * unit.z / Eu
    Rnl0 = EPS0 * chi3 * 3 / 4 * Eu ** 3
    return QZ0 * abs(Rnl0)


def phi_plasma(unit, medium, w0, mr, nuc):
    """AdaptiveSteps.jl:60-72."""
    mu = medium.permeability(w0)
    n0 = Media.refractive_index(medium, w0)
    k0 = Media.k_func(medium, w0)
    MR = mr * ME
    Eu = Units.E(unit, n0.real)
    QZ0 = MU0 * mu * w0 ** 2 / (2 * k0) * unit.z / Eu
    Rnl0 = 1j / w0 * QE ** 2 / MR / (nuc - 1j * w0) * unit.rho * Eu
    return QZ0 * abs(Rnl0.real)


class Problem:
    """Host image of one problem.  Keeps every numpy table alive for as long
    as the ctypes structs point at it."""

    def __init__(self, geometry, unit, grid, w0, medium, guard, responses,
                 plasma_eq, keys, dzparams, precision="mixed"):
        self.geometry = geometry
        self.unit = unit
        self.grid = grid
        self.w0 = w0
        self.medium = medium
        self.guard = guard
        self.responses = list(responses)
        self.pe = plasma_eq
        self.keys = dict(keys)
        self.precision = precision
        self._arrays = {}
        self._build(dzparams)

    # ------------------------------------------------------------------
    def _keep(self, name, arr):
        self._arrays[name] = arr
        return arr

    def _build(self, dzparams):
        g, unit, grid, medium, w0 = self.geometry, self.unit, self.grid, self.medium, self.w0
        keys = self.keys
        cfg = _abi.fil_config()
        cfg.abi_version = _abi.FIL_ABI_VERSION
        cfg.geometry = _abi.GEOM[g]
        cfg.precision = _abi.PREC[self.precision]
        cfg.alg = _abi.ALG[keys["ALG"]]
        cfg.nonlinearity = int(bool(keys["NONLINEARITY"]))
        cfg.plasma = int(bool(keys.get("PLASMA", False)))
        cfg.kparaxial = int(bool(keys["KPARAXIAL"]))
        cfg.qparaxial = int(bool(keys["QPARAXIAL"]))
        zu = unit.z
        n0 = Media.refractive_index(medium, w0)
        Eu = Units.E(unit, n0.real)
        self.Eu = Eu
        vf = Media.group_velocity(medium, w0)
        self.vf = vf

        has_t = g in ("T", "RT", "XYT")
        if has_t:
            w = grid.w * unit.w
            nt = grid.Nt
            cfg.dt = grid.dt
        else:
            w = np.array([w0])
            nt = 1
            cfg.dt = 1.0
        cfg.nt = nt
        if g in ("R", "RT"):
            cfg.n1, cfg.n2 = grid.Nr, 1
        elif g in ("XY", "XYT"):
            cfg.n1, cfg.n2 = grid.Nx, grid.Ny
            cfg.dxdy = grid.dx * grid.dy
        else:
            cfg.n1, cfg.n2 = 1, 1

        # propagation constants: KZ = dfr - kt^2/(beta + sqrt(beta^2 - kt^2))
        beta = np.array([Media.beta_func(medium, wj) for wj in w]) * zu
        # moving frame (spectral.jl:44-47, 90-91): - w/vf
        dfr = beta - w / vf * zu
        tab = _abi.fil_tables()
        tab.beta = _abi.dptr(self._keep("beta", _c(beta)))
        tab.dfr = _abi.dptr(self._keep("dfr", _c(dfr)))
        if g in ("R", "RT"):
            tab.kt1 = _abi.dptr(self._keep("kt1", _f(grid.k * unit.k * zu)))
            tab.guard1 = _abi.dptr(self._keep("guard1", _f(self.guard.R)))
            tab.kmax = _abi.dptr(self._keep("kmax", _f(self.guard.kmax * zu)))
            T, J1 = dht_matrix(grid.jzeros)
            tab.dht = _abi.dptr(self._keep("dht", _f(T)))
            tab.dht_s = _abi.dptr(self._keep("dht_s", _f(grid.rmax / J1)))
            tab.rdr = _abi.dptr(self._keep("rdr", _f(grid.r * grid.dr)))
        elif g in ("XY", "XYT"):
            tab.kt1 = _abi.dptr(self._keep("kt1", _f(grid.kx * unit.kx * zu)))
            tab.kt2 = _abi.dptr(self._keep("kt2", _f(grid.ky * unit.ky * zu)))
            tab.guard1 = _abi.dptr(self._keep("guard1", _f(self.guard.X)))
            tab.guard2 = _abi.dptr(self._keep("guard2", _f(self.guard.Y)))
            tab.sguard1 = _abi.dptr(self._keep("sguard1", _f(self.guard.KX)))
            tab.sguard2 = _abi.dptr(self._keep("sguard2", _f(self.guard.KY)))
        else:  # T
            tab.kt1 = _abi.dptr(self._keep("kt1", _f([0.0])))
            tab.guard1 = _abi.dptr(self._keep("guard1", _f([1.0])))
        if has_t:
            tab.guardt = _abi.dptr(self._keep("guardt", _f(self.guard.T)))
        if getattr(self.guard, "W", None) is not None:
            tab.wguard = _abi.dptr(self._keep("wguard", _f(self.guard.W)))

        # nonlinear prefactor and responses
        if cfg.nonlinearity:
            # the paraxial QZ(w); with QPARAXIAL = false the library forms
            # QZ(kt, w) = QZ(w) beta(w) / sqrt(beta^2 - kt^2)
            # (Qfunc_nonparaxial, nonlinear_propagators.jl:232-241)
            qz = np.array([qfunc_paraxial(medium, wj) for wj in w]) * zu / Eu
            tab.qz = _abi.dptr(self._keep("qz", _c(qz)))
            chan = {"cubic": np.zeros(nt, complex), "free": np.zeros(nt, complex),
                    "losses": np.zeros(nt, complex), "raman": np.zeros(nt, complex)}
            mask = 0
            for r in self.responses:
                kind = r.kind
                if kind in ("cubic", "cubic_spatial"):
                    chan["cubic"] += r.Rnl
                    mask |= _abi.RESP_CUBIC
                    cfg.cubic_thg = int(kind == "cubic" and r.p["THG"])
                elif kind == "free":
                    chan["free"] += r.Rnl
                    mask |= _abi.RESP_FREE
                elif kind == "losses":
                    chan["losses"] += r.Rnl
                    mask |= _abi.RESP_LOSSES
                    cfg.losses_ereal = int(r.p["EREAL"])
                elif kind == "raman":
                    chan["raman"] += r.Rnl
                    mask |= _abi.RESP_RAMAN
                    cfg.raman_thg = int(r.p["THG"])
                    tab.raman_h = _abi.dptr(self._keep("raman_h", _c(r.p["H"])))
                else:
                    raise ValueError("unknown response kind %r" % kind)
            cfg.resp_mask = mask
            tab.rnl_cubic = _abi.dptr(self._keep("rnl_cubic", _c(chan["cubic"])))
            tab.rnl_free = _abi.dptr(self._keep("rnl_free", _c(chan["free"])))
            tab.rnl_losses = _abi.dptr(self._keep("rnl_losses", _c(chan["losses"])))
            tab.rnl_raman = _abi.dptr(self._keep("rnl_raman", _c(chan["raman"])))

        # plasma
        pe = self.pe
        if cfg.plasma:
            cfg.plasma_alg = _abi.ALG[pe.alg]
            cfg.plasma_ereal = int(pe.EREAL)
            cfg.plasma_kdep = int(pe.KDEP)
            cfg.plasma_ncomp = len(pe.rho_nt)
            cfg.rate_n = pe.rate_n
            cfg.rho0 = pe.rho0
            tab.rho_nt = _abi.dptr(self._keep("rho_nt", _f(pe.rho_nt)))
            tab.rava = _abi.dptr(self._keep("rava", _f(pe.rava)))
            tab.kfix = _abi.dptr(self._keep("kfix", _f(pe.kfix)))
            tab.rate_lx = _abi.dptr(self._keep("rate_lx", _f(pe.rate_lx)))
            tab.rate_ly = _abi.dptr(self._keep("rate_ly", _f(pe.rate_ly)))

        # adaptive step (AdaptiveSteps.jl:29-44)
        dz0, phimax = dzparams[0], dzparams[1]
        cfg.dz0 = dz0
        cfg.phimax = phimax
        cfg.phik = phi_kerr(unit, medium, w0)
        if len(dzparams) >= 4:
            mr, nuc = dzparams[2], dzparams[3]
            cfg.phip = phi_plasma(unit, medium, w0, mr, nuc)
        else:
            cfg.phip = 0.0
        cfg.istop = float(keys.get("Istop", math.inf))
        self.config = cfg
        self.tables = tab

    # ------------------------------------------------------------------
    @property
    def field_shape(self):
        c = self.config
        g = self.geometry
        if g == "R":
            return (c.n1,)
        if g == "T":
            return (c.nt,)
        if g == "RT":
            return (c.n1, c.nt)
        if g == "XY":
            return (c.n1, c.n2)
        return (c.n1, c.n2, c.nt)
