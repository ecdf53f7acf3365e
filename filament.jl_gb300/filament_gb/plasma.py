"""Plasma equation set-up (src/modules/plasma_equations/photoionization_avalanche.jl:1-116)
and tabulated ionisation rates.

The rate tables use the reference's TabulatedFunctions dependency, which is
not vendored.  Its documented use is a rate W(I) tabulated over many decades
(examples/RT/multiphoton_O2.tf) and `tfpower`, the local multiphoton order.
This restatement interpolates linearly in (ln I, ln W) and defines
tfpower = d ln W / d ln I of the same segment; outside the table the end
segments are extended; W(I <= 0) = 0.  For the power-law tables of the
reference's decks the interpolation is exact.
"""
import math

import numpy as np

from .constants import HBAR, ME, QE


class TFunction:
    """Tabulated function y(x) with log-log interpolation.
    TFunction(T, fname, xu, yu) of the reference scales x by xu and y by yu
    (photoionization_avalanche.jl:34: xu = 1/Iu, yu = tu)."""

    def __init__(self, x, y, xu=1.0, yu=1.0):
        x = np.asarray(x, dtype=np.float64) * xu
        y = np.asarray(y, dtype=np.float64) * yu
        if len(x) < 2 or np.any(x <= 0) or np.any(y <= 0) or np.any(np.diff(x) <= 0):
            raise ValueError("rate table needs >= 2 increasing positive points")
        self.lx = np.log(x)
        self.ly = np.log(y)

    @classmethod
    def from_file(cls, fname, xu=1.0, yu=1.0):
        data = np.loadtxt(fname)
        return cls(data[:, 0], data[:, 1], xu, yu)

    def _seg(self, lx):
        i = int(np.searchsorted(self.lx, lx, side="right")) - 1
        return min(max(i, 0), len(self.lx) - 2)

    def __call__(self, x):
        if x <= 0:
            return 0.0
        lx = math.log(x)
        i = self._seg(lx)
        s = (self.ly[i + 1] - self.ly[i]) / (self.lx[i + 1] - self.lx[i])
        return math.exp(self.ly[i] + (lx - self.lx[i]) * s)

    def power(self, x):
        """tfpower: local slope d ln W / d ln I."""
        lx = math.log(x) if x > 0 else -math.inf
        i = self._seg(lx)
        return (self.ly[i + 1] - self.ly[i]) / (self.lx[i + 1] - self.lx[i])


def power_law_rate(K, I_ref, W_ref, Imin=1e9, Imax=1e20, n=10):
    """Multiphoton rate W = W_ref (I/I_ref)^K tabulated on a log grid (SI
    units, W/m^2 -> 1/s), the form of the reference's .tf tables."""
    I = np.logspace(math.log10(Imin), math.log10(Imax), n)
    return I, W_ref * (I / I_ref) ** K


class PlasmaEquation:
    """Device-independent image of the reference's plasma-equation objects
    (integrators, extract, kdrho_func and their parameter tuples)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def init_photoionization_avalanche(t, E, w0, units, params):
    """photoionization_avalanche.jl:1-116 restated: per species the rate
    table, fraction*rho_nt/rhou, the avalanche coefficient
    Rava = e^2/MR nuc/(nuc^2+w0^2)/Ui tu Eu^2 and K = ceil(Ui/(hbar w0))."""
    tu, Eu, Iu, rhou = units
    comps = params["components"]
    tfs, frhonts, Ravas, Ks = [], [], [], []
    for comp in comps:
        frac = comp["fraction"]
        Uiev = comp["ionization_energy"]
        rate = comp["ionization_rate"]
        if isinstance(rate, str):
            tf = TFunction.from_file(rate, 1.0 / Iu, tu)
        else:
            x, y = rate
            tf = TFunction(x, y, 1.0 / Iu, tu)
        tfs.append(tf)
        frhonts.append(frac * params["rho_nt"] / rhou)
        Ui = Uiev * QE
        MR = params["mr"] * ME
        sigmaB = QE ** 2 / MR * params["nuc"] / (params["nuc"] ** 2 + w0 ** 2)
        Ravas.append(sigmaB / Ui * tu * Eu ** 2)
        Ks.append(math.ceil(Ui / (HBAR * w0)))
    n = len(tfs[0].lx)
    if any(len(tf.lx) != n for tf in tfs):
        raise ValueError("all species' rate tables need the same length")
    alg = params.get("ALG", "RK3")
    return PlasmaEquation(
        alg=alg, EREAL=bool(params["EREAL"]), KDEP=bool(params["KDEP"]),
        rho0=params["rho0"] / rhou, tfs=tfs,
        rho_nt=np.array(frhonts), rava=np.array(Ravas), kfix=np.array(Ks, dtype=np.float64),
        rate_lx=np.concatenate([tf.lx for tf in tfs]),
        rate_ly=np.concatenate([tf.ly for tf in tfs]), rate_n=n)
