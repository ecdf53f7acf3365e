"""Absorbing guards (src/modules/Guards.jl:1-390), host FP64 tables.

The device applies them; here only the windows and cut-off tables are built.
"""
import math

import numpy as np

from . import media as Media


def guard_window_left(x, width, p=6):
    """Guards.jl:322-347: super-Gaussian window at the left edge."""
    x = np.asarray(x, dtype=np.float64)
    if width >= (x[-1] - x[0]):
        raise ValueError("Guard width is larger or equal than the grid size.")
    if width == 0:
        return np.ones_like(x)
    xloc1 = x[0]
    xloc2 = x[0] + width
    g1 = np.where(x >= xloc1, 1.0 - np.exp(-((x - xloc1) / (width / 2)) ** p), 0.0)
    g2 = np.where(x <= xloc2, np.exp(-((x - xloc2) / (width / 2)) ** p), 1.0)
    return (g1 + g2) / 2


def guard_window_right(x, width, p=6):
    """Guards.jl:350-375: super-Gaussian window at the right edge."""
    x = np.asarray(x, dtype=np.float64)
    if width >= (x[-1] - x[0]):
        raise ValueError("Guard width is larger or equal than the grid size.")
    if width == 0:
        return np.ones_like(x)
    xloc1 = x[-1] - width
    xloc2 = x[-1]
    g1 = np.where(x >= xloc1, np.exp(-((x - xloc1) / (width / 2)) ** p), 1.0)
    g2 = np.where(x <= xloc2, 1.0 - np.exp(-((x - xloc2) / (width / 2)) ** p), 0.0)
    return (g1 + g2) / 2


def guard_window_both(x, width, p=6):
    """Guards.jl:378-387."""
    x = np.asarray(x, dtype=np.float64)
    if width >= (x[-1] - x[0]) / 2:
        raise ValueError("Guard width is larger or equal than the grid size.")
    return guard_window_left(x, width, p) + guard_window_right(x, width, p) - 1


def sind(deg):
    return math.sin(math.radians(deg)) if deg % 180 != 0 else 0.0


def spectral_cutoff(w, wguard):
    """Wguard = exp(-((w/wguard)^2)^20) (Guards.jl:85,115,185)."""
    w = np.asarray(w, dtype=np.float64)
    return np.exp(-((w ** 2 / wguard ** 2) ** 20))


class Guard:
    """Host-side guard tables.  `field` holds the field-filter factors per
    axis; `spectral` the spectral-filter data.  Which entries exist depends on
    the geometry (Guards.jl:41-193)."""

    def __init__(self, **kw):
        self.__dict__.update(kw)


def Guard_build(geometry, unit, grid, w0, medium, p):
    """Guards.Guard(unit, grid, field, medium, p...) for each geometry."""
    if geometry == "R":                               # Guards.jl:41-58
        rguard, kguard = p
        R = guard_window_right(grid.r, rguard)
        k0 = Media.k_func(medium, w0)
        kmax = k0 * sind(kguard)
        return Guard(R=R, kmax=np.array([kmax]), W=None)
    if geometry == "T":                               # Guards.jl:78-89
        tguard, wguard = p
        Tg = guard_window_both(grid.t, tguard)
        W = spectral_cutoff(grid.w * unit.w, wguard)
        return Guard(T=Tg, W=W)
    if geometry == "RT":                              # Guards.jl:95-126
        rguard, tguard, kguard, wguard = p
        R = guard_window_right(grid.r, rguard)
        Tg = guard_window_both(grid.t, tguard)
        kmax = np.array([Media.k_func(medium, wj * unit.w) * sind(kguard)
                         for wj in grid.w])
        W = spectral_cutoff(grid.w * unit.w, wguard)
        return Guard(R=R, T=Tg, kmax=kmax, W=W)
    if geometry == "XY":                              # Guards.jl:132-156
        xguard, yguard, kxguard, kyguard = p
        X = guard_window_both(grid.x, xguard)
        Y = guard_window_both(grid.y, yguard)
        k0 = Media.k_func(medium, w0)
        kxmax = k0 * sind(kxguard)
        kymax = k0 * sind(kyguard)
        KX = np.exp(-(((grid.kx * unit.kx) ** 2 / kxmax ** 2) ** 20))
        KY = np.exp(-(((grid.ky * unit.ky) ** 2 / kymax ** 2) ** 20))
        return Guard(X=X, Y=Y, KX=KX, KY=KY, W=None)
    if geometry == "XYT":                             # Guards.jl:162-193
        xguard, yguard, tguard, kxguard, kyguard, wguard = p
        X = guard_window_both(grid.x, xguard)
        Y = guard_window_both(grid.y, yguard)
        Tg = guard_window_both(grid.t, tguard)
        # The reference forces the k-guards of XYT to 1 (Guards.jl:177-184).
        KX = np.ones(grid.Nx)
        KY = np.ones(grid.Ny)
        W = spectral_cutoff(grid.w * unit.w, wguard)
        return Guard(X=X, Y=Y, T=Tg, KX=KX, KY=KY, W=W)
    raise ValueError("Wrong grid geometry.")
