"""Field analyzers (src/modules/FieldAnalyzers.jl:1-383) on top of the
library's FP64 device reductions (fil_analyze).  The host part (radius,
maxima of the reduced arrays) is the reference's host logic."""
import math

import numpy as np


def radius(x, y, level=math.exp(-1)):
    """FieldAnalyzers.jl:357-380: half the distance between the outermost
    points where y >= level*max(y), as (|left| + |right|)/2."""
    x = np.asarray(x)
    y = np.asarray(y)
    ylevel = np.max(y) * level
    idx = np.nonzero(y >= ylevel)[0]
    if len(idx) == 0:
        return 0.0
    return (abs(x[idx[0]]) + abs(x[idx[-1]])) / 2


class FieldAnalyzer:
    """Per-geometry observed variables, updated by analyze(z)."""

    def __init__(self, geometry, grid, handle, z):
        self.geometry = geometry
        self.grid = grid
        self.handle = handle
        self.z = z
        self.Imax = 0.0
        self.rhomax = 0.0
        if geometry in ("R", "RT"):
            self.rdr = grid.r * grid.dr

    def analyze(self, z):
        self.z = z
        d = self.handle.analyze()
        g, grid = self.geometry, self.grid
        self.Imax = d["imax"]
        self.rhomax = d["rhomax"]
        F, P, rho_end = d["fluence"], d["power"], d["rho_end"]
        if g == "R":                                   # FieldAnalyzers.jl:46-60
            self.rfil = 2 * radius(grid.r, F)
            self.P = P[0]
        elif g == "T":                                 # FieldAnalyzers.jl:92-107
            self.duration = radius(grid.t, P)
            self.F = d["energy"]
        elif g == "RT":                                # FieldAnalyzers.jl:166-215
            self.Fr, self.Ft, self.rho = F, P, rho_end
            self.Fmax = np.max(F)
            self.De = 2 * math.pi * np.sum(rho_end * self.rdr)
            self.rfil = 2 * radius(grid.r, F)
            self.rpl = 2 * radius(grid.r, rho_end)
            self.tau = radius(grid.t, P)
            self.W = d["energy"]
            self.S = self.handle.spectrum()           # FieldAnalyzers.jl:180-197
        elif g == "XY":                                # FieldAnalyzers.jl:240-255
            I = F.reshape(grid.Nx, grid.Ny)
            self.I = I
            ix, iy = np.unravel_index(np.argmax(I), I.shape)
            self.ax = radius(grid.x, I[:, iy])
            self.ay = radius(grid.y, I[ix, :])
            self.P = P[0]
        elif g == "XYT":                               # FieldAnalyzers.jl:299-353
            Fxy = F.reshape(grid.Nx, grid.Ny)
            self.Fxy, self.Ft = Fxy, P
            self.Fmax = np.max(Fxy)
            ix, iy = np.unravel_index(np.argmax(Fxy), Fxy.shape)
            self.De = np.sum(rho_end) * grid.dx * grid.dy
            self.ax = radius(grid.x, Fxy[:, iy])
            self.ay = radius(grid.y, Fxy[ix, :])
            self.W = d["energy"]
            self.rho = rho_end.reshape(grid.Nx, grid.Ny)
            self.S = self.handle.spectrum()           # FieldAnalyzers.jl:320-336
        return self
