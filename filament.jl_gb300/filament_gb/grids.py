"""Grids (src/modules/Grids.jl:1-240), computed in FP64 on the host.

The Hankel grid follows the quasi-discrete Hankel transform of order 0
(Guizar-Sicairos and Gutierrez-Vega, JOSA A 21, 53 (2004)), which is what the
reference's HankelTransforms dependency provides (dhtcoord / dhtfreq,
Grids.jl:204-215):  r_i = j_i R / j_{N+1},  k_i = 2 pi dhtfreq_i = j_i / R,
with j_i the positive zeros of J0.
"""
from dataclasses import dataclass, field
import math

import numpy as np
from scipy import special


def bessel_j0_zeros(n):
    """First n positive zeros of J0."""
    return np.asarray(special.jn_zeros(0, n), dtype=np.float64)


def fftfreq(n, d):
    """FFTW.fftfreq(n, 1/d) restated: k/(n d) in FFTW order."""
    k = np.arange(n, dtype=np.float64)
    k[k >= (n + 1) // 2] -= n
    return k / (n * d)


def _step(i, x):
    """Grids.jl:227-238: local step of a non-uniform grid (0-based i)."""
    n = len(x)
    if i == 0:
        return x[1] - x[0]
    if i == n - 1:
        return x[n - 1] - x[n - 2]
    return (x[i + 1] - x[i - 1]) / 2.0


def _grid_spatial_axial(rmax, Nr):
    """Grids.jl:204-215."""
    j = bessel_j0_zeros(Nr + 1)
    r = j[:Nr] * rmax / j[Nr]
    k = j[:Nr] / rmax            # 2 pi * dhtfreq
    dr = np.array([_step(i, r) for i in range(Nr)]) if Nr > 1 else np.array([rmax])
    return r, dr, k, j


def _grid_temporal(tmin, tmax, Nt):
    """Grids.jl:218-223: range(tmin, tmax, length=Nt) and 2 pi fftfreq."""
    t = np.linspace(tmin, tmax, Nt)
    dt = (tmax - tmin) / (Nt - 1)
    w = 2.0 * math.pi * fftfreq(Nt, dt)
    return t, dt, w


def _grid_spatial_rectangular(xmin, xmax, Nx):
    """Grids.jl:196-201."""
    x = np.linspace(xmin, xmax, Nx)
    dx = (xmax - xmin) / (Nx - 1)
    kx = 2.0 * math.pi * fftfreq(Nx, dx)
    return x, dx, kx


@dataclass
class GridR:
    rmax: float
    Nr: int
    r: np.ndarray = field(repr=False)
    dr: np.ndarray = field(repr=False)
    k: np.ndarray = field(repr=False)
    jzeros: np.ndarray = field(repr=False)


@dataclass
class GridT:
    tmin: float
    tmax: float
    Nt: int
    t: np.ndarray = field(repr=False)
    dt: float
    w: np.ndarray = field(repr=False)


@dataclass
class GridRT:
    rmax: float
    Nr: int
    r: np.ndarray = field(repr=False)
    dr: np.ndarray = field(repr=False)
    k: np.ndarray = field(repr=False)
    jzeros: np.ndarray = field(repr=False)
    tmin: float
    tmax: float
    Nt: int
    t: np.ndarray = field(repr=False)
    dt: float
    w: np.ndarray = field(repr=False)


@dataclass
class GridXY:
    xmin: float
    xmax: float
    Nx: int
    x: np.ndarray = field(repr=False)
    dx: float
    kx: np.ndarray = field(repr=False)
    ymin: float
    ymax: float
    Ny: int
    y: np.ndarray = field(repr=False)
    dy: float
    ky: np.ndarray = field(repr=False)


@dataclass
class GridXYT:
    xmin: float
    xmax: float
    Nx: int
    x: np.ndarray = field(repr=False)
    dx: float
    kx: np.ndarray = field(repr=False)
    ymin: float
    ymax: float
    Ny: int
    y: np.ndarray = field(repr=False)
    dy: float
    ky: np.ndarray = field(repr=False)
    tmin: float
    tmax: float
    Nt: int
    t: np.ndarray = field(repr=False)
    dt: float
    w: np.ndarray = field(repr=False)


def Grid(geometry, p):
    """Grids.Grid(geometry, p) (Grids.jl:10-27).  Rn is not built (TDMA path)."""
    if geometry == "R":
        rmax, Nr = p
        r, dr, k, j = _grid_spatial_axial(float(rmax), int(Nr))
        return GridR(float(rmax), int(Nr), r, dr, k, j)
    if geometry == "T":
        tmin, tmax, Nt = p
        t, dt, w = _grid_temporal(float(tmin), float(tmax), int(Nt))
        return GridT(float(tmin), float(tmax), int(Nt), t, dt, w)
    if geometry == "RT":
        rmax, Nr, tmin, tmax, Nt = p
        r, dr, k, j = _grid_spatial_axial(float(rmax), int(Nr))
        t, dt, w = _grid_temporal(float(tmin), float(tmax), int(Nt))
        return GridRT(float(rmax), int(Nr), r, dr, k, j,
                      float(tmin), float(tmax), int(Nt), t, dt, w)
    if geometry == "XY":
        xmin, xmax, Nx, ymin, ymax, Ny = p
        x, dx, kx = _grid_spatial_rectangular(float(xmin), float(xmax), int(Nx))
        y, dy, ky = _grid_spatial_rectangular(float(ymin), float(ymax), int(Ny))
        return GridXY(float(xmin), float(xmax), int(Nx), x, dx, kx,
                      float(ymin), float(ymax), int(Ny), y, dy, ky)
    if geometry == "XYT":
        xmin, xmax, Nx, ymin, ymax, Ny, tmin, tmax, Nt = p
        x, dx, kx = _grid_spatial_rectangular(float(xmin), float(xmax), int(Nx))
        y, dy, ky = _grid_spatial_rectangular(float(ymin), float(ymax), int(Ny))
        t, dt, w = _grid_temporal(float(tmin), float(tmax), int(Nt))
        return GridXYT(float(xmin), float(xmax), int(Nx), x, dx, kx,
                       float(ymin), float(ymax), int(Ny), y, dy, ky,
                       float(tmin), float(tmax), int(Nt), t, dt, w)
    raise ValueError("Wrong grid geometry: %r" % (geometry,))


def dht_matrix(jzeros):
    """Order-0 QDHT kernel (Guizar-Sicairos & Gutierrez-Vega 2004, eq. 11):
    T_ij = 2/S J0(j_i j_j / S) / (|J1(j_i)| |J1(j_j)|), S = j_{N+1}.

    Returns (T, J1abs) with T of shape (N, N).  The reference applies the
    forward transform as (J/V) T (R/J) f and the inverse as (J/R) T (V/J) F, so
    a propagation iDHT(D * DHT(f)) equals diag(J/R) T D T diag(R/J) f.
    """
    N = len(jzeros) - 1
    j = jzeros[:N]
    S = jzeros[N]
    J1 = np.abs(special.j1(j))
    T = (2.0 / S) * special.j0(np.outer(j, j) / S) / np.outer(J1, J1)
    return T, J1
