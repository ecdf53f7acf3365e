"""Nonlinear response plug-ins (src/modules/medium_responses/*.jl).

Each `init_*` has the reference's plug-in signature
`init(unit, grid, field, medium, p) -> NonlinearResponse` and computes the
response's Rnl prefactor in FP64.  The per-point evaluation `calc_*` runs on
the device; `kind` selects the device channel.
"""
import math

import numpy as np

from .constants import C0, EPS0, HBAR, ME, QE
from . import media as Media
from . import units as Units
from .media import NonlinearResponse


def _Eu(unit, medium, w0):
    n0 = Media.refractive_index(medium, w0)
    return Units.E(unit, n0.real)


def _spatial(grid):
    return type(grid).__name__ in ("GridR", "GridXY")


def init_cubic(unit, grid, field, medium, p):
    """cubic.jl:4-30.  Rnl = eps0 chi3 Eu^3, chi3 = 4/3 n0^2 eps0 c n2."""
    THG = p["THG"]
    n2 = p["n2"]
    w0 = field.w0
    n0 = Media.refractive_index(medium, w0)
    Eu = Units.E(unit, n0.real)
    chi3 = 4.0 / 3.0 * n0.real ** 2 * EPS0 * C0 * n2
    Rnl = EPS0 * chi3 * Eu ** 3
    if _spatial(grid):
        kind = "cubic_spatial"         # calc_cubic_nothg_spatial (cubic.jl:49-54)
    else:
        kind = "cubic"                 # calc_cubic / calc_cubic_nothg
    return NonlinearResponse(kind, complex(Rnl), {"THG": bool(THG)})


def init_current_free(unit, grid, field, medium, p):
    """current_free.jl:4-28.
    Rnl(w) = i/w e^2/MR / (nuc - i w) rhou Eu, 0 at w = 0."""
    nuc = p["nuc"]
    mr = p["mr"]
    w0 = field.w0
    Eu = _Eu(unit, medium, w0)
    MR = mr * ME
    w = grid.w * unit.w
    Rnl = np.zeros(grid.Nt, dtype=np.complex128)
    nz = w != 0
    Rnl[nz] = (1j / w[nz] * QE ** 2 / MR / (nuc - 1j * w[nz]) * unit.rho * Eu)
    return NonlinearResponse("free", Rnl, {})


def init_current_losses(unit, grid, field, medium, p):
    """current_losses.jl:4-33.  Rnl(w) = i/w hbar w0 rhou/(tu Eu)."""
    EREAL = p["EREAL"]
    w0 = field.w0
    Eu = _Eu(unit, medium, w0)
    w = grid.w * unit.w
    Rnl = np.zeros(grid.Nt, dtype=np.complex128)
    nz = w != 0
    Rnl[nz] = 1j / w[nz] * HBAR * w0 * unit.rho / (unit.t * Eu)
    return NonlinearResponse("losses", Rnl, {"EREAL": bool(EREAL)})


def init_raman(unit, grid, field, medium, p):
    """raman.jl:4-43.  Rnl as in cubic; H(w) = Nt dt ifft(ifftshift(H(t) tu))
    with H(t) centred on the window."""
    THG = p["THG"]
    n2 = p["n2"]
    raman_response = p["raman_response"]
    w0 = field.w0
    n0 = Media.refractive_index(medium, w0)
    Eu = Units.E(unit, n0.real)
    chi3 = 4.0 / 3.0 * n0.real ** 2 * EPS0 * C0 * n2
    Rnl = EPS0 * chi3 * Eu ** 3
    tshift = grid.tmin + 0.5 * (grid.tmax - grid.tmin)
    H = np.array([raman_response((tj - tshift) * unit.t) for tj in grid.t],
                 dtype=np.float64) * unit.t
    H = np.fft.ifft(np.fft.ifftshift(H.astype(np.complex128))) * grid.Nt * grid.dt
    return NonlinearResponse("raman", complex(Rnl), {"THG": bool(THG), "H": H})


def raman_response_air(t):
    """Mlejnek, Wright, Moloney, Opt. Lett. 23, 382 (1998) response of air
    (examples/RT/air.jl:46-58)."""
    if t < 0.0:
        return 0.0
    Omega = 20.6e12
    Gamma = 26e12
    Lambda = math.sqrt(Omega ** 2 - Gamma ** 2 / 4.0)
    return Omega ** 2 * math.exp(-0.5 * Gamma * t) * math.sin(Lambda * t) / Lambda
