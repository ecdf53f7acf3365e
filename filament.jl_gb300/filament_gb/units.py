"""Dimensionless units per geometry (src/modules/Units.jl:1-144)."""
from dataclasses import dataclass
import math

from .constants import C0, EPS0


@dataclass
class UnitR:          # Units.jl:31-43
    r: float
    k: float
    z: float
    I: float


@dataclass
class UnitT:          # Units.jl:49-64
    z: float
    t: float
    w: float
    lam: float
    I: float
    rho: float


@dataclass
class UnitRT:         # Units.jl:67-87
    r: float
    k: float
    z: float
    t: float
    w: float
    lam: float
    I: float
    rho: float


@dataclass
class UnitXY:         # Units.jl:93-108
    x: float
    y: float
    kx: float
    ky: float
    z: float
    I: float


@dataclass
class UnitXYT:        # Units.jl:114-133
    x: float
    y: float
    kx: float
    ky: float
    z: float
    t: float
    w: float
    lam: float
    I: float
    rho: float


def Unit(geometry, p):
    """Units.Unit(geometry, p) (Units.jl:10-25)."""
    if geometry in ("R", "Rn"):
        ru, zu, Iu = p
        return UnitR(ru, 1.0 / ru, zu, Iu)
    if geometry == "T":
        zu, tu, Iu, rhou = p
        return UnitT(zu, tu, 1.0 / tu, tu, Iu, rhou)
    if geometry == "RT":
        ru, zu, tu, Iu, rhou = p
        return UnitRT(ru, 1.0 / ru, zu, tu, 1.0 / tu, tu, Iu, rhou)
    if geometry == "XY":
        xu, yu, zu, Iu = p
        return UnitXY(xu, yu, 1.0 / xu, 1.0 / yu, zu, Iu)
    if geometry == "XYT":
        xu, yu, zu, tu, Iu, rhou = p
        return UnitXYT(xu, yu, 1.0 / xu, 1.0 / yu, zu, tu, 1.0 / tu, tu, Iu, rhou)
    raise ValueError("Wrong grid geometry.")


def E(unit, n0):
    """Unit of electric field, Eu = sqrt(Iu / (n0 eps0 c / 2)) (Units.jl:137-141)."""
    ksi = n0 * EPS0 * C0 / 2.0
    return math.sqrt(unit.I / ksi)
