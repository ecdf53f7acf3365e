"""Medium functions (src/modules/Media.jl:1-194), host FP64.

`permittivity(w)` and `permeability(w)` are user callables of the angular
frequency in rad/s, as in the reference's medium decks (examples/RT/air.jl).
"""
import cmath
import math

from .constants import C0, EPS0


class Medium:
    """Media.Medium (Media.jl:8-12)."""

    def __init__(self, permittivity, permeability, n2):
        self.permittivity = permittivity
        self.permeability = permeability
        self.n2 = n2


class NonlinearResponse:
    """Media.NonlinearResponse (Media.jl:15-19): the reference's response
    plug-in record.  Here `kind` names one of the built-in device channels
    (cubic, free, losses, raman) instead of a Julia closure, `Rnl` is a scalar
    or a per-frequency complex table, and `p` holds the channel's switches."""

    def __init__(self, kind, Rnl, p):
        self.kind = kind
        self.Rnl = Rnl
        self.p = p


def refractive_index(medium, w):
    """Media.jl:22-27."""
    eps = medium.permittivity(abs(w))
    mu = medium.permeability(abs(w))
    return cmath.sqrt(complex(eps * mu))


def beta_func(medium, w):
    """Media.jl:29-32."""
    return refractive_index(medium, w) * w / C0


def k_func(medium, w):
    """Media.jl:35-38."""
    return beta_func(medium, w).real


def derivative(f, x, n):
    """Five-point stencil N-th derivative (Media.jl:168-191)."""
    h = 0.01 if x == 0 else 0.001 * x
    if n == 1:
        return (f(x - 2 * h) - 8 * f(x - h) + 8 * f(x + h) - f(x + 2 * h)) / (12 * h)
    if n == 2:
        return (-f(x - 2 * h) + 16 * f(x - h) - 30 * f(x) + 16 * f(x + h)
                - f(x + 2 * h)) / (12 * h ** 2)
    if n == 3:
        return (-f(x - 2 * h) + 2 * f(x - h) - 2 * f(x + h) + f(x + 2 * h)) / (2 * h ** 3)
    if n == 4:
        return (f(x - 2 * h) - 4 * f(x - h) + 6 * f(x) - 4 * f(x + h)
                + f(x + 2 * h)) / (h ** 4)
    raise ValueError("Wrong derivative order.")


def k1_func(medium, w):
    return derivative(lambda x: k_func(medium, x), w, 1)


def k2_func(medium, w):
    return derivative(lambda x: k_func(medium, x), w, 2)


def k3_func(medium, w):
    return derivative(lambda x: k_func(medium, x), w, 3)


def group_velocity(medium, w):
    """Media.jl:76-79."""
    return 1.0 / k1_func(medium, w)


def phase_velocity(medium, w):
    return C0 / refractive_index(medium, w).real


def diffraction_length(medium, w, a0):
    return k_func(medium, w) * a0 ** 2


def dispersion_length(medium, w, t0):
    k2 = k2_func(medium, w)
    return math.inf if k2 == 0 else t0 ** 2 / abs(k2)


def dispersion_length3(medium, w, t0):
    """Media.jl:99-107 (t0^3 / |k3|)."""
    k3 = k3_func(medium, w)
    return math.inf if k3 == 0 else t0 ** 3 / abs(k3)


def absorption_coefficient(medium, w):
    """Media.jl:64-67: Im(beta), by field."""
    return beta_func(medium, w).imag


def absorption_length(medium, w):
    """Media.jl:110-118, as the reference states it (ga / 2 for ga != 0)."""
    ga = absorption_coefficient(medium, w)
    return math.inf if ga == 0 else ga / 2


def nonlinearity_length(medium, w, I0):
    """Media.jl:137-145: 1 / (|n2| I0 w / c)."""
    n2 = medium.n2
    return math.inf if n2 == 0 else 1.0 / (abs(n2.real if isinstance(n2, complex) else n2) * I0 * w / C0)


def chi3_func(medium, w):
    """Media.jl:121-125."""
    n = refractive_index(medium, w)
    return 4.0 / 3.0 * n.real ** 2 * EPS0 * C0 * medium.n2


def critical_power(medium, w):
    """Media.jl:128-134 (Rcr = 3.79)."""
    Rcr = 3.79
    lam = 2 * math.pi * C0 / w
    n = refractive_index(medium, w)
    den = 8.0 * math.pi * abs(n.real) * abs(medium.n2)
    return math.inf if den == 0 else Rcr * lam ** 2 / den      # a Kerr-free medium: infinite


def selffocusing_length(medium, w, a0, P):
    """Marburger formula (Media.jl:148-157)."""
    Ld = diffraction_length(medium, w, a0)
    PPcr = P / critical_power(medium, w)
    if PPcr > 1:
        return 0.367 * Ld / math.sqrt((math.sqrt(PPcr) - 0.852) ** 2 - 0.0219)
    return math.inf


def air_permittivity(w):
    """Peck and Reeder two-term dispersion of air (JOSA 62, 958 (1972)), the
    medium of the reference's decks (examples/RT/air.jl:4-17)."""
    if w == 0.0:
        sig = 0.0
    else:
        lam = 2.0 * math.pi * C0 / w
        sig = 1.0 / lam * 1e-6
    dum = 8060.51 + 2480990.0 / (132.247 - sig ** 2) + 17455.7 / (39.32957 - sig ** 2)
    n = 1.0 + dum * 1e-8
    return n * n


def unit_permeability(w):
    return 1.0
