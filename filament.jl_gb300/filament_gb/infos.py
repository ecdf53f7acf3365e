"""The run's info.txt (src/modules/Infos.jl:22-612): the deck files, the
derived parameters of the grid, the field and the medium at the central
frequency, then runtime messages and the per-phase timing table that
Filament.run appends (src/Filament.jl:88-89, 160-181).

The sections are the reference's, with its names, units and descriptions;
the layout of each is a list of rows (name, value in SI, unit, text)."""
import datetime
import math
import os
import subprocess
import time

import numpy as np

from . import media as Media
from .constants import C0, HBAR, QE

RULE = "*" * 80


def _fmt(x):
    """Infos.jl:14: %18.12e."""
    return "%18.12e" % float(x)


def _rows(rows):
    width = max(len(r[0]) for r in rows)
    return "".join("%s = %s [%s] - %s\n" % (n.ljust(width), _fmt(v), u, d) for n, v, u, d in rows)


def _banner(title):
    return "%s\n%s\n%s\n" % (RULE, title.center(80).rstrip(), RULE)


def vcs_revision():
    """Infos.jl:85-98: branch and commit of the source tree, if any."""
    here = os.path.dirname(os.path.abspath(__file__))
    try:
        b = subprocess.run(["git", "rev-parse", "--abbrev-ref", "HEAD"], cwd=here, capture_output=True,
                           text=True, timeout=10)
        h = subprocess.run(["git", "rev-parse", "HEAD"], cwd=here, capture_output=True, text=True, timeout=10)
        if b.returncode == 0 and h.returncode == 0:
            return "%s %s" % (b.stdout.strip(), h.stdout.strip())
    except (OSError, subprocess.SubprocessError):
        pass
    return "unavailable"


def grid_rows(geometry, unit, grid):
    """Infos.jl:101-208."""
    rows = []
    if geometry in ("R", "RT"):
        dr = float(np.mean(np.diff(grid.r)))
        dk = float(np.mean(np.diff(grid.k)))
        rows += [("dr", dr * unit.r, "m", "average spatial step"),
                 ("dk", dk * unit.k, "1/m", "average spatial frequency (angular) step"),
                 ("kc", 2 * math.pi * 0.5 / dr * unit.k, "1/m", "spatial Nyquist frequency (angular)")]
    if geometry in ("XY", "XYT"):
        dkx, dky = grid.kx[1] - grid.kx[0], grid.ky[1] - grid.ky[0]
        rows += [("dx", grid.dx * unit.x, "m", "x spatial step"),
                 ("dy", grid.dy * unit.y, "m", "y spatial step"),
                 ("dkx", dkx * unit.kx, "1/m", "x spatial frequency (angular) step"),
                 ("dky", dky * unit.ky, "1/m", "y spatial frequency (angular) step"),
                 ("kxc", 2 * math.pi * 0.5 / dkx * unit.kx, "1/m", "x spatial Nyquist frequency (angular)"),
                 ("kyc", 2 * math.pi * 0.5 / dky * unit.ky, "1/m", "y spatial Nyquist frequency (angular)")]
    if geometry in ("T", "RT", "XYT"):
        f = grid.w / (2 * math.pi)
        rows += [("dt", grid.dt * unit.t, "s", "temporal step"),
                 ("df", (f[1] - f[0]) * unit.w, "1/s", "temporal frequency step"),
                 ("fc", 0.5 / grid.dt * unit.w, "1/s", "temporal Nyquist frequency")]
    return rows


def _beam(geometry, unit, an):
    """The initial beam size a0 (1/e half width) in m, or None."""
    if geometry in ("R", "RT"):
        return an.rfil * unit.r
    if geometry == "XY":
        return math.sqrt(an.ax * an.ay * unit.x * unit.y)
    return None


def _duration(geometry, unit, an):
    if geometry == "RT":
        return an.tau * unit.t
    if geometry == "T":
        return an.duration * unit.t
    return None


def field_rows(geometry, unit, w0, an):
    """Infos.jl:211-401."""
    I0 = an.Imax * unit.I
    a0, t0 = _beam(geometry, unit, an), _duration(geometry, unit, an)
    s2, fw = math.sqrt(2), 2 * math.sqrt(math.log(2))
    rows = []
    if a0 is not None:
        rows += [("a0e", a0, "m", "initial beam size (half width 1/e)"),
                 ("a0e2", s2 * a0, "m", "initial beam size (half width 1/e^2)"),
                 ("a0fwhm", fw * a0, "m", "initial beam size (FWHM)")]
    if t0 is not None:
        rows += [("t0e", t0, "s", "initial pulse duration (half width 1/e)"),
                 ("t0e2", s2 * t0, "s", "initial pulse duration (half width 1/e^2)"),
                 ("t0fwhm", fw * t0, "s", "initial pulse duration (FWHM)")]
    rows += [("I0", I0, "W/m^2", "initial intensity"),
             ("lam0", 2 * math.pi * C0 / w0, "m", "central wavelength"),
             ("f0", w0 / (2 * math.pi), "1/s", "central frequency"),
             ("w0", w0, "1/s", "central frequency (angular)")]
    P = _peak_power(geometry, unit, an)
    if geometry == "RT":
        F = an.Fmax * unit.t * unit.I
        W = an.W * unit.r ** 2 * unit.t * unit.I
        rows += [("P", P, "W", "peak power"),
                 ("Pg", math.pi * a0 ** 2 * I0, "W", "Gaussian peak power (pi*a0^2*I0)"),
                 ("F", F, "J/m^2", "peak fluence"),
                 ("Fg", math.sqrt(math.pi) * t0 * I0, "J/m^2", "Gaussian peak fluence (pi^0.5*t0*I0)"),
                 ("W", W, "J", "pulse energy"),
                 ("Wg", math.pi ** 1.5 * t0 * a0 ** 2 * I0, "J", "Gaussian pulse energy (pi^1.5*t0*a0^2*I0)")]
    elif geometry in ("R", "XY"):
        rows += [("P", P, "W", "peak power"),
                 ("Pg", math.pi * a0 ** 2 * I0, "W", "Gaussian peak power (pi*a0^2*I0)")]
    elif geometry == "T":
        rows += [("F", an.F * unit.t * unit.I, "J/m^2", "peak fluence"),
                 ("Fg", math.sqrt(math.pi) * t0 * I0, "J/m^2", "Gaussian peak fluence (pi^0.5*t0*I0)")]
    Wph = HBAR * w0
    rows += [("Wph", Wph, "J", "energy of one photon"), ("Wph", Wph / QE, "eV", "energy of one photon")]
    return rows


def _peak_power(geometry, unit, an):
    if geometry == "RT":
        W = an.W * unit.r ** 2 * unit.t * unit.I
        return W / (an.tau * unit.t) / math.sqrt(math.pi)
    if geometry == "R":
        return an.P * unit.r ** 2 * unit.I
    if geometry == "XY":
        return an.P * unit.x * unit.y * unit.I
    return None


def medium_rows(geometry, unit, w0, medium, an):
    """Infos.jl:404-590 (values at the central frequency)."""
    n0 = Media.refractive_index(medium, w0)
    I0 = an.Imax * unit.I
    a0, t0 = _beam(geometry, unit, an), _duration(geometry, unit, an)
    rows = [("n0re", n0.real, "-", "refractive index (real part)"),
            ("n0im", n0.imag, "-", "refractive index (imaginary part)"),
            ("k0", Media.k_func(medium, w0), "1/m", "wave number"),
            ("k1", Media.k1_func(medium, w0), "s/m", "1st derivative of wave number: d(k0)/dw"),
            ("k2", Media.k2_func(medium, w0), "s^2/m", "2nd derivative of wave number: d(k1)/dw"),
            ("k3", Media.k3_func(medium, w0), "s^3/m", "3rd derivative of wave number: d(k2)/dw"),
            ("ga", Media.absorption_coefficient(medium, w0), "1/m", "linear absorption coefficient (by field)"),
            ("vp", Media.phase_velocity(medium, w0) / C0, "C0", "phase velocity"),
            ("vg", Media.group_velocity(medium, w0) / C0, "C0", "group velocity"),
            ("n2", medium.n2, "m^2/W", "Kerr nonlinear index"),
            ("chi3", Media.chi3_func(medium, w0), "m/V", "3rd order nonlinear susceptibility")]
    Pcr = Media.critical_power(medium, w0)
    P = _peak_power(geometry, unit, an)
    if P is not None:
        rows.append(("P", P / Pcr, "Pcr", "peak power"))
    if geometry != "T":
        rows.append(("Pcr", Pcr, "W", "critical power"))
    if a0 is not None:
        rows.append(("Ld", Media.diffraction_length(medium, w0, a0), "m", "diffraction length"))
    if t0 is not None:
        rows += [("Ldisp", Media.dispersion_length(medium, w0, t0), "m", "dispersion length"),
                 ("Ldisp3", Media.dispersion_length3(medium, w0, t0), "m",
                  "3rd order dispersion length (t0^3/k3)")]
    rows.append(("La", Media.absorption_length(medium, w0), "m", "linear absorption length"))
    if geometry != "XYT":
        rows.append(("Lnl", Media.nonlinearity_length(medium, w0, I0), "m", "length of Kerr nonlinearity"))
    if P is not None:
        rows.append(("zf", Media.selffocusing_length(medium, w0, a0, P), "m", "self-focusing distance"))
    return rows


class Info:
    """Infos.Info: writes the header and the parameters at construction;
    message() appends (and prints) runtime information."""

    def __init__(self, fname, geometry, unit, grid, w0, medium, analyzer, files):
        self.fname = fname
        parts = ["\n", _banner("jlFilament"),
                 "datetime: %s\nrevision: %s\n\n" % (datetime.datetime.now().isoformat(), vcs_revision())]
        for title, path in zip(("Input file", "Initial condition file", "Medium file"), files):
            with open(path) as fp:
                parts += [_banner(title), fp.read(), "\n"]
        parts += [_banner("Parameters"),
                  "# Grid " + "-" * 73 + "\n", _rows(grid_rows(geometry, unit, grid)),
                  "# Field " + "-" * 72 + "\n", _rows(field_rows(geometry, unit, w0, analyzer)),
                  "# Medium (all values are given at central frequency) " + "-" * 27 + "\n",
                  _rows(medium_rows(geometry, unit, w0, medium, analyzer)),
                  _banner("Runtime information")]
        with open(fname, "w") as fp:
            fp.write("".join(parts))

    def message(self, text):
        """Infos.write_message."""
        with open(self.fname, "a") as fp:
            fp.write(str(text) + "\n")
        print(text)


class PhaseTimer:
    """Wall time per phase of the main loop (the reference's TimerOutputs
    sections "zstep", "field analyzer", "writeDAT", "writeHDF"), without the
    first step."""

    def __init__(self):
        self.t = {}
        self.n = {}

    def add(self, name, seconds):
        self.t[name] = self.t.get(name, 0.0) + seconds
        self.n[name] = self.n.get(name, 0) + 1

    def reset(self):
        self.t.clear()
        self.n.clear()

    def table(self):
        total = sum(self.t.values())
        lines = ["%-20s %8s %14s %8s" % ("section", "ncalls", "time (s)", "%tot")]
        for name in self.t:
            share = 100.0 * self.t[name] / total if total > 0 else 0.0
            lines.append("%-20s %8d %14.6f %7.1f%%" % (name, self.n[name], self.t[name], share))
        return "\n".join(lines)


def clock():
    return time.perf_counter()
