"""plot.dat writer (src/modules/WritePlots.jl:18-216): three header lines
(names, SI units, dimensionless unit values) and one row per analyzer call,
every value as %18.12e."""


def fmt(x):
    return "%18.12e" % float(x)


def _columns(geometry, unit):
    if geometry == "R":
        return [("z", "m", unit.z, "z"), ("Imax", "W/m^2", unit.I, "Imax"),
                ("rfil", "m", unit.r, "rfil"), ("P", "W", unit.r ** 2 * unit.I, "P")]
    if geometry == "T":
        return [("z", "m", unit.z, "z"), ("Imax", "W/m^2", unit.I, "Imax"),
                ("Nemax", "1/m^3", unit.rho, "rhomax"), ("duration", "s", unit.t, "duration"),
                ("F", "J/m^2", unit.t * unit.I, "F")]
    if geometry == "RT":
        return [("z", "m", unit.z, "z"), ("Fmax", "J/m^2", unit.t * unit.I, "Fmax"),
                ("Imax", "W/m^2", unit.I, "Imax"), ("Nemax", "1/m^3", unit.rho, "rhomax"),
                ("De", "1/m", unit.r ** 2 * unit.rho, "De"), ("rfil", "m", unit.r, "rfil"),
                ("rpl", "m", unit.r, "rpl"), ("tau", "s", unit.t, "tau"),
                ("W", "J", unit.r ** 2 * unit.t * unit.I, "W")]
    if geometry == "XY":
        return [("z", "m", unit.z, "z"), ("Imax", "W/m^2", unit.I, "Imax"),
                ("ax", "m", unit.x, "ax"), ("ay", "m", unit.y, "ay"),
                ("P", "W", unit.x * unit.y * unit.I, "P")]
    if geometry == "XYT":
        return [("z", "m", unit.z, "z"), ("Fmax", "J/m^2", unit.t * unit.I, "Fmax"),
                ("Imax", "W/m^2", unit.I, "Imax"), ("Nemax", "1/m^3", unit.rho, "rhomax"),
                ("De", "1/m", unit.x * unit.y * unit.rho, "De"), ("ax", "m", unit.x, "ax"),
                ("ay", "m", unit.y, "ay"), ("W", "J", unit.x * unit.y * unit.t * unit.I, "W")]
    raise ValueError(geometry)


class PlotDAT:
    def __init__(self, fname, geometry, unit):
        self.fname = fname
        self.cols = _columns(geometry, unit)
        with open(fname, "w") as fp:
            fp.write("#" + "".join(" %-18s" % c[0] for c in self.cols) + "\n")
            fp.write("#" + "".join(" %-18s" % c[1] for c in self.cols) + "\n")
            fp.write("#" + "".join(" %-18s" % repr(float(c[2])) for c in self.cols) + "\n")

    def write(self, analyzer):
        with open(self.fname, "a") as fp:
            fp.write("  " + "".join(fmt(getattr(analyzer, c[3])) + " " for c in self.cols) + "\n")


def read_dat(fname):
    """readdlm(fname, comments=true) equivalent: the numeric rows."""
    import numpy as np
    return np.loadtxt(fname, comments="#", ndmin=2)
