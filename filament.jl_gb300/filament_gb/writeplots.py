"""plot.dat writer (src/modules/WritePlots.jl:18-216): three header lines
(names, SI units, dimensionless unit values) and one row per analyzer call,
every value as %18.12e.  PlotNPZ: the content of the reference's plot.h5
(WritePlots.jl:218-507) in NumPy containers, there being no HDF5 library
here: the z-data group as plot_zdata.npz and the field snapshots as
plot_field_NNN.npy."""


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


class PlotNPZ:
    """WritePlots.PlotHDF (WritePlots.jl:218-368) without HDF5.  zdata
    (every call with z >= znext_zdata, step dz_zdata = lam0/2/zu): z and,
    RT: Fzr, rhozr, Fzt, iSzf; XYT: Fzxy, rhozxy, iSzf; XY: Izx, Izy (the
    intensity through the grid centre), written to <prefix>plot_zdata.npz by
    flush()/close().  Fields (z >= znext_field, step dz_plothdf, and not at
    the previous z-data point): <prefix>plot_field_NNN.npy, Re(E) for RT and
    XYT, E otherwise, with the z values in <prefix>plot_fields_z.npy."""

    def __init__(self, prefix, geometry, unit, z, dz_field, dz_zdata):
        import numpy as np
        self.np = np
        self.prefix = prefix
        self.geometry = geometry
        self.unit = unit
        self.dz_field = dz_field
        self.znext_field = z
        self.zprev_field = None
        self.ifield = 1
        self.field_z = []
        self.dz_zdata = dz_zdata
        self.znext_zdata = z
        self.zdata = {}

    def write(self, handle, analyzer, z):
        """WritePlots.writeHDF (WritePlots.jl:286-307)."""
        if z != self.zprev_field and z >= self.znext_field:
            E = handle.get_field()
            if self.geometry in ("RT", "XYT"):
                E = E.real
            self.np.save("%splot_field_%03d.npy" % (self.prefix, self.ifield), E)
            self.field_z.append(z)
            self.np.save("%splot_fields_z.npy" % self.prefix, self.np.asarray(self.field_z))
            self.ifield += 1
            self.znext_field += self.dz_field
        if z >= self.znext_zdata:
            self._zdata(analyzer)
            self.zprev_field = z
            self.znext_zdata = z + self.dz_zdata

    def _add(self, name, v):
        self.zdata.setdefault(name, []).append(self.np.array(v, copy=True))

    def _zdata(self, a):
        g = self.geometry
        self._add("z", a.z)
        if g == "RT":
            self._add("Fzr", a.Fr)
            self._add("rhozr", a.rho)
            self._add("Fzt", a.Ft)
            self._add("iSzf", a.S)
        elif g == "XYT":
            self._add("Fzxy", a.Fxy)
            self._add("rhozxy", a.rho)
            self._add("iSzf", a.S)
        elif g == "XY":
            I = a.I
            self._add("Izx", I[:, I.shape[1] // 2])
            self._add("Izy", I[I.shape[0] // 2, :])

    def flush(self):
        if self.zdata:
            self.np.savez("%splot_zdata.npz" % self.prefix,
                          **{k: self.np.stack(v) for k, v in self.zdata.items()})

    close = flush
