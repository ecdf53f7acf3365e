"""Filament.run and main_loop (src/Filament.jl:51-184) over the device library.

The per-step work runs in the library; this module mirrors the reference's
construction sequence and its loop:
    dz = dzadaptive(analyzer); z += dz; zstep; analyze!; writeDAT; Istop test
With device_loop=True the whole loop (controller included) runs on the
device through fil_run and plot.dat receives the final state only.
"""
import datetime
import math
import os

import numpy as np

from . import media as Media
from . import units as Units
from .analyzers import FieldAnalyzer
from .backend import Handle
from .constants import C0
from .grids import Grid
from .guards import Guard_build
from .problem import Problem
from .writeplots import PlotDAT, PlotNPZ
from .infos import Info, PhaseTimer, clock


class Field:
    """Fields.Field host part (Fields.jl:31-160): w0 and the initial field
    evaluated on the host grid.  The analytic-signal conversion and all
    device state live in the library handle."""

    def __init__(self, geometry, unit, grid, p):
        lam0, initial_condition = p[0], p[1]
        self.w0 = 2 * math.pi * C0 / lam0
        if geometry == "R":
            E = initial_condition(grid.r, unit.r, unit.I)
        elif geometry == "T":
            E = initial_condition(grid.t, unit.t, unit.I)
        elif geometry == "RT":
            E = initial_condition(grid.r, grid.t, unit.r, unit.t, unit.I)
        elif geometry == "XY":
            E = initial_condition(grid.x, grid.y, unit.x, unit.y, unit.I)
        else:
            E = initial_condition(grid.x, grid.y, grid.t, unit.x, unit.y, unit.t, unit.I)
        self.E0 = np.asarray(E, dtype=np.complex128)


class AStep:
    """AdaptiveSteps (AdaptiveSteps.jl:20-107) on the host, for the host loop."""

    def __init__(self, cfg):
        self.cfg = cfg

    def __call__(self, analyzer):
        c = self.cfg
        if not c.nonlinearity:
            return c.dz0
        dz = min(c.dz0, c.phimax / (c.phik * analyzer.Imax) if analyzer.Imax > 0 else math.inf)
        if c.phip > 0 and analyzer.rhomax > 0:
            dz = min(dz, c.phimax / (c.phip * analyzer.rhomax))
        return dz


class Simulation:
    """Everything Filament.run builds (Filament.jl:72-79)."""

    def __init__(self, input, binding=None, precision="mixed", make_handle=True):
        g = input["geometry"]
        self.geometry = g
        self.unit = Units.Unit(g, input["p_unit"])
        self.grid = Grid(g, input["p_grid"])
        self.field = Field(g, self.unit, self.grid, input["p_field"])
        self.medium = Media.Medium(*input["p_medium"])
        self.guard = Guard_build(g, self.unit, self.grid, self.field.w0, self.medium, input["p_guard"])
        responses_list, plasma_dict, keys = input["p_model"]
        resps = [item["init"](self.unit, self.grid, self.field, self.medium, item)
                 for item in responses_list]
        pe = None
        if keys.get("PLASMA"):
            w0 = self.field.w0
            n0 = Media.refractive_index(self.medium, w0)
            Eu = Units.E(self.unit, n0.real)
            units = (self.unit.t, Eu, self.unit.I, self.unit.rho)
            pe = plasma_dict["init"](self.grid.t, None, w0, units, plasma_dict)
        self.problem = Problem(g, self.unit, self.grid, self.field.w0, self.medium, self.guard,
                               resps, pe, keys, input["p_dzadaptive"], precision)
        self.z = input["z"]
        self.zmax = input["zmax"]
        self.Istop = input["Istop"]
        self.dzadaptive = AStep(self.problem.config)
        self.handle = None
        if make_handle:
            self.attach(Handle(self.problem, binding))

    def attach(self, handle):
        """Uses `handle` (made from self.problem, e.g. a batch member) and
        uploads the initial field."""
        self.handle = handle
        self.handle.set_field(self.field.E0, analytic=False)
        self.analyzer = FieldAnalyzer(self.geometry, self.grid, self.handle, self.z)
        self.analyzer.analyze(self.z)

    def close(self):
        if self.handle is not None:
            self.handle.close()


def run(input, binding=None, precision="mixed", device_loop=False, write_files=True,
        outdir=None):
    """Filament.run (Filament.jl:51-108).  Returns the Simulation."""
    sim = Simulation(input, binding, precision)
    plotdat = plotnpz = info = None
    if write_files:
        prefix = input["prefix"]
        base = outdir if outdir is not None else input.get("deck_dir", ".")
        path = os.path.join(base, prefix)
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        # info.txt (Filament.jl:88-89)
        info = Info(path + "info.txt", sim.geometry, sim.unit, sim.grid, sim.field.w0, sim.medium,
                    sim.analyzer, input["p_info"])
        plotdat = PlotDAT(path + "plot.dat", sim.geometry, sim.unit)
        plotdat.write(sim.analyzer)
        # plot.h5's content (Filament.jl:95-99): z-data every lam0/2, fields every dz_plothdf
        plotnpz = PlotNPZ(path, sim.geometry, sim.unit, sim.z, input["dz_plothdf"],
                          input["lam0"] / 2 / sim.unit.z)
        plotnpz.write(sim.handle, sim.analyzer, sim.z)
    try:
        main_loop(sim, plotdat, device_loop, plotnpz, info)
    finally:
        if plotnpz is not None:
            plotnpz.close()
    return sim


def main_loop(sim, plotdat, device_loop=False, plotnpz=None, info=None):
    """Filament.jl:111-184.  With `info`, the per-phase wall times (without
    the first step) and the start, end and run times go to info.txt."""
    z = sim.z
    timer = PhaseTimer()
    start = datetime.datetime.now()

    def timed(name, f, *a):
        t0 = clock()
        r = f(*a)
        timer.add(name, clock() - t0)
        return r

    def write(zz):
        if plotdat is not None:
            timed("writeDAT", plotdat.write, sim.analyzer)
        if plotnpz is not None:
            timed("writeHDF", plotnpz.write, sim.handle, sim.analyzer, zz)

    code = 0
    if device_loop:
        code, st = timed("zstep", sim.handle.run, z, sim.zmax, 2 ** 62)
        sim.z = st["z"]
        timed("field analyzer", sim.analyzer.analyze, sim.z)
        write(sim.z)
    else:
        first = True
        while z < sim.zmax:
            dz = sim.dzadaptive(sim.analyzer)
            z = z + dz
            timed("zstep", sim.handle.step, z, dz)
            timed("field analyzer", sim.analyzer.analyze, z)
            write(z)
            if sim.analyzer.Imax > sim.Istop:
                if info is not None:
                    info.message("Stop (Imax >= Istop): z=%s[zu], z=%s[m]" % (z, z * sim.unit.z))
                break
            if first:          # the first step's set-up is not in the timings
                timer.reset()
                first = False
        sim.z = z
    if info is not None:
        end = datetime.datetime.now()
        info.message(timer.table())
        info.message("Start time: %s\nEnd time:   %s\nRun time:   %s" % (start.isoformat(), end.isoformat(),
                                                                           end - start))
    return code
