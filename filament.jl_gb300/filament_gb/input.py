"""Input decks (src/Input.jl:20-200).

The reference evaluates Julia input files with `include`; this mirror
evaluates Python files defining the same globals (prefix, geometry, units,
grid, model switches, guards, dzphimax, Istop, ALG, file_initial_condition,
file_medium, initial_condition, permittivity, permeability, n2, responses,
plasma_equation).  The returned dict has the reference's keys.  Values stay
FP64 (the reference rounds RT/XY/XYT set-up values to Float32).
"""
import math
import os

import numpy as np

from . import constants
from . import plasma as _plasma
from . import responses as _responses
from . import media as _media


def _namespace(deck_dir):
    ns = {
        "__name__": "filament_deck",
        "math": math, "np": np, "pi": math.pi,
        "C0": constants.C0, "EPS0": constants.EPS0, "MU0": constants.MU0,
        "QE": constants.QE, "ME": constants.ME, "HBAR": constants.HBAR,
        "RK2": "RK2", "RK3": "RK3", "RK4": "RK4", "Tsit5": "Tsit5", "ATsit5": "ATsit5",
        "init_cubic": _responses.init_cubic,
        "init_current_free": _responses.init_current_free,
        "init_current_losses": _responses.init_current_losses,
        "init_raman": _responses.init_raman,
        "raman_response_air": _responses.raman_response_air,
        "init_photoionization_avalanche": _plasma.init_photoionization_avalanche,
        "power_law_rate": _plasma.power_law_rate,
        "air_permittivity": _media.air_permittivity,
        "unit_permeability": _media.unit_permeability,
        "DECKDIR": deck_dir,
    }
    return ns


def _exec(path, ns):
    with open(path) as fp:
        code = compile(fp.read(), path, "exec")
    exec(code, ns)


def prepare(fname, **overrides):
    """Input.prepare (Input.jl:20-200).  Keyword overrides replace deck
    globals after the deck has run (e.g. Nr=64 for a quick test)."""
    file_input = os.path.abspath(fname)
    deck_dir = os.path.dirname(file_input)
    ns = _namespace(deck_dir)
    _exec(file_input, ns)
    ns.update(overrides)
    _exec(os.path.join(deck_dir, ns["file_initial_condition"]), ns)
    _exec(os.path.join(deck_dir, ns["file_medium"]), ns)
    ns.update(overrides)
    g = ns["geometry"]
    NONLINEARITY = ns["NONLINEARITY"]
    PLASMA = ns.get("PLASMA", False)
    responses = ns["responses"] if NONLINEARITY else []
    p_medium = (ns["permittivity"], ns["permeability"], ns["n2"])
    keys = dict(NONLINEARITY=NONLINEARITY, PLASMA=False,
                KPARAXIAL=ns.get("KPARAXIAL", True), QPARAXIAL=ns.get("QPARAXIAL", True),
                ALG=ns.get("ALG", "RK4"), Istop=ns["Istop"])
    plasma_equation = {}
    if g == "R":
        p_unit = (ns["ru"], ns["zu"], ns["Iu"])
        p_grid = (ns["rmax"], ns["Nr"])
        p_guard = (ns["rguard"], ns["kguard"])
        p_dz = (ns["dz_initial"], ns["dzphimax"], NONLINEARITY)
    elif g == "T":
        p_unit = (ns["zu"], ns["tu"], ns["Iu"], ns["rhou"])
        p_grid = (ns["tmin"], ns["tmax"], ns["Nt"])
        p_guard = (ns["tguard"], ns["wguard"])
        p_dz = (ns["dz_initial"], ns["dzphimax"], ns.get("mr", 1.0), ns.get("nuc", 0.0), NONLINEARITY)
        keys.update(PLASMA=PLASMA, KPARAXIAL=True, QPARAXIAL=True)
        plasma_equation = ns["plasma_equation"] if PLASMA else {}
    elif g == "RT":
        p_unit = (ns["ru"], ns["zu"], ns["tu"], ns["Iu"], ns["rhou"])
        p_grid = (ns["rmax"], ns["Nr"], ns["tmin"], ns["tmax"], ns["Nt"])
        p_guard = (ns["rguard"], ns["tguard"], ns["kguard"], ns["wguard"])
        p_dz = (ns["dz_initial"], ns["dzphimax"], ns.get("mr", 1.0), ns.get("nuc", 0.0), NONLINEARITY)
        keys.update(PLASMA=PLASMA)
        plasma_equation = ns["plasma_equation"] if PLASMA else {}
    elif g == "XY":
        p_unit = (ns["xu"], ns["yu"], ns["zu"], ns["Iu"])
        p_grid = (ns["xmin"], ns["xmax"], ns["Nx"], ns["ymin"], ns["ymax"], ns["Ny"])
        p_guard = (ns["xguard"], ns["yguard"], ns["kxguard"], ns["kyguard"])
        p_dz = (ns["dz_initial"], ns["dzphimax"], NONLINEARITY)
    elif g == "XYT":
        p_unit = (ns["xu"], ns["yu"], ns["zu"], ns["tu"], ns["Iu"], ns["rhou"])
        p_grid = (ns["xmin"], ns["xmax"], ns["Nx"], ns["ymin"], ns["ymax"], ns["Ny"],
                  ns["tmin"], ns["tmax"], ns["Nt"])
        p_guard = (ns["xguard"], ns["yguard"], ns["tguard"], ns["kxguard"], ns["kyguard"], ns["wguard"])
        p_dz = (ns["dz_initial"], ns["dzphimax"], ns.get("mr", 1.0), ns.get("nuc", 0.0), NONLINEARITY)
        keys.update(PLASMA=PLASMA)
        plasma_equation = ns["plasma_equation"] if PLASMA else {}
    else:
        raise ValueError("Wrong grid geometry.")
    return {
        "prefix": ns.get("prefix", "results/"),
        "deck_dir": deck_dir,
        "geometry": g,
        "z": ns["z"] / ns["zu"],
        "zmax": ns["zmax"],
        "lam0": ns["lam0"],
        "Istop": ns["Istop"],
        "dz_plothdf": ns.get("dz_plothdf", ns["zmax"]),
        "p_unit": p_unit,
        "p_grid": p_grid,
        "p_field": (ns["lam0"], ns["initial_condition"]),
        "p_medium": p_medium,
        "p_guard": p_guard,
        "p_model": (responses, plasma_equation, keys),
        "p_dzadaptive": p_dz,
        "p_info": (file_input, os.path.join(deck_dir, ns["file_initial_condition"]),
                   os.path.join(deck_dir, ns["file_medium"])),
    }
