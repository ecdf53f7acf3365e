"""info.txt (src/modules/Infos.jl:22-612, written by Filament.run,
src/Filament.jl:88-89, 160-181): the deck files, the derived parameters of
the grid, field and medium, and the runtime information, for a short run of
each geometry on the oracle.  The values are checked against what they
state: the intensity is the analyzer's Imax in W/m^2, the photon energy of
800 nm is 1.5498 eV, the RT beam carries the deck's 3 critical powers, the
T pulse is 35 fs FWHM, the R beam is 1 mm at 1/e."""
import math
import os

import pytest

from conftest import DECKS
from gpu_helpers import FIL_DECK


def _sections(text):
    """{section: {name: (value, unit)}} of the Parameters block."""
    out, cur = {}, None
    block = text.split("Parameters", 1)[1].split("Runtime information", 1)[0]
    for line in block.splitlines():
        if line.startswith("# "):
            cur = line[2:].split(" (")[0].split(" -")[0].strip()
            out[cur] = {}
        elif cur and " = " in line and "[" in line:
            name, rest = line.split(" = ", 1)
            value, unit = rest.split(" [", 1)
            out[cur].setdefault(name.strip(), (float(value), unit.split("]")[0]))
        elif line.startswith("*") and cur:
            cur = None
    return out


CASES = {
    "RT": (FIL_DECK, dict(Nr=64, Nt=512, rmax=2.0, tmin=-100.0, tmax=100.0, zmax=0.003)),
    "T": (os.path.join(DECKS, "nonlinear_T", "input.py"), dict(Nt=1024, zmax=0.003)),
    "R": (os.path.join(DECKS, "nonlinear_R", "input.py"), dict(Nr=128, zmax=0.003)),
    "XY": (os.path.join(DECKS, "diffraction_XY", "input.py"), dict(Nx=128, Ny=64, zmax=0.003)),
}


@pytest.mark.parametrize("geom", list(CASES))
def test_info_file(oracle_binding, tmp_path, geom):
    import filament_gb as fg
    deck, kw = CASES[geom]
    inp = fg.prepare(deck, **kw)
    sim = fg.Simulation(inp, binding=oracle_binding)
    imax0 = sim.analyzer.Imax
    sim.close()
    run = fg.run(inp, binding=oracle_binding, write_files=True, outdir=str(tmp_path))
    run.close()
    path = os.path.join(str(tmp_path), inp["prefix"], "info.txt")
    text = open(path).read()
    for title in ("jlFilament", "Input file", "Initial condition file", "Medium file", "Parameters",
                  "Runtime information"):
        assert title in text
    assert open(inp["p_info"][0]).read() in text          # the deck itself
    assert "Start time:" in text and "Run time:" in text and "ncalls" in text
    s = _sections(text)
    field, medium, grid = s["Field"], s["Medium"], s["Grid"]
    Iu = inp["p_unit"][-1] if geom in ("R", "XY") else inp["p_unit"][-2]
    assert field["I0"] == (pytest.approx(imax0 * Iu, rel=1e-11), "W/m^2")
    assert field["lam0"][0] == pytest.approx(800e-9, rel=1e-12)
    assert field["Wph"][0] == pytest.approx(6.62607015e-34 * 299792458.0 / 800e-9, rel=1e-9)
    assert medium["n0re"][0] == pytest.approx(1.000275, abs=1e-5)
    if geom == "RT":
        assert medium["P"] == (pytest.approx(3.0, rel=0.03), "Pcr")
        assert set(grid) == {"dr", "dk", "kc", "dt", "df", "fc"}
    if geom == "T":
        assert field["t0fwhm"][0] == pytest.approx(35e-15, rel=0.02)
        assert set(grid) == {"dt", "df", "fc"}
    if geom == "R":
        assert field["a0e"][0] == pytest.approx(1e-3, rel=0.02)
    if geom == "XY":
        assert set(grid) == {"dx", "dy", "dkx", "dky", "kxc", "kyc"}
    assert math.isinf(medium["La"][0])                      # air without absorption


def test_stop_message_and_timings(oracle_binding, tmp_path):
    """A run that reaches Istop says so in info.txt (Filament.jl:160-163) and
    times its phases without the first step (Filament.jl:166-170)."""
    import filament_gb as fg
    deck, kw = CASES["RT"]
    inp = fg.prepare(deck, **dict(kw, zmax=0.01, Istop=0.5))     # Imax is 0.92 at z = 0
    run = fg.run(inp, binding=oracle_binding, write_files=True, outdir=str(tmp_path))
    run.close()
    text = open(os.path.join(str(tmp_path), inp["prefix"], "info.txt")).read()
    assert "Stop (Imax >= Istop): z=" in text
    inp = fg.prepare(deck, **dict(kw, zmax=0.005))
    run = fg.run(inp, binding=oracle_binding, write_files=True, outdir=str(tmp_path / "b"))
    run.close()
    text = open(os.path.join(str(tmp_path / "b"), inp["prefix"], "info.txt")).read()
    table = text.split("Runtime information", 1)[1]
    rows = {l.split()[0]: l.split() for l in table.splitlines() if l and l.split()[0] in
            ("zstep", "field", "writeDAT", "writeHDF")}
    assert int(rows["zstep"][1]) == 4                  # 5 steps of 1 mm, the first not timed
    assert set(rows) == {"zstep", "field", "writeDAT", "writeHDF"}
