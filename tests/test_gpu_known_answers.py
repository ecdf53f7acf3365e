"""The reference's physics tests (test/test_diffraction_r.jl,
test_diffraction_rt.jl, test_diffraction_xy.jl, test_dispersion_t.jl,
test_dispersion_rt.jl) run on the CUDA library, mixed and FP64 forms, with
the reference's tolerances."""
import math
import os

import numpy as np
import pytest

from conftest import DECKS

pytestmark = pytest.mark.gpu

LAM0 = 800e-9
A0 = 1e-3
ZD = 2 * math.pi / LAM0 * A0 ** 2
K2 = 2.131584978375e-29
TAU0 = 20e-15


def _run(deck, tmp_path, precision):
    import filament_gb as fg
    inp = fg.prepare(os.path.join(DECKS, deck, "input.py"))
    sim = fg.run(inp, precision=precision, outdir=str(tmp_path))
    sim.close()
    return np.loadtxt(os.path.join(str(tmp_path), "results", "plot.dat"), comments="#", ndmin=2).T


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_diffraction_rt(gpu_lib, tmp_path, precision):
    d = _run("diffraction_RT", tmp_path, precision)
    z, I, a = d[0], d[2], d[5] * 1e-3
    ath = A0 * np.sqrt(1 + (z / ZD) ** 2)
    Ith = (A0 / ath) ** 2
    assert np.max(np.abs(a - ath)) <= 0.02e-3
    assert np.max(np.abs(I - Ith)) <= 1e-3


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dispersion_rt(gpu_lib, tmp_path, precision):
    d = _run("dispersion_RT", tmp_path, precision)
    z, I = d[0], d[2]
    zd = TAU0 ** 2 / K2
    Ith = TAU0 / (TAU0 * np.sqrt(1 + (z / zd) ** 2))
    assert np.max(np.abs(I - Ith)) <= 1e-3


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_diffraction_xy(gpu_lib, tmp_path, precision):
    """test/test_diffraction_xy.jl:1-30 on the XY path (2048 x 2048)."""
    d = _run("diffraction_XY", tmp_path, precision)
    z, I, ax, ay = d[0], d[1], d[2] * 1e-3, d[3] * 1e-3
    ath = A0 * np.sqrt(1 + (z / ZD) ** 2)
    Ith = (A0 / ath) ** 2
    assert np.max(np.abs(ax - ath)) <= 0.01e-3
    assert np.max(np.abs(ay - ath)) <= 0.01e-3
    assert np.max(np.abs(I - Ith)) <= 1e-3


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_diffraction_r(gpu_lib, tmp_path, precision):
    """test/test_diffraction_r.jl:12-28 on the R path (Hankel matrix-vector
    products, 2000 points)."""
    d = _run("diffraction_R", tmp_path, precision)
    z, I, a = d[0], d[1], d[2] * 1e-3
    ath = A0 * np.sqrt(1 + (z / ZD) ** 2)
    Ith = (A0 / ath) ** 2
    assert np.max(np.abs(a - ath)) <= 0.02e-3
    assert np.allclose(I, Ith, rtol=1e-3)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_dispersion_t(gpu_lib, tmp_path, precision):
    """test/test_dispersion_t.jl:1-28 on the T path (one row, the linear step
    pointwise in w)."""
    d = _run("dispersion_T", tmp_path, precision)
    z, I, tau = d[0], d[1], d[3] * 1e-15
    zd = TAU0 ** 2 / K2
    tauth = TAU0 * np.sqrt(1 + (z / zd) ** 2)
    Ith = TAU0 / tauth
    assert np.max(np.abs(tau - tauth)) <= 0.1e-15
    assert np.max(np.abs(I - Ith)) <= 1e-3
