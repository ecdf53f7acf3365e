"""The reference's five physics tests (test/runtests.jl:8-29) run against the
FP64 oracle, with the reference's own tolerances.  They pin the oracle's
linear path (QDHT, KZ, t-FFT, analytic signal, guards) to closed-form
Gaussian-beam diffraction and pulse dispersion."""
import math
import os

import numpy as np
import pytest

from conftest import DECKS

LAM0 = 800e-9
A0 = 1e-3
ZD = 2 * math.pi / LAM0 * A0 ** 2          # diffraction length
K2 = 2.131584978375e-29                     # test/dispersion/T/runtests: d(k1)/dw of air
TAU0 = 20e-15


def _run(deck, binding, tmp_path):
    import filament_gb as fg
    inp = fg.prepare(os.path.join(DECKS, deck, "input.py"))
    sim = fg.run(inp, binding=binding, outdir=str(tmp_path))
    sim.close()
    return np.loadtxt(os.path.join(str(tmp_path), "results", "plot.dat"), comments="#", ndmin=2).T


def test_diffraction_r(oracle_binding, tmp_path):
    """test/test_diffraction_r.jl:12-28."""
    d = _run("diffraction_R", oracle_binding, tmp_path)
    z, I, a = d[0], d[1], d[2] * 1e-3
    ath = A0 * np.sqrt(1 + (z / ZD) ** 2)
    Ith = (A0 / ath) ** 2
    assert np.max(np.abs(a - ath)) <= 0.02e-3
    assert np.allclose(I, Ith, rtol=1e-3)


def test_diffraction_rt(oracle_binding, tmp_path):
    """test/test_diffraction_rt.jl:1-29."""
    d = _run("diffraction_RT", oracle_binding, tmp_path)
    z, I, a = d[0], d[2], d[5] * 1e-3
    ath = A0 * np.sqrt(1 + (z / ZD) ** 2)
    Ith = (A0 / ath) ** 2
    assert np.max(np.abs(a - ath)) <= 0.02e-3
    assert np.max(np.abs(I - Ith)) <= 1e-3


def test_diffraction_xy(oracle_binding, tmp_path):
    """test/test_diffraction_xy.jl:1-30."""
    d = _run("diffraction_XY", oracle_binding, tmp_path)
    z, I, ax, ay = d[0], d[1], d[2] * 1e-3, d[3] * 1e-3
    ath = A0 * np.sqrt(1 + (z / ZD) ** 2)
    Ith = (A0 / ath) ** 2
    assert np.max(np.abs(ax - ath)) <= 0.01e-3
    assert np.max(np.abs(ay - ath)) <= 0.01e-3
    assert np.max(np.abs(I - Ith)) <= 1e-3


def test_dispersion_t(oracle_binding, tmp_path):
    """test/test_dispersion_t.jl:1-28."""
    d = _run("dispersion_T", oracle_binding, tmp_path)
    z, I, tau = d[0], d[1], d[3] * 1e-15
    zd = TAU0 ** 2 / K2
    tauth = TAU0 * np.sqrt(1 + (z / zd) ** 2)
    Ith = TAU0 / tauth
    assert np.max(np.abs(tau - tauth)) <= 0.1e-15
    assert np.max(np.abs(I - Ith)) <= 1e-3


def test_dispersion_rt(oracle_binding, tmp_path):
    """test/test_dispersion_rt.jl:1-27."""
    d = _run("dispersion_RT", oracle_binding, tmp_path)
    z, I = d[0], d[2]
    zd = TAU0 ** 2 / K2
    tauth = TAU0 * np.sqrt(1 + (z / zd) ** 2)
    Ith = TAU0 / tauth
    assert np.max(np.abs(I - Ith)) <= 1e-3
