"""The integral power spectrum (FieldAnalyzers.jl:180-197 RT, :320-336 XYT)
and the plot.h5 content (WritePlots.jl:218-507) written as NumPy
containers, on the FP64 oracle: the spectrum against a numpy evaluation of
the analyzer's formula on the oracle's field, Parseval's identity against
the energy W, and the z-data / field files of a short run of the
reference's dispersion_RT deck."""
import math
import os

import numpy as np
import pytest

from conftest import DECKS


def _spectrum_numpy(E, w, dt):
    """S_k = sum_p w_p |2 Sr_k Nt dt|^2, Sa = ifft(E_p), Sr_0 = Sa_0,
    Sr_k = Sa_k / 2 (0 < k < Nt/2), the Nyquist bin as Sa holds it."""
    nt = E.shape[-1]
    Sa = np.fft.ifft(E, axis=-1)[..., : nt // 2 + 1]
    c = np.full(nt // 2 + 1, 0.5)
    c[0] = c[-1] = 1.0
    v = 2.0 * c * Sa * nt * dt
    return np.tensordot(w, np.abs(v) ** 2, axes=(0, 0))


def _close(S, ref):
    """Equal to FFT rounding: bins far down the spectrum's wings carry the
    transform's absolute error, ~1e-16 of the peak."""
    np.testing.assert_allclose(S, ref, rtol=1e-9, atol=1e-13 * float(np.max(ref)))


def test_rt_spectrum_formula_and_parseval(oracle_binding):
    import filament_gb as fg
    from gpu_helpers import rt_input
    sim = fg.Simulation(rt_input(), binding=oracle_binding)
    dt = float(sim.grid.dt)
    w = 2 * math.pi * sim.grid.r * sim.grid.dr
    S0 = sim.handle.spectrum()
    E0 = sim.handle.get_field()
    assert S0.shape == (sim.grid.Nt // 2 + 1,)
    _close(S0, _spectrum_numpy(E0, w, dt))
    # Parseval at z0 (the field is analytic: nothing above Nt/2, nothing at
    # w = 0): sum_k S_k / (Nt dt) = W = 2 pi sum_r r dr sum_t |E|^2 dt
    W = sim.handle.analyze()["energy"]
    assert np.sum(S0) / (sim.grid.Nt * dt) == pytest.approx(W, rel=1e-10)
    z = 0.0
    for _ in range(3):
        z += 2e-3
        sim.handle.step(z, 2e-3)
    S1 = sim.handle.spectrum()
    _close(S1, _spectrum_numpy(sim.handle.get_field(), w, dt))
    sim.close()


def test_xyt_spectrum_formula(oracle_binding):
    import filament_gb as fg
    from gpu_helpers import xyt_input
    sim = fg.Simulation(xyt_input(Nx=64, Ny=64, Nt=512), binding=oracle_binding)
    E = sim.handle.get_field().reshape(-1, sim.grid.Nt)
    w = np.full(E.shape[0], float(sim.grid.dx * sim.grid.dy))
    _close(sim.handle.spectrum(), _spectrum_numpy(E, w, float(sim.grid.dt)))
    sim.close()


def test_plot_npz_files(oracle_binding, tmp_path):
    import filament_gb as fg
    inp = fg.prepare(os.path.join(DECKS, "dispersion_RT", "input.py"), zmax=0.05)
    sim = fg.run(inp, binding=oracle_binding, outdir=str(tmp_path))
    out = os.path.join(str(tmp_path), "results")
    zd = np.load(os.path.join(out, "plot_zdata.npz"))
    nz = len(zd["z"])
    dat = np.loadtxt(os.path.join(out, "plot.dat"), comments="#", ndmin=2)
    assert nz == dat.shape[0] >= 2
    assert zd["Fzr"].shape == (nz, sim.grid.Nr) and zd["Fzt"].shape == (nz, sim.grid.Nt)
    assert zd["iSzf"].shape == (nz, sim.grid.Nt // 2 + 1) and zd["rhozr"].shape == (nz, sim.grid.Nr)
    assert np.all(np.isfinite(zd["iSzf"])) and np.all(zd["iSzf"] >= 0)
    np.testing.assert_allclose(zd["z"], dat[:, 0], rtol=1e-12)
    zf = np.load(os.path.join(out, "plot_fields_z.npy"))
    f1 = np.load(os.path.join(out, "plot_field_001.npy"))
    assert zf[0] == 0.0 and f1.shape == (sim.grid.Nr, sim.grid.Nt) and np.isrealobj(f1)
