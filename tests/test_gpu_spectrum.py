"""The integral power spectrum (fil_analyze_spectrum: k_rowspec + k_colsum,
FieldAnalyzers.jl:180-197, 320-336) on the GPU against the FP64 oracle
after a few steps (the field with its pending guard, both halves of the
spectrum), and Parseval's identity against the energy at z0."""
import numpy as np
import pytest

from gpu_helpers import pair, rel_l2, rt_input, step_both, t_input, xyt_input

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-5, "fp64": 1e-10}
INPUTS = {"RT": rt_input, "T": t_input, "XYT": xyt_input}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("geom", ["RT", "T", "XYT"])
def test_spectrum_matches_oracle(gpu_lib, geom, precision):
    g, r = pair(INPUTS[geom](), precision)
    S0 = g.handle.spectrum()
    W = g.handle.analyze()["energy"]
    nt, dt = g.grid.Nt, float(g.grid.dt)
    assert np.sum(S0) / (nt * dt) == pytest.approx(W, rel=10 * TOL[precision])
    step_both(g, r, 3, 2e-3)
    Sg, Sr = g.handle.spectrum(), r.handle.spectrum()
    assert Sg.shape == (nt // 2 + 1,)
    assert rel_l2(Sg, Sr) < 10 * TOL[precision]
    # the analyzer's other outputs are still right after the spectrum call
    ag, ar = g.handle.analyze(), r.handle.analyze()
    assert rel_l2(ag["power"], ar["power"]) < 10 * TOL[precision]
