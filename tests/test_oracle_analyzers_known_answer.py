"""Known answers of the oracle's analyzer reductions (FieldAnalyzers.jl:
166-215) on the RT deck's initial field, a Gaussian beam times a Gaussian
pulse on an 800 nm carrier: the analytic signal's |E|^2 is
I0/Iu exp(-r^2/a0^2) exp(-t^2/t0^2) (to e^-(w0 t0)^2), so
  fluence  F(r) = sum_t |E|^2 dt            (FieldAnalyzers.jl:171)
  power    P(t) = 2 pi sum_r |E|^2 r dr     (FieldAnalyzers.jl:174-175)
  energy   W    = 2 pi sum_r F(r) r dr      (FieldAnalyzers.jl:213)
  Imax     = max |E|^2                      (FieldAnalyzers.jl:201)
equal the same sums of the Gaussian on the grid to rounding, and W in
joules is the pulse's peak power P0 = PPcr Pcr times sqrt(pi) t0 to the
quadrature's accuracy."""
import math

import numpy as np
import pytest
import scipy.constants as sc

from gpu_helpers import rt_input

PPCR, A0 = 3.0, 1e-3


def test_initial_field_analyzers(oracle_binding):
    import filament_gb as fg
    inp = rt_input(Nr=256, rmax=5.0, Nt=1024, tmin=-200.0, tmax=200.0, PPcr=PPCR, beam_a0=A0)
    sim = fg.Simulation(inp, binding=oracle_binding)
    an = sim.handle.analyze()
    g = sim.problem.grid
    rdr = np.asarray(sim.problem._arrays["rdr"])
    ru, zu, tu, Iu, rhou = inp["p_unit"]
    perm, _, n2 = inp["p_medium"]
    lam0 = inp["lam0"]
    w0 = 2 * np.pi * sc.c / lam0
    n0 = math.sqrt(complex(perm(w0)).real)
    P0 = PPCR * 3.79 * lam0 ** 2 / (8 * np.pi * n0 * n2)        # Media.critical_power
    I0 = P0 / (np.pi * A0 ** 2)
    t0 = 35e-15 / (2 * math.sqrt(math.log(2)))
    env_r = np.exp(-(g.r * ru) ** 2 / A0 ** 2)
    env_t = np.exp(-(g.t * tu) ** 2 / t0 ** 2)

    F = I0 / Iu * env_r * np.sum(env_t) * g.dt
    P = I0 / Iu * env_t * 2 * np.pi * np.sum(env_r * rdr)
    assert np.max(np.abs(an["fluence"] - F)) <= 1e-12 * np.max(F)
    assert np.max(np.abs(an["power"] - P)) <= 1e-12 * np.max(P)
    assert an["energy"] == pytest.approx(2 * np.pi * np.sum(F * rdr), rel=1e-12)
    assert an["imax"] == pytest.approx(I0 / Iu * env_r.max() * env_t.max(), rel=1e-12)
    # the energy in joules against the pulse's peak power and duration
    assert an["energy"] * Iu * tu * ru ** 2 == pytest.approx(P0 * math.sqrt(math.pi) * t0, rel=1e-5)
    sim.close()
