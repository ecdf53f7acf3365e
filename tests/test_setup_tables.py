"""Host set-up (the FP64 tables both the library and the oracle consume)
checked against known values."""
import math

import numpy as np
import pytest
from scipy import special


def test_air_k2_matches_reference_value():
    """test/test_dispersion_t.jl:16: k2 of air at 800 nm."""
    from filament_gb import media
    from filament_gb.constants import C0
    m = media.Medium(media.air_permittivity, media.unit_permeability, 1e-23)
    w0 = 2 * math.pi * C0 / 800e-9
    assert media.k2_func(m, w0) == pytest.approx(2.131584978375e-29, rel=1e-9)


def test_bessel_zeros_and_dht_orthogonality():
    from filament_gb.grids import bessel_j0_zeros, dht_matrix
    j = bessel_j0_zeros(65)
    assert j[0] == pytest.approx(2.404825557695773, rel=1e-14)
    assert np.all(np.abs(special.j0(j)) < 1e-12)
    T, J1 = dht_matrix(j)
    # the QDHT kernel is symmetric and nearly orthogonal (T^2 ~ I)
    assert np.allclose(T, T.T)
    assert np.max(np.abs(T @ T - np.eye(64))) < 5e-3


def test_hankel_transform_of_gaussian():
    """diag(J/V) T diag(R/J) applied to exp(-a r^2) vs the analytic order-0
    transform pi/a exp(-pi^2 v^2/a)."""
    from filament_gb.grids import bessel_j0_zeros, dht_matrix
    N, R = 256, 5.0
    j = bessel_j0_zeros(N + 1)
    T, J1 = dht_matrix(j)
    S = j[N]
    V = S / (2 * math.pi * R)
    r = j[:N] * R / S
    v = j[:N] / (2 * math.pi * R)
    a = 1.0
    f = np.exp(-a * r ** 2)
    F = (J1 / V) * (T @ (f * R / J1))
    Fth = math.pi / a * np.exp(-(math.pi * v) ** 2 / a)
    assert np.max(np.abs(F - Fth)) < 1e-10


def test_guard_windows():
    from filament_gb import guards
    x = np.linspace(0, 10, 1001)
    g = guards.guard_window_right(x, 2.0)
    assert g[0] == pytest.approx(1.0) and g[-1] == pytest.approx(0.0, abs=1e-12)
    assert np.all(np.diff(g) <= 1e-15)
    gb = guards.guard_window_both(np.linspace(-5, 5, 1001), 1.0)
    assert gb[0] == pytest.approx(0.0, abs=1e-12) and gb[500] == pytest.approx(1.0)
    with pytest.raises(ValueError):
        guards.guard_window_both(x, 6.0)


def test_tabulated_rate_power_law_and_tfpower():
    from filament_gb.plasma import TFunction, power_law_rate
    I, W = power_law_rate(8.0, 1e18, 8.85e12)
    tf = TFunction(I, W, 1e-16, 1e-15)   # Iu = 1e16, tu = 1e-15
    assert tf(100.0) == pytest.approx(8.85e12 * 1e-15, rel=1e-12)
    assert tf.power(3.0) == pytest.approx(8.0, rel=1e-12)
    assert tf(0.0) == 0.0


def test_units_field_unit():
    from filament_gb import units
    from filament_gb.constants import C0, EPS0
    u = units.Unit("RT", (1e-3, 1.0, 1e-15, 1e16, 2.5e25))
    assert u.k == pytest.approx(1e3) and u.w == pytest.approx(1e15)
    assert units.E(u, 1.0) == pytest.approx(math.sqrt(1e16 / (EPS0 * C0 / 2)))


def test_problem_tables_rt_small():
    import filament_gb as fg
    import os
    from conftest import PKG_DECKS
    inp = fg.prepare(os.path.join(PKG_DECKS, "filament_RT", "input.py"), Nr=32, Nt=512)
    from filament_gb.filament import Field
    from filament_gb import units, grids, media, guards
    from filament_gb.problem import Problem
    g = inp["geometry"]
    u = units.Unit(g, inp["p_unit"])
    gr = grids.Grid(g, inp["p_grid"])
    f = Field(g, u, gr, inp["p_field"])
    m = media.Medium(*inp["p_medium"])
    gd = guards.Guard_build(g, u, gr, f.w0, m, inp["p_guard"])
    resp, pdict, keys = inp["p_model"]
    rs = [it["init"](u, gr, f, m, it) for it in resp]
    p = Problem(g, u, gr, f.w0, m, gd, rs, None, dict(keys, PLASMA=False), inp["p_dzadaptive"])
    c = p.config
    assert (c.n1, c.n2, c.nt) == (32, 1, 512)
    assert c.resp_mask == 7 and c.cubic_thg == 1
    # moving frame: KZ(k=0, w0) small compared with beta(w0)
    beta = p._arrays["beta"].view(np.complex128)
    dfr = p._arrays["dfr"].view(np.complex128)
    j0 = int(np.argmin(np.abs(gr.w * u.w - f.w0)))
    assert abs(dfr[j0]) < 1e-3 * abs(beta[j0])
