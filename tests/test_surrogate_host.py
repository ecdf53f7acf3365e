"""Host side of the learned plasma surrogate (no GPU): the CPU reference of
the network checked by finite differences, and the training targets, which
must reproduce the plasma solve exactly through the closed form the row
kernel uses."""
import numpy as np
import pytest


def test_reference_gradient_matches_finite_differences(monkeypatch):
    """The CPU reference's backward pass, with the BF16 rounding switched
    off so that the loss is smooth, against central differences."""
    import surrogate_ref as sr
    monkeypatch.setattr(sr, "bf16", lambda x: np.asarray(x, dtype=np.float64))
    rng = np.random.default_rng(3)
    p = rng.uniform(-0.3, 0.3, sr.nparams())
    f = rng.standard_normal((2, 3, 40))
    t = rng.standard_normal((2, 40))
    m = (rng.random((2, 40)) > 0.3).astype(float)
    _, g = sr.grad(p, f, t, m)
    offs = np.cumsum([0] + [co * ci * sr.K + co for ci, co in zip(sr.CI, sr.CO)])
    # a weight and a bias of every layer
    idx = [int(offs[l]) + 7 for l in range(4)] + [int(offs[l + 1]) - 1 for l in range(4)]
    for i in idx:
        eps = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[i] += eps
        pm[i] -= eps
        fd = (sr.grad(pp, f, t, m)[0] - sr.grad(pm, f, t, m)[0]) / (2 * eps)
        assert g[i] == pytest.approx(fd, rel=1e-6, abs=1e-9)


def test_reference_bf16_rounding():
    import surrogate_ref as sr
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 2 ** -9, -2.5e-3], dtype=np.float32)
    r = sr.bf16(x)
    # ties to even: 1 + 2^-8 is a tie between 1 and 1 + 2^-7 -> 1
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == 1.0
    assert abs(r[4] - (-2.5e-3)) <= 2.5e-3 * 2 ** -8


class _PE:
    """Plasma equation stand-in: one species, power law W = (I/1.5)^8,
    avalanche coefficient 0.05, RK3 in time."""

    def __init__(self):
        from filament_gb.plasma import TFunction
        I = np.logspace(-6, 2, 9)
        self.tfs = [TFunction(I, (I / 1.5) ** 8)]
        self.rho_nt = np.array([2.0])
        self.rava = np.array([0.05])
        self.rho0 = 0.0
        self.EREAL = False
        self.alg = "RK3"


def _rows(nt, dt):
    t = (np.arange(nt) - nt / 2) * dt
    return np.array([np.sqrt(a * np.exp(-(t / 2.0) ** 2)) * np.exp(1j * 3.0 * t) for a in (0.6, 0.8, 1.0)]), t


def test_training_targets_reconstruct_the_density():
    """A sequential solve whose avalanche term is amplified by a known factor
    c(t) > 0 gives targets g = ln c; the closed form of the row kernel with
    those g gives the density back, and without them (g = 0) it does not."""
    from filament_gb import surrogate as S
    pe = _PE()
    nt, dt = 256, 0.05
    E, t = _rows(nt, dt)
    wb = S.quad_rate(pe, E) * dt
    av = S.quad_ava(pe, E) * dt
    c = 1.0 + 0.8 * np.exp(-((t[:-1] - 1.0) / 1.5) ** 2)
    rho = np.zeros(E.shape)
    Sb = np.zeros(3)
    for j in range(nt - 1):
        w = wb[:, j] + av[:, j] * -np.expm1(-Sb) * c[j]
        rho[:, j + 1] = rho[:, j] + (2.0 - rho[:, j]) * -np.expm1(-w)
        Sb += wb[:, j]
    f, g, m = S.training_pairs(E, rho, pe, dt, floor=1.0)
    assert f.shape == (3, 3, nt) and g.shape == (3, nt)
    assert np.allclose(f[:, 1], (E.real ** 2 / np.maximum(np.abs(E) ** 2, 1e-30)), atol=1e-6)
    # f2: log of the base rate's exponent, log(1e-30) / 16 before the first step
    Sb = np.cumsum(S.quad_rate(pe, E) * dt, axis=1)
    assert np.allclose(f[:, 2, 1:], np.log(np.maximum(Sb, 1e-30)) / 16, atol=1e-6)
    assert np.allclose(f[:, 2, 0], np.log(1e-30) / 16)
    ok = m[:, :-1] > 0
    assert np.mean(ok) > 0.3
    assert np.allclose(g[:, :-1][ok], np.broadcast_to(np.log(c), ok.shape)[ok], atol=1e-4)
    rec = S.closed_form_density(E, g, pe, dt)
    assert np.max(np.abs(rec - rho)) <= 1e-6 * np.max(rho)
    rec0 = S.closed_form_density(E, np.zeros_like(g), pe, dt)
    assert np.max(np.abs(rec0 - rho)) > 1e-3 * np.max(rho)


def test_training_rows_below_the_threshold_are_dropped():
    from filament_gb import surrogate as S
    pe = _PE()
    nt = 64
    E = np.ones((2, nt), complex)
    rho = np.zeros((2, nt))
    rho[0] = np.linspace(0, 1e-3, nt)
    rho[1] = np.linspace(0, 1e-15, nt)
    f, d, m = S.training_pairs(E, rho, pe, 0.1)
    assert f.shape[0] == 1


def test_skipped_tiles_cannot_change_the_density():
    """The tile rule of the row reduction (surrogate.tile_flags): with g = 0
    on the tiles without bit 0 the closed-form density stays within 2^-24
    of its scale of the density with any g in range there, on rows where
    most tiles are skipped (ahead of the pulse S = 0, behind it A ~ 0)."""
    from filament_gb import surrogate as S
    pe = _PE()
    nt, dt = 2048, 0.05
    t = (np.arange(nt) - nt / 4) * dt
    E = np.array([np.sqrt(a * np.exp(-(t / 3.0) ** 2)) * np.exp(1j * 3.0 * t) for a in (0.5, 1.0, 2.0)])
    fl = S.tile_flags(E, pe, dt)
    assert fl.shape == (3, nt // 128)
    use, run = (fl & 1) > 0, (fl & 2) > 0
    assert np.all(run[use])                     # the tiles using g are run
    assert 0 < np.mean(run) < 0.5               # and most are skipped
    # every tile using g has both neighbours run (receptive field)
    assert np.all(run[:, 1:][use[:, :-1]]) and np.all(run[:, :-1][use[:, 1:]])
    rng = np.random.default_rng(5)
    mask = np.repeat(use, 128, axis=1)
    scale = np.max(S.closed_form_density(E, np.zeros((3, nt)), pe, dt))
    for g in (np.full((3, nt), S.G_RANGE[1]), np.full((3, nt), S.G_RANGE[0]),
              rng.uniform(*S.G_RANGE, size=(3, nt))):
        full = S.closed_form_density(E, g, pe, dt)
        masked = S.closed_form_density(E, np.where(mask, g, 0.0), pe, dt)
        assert np.max(np.abs(full - masked)) <= 2.0 ** -24 * scale
    # the rule is not vacuous: g on the tiles with bit 0 does change it
    g = np.full((3, nt), S.G_RANGE[1])
    assert np.max(np.abs(S.closed_form_density(E, g, pe, dt)
                         - S.closed_form_density(E, np.zeros((3, nt)), pe, dt))) > 1e-3 * scale
