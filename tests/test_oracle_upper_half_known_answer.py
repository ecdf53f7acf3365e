"""Known answer of the oracle's linear T step on a field with
negative-frequency content, which the reference keeps in its full-length
spectrum (Models.jl:152-171, spectral.jl:16-26): every bin of the spectrum,
the upper half included, is multiplied by Wguard(w) exp(i KZ(w) dz) with KZ
taken at that bin's (negative) frequency, and the field guard follows.  The
GPU library carries the upper half the same way (checked against this
oracle by the upper-half tests of tests/test_gpu_parity.py)."""
import numpy as np

from gpu_helpers import t_input


def _complex(v):
    return np.ascontiguousarray(v, dtype=np.float64).view(np.complex128)


def test_linear_step_carries_the_upper_half(oracle_binding):
    import filament_gb as fg
    inp = t_input(Nt=1024, NONLINEARITY=False, PLASMA=False, tguard=0.0)
    sim = fg.Simulation(inp, binding=oracle_binding)
    a = sim.problem._arrays
    nt = sim.problem.config.nt
    k = np.arange(nt)
    rng = np.random.default_rng(2)
    S0 = (rng.standard_normal(nt) + 1j * rng.standard_normal(nt)) * np.exp(-((k - 150) / 40.0) ** 2)
    S0 += 0.1 * (rng.standard_normal(nt) + 1j * rng.standard_normal(nt)) * np.exp(-((k - (nt - 150)) / 40.0) ** 2)
    E0 = np.fft.fft(S0)
    sim.handle.set_field(E0, analytic=True)
    dz = 0.05
    sim.handle.step(dz, dz)
    E1 = sim.handle.get_field()
    D = np.asarray(a["wguard"]) * np.exp(1j * _complex(a["dfr"]) * dz)
    E = np.asarray(a["guardt"]) * np.fft.fft(D * np.fft.ifft(E0))
    assert np.linalg.norm(E - E1) <= 1e-13 * np.linalg.norm(E1)
    S1 = np.fft.ifft(E1)
    assert np.linalg.norm(S1[nt // 2:]) > 0.05 * np.linalg.norm(S1)     # the upper half is carried
    sim.close()
