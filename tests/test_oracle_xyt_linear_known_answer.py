"""Known answer of the oracle's XYT linear step (spectral.jl:16-26 with the
XYT propagator of spectral.jl:130-158, Kfunc of spectral.jl:160-184; the
guards of Guards.jl:162-193): the step is diagonal in (kx, ky, w),
  E1 = G(x) G(y) G(t) F^-1[ exp(i KZ dz) Wguard(w) KXguard KYguard F[E0] ],
  KZ = sqrt(beta(w)^2 - kx^2 - ky^2) - w / vf        (KPARAXIAL = false)
     = beta - (kx^2 + ky^2) / (2 beta) - w / vf      (KPARAXIAL = true),
with t -> w by the inverse FFT (Models.jl:152-171) and the transverse
transform by the 2-D FFT.  The reference's diffraction and dispersion tests
cover XY and T separately; this checks their space-time coupling in XYT."""
import numpy as np
import pytest

from gpu_helpers import XYT_DECK


def _complex(v):
    return np.ascontiguousarray(v, dtype=np.float64).view(np.complex128)


@pytest.mark.parametrize("kparaxial", [False, True])
def test_xyt_linear_step(oracle_binding, kparaxial):
    import filament_gb as fg
    inp = fg.prepare(XYT_DECK, Nx=32, Ny=32, Nt=256, zmax=0.02, NONLINEARITY=False, KPARAXIAL=kparaxial)
    assert inp["p_model"][2]["KPARAXIAL"] == kparaxial
    sim = fg.Simulation(inp, binding=oracle_binding)
    a = sim.problem._arrays
    E0 = sim.handle.get_field()
    dz = 2e-3
    sim.handle.step(dz, dz)
    E1 = sim.handle.get_field()

    beta, dfr = _complex(a["beta"]), _complex(a["dfr"])
    kx, ky = np.asarray(a["kt1"]), np.asarray(a["kt2"])
    kt2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2
    b = beta[None, None, :]
    if kparaxial:
        with np.errstate(divide="ignore", invalid="ignore"):
            kz = np.where(b != 0, b - kt2 / (2 * b), 0)
    else:
        kz = np.sqrt(b ** 2 - kt2 + 0j)
    kz = kz - (beta - dfr)[None, None, :]
    D = (np.exp(1j * kz * dz) * np.asarray(a["wguard"])[None, None, :]
         * np.asarray(a["sguard1"])[:, None, None] * np.asarray(a["sguard2"])[None, :, None])
    G = (np.asarray(a["guard1"])[:, None, None] * np.asarray(a["guard2"])[None, :, None]
         * np.asarray(a["guardt"])[None, None, :])
    S = np.fft.fft2(np.fft.ifft(E0, axis=2), axes=(0, 1))
    E = G * np.fft.fft(np.fft.ifft2(D * S, axes=(0, 1)), axis=2)
    assert np.linalg.norm(E - E1) <= 1e-13 * np.linalg.norm(E1)
    assert np.linalg.norm(G * E0 - E1) > 1e-2 * np.linalg.norm(E1)      # the step does something
    sim.close()
