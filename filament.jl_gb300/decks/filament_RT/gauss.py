# Gaussian beam (1/e intensity radius a0 = beam_a0, 1 mm by default) x
# Gaussian pulse of 35 fs
# FWHM at 800 nm with peak power PPcr * Pcr, the conventions of the
# reference's examples/RT/gauss.jl (field ~ exp(-r^2/(2 a0^2)) exp(-t^2/(2 t0^2))
# cos(w0 t), t0 = FWHM / (2 sqrt(ln 2))).
z = 0.0
lam0 = 0.8e-6

def initial_condition(r, t, ru, tu, Iu):
    a0 = beam_a0
    t0 = 35e-15 / (2 * math.sqrt(math.log(2)))
    w0 = 2 * pi * C0 / lam0
    n0 = math.sqrt(permittivity(w0))
    Pcr = 3.79 * lam0 ** 2 / (8 * pi * n0 * n2)      # Media.critical_power
    I0 = PPcr * Pcr / (pi * a0 ** 2)
    # separable: beam factor of r times pulse factor of t, each evaluated on
    # its axis (element by element the same products as on the full grid)
    r = np.asarray(r, dtype=float)
    t = np.asarray(t, dtype=float)
    beam = np.sqrt(I0 / Iu) * np.exp(-0.5 * (r * ru) ** 2 / a0 ** 2)
    if chirp_fs2 != 0.0:
        # the transform-limited spectrum times exp(i phi2 (w - w0)^2 / 2):
        # complex envelope (t0 / tau) exp(-t^2 / (2 tau^2)), tau^2 = t0^2 - i phi2
        tau2 = t0 ** 2 - 1j * chirp_fs2 * 1e-30
        env = np.sqrt(t0 ** 2 / tau2) * np.exp(-0.5 * (t * tu) ** 2 / tau2)
        return (beam[:, None] * np.real(env * np.exp(1j * w0 * t * tu))[None, :]) + 0j
    return (beam[:, None] * np.exp(-0.5 * (t * tu) ** 2 / t0 ** 2)[None, :]
            * np.cos(w0 * t * tu)[None, :]) + 0j
