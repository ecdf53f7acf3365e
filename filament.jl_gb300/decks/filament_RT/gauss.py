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
    R, T = np.meshgrid(r, t, indexing="ij")
    if chirp_fs2 != 0.0:
        # the transform-limited spectrum times exp(i phi2 (w - w0)^2 / 2):
        # complex envelope (t0 / tau) exp(-t^2 / (2 tau^2)), tau^2 = t0^2 - i phi2
        tau2 = t0 ** 2 - 1j * chirp_fs2 * 1e-30
        env = np.sqrt(t0 ** 2 / tau2) * np.exp(-0.5 * (T * tu) ** 2 / tau2)
        return (np.sqrt(I0 / Iu) * np.exp(-0.5 * (R * ru) ** 2 / a0 ** 2)
                * np.real(env * np.exp(1j * w0 * T * tu))) + 0j
    return (np.sqrt(I0 / Iu) * np.exp(-0.5 * (R * ru) ** 2 / a0 ** 2)
            * np.exp(-0.5 * (T * tu) ** 2 / t0 ** 2) * np.cos(w0 * T * tu)) + 0j
