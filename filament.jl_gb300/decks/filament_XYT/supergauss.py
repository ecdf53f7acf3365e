# Super-Gaussian beam of order 4 (w0 = 3 mm) x Gaussian pulse of 50 fs FWHM at
# 800 nm with peak power PPcr * Pcr, multiplied by (1 + noise * U(-1, 1)) with
# a fixed numpy PCG64 seed; conventions of the reference's examples/XYT decks
# (field ~ exp(-(r^2/w0^2)^m / 2) exp(-t^2/(2 t0^2)) cos(w0 t)).
z = 0.0
lam0 = 0.8e-6

def initial_condition(x, y, t, xu, yu, tu, Iu):
    w0 = 3e-3
    m = 4
    t0 = 50e-15 / (2 * math.sqrt(math.log(2)))
    om0 = 2 * pi * C0 / lam0
    n0 = math.sqrt(permittivity(om0))
    Pcr = 3.79 * lam0 ** 2 / (8 * pi * n0 * n2)      # Media.critical_power
    # peak intensity of a super-Gaussian of power P: P / (pi w0^2 Gamma(1 + 1/m))
    I0 = PPcr * Pcr / (pi * w0 ** 2 * math.gamma(1 + 1 / m))
    X, Y = np.meshgrid(x * xu, y * yu, indexing="ij")
    r2 = (X ** 2 + Y ** 2) / w0 ** 2
    A = np.sqrt(I0 / Iu) * np.exp(-0.5 * r2 ** m)
    rng = np.random.Generator(np.random.PCG64(seed))
    A = A * (1 + noise * rng.uniform(-1, 1, size=A.shape))
    T = t * tu
    P = np.exp(-0.5 * T ** 2 / t0 ** 2) * np.cos(om0 * T)
    return (A[:, :, None] * P[None, None, :]) + 0j
