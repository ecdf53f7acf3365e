# test/dispersion/T/gauss.jl: t0 = 20 fs, I0 = 1e12 W/cm^2.
z = 0.0
lam0 = 800e-9
def initial_condition(t, tu, Iu):
    t0 = 20e-15
    I0 = 1e12 * 1e4
    w0 = 2 * pi * C0 / lam0
    return np.sqrt(I0 / Iu) * np.exp(-0.5 * (t * tu) ** 2 / t0 ** 2) * np.cos(w0 * t * tu) + 0j
