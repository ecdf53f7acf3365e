# test/diffraction/RT/gauss.jl: a0 = 1 mm, t0 = 100 fs, I0 = 1e12 W/cm^2.
z = 0.0
lam0 = 800e-9
def initial_condition(r, t, ru, tu, Iu):
    a0 = 1e-3
    t0 = 100e-15
    I0 = 1e12 * 1e4
    w0 = 2 * pi * C0 / lam0
    R, T = np.meshgrid(r, t, indexing="ij")
    return (np.sqrt(I0 / Iu) * np.exp(-0.5 * (R * ru) ** 2 / a0 ** 2)
            * np.exp(-0.5 * (T * tu) ** 2 / t0 ** 2) * np.cos(w0 * T * tu)) + 0j
