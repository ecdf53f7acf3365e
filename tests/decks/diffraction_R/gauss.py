# test/diffraction/R/gauss.jl: a0 = 1 mm, I0 = 1e12 W/cm^2.
z = 0.0
lam0 = 800e-9
def initial_condition(r, ru, Iu):
    a0 = 1e-3
    I0 = 1e12 * 1e4
    return np.sqrt(I0 / Iu) * np.exp(-0.5 * (r * ru) ** 2 / a0 ** 2) + 0j
