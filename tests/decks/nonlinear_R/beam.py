# Gaussian beam a0 = 1 mm, I0 = 1e17 W/m^2 at 800 nm.
z = 0.0
lam0 = 800e-9
def initial_condition(r, ru, Iu):
    a0 = 1e-3
    I0 = 1e17
    return np.sqrt(I0 / Iu) * np.exp(-0.5 * (r * ru) ** 2 / a0 ** 2) + 0j
