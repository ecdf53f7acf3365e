# test/diffraction/XY/gauss.jl: a0 = 1 mm, I0 = 1e12 W/cm^2.
z = 0.0
lam0 = 800e-9
def initial_condition(x, y, xu, yu, Iu):
    a0 = 1e-3
    I0 = 1e12 * 1e4
    X, Y = np.meshgrid(x, y, indexing="ij")
    return np.sqrt(I0 / Iu) * np.exp(-0.5 * ((X * xu) ** 2 + (Y * yu) ** 2) / a0 ** 2) + 0j
