# 35 fs FWHM pulse at 800 nm, peak intensity 5e17 W/m^2.
z = 0.0
lam0 = 800e-9
def initial_condition(t, tu, Iu):
    t0 = 35e-15 / (2 * math.sqrt(math.log(2)))
    I0 = 5e17
    w0 = 2 * pi * C0 / lam0
    return np.sqrt(I0 / Iu) * np.exp(-0.5 * (t * tu) ** 2 / t0 ** 2) * np.cos(w0 * t * tu) + 0j
