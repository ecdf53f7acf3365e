# Air: Peck-Reeder two-term dispersion, n2 = 1e-23 m^2/W, one ionising
# species with a multiphoton rate W = sigma_8 I^8 (Ui = 12.06 eV, neutral
# density 5.4e24 m^-3), Drude plasma (nuc = 5e12 1/s, mr = 1).  sigma_8 is
# fixed by W(1e18 W/m^2) = 8.85e12 1/s, the O2 rate of the reference's
# examples/RT/multiphoton_O2.tf at that intensity.  Responses: cubic with
# third-harmonic generation, free current, multiphoton losses (no Raman).
permittivity = air_permittivity
permeability = unit_permeability
n2 = 1e-23
nuc = 5e12
mr = 1.0
cubic = {"init": init_cubic, "THG": True, "n2": n2}
current_free = {"init": init_current_free, "nuc": nuc, "mr": mr}
current_losses = {"init": init_current_losses, "EREAL": False}
responses = [cubic, current_free, current_losses]
single = {"fraction": 1.0, "ionization_energy": 12.06,
          "ionization_rate": power_law_rate(8.0, 1e18, 8.85e12)}
plasma_equation = {
    "init": init_photoionization_avalanche,
    "ALG": RK3, "EREAL": False, "KDEP": True,
    "rho0": 0.0, "rho_nt": 5.4e24, "nuc": nuc, "mr": mr,
    "components": [single],
}
