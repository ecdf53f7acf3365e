# Air for the linear known-answer decks (test/diffraction/*/air.jl,
# test/dispersion/*/air.jl): Peck-Reeder dispersion, n2 = 1e-23 m^2/W,
# cubic response without third-harmonic generation.
permittivity = air_permittivity
permeability = unit_permeability
n2 = 1e-23
cubic = {"init": init_cubic, "THG": False, "n2": n2}
responses = [cubic]
