# Femtosecond pulse in air on one time row (T geometry): Kerr, plasma,
# Drude current and multiphoton losses (the layout of the reference's
# T decks, test/dispersion/T/input.jl).
prefix = "results/"
file_initial_condition = "pulse.py"
file_medium = "air.py"
zu = 1.0; tu = 1e-15; Iu = 1e12 * 1e4; rhou = 2.5e25
geometry = "T"
tmin, tmax = -100.0, 100.0; Nt = 1024
zmax = 0.02; dz_initial = 1e-3
NONLINEARITY = True; PLASMA = True
tguard = 10.0; wguard = 1e16
dzphimax = pi / 100.0; Istop = 1e3
ALG = RK4
