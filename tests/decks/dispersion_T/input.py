# Gaussian-pulse dispersion, T geometry (test/dispersion/T/input.jl).
prefix = "results/"
file_initial_condition = "gauss.py"
file_medium = "../air_linear.py"
zu = 1.0; tu = 1e-15; Iu = 1e12 * 1e4; rhou = 2.5e25
geometry = "T"
tmin, tmax = -100.0, 100.0; Nt = 2048
zmax = 20.0; dz_initial = zmax / 100.0
NONLINEARITY = False; PLASMA = False
tguard = 10.0; wguard = 1e16
dzphimax = pi / 100.0; Istop = 1e3
ALG = RK3
