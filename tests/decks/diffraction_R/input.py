# Gaussian-beam diffraction, R geometry (test/diffraction/R/input.jl).
prefix = "results/"
file_initial_condition = "gauss.py"
file_medium = "../air_linear.py"
ru = 1e-3; zu = 1.0; Iu = 1e12 * 1e4
geometry = "R"
rmax = 10.0; Nr = 2000
zmax = 10.0; dz_initial = zmax / 100.0
NONLINEARITY = False
KPARAXIAL = False; QPARAXIAL = True
rguard = 0.0; kguard = 90.0
dzphimax = pi / 100.0; Istop = 1e3
ALG = RK4
