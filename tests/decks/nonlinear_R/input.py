# Gaussian beam with Kerr self-focusing, R geometry (the layout of the
# reference's R decks, test/diffraction/R/input.jl).
prefix = "results/"
file_initial_condition = "beam.py"
file_medium = "../air_linear.py"
ru = 1e-3; zu = 1.0; Iu = 1e12 * 1e4
geometry = "R"
rmax = 4.0; Nr = 256
zmax = 0.02; dz_initial = 1e-3
NONLINEARITY = True
KPARAXIAL = False; QPARAXIAL = True
rguard = 0.5; kguard = 45.0
dzphimax = pi / 100.0; Istop = 1e3
ALG = RK4
