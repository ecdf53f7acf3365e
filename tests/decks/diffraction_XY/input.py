# Gaussian-beam diffraction, XY geometry (test/diffraction/XY/input.jl).
prefix = "results/"
file_initial_condition = "gauss.py"
file_medium = "../air_linear.py"
xu = 1e-3; yu = 1e-3; zu = 1.0; Iu = 1e12 * 1e4
geometry = "XY"
xmin, xmax = -10.0, 10.0; Nx = 2048
ymin, ymax = -10.0, 10.0; Ny = 2048
zmax = 10.0; dz_initial = zmax / 100.0
NONLINEARITY = False
KPARAXIAL = False; QPARAXIAL = True
xguard = 0.0; yguard = 0.0; kxguard = 90.0; kyguard = 90.0
dzphimax = pi / 100.0; Istop = 1e3
ALG = RK4
