# Diffraction of a Gaussian pulse, RT geometry (test/diffraction/RT/input.jl).
prefix = "results/"
file_initial_condition = "gauss.py"
file_medium = "../air_linear.py"
ru = 1e-3; zu = 1.0; tu = 1e-15; Iu = 1e12 * 1e4; rhou = 2.5e25
geometry = "RT"
rmax = 10.0; Nr = 500
tmin, tmax = -400.0, 400.0; Nt = 4096
zmax = 10.0; dz_initial = zmax / 100.0
NONLINEARITY = False; PLASMA = False
KPARAXIAL = False; QPARAXIAL = True
rguard = 1.0; tguard = 20.0; kguard = 45.0; wguard = 1e16
dzphimax = pi / 100.0; Istop = 1e3
ALG = RK3
