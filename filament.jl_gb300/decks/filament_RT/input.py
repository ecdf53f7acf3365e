# Filamentation of a femtosecond pulse in air, RT geometry.
# Default values: Nr = 256 Hankel grid to R = 5 mm, Nt = 1024 over +-200 fs,
# 3 Pcr, RK2, fixed dz = 1 mm over 1 m (dzphimax = inf).  The 1000 x 4096
# workload overrides Nr, Nt, PPcr = 5, ALG = RK4, dzphimax = 0.1, zmax = 3.
# Layout and keys follow the reference's RT deck (examples/RT/input.jl).
prefix = "results/"
file_initial_condition = "gauss.py"
file_medium = "air.py"
ru = 1e-3; zu = 1.0; tu = 1e-15; Iu = 1e12 * 1e4; rhou = 2.5e25
geometry = "RT"
rmax = 5.0; Nr = 256
tmin, tmax = -200.0, 200.0; Nt = 1024
zmax = 1.0; dz_initial = 1e-3
NONLINEARITY = True; PLASMA = True
KPARAXIAL = False; QPARAXIAL = True
rguard = 1.0; tguard = 20.0; kguard = 45.0; wguard = 1e16
dzphimax = math.inf
Istop = 1e3
ALG = RK2
PPcr = 3.0          # peak power in units of the critical power
beam_a0 = 1e-3      # 1/e intensity radius of the beam (m)
chirp_fs2 = 0.0     # spectral phase phi2 (w - w0)^2 / 2 of the pulse (fs^2)
