# Multifilamentation of a femtosecond pulse in air, XYT geometry.
# Default values: 512 x 512 over +-5 mm, Nt = 512 over +-200 fs, order-4
# super-Gaussian beam (w0 = 3 mm) x 50 fs pulse at 20 Pcr with 5 % seeded
# amplitude noise, RK3, adaptive dz (max nonlinear phase 0.1 rad) over 2 m.
# Layout and keys follow the reference's XYT decks (examples/XYT/input.jl).
prefix = "results/"
file_initial_condition = "supergauss.py"
file_medium = "../filament_RT/air.py"
xu = 1e-3; yu = 1e-3; zu = 1.0; tu = 1e-15; Iu = 1e12 * 1e4; rhou = 2.5e25
geometry = "XYT"
xmin, xmax = -5.0, 5.0; Nx = 512
ymin, ymax = -5.0, 5.0; Ny = 512
tmin, tmax = -200.0, 200.0; Nt = 512
zmax = 2.0; dz_initial = 1e-2
NONLINEARITY = True; PLASMA = True
KPARAXIAL = False; QPARAXIAL = True
xguard = 1.0; yguard = 1.0; tguard = 20.0; kxguard = 45.0; kyguard = 45.0; wguard = 1e16
dzphimax = 0.1
Istop = 1e3
ALG = RK3
PPcr = 20.0         # peak power in units of the critical power
noise = 0.05        # uniform amplitude noise, +-5 %
seed = 1234         # numpy PCG64 seed of the noise
