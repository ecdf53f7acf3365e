"""CODATA 2018 constants, as used by the reference (src/modules/Constants.jl:1-16).

PhysicalConstants.jl's CODATA2018 values are restated here numerically.  The
reduced Planck constant is h/(2 pi) with the exact SI value of h.
"""
import math

C0 = 299792458.0                  # speed of light in vacuum [m/s]
EPS0 = 8.8541878128e-12           # vacuum electric permittivity [F/m]
MU0 = 1.25663706212e-6            # vacuum magnetic permeability [N/A^2]
QE = 1.602176634e-19              # elementary charge [C]
ME = 9.1093837015e-31             # electron mass [kg]
HBAR = 6.62607015e-34 / (2.0 * math.pi)  # reduced Planck constant [J s]
