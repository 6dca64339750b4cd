"""Physical constants (CODATA 2022, the values scipy.constants carries and the
reference uses through it).  libsbe_gb300 compiles in the same numbers; the
``sbe_constants`` entry point returns them for a consistency check."""

HBAR = 1.0545718176461565e-34   # J s
E0 = 1.602176634e-19            # C
EPS0 = 8.8541878188e-12         # F/m
ME0 = 9.1093837139e-31          # kg
KB = 1.380649e-23               # J/K
C0 = 299792458.0                # m/s
PI = 3.141592653589793
TWOPI = 2.0 * PI
