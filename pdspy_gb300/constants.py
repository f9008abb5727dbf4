"""Physical and astronomical constants with pdspy's values.

The values must equal pdspy's (pdspy/constants/physics.py:1-15,
pdspy/constants/astronomy.py:1-9, pdspy/constants/math.py) so that grids, stellar
radii and disk normalisations built here agree with pdspy's to the last bit.
"""
# physics
c = 2.99792458e10           # cm s^-1
h = 6.6260755e-27           # erg s
k = 1.380658e-16            # erg K^-1
G = 6.67259e-8              # cm^3 g^-1 s^-2
m_p = 1.6726231e-24         # g
sigma = 5.67051e-5          # erg cm^-2 K^-4 s^-1

# astronomy
AU = 1.495978707e13         # cm
pc = 3.085677581e18         # cm
M_sun = 1.99e33             # g
R_sun = 6.96e10             # cm
L_sun = 3.9e33              # erg s^-1
Jy = 1.0e-23                # erg s^-1 cm^-2 Hz^-1
arcsec = 4.84813681e-6      # radians

# pdspy's own value of pi (pdspy/constants/math.py), used in its disk normalisation
pi_pdspy = 3.14159265
