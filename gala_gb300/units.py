"""Fixed galactic unit system (kpc, Myr, Msun, radian), as plain floats.

gala's ``galactic`` unit system (src/gala/units.py) is kpc, Myr, Msun, radian
with velocities reported in km/s.  Without astropy the library works in these
units throughout; inputs and outputs are floats in them.
"""

# Gravitational constant in kpc^3 / (Msun Myr^2): CODATA-2018 G with the IAU
# nominal solar mass parameter and Julian-year Myr, as astropy decomposes it.
G = 4.498502151469553e-12

# 1 km/s in kpc/Myr
KMS_TO_KPC_MYR = 1.022712165045695e-3


class UnitSystem:
    """Minimal stand-in for gala's UnitSystem: names only, values are floats."""

    def __init__(self, length="kpc", time="Myr", mass="Msun", angle="radian"):
        self.length, self.time, self.mass, self.angle = length, time, mass, angle

    def __getitem__(self, key):
        return {"length": self.length, "time": self.time, "mass": self.mass, "angle": self.angle}[key]

    def __repr__(self):
        return f"UnitSystem({self.length}, {self.time}, {self.mass}, {self.angle})"


galactic = UnitSystem()
