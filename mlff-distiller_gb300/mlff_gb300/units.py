"""Physical units and atomic masses for the MD driver.

Units follow the convention the reference's MD path runs in (ASE's:
Angstrom, eV, atomic mass unit; time in Angstrom * sqrt(amu / eV)).  The
constants are CODATA 2018 values; the masses are IUPAC standard atomic
weights (conventional / abridged values, mass number of the most stable
isotope for elements without a standard weight).
"""
import math

import numpy as np

_AMU_KG = 1.66053906660e-27
_EV_J = 1.602176634e-19
_ANGSTROM_M = 1e-10

#: one internal time unit in seconds: Angstrom * sqrt(amu / eV)
TIME_UNIT_S = _ANGSTROM_M * math.sqrt(_AMU_KG / _EV_J)
#: femtosecond in internal time units (nve_harness.py:106 uses timestep * units.fs)
fs = 1e-15 / TIME_UNIT_S
#: Boltzmann constant, eV / K
kB = 8.617333262e-5

# index = atomic number; entry 0 is the dummy element
ATOMIC_MASSES = np.array([
    1.0,
    1.008, 4.002602, 6.94, 9.0121831, 10.81, 12.011, 14.007, 15.999, 18.998403163, 20.1797,
    22.98976928, 24.305, 26.9815385, 28.085, 30.973761998, 32.06, 35.45, 39.948, 39.0983, 40.078,
    44.955908, 47.867, 50.9415, 51.9961, 54.938044, 55.845, 58.933194, 58.6934, 63.546, 65.38,
    69.723, 72.630, 74.921595, 78.971, 79.904, 83.798, 85.4678, 87.62, 88.90584, 91.224,
    92.90637, 95.95, 97.0, 101.07, 102.90550, 106.42, 107.8682, 112.414, 114.818, 118.710,
    121.760, 127.60, 126.90447, 131.293, 132.90545196, 137.327, 138.90547, 140.116, 140.90766, 144.242,
    145.0, 150.36, 151.964, 157.25, 158.92535, 162.500, 164.93033, 167.259, 168.93422, 173.054,
    174.9668, 178.49, 180.94788, 183.84, 186.207, 190.23, 192.217, 195.084, 196.966569, 200.592,
    204.38, 207.2, 208.98040, 209.0, 210.0, 222.0, 223.0, 226.0, 227.0, 232.0377,
    231.03588, 238.02891, 237.0, 244.0, 243.0, 247.0, 247.0, 251.0, 252.0, 257.0,
    258.0, 259.0, 262.0, 267.0, 270.0, 269.0, 270.0, 270.0, 278.0, 281.0,
    281.0, 285.0, 286.0, 289.0, 289.0, 293.0, 293.0, 294.0,
], dtype=np.float64)
assert ATOMIC_MASSES.shape[0] == 119


def masses_of(numbers) -> np.ndarray:
    z = np.asarray(numbers, dtype=np.int64)
    if z.size and (z.min() < 0 or z.max() > 118):
        raise ValueError(f"atomic numbers must be in 0..118, got {z.min()}..{z.max()}")
    return ATOMIC_MASSES[z]
