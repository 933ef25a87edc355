"""Atomic units, with the conversion factors MicMec takes from ``molmod.units``.

MicMec works in atomic units throughout (Hartree, bohr, electron mass, atomic
time). The reference imports its factors from the third-party ``molmod``
package (molmod 1.4.8, pinned in the reference's docs/installation.rst:12),
which is not available here. The factors below restate molmod's definitions:
CODATA-1998 values for the atomic units of length, mass and energy, CODATA-2002
values for the atomic unit of time and the Avogadro and Boltzmann constants; the
atomic mass unit is defined as gram / Avogadro's number. Two of them are pinned by
the reference's own data files: every ``*_micmec.chk`` stores lengths in bohr, and a
10 Å cell edge appears as 18.89726133921252, i.e. ``angstrom`` below (e.g.
data/3x3x3_test_micmec.chk:165-168); the 'fcu' type mass of
data/type_1x1x1_fcu_atomic.pickle (12133589.4468533) is the standard atomic weights
of its 456 atoms (6656.24288) times ``amu`` below.
"""

# base SI values of the atomic units and constants (as molmod.units / molmod.constants)
_BOHR_M = 0.5291772083e-10
_HARTREE_J = 4.35974381e-18
_ME_KG = 9.10938188e-31
_AUTIME_S = 2.418884326505e-17
_E_C = 1.602176462e-19
_AVOGADRO = 6.0221415e23
_KB_J = 1.3806505e-23

au = 1.0

# length
meter = 1.0 / _BOHR_M
angstrom = 1.0e-10 * meter
nanometer = 1.0e-9 * meter
bohr = 1.0

# mass
kilogram = 1.0 / _ME_KG
gram = 1.0e-3 * kilogram
unified = gram / _AVOGADRO
amu = unified

# energy
joule = 1.0 / _HARTREE_J
kjmol = 1.0e3 * joule / _AVOGADRO
kcalmol = 4.184 * kjmol
electronvolt = _E_C * joule
ev = electronvolt

# time
second = 1.0 / _AUTIME_S
femtosecond = 1.0e-15 * second
picosecond = 1.0e-12 * second
nanosecond = 1.0e-9 * second

# temperature
kelvin = 1.0

# pressure
pascal = joule / meter**3
bar = 1.0e5 * pascal
atm = 101325.0 * pascal
gigapascal = 1.0e9 * pascal

# Boltzmann constant in Hartree per kelvin
boltzmann = _KB_J * joule

__all__ = [
    "au", "meter", "angstrom", "nanometer", "bohr", "kilogram", "gram",
    "unified", "amu", "joule", "kjmol", "kcalmol", "electronvolt", "ev",
    "second", "femtosecond", "picosecond", "nanosecond", "kelvin", "pascal",
    "bar", "atm", "gigapascal", "boltzmann",
]
