"""molmod.units / molmod.constants stand-in: molmod 1.4.8's unit factors, written out.

The reference imports its unit factors from molmod 1.4.8 (pinned in the reference's
docs/installation.rst:12), which is absent here. This file restates molmod's own
definitions (molmod/units.py and molmod/constants.py of that release: CODATA-1998
values for the atomic units of length, mass and energy, CODATA-2002 values for the
atomic unit of time, the Avogadro and the Boltzmann constants) as literal
expressions, independently of the package under test, so that a wrong factor in the
package cannot be reproduced in the fixtures the reference generates with this file.
Two of these factors are also pinned by the reference's own data files:

* angstrom: every ``data/*_micmec.chk`` stores a 10 A lattice edge as 18.89726133921252 bohr;
* amu: the 'fcu' type mass in ``data/type_1x1x1_fcu_atomic.pickle`` (12133589.4468533)
  is the sum of the standard atomic weights of the 456 atoms of
  ``data/1x1x1_fcu_atomic.chk`` (Zr24 O128 C192 H112: 6656.24288) times amu = gram/avogadro.

tests/test_units_pinned.py compares the package's factors with these.
"""

# molmod/constants.py
avogadro = 6.0221415e23
boltzmann = 1.3806505e-23 / 4.35974381e-18  # J/K over the hartree in J: 3.1668154051341965e-06

# molmod/units.py
au = 1.0
coulomb = 1.0 / 1.602176462e-19
kilogram = 1.0 / 9.10938188e-31
gram = 1.0e-3 * kilogram
unified = gram / avogadro
amu = unified
meter = 1.0 / 0.5291772083e-10
nanometer = 1.0e-9 * meter
angstrom = 1.0e-10 * meter
bohr = 1.0
joule = 1.0 / 4.35974381e-18
calorie = 4.184 * joule
kjmol = 1.0e3 * joule / avogadro
kcalmol = 1.0e3 * calorie / avogadro
electronvolt = (1.0 / coulomb) * joule
newton = joule / meter
second = 1.0 / 2.418884326505e-17
nanosecond = 1e-9 * second
picosecond = 1e-12 * second
femtosecond = 1e-15 * second
pascal = newton / meter**2
bar = 100000 * pascal
atm = 1.01325 * bar
kelvin = 1.0
