"""The package's unit factors against molmod 1.4.8's, written out independently.

The golden fixtures were made by running the reference with a molmod stand-in
(tests/golden/standin/molmod/units.py) whose factors are literal restatements of
molmod's definitions, not imports of this package; a wrong factor here would show
as a mismatch below instead of being reproduced in the fixtures. The atomic mass
unit is also pinned by the reference's own data (the 'fcu' type mass is the sum of
the standard atomic weights of its 456 atoms), and the angstrom by its CHK files.
"""
import importlib.util
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

# IUPAC standard atomic weights (2001 table), the values molmod's periodic table carries
ATOMIC_WEIGHT = {1: 1.00794, 6: 12.0107, 8: 15.9994, 40: 91.224}


def _standin_units():
    path = os.path.join(GOLDEN, "standin", "molmod", "units.py")
    spec = importlib.util.spec_from_file_location("molmod_units_standin", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.mark.parametrize("name", ["boltzmann", "kjmol", "femtosecond", "picosecond", "amu", "pascal", "bar",
                                  "angstrom", "kelvin", "electronvolt", "kcalmol", "atm"])
def test_factor_equals_molmod_definition(name):
    from micmec_gb300 import units

    ref = getattr(_standin_units(), name)
    assert getattr(units, name) == pytest.approx(ref, rel=1e-15, abs=0.0)


def test_amu_pinned_by_reference_type_mass():
    from micmec_gb300 import units

    pin = load_golden("units_pin")
    weights = sum(ATOMIC_WEIGHT[int(z)] * int(n) for z, n in zip(pin["numbers"], pin["counts"]))
    assert int(pin["counts"].sum()) == 456
    assert float(pin["fcu_mass"]) == pytest.approx(weights * units.amu, rel=1e-14)


def test_angstrom_pinned_by_chk_lattice_edge():
    from micmec_gb300 import units

    assert 10.0 * units.angstrom == pytest.approx(18.89726133921252, rel=1e-15)


def test_boltzmann_in_hartree_per_kelvin():
    from micmec_gb300 import units

    # k_B = 1.3806505e-23 J/K with the hartree 4.35974381e-18 J (molmod.constants)
    assert units.boltzmann == pytest.approx(3.1668154051341965e-06, rel=1e-15)
    assert np.isclose(units.boltzmann * 300.0 / units.kjmol * 1000.0 / 8.314472, 300.0, rtol=1e-6)
