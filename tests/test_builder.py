"""Host-side system construction and I/O against the reference's builder output."""
import os

import numpy as np
import pytest

from conftest import load_golden
from micmec_gb300 import units
from micmec_gb300.chk import dump_chk, load_chk
from micmec_gb300.lattices import standard_types
from micmec_gb300.utils import build_system, voigt, voigt_inv

B = load_golden("builder")


@pytest.mark.parametrize("tag,pbc", [("pbc", True), ("nopbc", False)])
def test_build_system_matches_reference(tag, pbc):
    grid = B[f"{tag}/grid"]
    d = build_system(standard_types(nstates=2), grid, pbc=pbc)
    for k in ("surrounding_cells", "surrounding_nodes", "boundary_nodes", "types"):
        assert np.array_equal(np.asarray(d[k]), B[f"{tag}/{k}"]), k
    assert np.array_equal(d["masses"], B[f"{tag}/masses"])  # same accumulation order: bitwise
    assert np.array_equal(d["pos"], B[f"{tag}/pos"])
    assert np.array_equal(np.asarray(d["rvecs"]).reshape(-1, 3), B[f"{tag}/rvecs"].reshape(-1, 3))


def test_units_pinned_by_chk_data():
    # data/3x3x3_test_micmec.chk stores a 10 angstrom cell as 18.89726133921252 bohr
    assert abs(10 * units.angstrom - 18.89726133921252) < 1e-13


def test_voigt_roundtrip():
    rng = np.random.default_rng(0)
    m = rng.normal(size=(6, 6))
    m = m + m.T
    assert np.allclose(voigt(voigt_inv(m, mode="elasticity"), mode="elasticity"), m)


def test_chk_roundtrip(tmp_path):
    data = {"pos": np.arange(12.0).reshape(4, 3), "types": np.array([1, 2, 1]), "name": "x", "mass": 3,
            "temp": 300.0}
    fn = os.path.join(tmp_path, "t.chk")
    dump_chk(fn, data)
    back = load_chk(fn)
    assert np.array_equal(back["pos"], data["pos"]) and np.array_equal(back["types"], data["types"])
    assert back["name"] == "x" and back["mass"] == 3 and back["temp"] == 300.0
