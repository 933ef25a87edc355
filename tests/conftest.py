import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)


def system_dict(npz, prefix):
    """System description stored under ``prefix`` in a golden file (as the oracle takes it)."""
    d = {}
    params = {}
    for key in npz.files:
        if not key.startswith(prefix):
            continue
        sub = key[len(prefix):]
        if sub.startswith("param:"):
            name = sub[len("param:"):]
            val = npz[key]
            params[name] = val if val.ndim else float(val)
        else:
            d[sub] = npz[key]
    d["params"] = params
    return d


def make_system(d):
    from micmec_gb300.system import System

    return System(
        pos=d["pos"].copy(), masses=d["masses"], rvecs=d["rvecs"], surrounding_cells=d["surrounding_cells"],
        surrounding_nodes=d["surrounding_nodes"], grid=d["grid"], types=d["types"], params=d["params"],
    )


@pytest.fixture(scope="session")
def forces_golden():
    return load_golden("forces")
