"""System construction on the device (mm_build_topology) against the reference's builder
output and the host builder, bit for bit."""
import numpy as np
import pytest

from conftest import load_golden
from micmec_gb300.lattices import defect_grid, standard_types
from micmec_gb300.utils import build_system

pytestmark = pytest.mark.gpu

KEYS = ("surrounding_cells", "surrounding_nodes", "boundary_nodes", "types", "masses", "pos", "rvecs")


def _same(a, b):
    for k in KEYS:
        x, y = np.asarray(a[k]), np.asarray(b[k])
        assert x.shape == y.shape and np.array_equal(x, y), k
        assert x.dtype == y.dtype or k == "boundary_nodes", k


@pytest.mark.parametrize("tag,pbc", [("pbc", True), ("nopbc", False)])
def test_device_build_matches_reference(tag, pbc):
    B = load_golden("builder")
    grid = B[f"{tag}/grid"]
    d = build_system(standard_types(nstates=2), grid, pbc=pbc, device=True)
    for k in ("surrounding_cells", "surrounding_nodes", "boundary_nodes", "types", "masses", "pos"):
        assert np.array_equal(np.asarray(d[k]), B[f"{tag}/{k}"]), k
    assert np.array_equal(np.asarray(d["rvecs"]).reshape(-1, 3), B[f"{tag}/rvecs"].reshape(-1, 3))


@pytest.mark.parametrize("shape,pbc,vacancy", [
    ((1, 1, 1), True, 0.0), ((2, 3, 1), [True, False, True], 0.0), ((1, 4, 2), False, 0.0),
    ((5, 4, 3), [False, True, True], 0.3), ((7, 7, 7), True, 0.25), ((9, 6, 8), False, 0.4),
    ((20, 17, 13), True, 0.1),
])
def test_device_build_matches_host_with_vacancies_and_mixed_periodicity(shape, pbc, vacancy):
    rng = np.random.default_rng(sum(shape))
    grid = rng.integers(1, 3, size=shape)
    grid[rng.random(shape) < vacancy] = 0
    if not grid.any():
        grid[0, 0, 0] = 1
    data = standard_types(nstates=2)
    _same(build_system(data, grid, pbc=pbc, device=True), build_system(data, grid, pbc=pbc))


def test_device_build_large_clustered_lattice():
    """96^3 with clustered defects: past a single scan tile in every pass, equal to the host."""
    rng = np.random.default_rng(3)
    grid = defect_grid(96, 0.2, rng, clustered=True)
    data = standard_types(nstates=2)
    _same(build_system(data, grid, pbc=True, device=True), build_system(data, grid, pbc=True))


def test_device_build_rejects_type_ids_outside_the_mass_table():
    """A grid value at or above ntype_ids is reported as MM_ERR_ARG (checked on the device)."""
    import torch

    from micmec_gb300 import _native as nat

    grid = np.ones((4, 4, 4), dtype=np.int32)
    grid[1, 2, 3] = 3
    g_d = torch.from_numpy(grid).cuda()
    n = grid.size
    outs = [torch.empty((n, 8), dtype=torch.int64, device="cuda"), torch.empty((n, 8), dtype=torch.int64, device="cuda"),
            torch.empty(n, dtype=torch.float64, device="cuda"), torch.empty((n, 3), dtype=torch.float64, device="cuda"),
            torch.empty(n, dtype=torch.int32, device="cuda"), torch.empty(n, dtype=torch.uint8, device="cuda")]
    pbc = np.ones(3, dtype=np.int32)
    mass = np.array([0.0, 1.0, 2.0, 3.0])
    size = np.ones(3)
    counts = np.zeros(2, dtype=np.int64)
    args = [g_d.data_ptr(), 4, 4, 4, pbc.ctypes.data, mass.ctypes.data, 4, size.ctypes.data] + \
        [o.data_ptr() for o in outs] + [counts.ctypes.data, torch.cuda.current_stream().cuda_stream]
    assert nat.lib().mm_build_topology(*args) == 0 and tuple(counts) == (64, 64)
    args[6] = 3  # type ids 0 .. 2 only
    assert nat.lib().mm_build_topology(*args) != 0
    assert b"type id" in nat.lib().mm_last_error()
