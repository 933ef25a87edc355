"""mm_compute_noalloc: the force evaluation for callers that cannot allocate device memory.

Such callers (code inside another framework's memory pool or a fixed-budget arena,
plugins whose host owns all device allocations) cannot use mm_create, which
allocates. mm_compute_noalloc keeps its working memory in a static device array
instead. These tests call it through the C ABI and check it against the regular
entry point (mm_compute via ForcePartMechanical) on two calls in a row, with the
tolerances of the other force tests. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MM_OK, MM_ERR_ARG = 0, 2


def _lib():
    from micmec_gb300 import _native as nat

    L = nat.lib()
    P = ctypes.c_void_p
    L.mm_compute_noalloc.argtypes = [P, P, ctypes.c_int, P, P, P, P, P, P, ctypes.c_int, ctypes.c_int, P, P, P, P, P]
    L.mm_compute_noalloc.restype = ctypes.c_int
    return L


def _system(n, seed):
    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    d = lattices.make_lattice(lattices.defect_grid(n, 0.2, rng), nstates=2)
    d["pos"] = lattices.displace(d["pos"], 0.1 * units.angstrom, rng)
    return System.from_dict(d), rng


def _noalloc(L, s, fp, pos, precision):
    import torch

    from micmec_gb300.pes.mmff import type_parameters

    dev = fp.device
    ids = fp.type_ids
    index = {k: i for i, k in enumerate(ids)}
    ctype = torch.tensor([index[int(t)] for t in s.types], dtype=torch.int32, device=dev)
    nstates, h0, C, df, temp = type_parameters(s.params, ids)
    shape = np.ascontiguousarray(fp.lattice_shape, dtype=np.int32)
    rvecs = np.ascontiguousarray(s.domain.rvecs, dtype=np.float64)
    pos_d = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
    gpos = torch.zeros((s.nnodes, 3), dtype=torch.float64, device=dev)
    vtens = torch.zeros((3, 3), dtype=torch.float64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    st = L.mm_compute_noalloc(
        shape.ctypes.data, ctype.data_ptr(), len(ids), nstates.ctypes.data, h0.ctypes.data, C.ctypes.data,
        df.ctypes.data, temp.ctypes.data, rvecs.ctypes.data, 1, {"fp64": 0, "fp32": 1}[precision],
        pos_d.data_ptr(), gpos.data_ptr(), vtens.data_ptr(), energy.data_ptr(),
        torch.cuda.current_stream().cuda_stream)
    assert st == MM_OK, L.mm_last_error()
    torch.cuda.synchronize()
    return float(energy.item()), gpos.cpu().numpy(), vtens.cpu().numpy()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_noalloc_matches_regular_entry_point(precision, tol):
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    L = _lib()
    s, rng = _system(12, 5)
    fp = ForcePartMechanical(s, model="nanocell", precision=precision)
    ff = MicMecForceField(s, [fp])
    pos0 = s.pos.copy()
    for call in range(2):  # two calls in a row, different positions
        pos = pos0 + rng.normal(0.0, 0.02 * units.angstrom, pos0.shape) * call
        ff.update_pos(pos)
        g_ref = np.zeros((s.nnodes, 3))
        v_ref = np.zeros((3, 3))
        e_ref = ff.compute(g_ref, v_ref)
        e, g, v = _noalloc(L, s, fp, pos, precision)
        assert abs(e - e_ref) <= tol * abs(e_ref)
        assert np.abs(g - g_ref).max() <= tol * np.abs(g_ref).max()
        assert np.abs(v - v_ref).max() <= tol * np.abs(v_ref).max()


def test_noalloc_rejects_lattices_beyond_the_scratch_size():
    import torch

    L = _lib()
    shape = np.array([33, 33, 33], dtype=np.int32)  # 35,937 cells > 32,768
    n = int(np.prod(shape))
    dev = torch.device("cuda")
    ctype = torch.zeros(n, dtype=torch.int32, device=dev)
    pos = torch.zeros((n, 3), dtype=torch.float64, device=dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    one = np.array([1], dtype=np.int32)
    h0 = np.tile(np.eye(3).ravel(), (4, 1))
    C = np.zeros((4, 81))
    df = np.zeros(4)
    temp = np.array([300.0])
    rvecs = np.eye(3) * 100.0
    st = L.mm_compute_noalloc(shape.ctypes.data, ctype.data_ptr(), 1, one.ctypes.data, h0.ctypes.data,
                              C.ctypes.data, df.ctypes.data, temp.ctypes.data, rvecs.ctypes.data, 1, 0,
                              pos.data_ptr(), None, None, energy.data_ptr(), None)
    assert st == MM_ERR_ARG
    assert b"32768" in L.mm_last_error()
