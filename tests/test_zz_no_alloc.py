"""mm_compute_noalloc: the force evaluation for callers that cannot allocate device memory.

Such callers (code inside another framework's memory pool or a fixed-budget arena,
plugins whose host owns all device allocations) cannot use mm_create, which
allocates. mm_compute_noalloc keeps its working memory in a static device array
instead. These tests call it through the C ABI and check it against the regular
entry point (mm_compute via ForcePartMechanical) on two calls in a row, with the
tolerances of the other force tests, for both energy models; the gradient and
virial buffers start nonzero, since the call adds into them. The largest lattice
the static array holds (32^3 cells, FP64) is run too, and an out-of-range cell type
is refused before any energy is evaluated, and so is a call on a stream that is being
captured into a CUDA graph. This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MM_OK, MM_ERR_NAN, MM_ERR_ARG = 0, 1, 2
MODELS = {"original": 0, "nanocell": 1}
_CAPTURE_BUFFERS = {}


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


def _noalloc(L, s, fp, pos, precision, model, g0, v0, ctype=None):
    import torch

    from micmec_gb300.pes.mmff import type_parameters

    dev = fp.device
    ids = fp.type_ids
    index = {k: i for i, k in enumerate(ids)}
    if ctype is None:
        ctype = torch.tensor([index[int(t)] for t in s.types], dtype=torch.int32, device=dev)
    nstates, h0, C, df, temp = type_parameters(s.params, ids)
    shape = np.ascontiguousarray(fp.lattice_shape, dtype=np.int32)
    rvecs = np.ascontiguousarray(s.domain.rvecs, dtype=np.float64)
    pos_d = torch.from_numpy(np.ascontiguousarray(pos)).to(dev)
    gpos = torch.from_numpy(np.array(g0, dtype=np.float64)).to(dev)
    vtens = torch.from_numpy(np.array(v0, dtype=np.float64)).to(dev)
    energy = torch.zeros(1, dtype=torch.float64, device=dev)
    st = L.mm_compute_noalloc(
        shape.ctypes.data, ctype.data_ptr(), len(ids), nstates.ctypes.data, h0.ctypes.data, C.ctypes.data,
        df.ctypes.data, temp.ctypes.data, rvecs.ctypes.data, MODELS[model], {"fp64": 0, "fp32": 1}[precision],
        pos_d.data_ptr(), gpos.data_ptr(), vtens.data_ptr(), energy.data_ptr(),
        torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return st, float(energy.item()), gpos.cpu().numpy(), vtens.cpu().numpy()


def _check_against_regular(L, n, seed, model, precision, tol):
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    s, rng = _system(n, seed)
    fp = ForcePartMechanical(s, model=model, precision=precision)
    ff = MicMecForceField(s, [fp])
    pos0 = s.pos.copy()
    for call in range(2):  # two calls in a row, different positions
        pos = pos0 + rng.normal(0.0, 0.02 * units.angstrom, pos0.shape) * call
        ff.update_pos(pos)
        g_ref = np.zeros((s.nnodes, 3))
        v_ref = np.zeros((3, 3))
        e_ref = ff.compute(g_ref, v_ref)
        # nonzero starting buffers: the call adds its gradient and virial to them
        g0 = rng.normal(0.0, np.abs(g_ref).max(), g_ref.shape)
        v0 = rng.normal(0.0, np.abs(v_ref).max(), (3, 3))
        st, e, g, v = _noalloc(L, s, fp, pos, precision, model, g0, v0)
        assert st == MM_OK, L.mm_last_error()
        assert abs(e - e_ref) <= tol * abs(e_ref)
        assert np.abs((g - g0) - g_ref).max() <= tol * np.abs(g_ref).max()
        assert np.abs((v - v0) - v_ref).max() <= tol * np.abs(v_ref).max()


@pytest.mark.parametrize("model", ["nanocell", "original"])
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_noalloc_matches_regular_entry_point(precision, tol, model):
    _check_against_regular(_lib(), 12, 5, model, precision, tol)


def test_noalloc_largest_lattice_fp64():
    """32^3 = 32,768 cells in FP64: the layout that fills most of the static array."""
    _check_against_regular(_lib(), 32, 6, "nanocell", "fp64", 1e-10)


def test_noalloc_rejects_out_of_range_cell_type_and_recovers():
    """A type id >= ntypes is refused with MM_ERR_ARG (no kernel reads the parameter table
    with it); the next call with valid types succeeds."""
    import torch

    from micmec_gb300.pes.mmff import ForcePartMechanical

    L = _lib()
    s, _ = _system(4, 7)
    fp = ForcePartMechanical(s, model="nanocell", precision="fp64")
    index = {k: i for i, k in enumerate(fp.type_ids)}
    good = [index[int(t)] for t in s.types]
    zeros_g, zeros_v = np.zeros((s.nnodes, 3)), np.zeros((3, 3))
    for badval in (len(fp.type_ids), 255, -1):
        bad = list(good)
        bad[5] = badval
        ctype = torch.tensor(bad, dtype=torch.int32, device=fp.device)
        st, _, _, _ = _noalloc(L, s, fp, s.pos, "fp64", "nanocell", zeros_g, zeros_v, ctype=ctype)
        assert st == MM_ERR_ARG
        assert b"cell type" in L.mm_last_error()
    st, e, _, _ = _noalloc(L, s, fp, s.pos, "fp64", "nanocell", zeros_g, zeros_v)
    assert st == MM_OK and np.isfinite(e)


def test_noalloc_reports_nan_and_recovers():
    """A NaN position gives MM_ERR_NAN (the reference raises ValueError); the status words
    are cleared by the next call."""
    from micmec_gb300.pes.mmff import ForcePartMechanical

    L = _lib()
    s, _ = _system(4, 8)
    fp = ForcePartMechanical(s, model="nanocell", precision="fp32")
    zeros_g, zeros_v = np.zeros((s.nnodes, 3)), np.zeros((3, 3))
    pos = s.pos.copy()
    pos[3, 1] = np.nan
    st, _, _, _ = _noalloc(L, s, fp, pos, "fp32", "nanocell", zeros_g, zeros_v)
    assert st == MM_ERR_NAN
    st, e, _, _ = _noalloc(L, s, fp, s.pos, "fp32", "nanocell", zeros_g, zeros_v)
    assert st == MM_OK and np.isfinite(e)


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


@pytest.mark.filterwarnings("ignore:The CUDA Graph is empty")  # nothing is captured, by design
def test_noalloc_refuses_a_stream_under_capture():
    import torch

    from micmec_gb300.pes.mmff import ForcePartMechanical

    L = _lib()
    s, _ = _system(4, 17)
    fp = ForcePartMechanical(s)
    zeros_g, zeros_v = np.zeros((s.nnodes, 3)), np.zeros((3, 3))
    index = {k: i for i, k in enumerate(fp.type_ids)}
    _CAPTURE_BUFFERS.update(
        ctype=torch.tensor([index[int(t)] for t in s.types], dtype=torch.int32, device=fp.device),
        pos=torch.from_numpy(np.ascontiguousarray(s.pos)).to(fp.device),
        energy=torch.zeros(1, dtype=torch.float64, device=fp.device))
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        status = []
        with torch.cuda.graph(graph, stream=side):
            status.append(_noalloc_on_stream(L, s, fp, side))
    assert status == [MM_ERR_ARG]
    assert b"captured" in L.mm_last_error()
    st, e, _, _ = _noalloc(L, s, fp, s.pos, "fp64", "nanocell", zeros_g, zeros_v)  # usable afterwards
    assert st == MM_OK and np.isfinite(e)


def _noalloc_on_stream(L, s, fp, stream):
    """One call with buffers allocated before the capture began (only the call is captured)."""
    from micmec_gb300.pes.mmff import type_parameters

    ids = fp.type_ids
    nstates, h0, C, df, temp = type_parameters(s.params, ids)
    shape = np.ascontiguousarray(fp.lattice_shape, dtype=np.int32)
    rvecs = np.ascontiguousarray(s.domain.rvecs, dtype=np.float64)
    b = _CAPTURE_BUFFERS
    return L.mm_compute_noalloc(shape.ctypes.data, b["ctype"].data_ptr(), len(ids), nstates.ctypes.data,
                                h0.ctypes.data, C.ctypes.data, df.ctypes.data, temp.ctypes.data, rvecs.ctypes.data,
                                1, 0, b["pos"].data_ptr(), None, None, b["energy"].data_ptr(), stream.cuda_stream)
