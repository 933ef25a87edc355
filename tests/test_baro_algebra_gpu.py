"""The batch kernels' warp-parallel barostat algebra (lane e forming entry e of each 3x3
result) against the one-thread form it replaces, bit for bit, and against scipy's expm."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _matrices():
    rng = np.random.default_rng(11)
    mats = []
    # barostat-like arguments (dt/2 times a barostat velocity): tiny, a few Taylor terms
    for scale in (1e-6, 1e-4, 1e-2):
        a = rng.normal(size=(40, 3, 3)) * scale
        mats.append(0.5 * (a + a.transpose(0, 2, 1)))
    # norms above 1/8: scaling and squaring steps
    a = rng.normal(size=(40, 3, 3)) * rng.uniform(0.2, 3.0, size=(40, 1, 1))
    mats.append(0.5 * (a + a.transpose(0, 2, 1)))
    # zero, identity multiple, a non-symmetric matrix, a diagonal one
    mats.append(np.stack([np.zeros((3, 3)), 0.3 * np.eye(3), rng.normal(size=(3, 3)) * 0.05,
                          np.diag([1e-3, -2e-3, 5e-4])]))
    return np.concatenate(mats)


@pytest.mark.parametrize("f", [1.0, -0.5, 0.25])
def test_warp_matrix_exponential_equals_one_thread_form(f):
    import torch
    from scipy.linalg import expm

    from micmec_gb300 import _native as nat

    S = _matrices()
    n = len(S)
    dev = torch.device("cuda", 0)
    s_d = torch.from_numpy(np.ascontiguousarray(S)).to(dev)
    rt = torch.full((n, 3, 3), np.nan, dtype=torch.float64, device=dev)
    rw = torch.full((n, 3, 3), np.nan, dtype=torch.float64, device=dev)
    nat.check(nat.lib().mm_selftest_sym_exp(s_d.data_ptr(), n, f, rt.data_ptr(), rw.data_ptr(),
                                            torch.cuda.current_stream().cuda_stream), "mm_selftest_sym_exp")
    torch.cuda.synchronize()
    rt, rw = rt.cpu().numpy(), rw.cpu().numpy()
    assert np.array_equal(rt, rw)
    for k in range(n):
        ref = expm(f * S[k])
        # normwise: ~1 ulp for the barostat-sized arguments (no squaring); the squarings of
        # the larger ones amplify rounding (a CPU restatement of the same steps: <= 5e-13)
        big = np.abs(f * S[k]).sum(axis=0).max() > 0.125
        assert np.abs(rw[k] - ref).max() <= (2e-12 if big else 1e-14) * np.abs(ref).max(), k


def test_selftest_rejects_bad_arguments():
    from micmec_gb300 import _native as nat

    assert nat.lib().mm_selftest_sym_exp(None, 4, 1.0, None, None, None) != 0
    assert b"sym_exp" in nat.lib().mm_last_error()
    assert nat.lib().mm_selftest_sym_exp(None, 0, 1.0, None, None, None) == 0


def test_exp_small_against_library_exp():
    """The hook algebra's exponential: a Taylor polynomial below |x| = 2^-5, the library exp
    above; within 2 ulp of CUDA's exp (and of numpy's) everywhere on the tested range."""
    import ctypes

    import torch

    from micmec_gb300 import _native as nat

    L = nat.lib()
    L.mm_selftest_exp_small.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    L.mm_selftest_exp_small.restype = ctypes.c_int
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-2.0**-5, 2.0**-5, 20000), rng.normal(size=2000) * 1e-6,
                        rng.uniform(-3.0, 3.0, 2000), [0.0, -0.0, 2.0**-5, -2.0**-5, 2.0**-6, 1e-300, -1e-310]])
    xd = torch.tensor(x, dtype=torch.float64, device="cuda")
    out = torch.empty_like(xd)
    nat.check(L.mm_selftest_exp_small(xd.data_ptr(), out.data_ptr(), len(x), None), "mm_selftest_exp_small")
    got = out.cpu().numpy()
    ref_cuda = torch.exp(xd).cpu().numpy()
    assert (np.abs(got - ref_cuda) <= 2 * np.spacing(np.abs(ref_cuda))).all()
    assert (np.abs(got - np.exp(x)) <= 2 * np.spacing(np.exp(x))).all()
