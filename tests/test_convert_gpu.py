"""Device FP64 <-> FP32 conversions of the FP32 node update against IEEE 754 casts."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cases():
    rng = np.random.default_rng(3)
    d = [rng.normal(size=20000) * 10.0 ** rng.integers(-50, 45, 20000),
         rng.normal(size=20000) * 2.0 ** rng.integers(-160, -120, 20000)]
    # values half-way between neighbouring binary32 numbers (ties), and their neighbours
    f = (rng.normal(size=4000) * 2.0 ** rng.integers(-149, 100, 4000)).astype(np.float32)
    nxt = np.nextafter(f, np.float32(np.inf))
    mid = (f.astype(np.float64) + nxt.astype(np.float64)) / 2
    d += [mid, np.nextafter(mid, 0), np.nextafter(mid, np.inf), -mid]
    d.append(np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 2.0 ** -150, 2.0 ** -149, 3 * 2.0 ** -150,
                       3.4028235677973366e38, 3.40282356779733e38, 1e-320, -1e-320, 1e300]))
    din = np.concatenate(d)
    with np.errstate(all="ignore"):
        fin = np.concatenate([(rng.normal(size=20000) * 10.0 ** rng.integers(-45, 38, 20000)).astype(np.float32),
                              np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-45, 1e-40, 1.17e-38],
                                       dtype=np.float32)])
    n = min(len(din), len(fin))
    return din[:n], fin[:n]


def test_conversions_match_ieee_casts():
    import torch

    from micmec_gb300 import _native as nat

    din, fin = _cases()
    n = len(din)
    dev = torch.device("cuda", 0)
    td = torch.from_numpy(din).to(dev)
    tf = torch.from_numpy(fin).to(dev)
    od = torch.empty(n, dtype=torch.float32, device=dev)
    of = torch.empty(n, dtype=torch.float64, device=dev)
    nat.check(nat.lib().mm_selftest_convert(td.data_ptr(), od.data_ptr(), tf.data_ptr(), of.data_ptr(), n,
                                            torch.cuda.current_stream().cuda_stream), "mm_selftest_convert")
    torch.cuda.synchronize()
    got_f = od.cpu().numpy()
    got_d = of.cpu().numpy()
    with np.errstate(all="ignore"):
        want_f = din.astype(np.float32)
    want_d = fin.astype(np.float64)
    nan_f = np.isnan(want_f)
    assert np.array_equal(np.isnan(got_f), nan_f)
    assert np.array_equal(got_f[~nan_f].view(np.uint32), want_f[~nan_f].view(np.uint32))
    nan_d = np.isnan(want_d)
    assert np.array_equal(np.isnan(got_d), nan_d)
    assert np.array_equal(got_d[~nan_d].view(np.uint64), want_d[~nan_d].view(np.uint64))
