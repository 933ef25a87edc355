"""The host-buffer MD step (mm_md_step_host) against the device MD loop (mm_md_run).

Pageable (NumPy) caller buffers are staged through device memory; pinned buffers are
read and written in place by the kernels. Both must give the same trajectory, and
NVE steps must follow the device loop's trajectory.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

THERMO_NONE, THERMO_LANGEVIN = 0, 1


def _system(n=6, seed=3):
    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    grid = lattices.defect_grid(n, 0.2, rng)
    d = lattices.make_lattice(grid, nstates=2)
    d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
    s = System.from_dict(d)
    kT = units.boltzmann * 300.0
    vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(kT / s.masses)[:, None]
    return s, vel


def _host_steps(fp, pos, vel, nsteps, thermo, pinned, seed=11):
    import torch

    from micmec_gb300 import _native as nat, units

    dt, temp, tau = 1.0 * units.femtosecond, 300.0, 100.0 * units.femtosecond
    g = np.zeros_like(pos)
    fp.system.pos[:] = pos
    fp.compute(g)
    arrays = [np.ascontiguousarray(pos.copy()), np.ascontiguousarray(vel.copy()), g,
              np.zeros(nat.MM_REC_LEN)]
    if pinned:
        arrays = [torch.from_numpy(a).pin_memory() for a in arrays]
        ptrs = [a.data_ptr() for a in arrays]
    else:
        ptrs = [a.ctypes.data for a in arrays]
    recs = []
    for i in range(nsteps):
        nat.check(nat.lib().mm_md_step_host(fp.handle, ptrs[0], ptrs[1], ptrs[2], ptrs[3], dt, thermo, temp, tau,
                                            seed, 1 + i), "mm_md_step_host")
        recs.append(arrays[3].numpy().copy() if pinned else arrays[3].copy())
    out = [a.numpy().copy() if pinned else a.copy() for a in arrays[:3]]
    return out[0], out[1], out[2], np.array(recs)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
@pytest.mark.parametrize("thermo", [THERMO_NONE, THERMO_LANGEVIN])
def test_pinned_and_pageable_buffers_agree(precision, thermo):
    from micmec_gb300.pes.mmff import ForcePartMechanical

    s, vel = _system()
    fp = ForcePartMechanical(s, precision=precision)
    pos0 = s.pos.copy()
    a = _host_steps(fp, pos0, vel, 5, thermo, pinned=False)
    b = _host_steps(fp, pos0, vel, 5, thermo, pinned=True)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert np.isfinite(a[3]).all()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-6)])
def test_nve_host_steps_follow_device_loop(precision, tol):
    import torch

    from micmec_gb300 import _native as nat, units
    from micmec_gb300.pes.mmff import ForcePartMechanical

    s, vel = _system()
    fp = ForcePartMechanical(s, precision=precision)
    pos0 = s.pos.copy()
    nsteps = 5
    hp, hv, hg, _ = _host_steps(fp, pos0, vel, nsteps, THERMO_NONE, pinned=True)
    dev = torch.device("cuda", 0)
    pd = torch.from_numpy(pos0.copy()).to(dev)
    vd = torch.from_numpy(vel.copy()).to(dev)
    nat.check(nat.lib().mm_md_run(fp.handle, pd.data_ptr(), vd.data_ptr(), nsteps, 1.0 * units.femtosecond,
                                  THERMO_NONE, 300.0, 100.0 * units.femtosecond, 11, None, None, 1,
                                  torch.cuda.current_stream().cuda_stream), "mm_md_run")
    torch.cuda.synchronize()
    dp, dv = pd.cpu().numpy(), vd.cpu().numpy()
    assert np.abs(hp - dp).max() <= tol * np.abs(dp - dp.mean(axis=0)).max()
    assert np.abs(hv - dv).max() <= tol * np.abs(dv).max() * 10
