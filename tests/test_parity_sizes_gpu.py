"""GPU paths against the CPU oracle at the sizes of the standard workloads.

The golden-fixture tests run on lattices of at most 5^3 cells. These run the same
comparisons where the kernels use grid-stride passes, several waves of blocks,
block partial sums over many blocks and corner-gradient buffers of tens of MB:

* the 64^3 two-type two-state lattice (10% 'reo' cells, uniform): energy, gradient
  and virial of ForcePartMechanical.compute for both models, FP64 and FP32 cells;
* ten Langevin steps of that lattice on the fused device path, with the normals
  replayed into the oracle's step (micmec/sampling/verlet.py:140-166, nvt.py:196-218);
* sixteen uneven periodic systems as in the batched strain-scan workload (n = 3..12,
  0-30% defects, uniaxial strains 0-5%) through BatchSystems: static energy and
  virial, then five NVE steps, per system;
* a 96^3 lattice with 20% clustered defects through the grid-wide lattice engine
  (mm_md_engine): three NVE steps.

The oracle (oracle/mmff.py, oracle/md.py) is pinned to the reference by the golden
fixtures; here it runs split over worker processes started with 'spawn'.
Tolerances: FP64 cells 1e-10 relative to the largest component for one evaluation
and 1e-8 along trajectories (as the reference-trajectory tests); FP32 cells 1e-5.
"""
import multiprocessing as mp
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FS = 1e-15 / 2.418884326505e-17  # femtosecond in atomic time units


@pytest.fixture(scope="module")
def pool():
    n = max(1, min(16, os.cpu_count() or 1))
    ctx = mp.get_context("spawn")
    p = ctx.Pool(n)
    p.nproc = n
    yield p
    p.close()
    p.join()


def _lattice(n, fraction, seed, clustered=False, sigma=0.05):
    from micmec_gb300 import lattices, units

    rng = np.random.default_rng(seed)
    grid = lattices.defect_grid(n, fraction, rng, clustered=clustered)
    d = lattices.make_lattice(grid, nstates=2)
    d["pos"] = lattices.displace(d["pos"], sigma * units.angstrom, rng)
    d["params"] = {k: v for k, v in d.items() if "/" in k}
    return d, rng


def _thermal_velocities(masses, rng, temp=300.0):
    from micmec_gb300 import units

    m = np.asarray(masses)
    v = rng.normal(0.0, 1.0, (len(m), 3)) * np.sqrt(units.boltzmann * temp / m)[:, None]
    v -= (m @ v) / m.sum()  # no centre-of-mass motion (as the thermostat's init leaves it)
    return v


def _oracle_compute(d, model, pool):
    """Energy, gradient and virial from the oracle, cells split over the pool."""
    from oracle import md as omd
    from oracle import mmff as om

    sn = np.asarray(d["surrounding_nodes"])
    shifts = om.cell_shifts(d["grid"], sn, True)
    e, g, verts = omd.pooled_deformation(pool, pool.nproc, np.asarray(d["pos"]), np.asarray(d["rvecs"]), sn,
                                         np.asarray(d["types"]), shifts, d["params"], model)
    return float(e.sum()), om.gather_gpos(g, d["surrounding_cells"]), np.einsum("ijk,ijl->kl", g, verts)


class _ReplayLangevin(object):
    """The oracle's velocity-Verlet step with the Langevin thermostat fed given normals."""

    def __init__(self, d, vel, model, noise, temp, timecon, dt, pool):
        from oracle import md as omd

        self.noise = noise
        self.calls = 0
        self.state = omd.LangevinState(d, vel, model=model, temp=temp, timecon_fs=timecon / FS, dt_fs=dt / FS,
                                       pool=pool, nproc=pool.nproc)
        st = self.state
        noise_src = self

        def thermo():
            if st.temp is None:
                return
            c1 = np.exp(-st.dt / st.tau / 2)
            c2 = np.sqrt((1.0 - c1**2) * st.temp * 1.3806505e-23 / 4.35974381e-18 / st.masses).reshape(-1, 1)
            st.vel = c1 * st.vel + c2 * noise_src.noise[noise_src.calls]
            noise_src.calls += 1

        st.thermo = thermo


def _recorder():
    from micmec_gb300.sampling.iterative import Hook

    class H(Hook):
        def __init__(self):
            Hook.__init__(self, 0, 1)
            self.rows = []

        def __call__(self, it):
            self.rows.append((it.counter, it.epot, it.ekin))

    return H()


# ---------------------------------------------------------------- 64^3 forces


@pytest.fixture(scope="module")
def lattice64():
    return _lattice(64, 0.1, 2026)[0]


@pytest.mark.parametrize("model", ["nanocell", "original"])
def test_lattice64_forces_match_oracle(lattice64, model, pool):
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.system import System

    d = lattice64
    e_ref, g_ref, v_ref = _oracle_compute(d, model, pool)
    for precision, tol in (("fp64", 1e-10), ("fp32", 1e-5)):
        s = System.from_dict(d)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model=model, precision=precision)])
        gpos = np.zeros((s.nnodes, 3))
        vtens = np.zeros((3, 3))
        e = ff.compute(gpos, vtens)
        assert abs(e - e_ref) <= tol * abs(e_ref), (precision, e, e_ref)
        assert np.abs(gpos - g_ref).max() <= tol * np.abs(g_ref).max(), precision
        assert np.abs(vtens - v_ref).max() <= tol * np.abs(v_ref).max(), precision


# ---------------------------------------------------------------- 64^3 Langevin


def test_lattice64_langevin_steps_match_oracle_with_replayed_noise(lattice64, pool):
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.nvt import LangevinThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator
    from micmec_gb300.system import System

    d = lattice64
    nsteps, temp, timecon, dt = 10, 300.0, 100 * FS, 1.0 * FS
    rng = np.random.default_rng(77)
    vel0 = _thermal_velocities(d["masses"], rng)
    noise = rng.normal(size=(2 * nsteps, len(vel0), 3))
    ref = _ReplayLangevin(d, vel0, "nanocell", noise, temp, timecon, dt, pool)
    ref_epot = [ref.state.step() for _ in range(nsteps)]
    for precision, tol in (("fp64", 1e-8), ("fp32", 1e-5)):
        s = System.from_dict(d)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision=precision)])
        rec = _recorder()
        lt = LangevinThermostat(temp, timecon=timecon, replay_noise=noise)
        vi = VerletIntegrator(ff, dt, hooks=[lt, rec], vel0=vel0.copy(), device=True)
        assert vi._device_plan() is lt  # the fused node-kernel path
        vi.run(nsteps)
        got = np.array([r[1] for r in rec.rows[1:]])
        assert np.abs(got - ref_epot).max() <= tol * np.abs(ref_epot).max(), precision
        dpos = vi.pos - ref.state.pos
        assert np.abs(dpos).max() <= tol * 100.0, precision  # bohr, as the trajectory tests
        assert np.abs(vi.vel - ref.state.vel).max() <= tol * np.abs(ref.state.vel).max(), precision


# ---------------------------------------------------------------- batched systems


def _uneven_systems(count, seed):
    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    strains = np.arange(0, 21) * 0.0025
    out = []
    for _ in range(count):
        n = int(rng.integers(3, 13))
        frac = float(rng.uniform(0.0, 0.3))
        d = lattices.make_lattice(lattices.defect_grid(n, frac, rng), nstates=2)
        F = np.eye(3)
        F[0, 0] += strains[rng.integers(0, len(strains))]
        d["pos"] = d["pos"] @ F
        d["rvecs"] = d["rvecs"] @ F
        d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
        d["params"] = {k: v for k, v in d.items() if "/" in k}
        out.append((d, System.from_dict(d)))
    return out, rng


@pytest.mark.parametrize("precision,tol,tol_md", [("fp64", 1e-10, 1e-8), ("fp32", 1e-5, 1e-5)])
def test_uneven_batch_matches_oracle(precision, tol, tol_md, pool):
    from micmec_gb300.batch import REC, BatchSystems
    from oracle import md as omd

    systems, rng = _uneven_systems(16, 31)
    assert len({s.ncells for _, s in systems}) > 4  # uneven sizes
    b = BatchSystems([s for _, s in systems], model="nanocell", precision=precision)
    b.relax(max_iter=0, gtol=1e-3)  # one force evaluation, no step
    E = b.energies()
    W = b.stress()
    vols = b.control()[:, 18]
    vel0 = [_thermal_velocities(s.masses, rng) for _, s in systems]
    nsteps, dt = 5, 1.0 * FS
    b.set_state([s.pos for _, s in systems], vel0, [s.domain.rvecs for _, s in systems])
    rec = b.md(nsteps, timestep=dt, record=True, use_graph=False)
    pos, vel, _ = b.get_state()
    for i, (d, s) in enumerate(systems):
        e_ref, _, v_ref = _oracle_compute(d, "nanocell", pool)
        assert abs(E[i] - e_ref) <= tol * abs(e_ref), i
        assert np.abs(W[i] * vols[i] - v_ref).max() <= tol * np.abs(v_ref).max(), i
        ref = omd.LangevinState(d, vel0[i], model="nanocell", temp=None, dt_fs=1.0)
        ref_epot = [ref.step() for _ in range(nsteps)]
        assert np.abs(rec[i, :, REC["epot"]] - ref_epot).max() <= tol_md * np.abs(ref_epot).max(), i
        assert np.abs(pos[i] - ref.pos).max() <= tol_md * 100.0, i
        assert np.abs(vel[i] - ref.vel).max() <= tol_md * np.abs(ref.vel).max(), i


# ---------------------------------------------------------------- lattice engine, 96^3


@pytest.fixture(scope="module")
def engine96(pool):
    """96^3 lattice with 20% clustered defects, initial velocities and the oracle's 3 NVE steps."""
    from oracle import md as omd

    d, rng = _lattice(96, 0.2, 55, clustered=True)
    vel0 = _thermal_velocities(d["masses"], rng)
    ref = omd.LangevinState(d, vel0, model="nanocell", temp=None, dt_fs=1.0, pool=pool, nproc=pool.nproc)
    epot = [ref.step() for _ in range(3)]
    return d, vel0, epot, ref.pos.copy(), ref.vel.copy()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-8), ("fp32", 1e-5)])
def test_lattice_engine_96_clustered_matches_oracle(precision, tol, engine96):
    import torch

    from micmec_gb300 import _native as nat
    from micmec_gb300.batch import CTL, CTL_LEN, REC_LEN
    from micmec_gb300.pes.mmff import ForcePartMechanical
    from micmec_gb300.system import System

    d, vel0, ref_epot, ref_pos, ref_vel = engine96
    nsteps, dt = len(ref_epot), 1.0 * FS
    s = System.from_dict(d)
    part = ForcePartMechanical(s, model="nanocell", precision=precision)
    dev = part.device
    pos_d = torch.from_numpy(np.ascontiguousarray(s.pos)).to(dev)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel0)).to(dev)
    recs = torch.zeros((nsteps, REC_LEN), dtype=torch.float64, device=dev)
    ctl = np.zeros(CTL_LEN)
    ctl[CTL["ndof"]] = 3 * s.nnodes
    L = nat.lib()
    st = L.mm_md_engine(part.handle, pos_d.data_ptr(), vel_d.data_ptr(), nsteps, dt, 0, 0.0, 1.0, 0, 0.0, 3, 0,
                        None, None, ctl.ctypes.data, recs.data_ptr(), 0, torch.cuda.current_stream().cuda_stream)
    nat.check(st, "mm_md_engine")
    got = recs.cpu().numpy()[:, 0]
    assert np.abs(got - ref_epot).max() <= tol * np.abs(ref_epot).max()
    assert np.abs(pos_d.cpu().numpy() - ref_pos).max() <= tol * 100.0
    assert np.abs(vel_d.cpu().numpy() - ref_vel).max() <= tol * np.abs(ref_vel).max()
