"""MD on the GPU against trajectories of the reference's VerletIntegrator and hooks.

Golden files hold the reference's per-step (counter, epot, ekin, econs, temp, press,
vtens, ptens, rvecs, volume) rows and position/velocity snapshots. Stochastic runs
replay the reference's recorded normal draws.
"""
import numpy as np
import pytest

from conftest import load_golden, make_system, system_dict

pytestmark = pytest.mark.gpu


def _setup(name, precision="fp64"):
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    g = load_golden(name)
    s = make_system(system_dict(g, "sys/"))
    fp = ForcePartMechanical(s, model=str(g["model"]), precision=precision)
    return g, s, MicMecForceField(s, [fp])


class Rec(object):
    def __init__(self):
        from micmec_gb300.sampling.iterative import Hook

        class H(Hook):
            def __init__(self, rows, snaps):
                Hook.__init__(self, 0, 1)
                self.rows, self.snaps = rows, snaps

            def __call__(self, it):
                self.rows.append([it.counter, it.epot, it.ekin, it.econs, it.temp, getattr(it, "press", 0.0)]
                                 + list(np.asarray(it.vtens).ravel()) + list(np.asarray(it.ptens).ravel())
                                 + list(np.asarray(it.mmf.system.domain.rvecs).ravel())
                                 + [it.mmf.system.domain.volume])
                self.snaps[it.counter] = (it.pos.copy(), it.vel.copy())

        self.rows, self.snaps = [], {}
        self.hook = H(self.rows, self.snaps)


def _compare(g, rec, nsteps, rtol):
    ref = g["records"][: nsteps + 1]
    got = np.array(rec.rows)[: nsteps + 1]
    assert got.shape == ref.shape
    for col, name in ((1, "epot"), (2, "ekin"), (3, "econs")):
        scale = np.abs(ref[:, col]).max()
        assert np.abs(got[:, col] - ref[:, col]).max() <= rtol * scale, name
    vt = slice(6, 15)
    assert np.abs(got[1:, vt] - ref[1:, vt]).max() <= rtol * np.abs(ref[1:, vt]).max()
    for key in g.files:
        if key.startswith("pos_"):
            c = int(key[4:])
            if c in rec.snaps and c <= nsteps:
                p, v = rec.snaps[c]
                assert np.abs(p - g[key]).max() <= rtol * 100.0
                assert np.abs(v - g["vel_%d" % c]).max() <= rtol * np.abs(g["vel_%d" % c]).max()


@pytest.mark.parametrize("device", [True, False])
@pytest.mark.parametrize("name", ["md_nve_original", "md_nve_nanocell"])
def test_nve_matches_reference(name, device):
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup(name)
    rec = Rec()
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=[rec.hook], vel0=g["vel0"].copy(), device=device)
    n = 1000 if device else 200
    vi.run(n)
    _compare(g, rec, n, 1e-8)


@pytest.mark.parametrize("device", [True, False])
def test_langevin_replay_matches_reference(device):
    from micmec_gb300.sampling.nvt import LangevinThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup("md_langevin_nanocell")
    rec = Rec()
    lt = LangevinThermostat(float(g["meta/temp"]), timecon=float(g["meta/timecon"]), replay_noise=g["noise"])
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=[lt, rec.hook], vel0=g["vel0"].copy(), device=device)
    vi.run(200)
    _compare(g, rec, 200, 1e-8)


@pytest.mark.parametrize("device", ["batch", "engine", "host"])
def test_nhc_matches_reference(device):
    from micmec_gb300.sampling.nvt import NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup("md_nhc_nanocell")
    rec = Rec()
    t = NHCThermostat(float(g["meta/temp"]), timecon=float(g["meta/timecon"]), chainlength=3,
                      chain_vel0=g["meta/chain_vel0"].copy())
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=[t, rec.hook], vel0=g["vel0"].copy(),
                          device=device != "host")
    if device == "engine":
        vi.batch_max_cells = 0
    vi.run(200)
    _compare(g, rec, 200, 1e-8)
    assert np.allclose(t.chain.pos, g["chain_pos_end"], rtol=1e-7, atol=1e-12)


@pytest.mark.parametrize("device", ["batch", "engine", "host"])
@pytest.mark.parametrize("name", ["md_mtk_nanocell", "md_nhc_mtk_nanocell", "md_langevin_mtk_nanocell"])
def test_mtk_matches_reference(name, device):
    from micmec_gb300.sampling.npt import MTKBarostat
    from micmec_gb300.sampling.nvt import LangevinThermostat, NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup(name)
    rec = Rec()
    T = float(g["meta/temp"])
    hooks = []
    if name == "md_mtk_nanocell":
        hooks.append(MTKBarostat(ff, T, float(g["meta/press"]), timecon=float(g["meta/timecon"]),
                                 vel_press0=g["meta/vel_press0"].copy()))
    elif name == "md_nhc_mtk_nanocell":
        hooks.append(NHCThermostat(T, timecon=float(g["meta/timecon_thermo"]), chainlength=3,
                                   chain_vel0=g["meta/chain_vel0"].copy()))
        hooks.append(MTKBarostat(ff, T, float(g["meta/press"]), timecon=float(g["meta/timecon_baro"]),
                                 vel_press0=g["meta/vel_press0"].copy()))
    else:
        hooks.append(LangevinThermostat(T, timecon=float(g["meta/timecon_thermo"]), replay_noise=g["noise"]))
        hooks.append(MTKBarostat(ff, T, float(g["meta/press"]), timecon=float(g["meta/timecon_baro"]),
                                 vel_press0=g["meta/vel_press0"].copy()))
    n = len(g["records"]) - 1
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=hooks + [rec.hook], vel0=g["vel0"].copy(),
                          device=device != "host")
    if device == "engine":
        vi.batch_max_cells = 0
    vi.run(n)
    _compare(g, rec, n, 1e-7)
    assert np.allclose(s.domain.rvecs, g["rvecs_end"], rtol=1e-9)


BARO_OPTION_NAMES = ["md_mtk_iso_nanocell", "md_nhc_mtk_volc_nanocell", "md_nhc_mtk_bthermo_nanocell",
                     "md_nhc_bbaro_iso_nanocell", "md_nhc_bbaro_volc_nanocell", "md_lbaro_iso_nanocell",
                     "md_nhc_lbaro_volc_nanocell"]


@pytest.mark.parametrize("device,precision", [("batch", "fp64"), ("engine", "fp64"), ("host", "fp64"),
                                              ("batch", "fp32"), ("engine", "fp32")])
@pytest.mark.parametrize("name", BARO_OPTION_NAMES)
def test_barostat_options_match_reference(name, device, precision):
    """The MTK, Berendsen and Langevin barostats isotropic and under a volume constraint, and
    the MTK barostat with a chain of its own."""
    from test_hooks_cpu import hooks_for

    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup(name, precision)
    tol, vtol = (1e-7, 1e-6) if precision == "fp64" else (2e-5, 1e-3)
    rec = Rec()
    n = len(g["records"]) - 1
    hooks = hooks_for(name, g, ff)
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=hooks + [rec.hook], vel0=g["vel0"].copy(),
                          device=device != "host")
    if device == "engine":
        vi.batch_max_cells = 0
    if device != "host":
        assert vi._device_plan()[1]["engine"] == ("batch" if device == "batch" else "lattice")
    vi.run(n)
    _compare(g, rec, n, tol)
    ref = g["rvecs_end"]
    assert np.abs(s.domain.rvecs - ref).max() <= (1e-9 if precision == "fp64" else 1e-7) * np.abs(ref).max()
    baro = hooks[-1]

    def close(a, b, atol):
        a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
        return np.abs(a - b).max() <= vtol * np.abs(b).max() + atol

    if "vel_press_end" in g.files:
        assert close(baro.vel_press, g["vel_press_end"], 1e-14)
    if "chain_pos_end" in g.files:
        assert close(hooks[0].chain.pos, g["chain_pos_end"], 1e-12)
        assert close(hooks[0].chain.vel, g["chain_vel_end"], 1e-14)
    if "baro_chain_pos_end" in g.files:
        assert close(baro.baro_thermo.chain.pos, g["baro_chain_pos_end"], 1e-12)
        assert close(baro.baro_thermo.chain.vel, g["baro_chain_vel_end"], 1e-14)


def _lattice(n, nstates, seed, sigma=0.05):
    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    d = lattices.make_lattice(lattices.defect_grid(n, 0.1, rng), nstates=nstates)
    d["pos"] = lattices.displace(d["pos"], sigma * units.angstrom, rng)
    s = System.from_dict(d)
    kT = units.boltzmann * 300.0
    vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(kT / s.masses)[:, None]
    vel -= (s.masses @ vel) / s.masses.sum()
    return s, vel


def test_fp32_nve_tracks_fp64_and_conserves_energy():
    """FP32 cells / FP64 state vs the FP64 path on a 10^3 two-state lattice, 500 NVE steps."""
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.verlet import VerletIntegrator

    out = {}
    for prec in ("fp64", "fp32"):
        s, vel = _lattice(10, 2, 3)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision=prec)])
        rec = Rec()
        vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=[rec.hook], vel0=vel)
        vi.run(500)
        out[prec] = np.array(rec.rows)
    a, b = out["fp64"], out["fp32"]
    econs64, econs32 = a[:, 3], b[:, 3]
    scale = np.abs(a[:, 2]).max()  # kinetic energy scale
    # conserved quantity: fluctuation relative to the kinetic energy stays small in both
    assert np.ptp(econs64) < 5e-3 * scale
    assert np.ptp(econs32) < 5e-3 * scale
    # short-time trajectories agree
    assert np.abs(a[:50, 1] - b[:50, 1]).max() < 1e-5 * np.abs(a[:50, 1]).max()


def test_langevin_generator_reaches_target_temperature():
    """Philox noise, no replay: the kinetic temperature settles at the thermostat temperature."""
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.nvt import LangevinThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    s, vel = _lattice(12, 2, 4)
    ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision="fp32")])
    rec = Rec()
    lt = LangevinThermostat(600.0, timecon=20 * units.femtosecond, seed=7)
    vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=[lt, rec.hook], vel0=vel)
    vi.run(3000)
    temps = np.array(rec.rows)[1000:, 4]
    assert abs(temps.mean() - 600.0) < 0.05 * 600.0


def test_device_and_host_langevin_paths_agree_with_replayed_noise_fp32():
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.nvt import LangevinThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    rows = {}
    noise = np.random.default_rng(9).normal(size=(2 * 100, 6 ** 3, 3))
    for device in (True, False):
        s, vel = _lattice(6, 2, 5)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision="fp32")])
        rec = Rec()
        lt = LangevinThermostat(300.0, timecon=100 * units.femtosecond, replay_noise=noise)
        vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=[lt, rec.hook], vel0=vel, device=device)
        vi.run(100)
        rows[device] = np.array(rec.rows)
    a, b = rows[True], rows[False]
    for col in (1, 2, 3):
        assert np.abs(a[:, col] - b[:, col]).max() <= 1e-6 * np.abs(b[:, col]).max()


@pytest.mark.parametrize("hooks", ["nhc+mtk", "langevin+mtk", "berendsen+bbaro", "csvr", "nhc+lbaro"])
def test_engine_fp32_tracks_fp64_with_hooks(hooks):
    """Lattice engine with thermostat / barostat hooks (100 MPa): FP32 cells (gather fused into
    the kicks, FP32 increments, compensated FP32 kinetic sums) against FP64 cells, with the same
    generated draws for the stochastic hooks."""
    from micmec_gb300 import units
    from micmec_gb300.sampling.npt import BerendsenBarostat, LangevinBarostat, MTKBarostat
    from micmec_gb300.sampling.nvt import BerendsenThermostat, CSVRThermostat, LangevinThermostat, NHCThermostat
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.verlet import VerletIntegrator

    fs = units.femtosecond
    P = 100e6 * units.pascal
    out = {}
    for prec in ("fp64", "fp32"):
        s, vel = _lattice(10, 2, 5)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision=prec)])
        rec = Rec()
        # fixed initial chain and barostat velocities (by default both are drawn at random)
        nhc = NHCThermostat(300.0, timecon=100 * fs, chain_vel0=np.array([1e-5, -2e-5, 1e-5]))
        hs = {
            "nhc+mtk": lambda: [nhc, MTKBarostat(ff, 300.0, P, timecon=1000 * fs, vel_press0=np.zeros((3, 3)))],
            "langevin+mtk": lambda: [LangevinThermostat(300.0, timecon=100 * fs, seed=3),
                                     MTKBarostat(ff, 300.0, P, timecon=1000 * fs, vel_press0=np.zeros((3, 3)))],
            "berendsen+bbaro": lambda: [BerendsenThermostat(300.0, timecon=100 * fs),
                                        BerendsenBarostat(ff, 300.0, P, timecon=1000 * fs)],
            "csvr": lambda: [CSVRThermostat(300.0, timecon=100 * fs, seed=5)],
            "nhc+lbaro": lambda: [nhc, LangevinBarostat(ff, 300.0, P, timecon=2000 * fs, vel_press0=np.zeros((3, 3)),
                                                        seed=7)],
        }[hooks]()
        vi = VerletIntegrator(ff, 1.0 * fs, hooks=hs + [rec.hook], vel0=vel, device=True)
        vi.batch_max_cells = 0
        assert vi._device_plan()[1]["engine"] == "lattice"
        vi.run(60)
        out[prec] = np.array(rec.rows)
    a, b = out["fp64"], out["fp32"]
    assert np.isfinite(b).all()
    # epot, ekin and the cell volume follow the FP64 run at FP32 precision
    de = np.abs(a[:20, 1] - b[:20, 1]).max() / np.abs(a[:20, 1]).max()
    dk = np.abs(a[:20, 2] - b[:20, 2]).max() / np.abs(a[:20, 2]).max()
    dv = np.abs(a[:, -1] - b[:, -1]).max() / np.abs(a[:, -1]).max()
    assert de < 1e-5 and dk < 1e-5 and dv < 1e-6, (de, dk, dv)


def test_engine_on_lattice_with_vacancies_follows_host_path():
    """Lattice engine with the general topology tables (cells removed from a periodic
    lattice): NHC thermostat, FP64 and FP32 cells, against the host path (FP64)."""
    from micmec_gb300 import lattices, units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.nvt import NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator
    from micmec_gb300.system import System

    rng = np.random.default_rng(21)
    grid = lattices.defect_grid(8, 0.2, rng)
    flat = grid.reshape(-1)
    flat[rng.permutation(flat.size)[:20]] = 0  # vacancies
    d = lattices.make_lattice(grid, nstates=2)
    d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
    kT = units.boltzmann * 300.0
    s0 = System.from_dict(d)
    vel = rng.normal(0.0, 1.0, s0.pos.shape) * np.sqrt(kT / s0.masses)[:, None]
    out = {}
    for route, prec in (("host", "fp64"), ("engine", "fp64"), ("engine", "fp32")):
        s = System.from_dict(d)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision=prec)])
        rec = Rec()
        t = NHCThermostat(300.0, timecon=100 * units.femtosecond, chain_vel0=np.array([1e-5, -2e-5, 1e-5]))
        vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=[t, rec.hook], vel0=vel.copy(),
                              device=(route == "engine"))
        vi.batch_max_cells = 0
        vi.run(30)
        out[route, prec] = np.array(rec.rows)
    h, e64, e32 = out["host", "fp64"], out["engine", "fp64"], out["engine", "fp32"]
    for col in (1, 2, 3):  # epot, ekin, econs
        scale = np.abs(h[:, col]).max()
        assert np.abs(e64[:, col] - h[:, col]).max() <= 1e-9 * scale
        assert np.abs(e32[:, col] - h[:, col]).max() <= 1e-5 * scale


HOOK_NAMES = ["md_berendsen_nanocell", "md_csvr_nanocell", "md_berendsen_mtk_nanocell", "md_nhc_bbaro_nanocell",
              "md_lbaro_nanocell", "md_nhc_lbaro_nanocell"]


@pytest.mark.parametrize("device", ["batch", "engine", "host"])
@pytest.mark.parametrize("name", HOOK_NAMES)
def test_hooks_match_reference(name, device):
    """Berendsen / CSVR thermostats and Berendsen / Langevin barostats on the device paths."""
    from test_hooks_cpu import hooks_for

    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup(name)
    rec = Rec()
    n = len(g["records"]) - 1
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=hooks_for(name, g, ff) + [rec.hook], vel0=g["vel0"].copy(),
                          device=device != "host")
    if device == "engine":
        vi.batch_max_cells = 0
    if device != "host":
        assert vi._device_plan()[1]["engine"] == ("batch" if device == "batch" else "lattice")
    vi.run(n)
    _compare(g, rec, n, 1e-7)
    assert np.allclose(s.domain.rvecs, g["rvecs_end"], rtol=1e-9)
    if "chain_pos_end" in g.files:
        hook = [h for h in vi.hooks if hasattr(h, "thermostat")][0]
        assert np.allclose(hook.thermostat.chain.pos, g["chain_pos_end"], rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("hooks", ["csvr", "nhc_lbaro"])
def test_generated_hook_draws_agree_between_batch_and_engine(hooks):
    """Without replay, the batch kernel and the lattice engine draw the same CSVR and
    Langevin-barostat numbers (the same generator stream keyed by system, step and call)."""
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.npt import LangevinBarostat
    from micmec_gb300.sampling.nvt import CSVRThermostat, NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    rows = {}
    for engine in ("batch", "lattice"):
        s, vel = _lattice(4, 2, 12)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision="fp64")])
        if hooks == "csvr":
            hs = [CSVRThermostat(600.0, timecon=50 * units.femtosecond, seed=11)]
        else:
            hs = [NHCThermostat(300.0, timecon=100 * units.femtosecond, chain_vel0=np.zeros(3)),
                  LangevinBarostat(ff, 300.0, 1e8 * units.pascal, timecon=2000 * units.femtosecond,
                                   vel_press0=np.zeros((3, 3)), seed=11)]
        rec = Rec()
        vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=hs + [rec.hook], vel0=vel, device=True)
        if engine == "lattice":
            vi.batch_max_cells = 0
        assert vi._device_plan()[1]["engine"] == engine
        vi.run(60)
        rows[engine] = np.array(rec.rows)
    a, b = rows["batch"], rows["lattice"]
    assert np.isfinite(a).all()
    for col in (1, 2, 3):
        assert np.abs(a[:, col] - b[:, col]).max() <= 1e-7 * np.abs(b[:, col]).max()


def test_csvr_generator_samples_canonical_kinetic_energy():
    """CSVR with the device generator (normal R, chi-squared S by Marsaglia-Tsang): the
    kinetic energy follows the canonical Gamma(ndof/2, kT) law in mean and variance."""
    from micmec_gb300 import units
    from micmec_gb300.batch import REC, BatchSystems

    systems = [_lattice(4, 1, 20 + i)[0] for i in range(48)]
    b = BatchSystems(systems, model="nanocell", precision="fp64")
    T = 600.0
    b.setup_md(temp=300.0, thermostat="csvr", seed=3)
    rec = b.md(4000, timestep=1.0 * units.femtosecond, thermostat="csvr", temp=T,
               timecon=50 * units.femtosecond, seed=5, record=True)
    ndof = 3 * systems[0].nnodes - 3
    kT = units.boltzmann * T
    ek = rec[:, 1000:, REC["ekin"]].ravel()
    assert abs(ek.mean() / (0.5 * ndof * kT) - 1.0) < 0.02
    assert abs(ek.var() / (0.5 * ndof * kT ** 2) - 1.0) < 0.15


def test_device_writers_run_on_snapshots_while_the_gpu_steps(tmp_path):
    """Writers (read-only hooks) run on pinned snapshots while the next chunk steps; their
    records equal those of a run whose hooks force synchronous chunks."""
    from micmec_gb300 import h5lite, units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.iterative import Hook
    from micmec_gb300.sampling.nvt import LangevinThermostat
    from micmec_gb300.sampling.trajectory import HDF5Writer, XYZWriter
    from micmec_gb300.sampling.verlet import VerletIntegrator

    noise = np.random.default_rng(4).normal(size=(2 * 60, 6 ** 3, 3))

    class Touch(Hook):  # may modify the state (the default): chunks run synchronously
        def __call__(self, it):
            pass

    out = {}
    for mode in ("overlap", "sync"):
        s, vel = _lattice(6, 2, 5)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision="fp64")])
        f = h5lite.File(str(tmp_path / ("%s.h5" % mode)), "w")
        xyz = XYZWriter(str(tmp_path / ("%s.xyz" % mode)), step=10)
        hooks = [LangevinThermostat(300.0, timecon=100 * units.femtosecond, replay_noise=noise),
                 HDF5Writer(f, step=10), xyz]
        if mode == "sync":
            hooks.append(Touch(0, 10))
        vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=hooks, vel0=vel)
        assert vi._hooks_read_only(10) == (mode == "overlap")
        vi.run(60)
        f.close()
        xyz.close()
        with h5lite.File(str(tmp_path / ("%s.h5" % mode)), "r") as h:
            out[mode] = {k: np.array(h["trajectory/" + k][:]) for k in ("counter", "pos", "vel", "epot", "econs")}
        out[mode]["xyz"] = open(str(tmp_path / ("%s.xyz" % mode))).read()
    a, b = out["overlap"], out["sync"]
    assert list(a["counter"]) == [0, 10, 20, 30, 40, 50, 60]
    for k in ("counter", "pos", "vel", "epot", "econs"):
        assert np.array_equal(a[k], b[k]), k
    assert a["xyz"] == b["xyz"]


def test_state_changes_by_hooks_reach_the_device_path():
    """A hook that changes the velocities between device chunks: the device path continues
    from the changed state, as the host path does."""
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.iterative import Hook
    from micmec_gb300.sampling.verlet import VerletIntegrator

    class Cool(Hook):
        def __call__(self, it):
            it.vel[:] *= 0.5

    rows = {}
    for device in (True, False):
        s, vel = _lattice(5, 2, 6)
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision="fp64")])
        rec = Rec()
        vi = VerletIntegrator(ff, 1.0 * units.femtosecond, hooks=[Cool(20, 1000), rec.hook], vel0=vel, device=device)
        vi.run(40)
        rows[device] = np.array(rec.rows)
    a, b = rows[True], rows[False]
    assert a[30, 2] < 0.6 * a[19, 2]  # the cooling took effect
    for col in (1, 2):
        assert np.abs(a[:, col] - b[:, col]).max() <= 1e-9 * np.abs(b[:, col]).max()
