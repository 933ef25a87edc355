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


def test_nhc_matches_reference():
    from micmec_gb300.sampling.nvt import NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g, s, ff = _setup("md_nhc_nanocell")
    rec = Rec()
    t = NHCThermostat(float(g["meta/temp"]), timecon=float(g["meta/timecon"]), chainlength=3,
                      chain_vel0=g["meta/chain_vel0"].copy())
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=[t, rec.hook], vel0=g["vel0"].copy())
    vi.run(200)
    _compare(g, rec, 200, 1e-8)
    assert np.allclose(t.chain.pos, g["chain_pos_end"], rtol=1e-7, atol=1e-12)


@pytest.mark.parametrize("name", ["md_mtk_nanocell", "md_nhc_mtk_nanocell", "md_langevin_mtk_nanocell"])
def test_mtk_matches_reference(name):
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
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=hooks + [rec.hook], vel0=g["vel0"].copy())
    vi.run(n)
    _compare(g, rec, n, 1e-7)
    assert np.allclose(s.domain.rvecs, g["rvecs_end"], rtol=1e-9)
