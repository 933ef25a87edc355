"""Host thermostat / barostat hooks against the reference's trajectories, without a GPU.

The force field is the NumPy oracle (``oracle/mmff.py``) behind the ``ForcePart``
interface, so the hook classes of ``micmec_gb300.sampling`` run their host path on the
CPU. The golden files hold the reference's per-step records for every thermostat and
barostat ``TBCombination`` accepts (alone and combined), the CSVR and the GLE thermostats;
the stochastic hooks replay the reference's recorded draws.
"""
import numpy as np
import pytest

from conftest import load_golden, make_system, system_dict
from oracle import mmff as om


def _oracle_ff(g):
    from micmec_gb300.pes.mmff import ForcePart, MicMecForceField

    d = system_dict(g, "sys/")
    s = make_system(d)
    model = str(g["model"])

    class OraclePart(ForcePart):
        def __init__(self, system):
            ForcePart.__init__(self, "oracle", system)
            self.sys = system

        def _internal_compute(self, gpos, vtens):
            d["pos"] = self.sys.pos
            d["rvecs"] = self.sys.domain.rvecs
            e, gp, vt = om.compute(d, model)
            if gpos is not None:
                gpos += gp
            if vtens is not None:
                vtens += vt
            return e

    return s, MicMecForceField(s, [OraclePart(s)])


class Rows(object):
    def __init__(self):
        from micmec_gb300.sampling.iterative import Hook

        rows = self.rows = []

        class H(Hook):
            def __call__(self, it):
                rows.append([it.counter, it.epot, it.ekin, it.econs] + list(np.asarray(it.vtens).ravel())
                            + list(np.asarray(it.mmf.system.domain.rvecs).ravel()))

        self.hook = H(0, 1)


def hooks_for(name, g, ff):
    """The hooks of golden run ``name``, built from its stored constants and draws."""
    from micmec_gb300.sampling.npt import BerendsenBarostat, LangevinBarostat, MTKBarostat
    from micmec_gb300.sampling.nvt import BerendsenThermostat, CSVRThermostat, LangevinThermostat, NHCThermostat

    T = float(g["meta/temp"])
    if name == "md_andersen_nanocell":
        from micmec_gb300.sampling.nvt import AndersenThermostat

        return [AndersenThermostat(T, step=int(g["meta/step"]), select=np.arange(0, 27, 2),
                                   annealing=float(g["meta/annealing"]))]
    if name == "md_gle_nanocell":
        from micmec_gb300.sampling.nvt import GLEThermostat

        return [GLEThermostat(T, g["meta/a_p"], replay_noise=[g["gle_s0"]] + list(g["gle_noise"]))]
    if name == "md_langevin_nanocell":
        return [LangevinThermostat(T, timecon=float(g["meta/timecon"]), replay_noise=g["noise"])]
    if name == "md_nhc_nanocell":
        return [NHCThermostat(T, timecon=float(g["meta/timecon"]), chainlength=3,
                              chain_vel0=g["meta/chain_vel0"].copy())]
    if name == "md_mtk_nanocell":
        return [MTKBarostat(ff, T, float(g["meta/press"]), timecon=float(g["meta/timecon"]),
                            vel_press0=g["meta/vel_press0"].copy())]
    if name == "md_berendsen_nanocell":
        return [BerendsenThermostat(T, timecon=float(g["meta/timecon"]))]
    if name == "md_csvr_nanocell":
        return [CSVRThermostat(T, timecon=float(g["meta/timecon"]), replay_noise=g["csvr_noise"])]
    press = float(g["meta/press"])
    if name == "md_lbaro_nanocell":
        return [LangevinBarostat(ff, T, press, timecon=float(g["meta/timecon"]), vel_press0=g["vel_press0"],
                                 replay_noise=g["baro_noise"])]
    if name == "md_lbaro_iso_nanocell":
        return [LangevinBarostat(ff, T, press, timecon=float(g["meta/timecon"]), anisotropic=False,
                                 vel_press0=g["vel_press0"], replay_noise=g["baro_noise"])]
    if name == "md_mtk_iso_nanocell":
        return [MTKBarostat(ff, T, press, timecon=float(g["meta/timecon"]), anisotropic=False,
                            vel_press0=float(g["meta/vel_press0"]))]
    tb, tt = float(g["meta/timecon_baro"]), float(g["meta/timecon_thermo"])
    if name == "md_langevin_mtk_nanocell":
        return [LangevinThermostat(T, timecon=tt, replay_noise=g["noise"]),
                MTKBarostat(ff, T, press, timecon=tb, vel_press0=g["meta/vel_press0"].copy())]
    if name == "md_berendsen_mtk_nanocell":
        return [BerendsenThermostat(T, timecon=tt), MTKBarostat(ff, T, press, timecon=tb,
                                                                vel_press0=g["meta/vel_press0"].copy())]
    nhc = NHCThermostat(T, timecon=tt, chainlength=3, chain_vel0=g["meta/chain_vel0"].copy())
    if name == "md_nhc_mtk_nanocell":
        return [nhc, MTKBarostat(ff, T, press, timecon=tb, vel_press0=g["meta/vel_press0"].copy())]
    if name == "md_nhc_mtk_volc_nanocell":
        return [nhc, MTKBarostat(ff, T, press, timecon=tb, vol_constraint=True,
                                 vel_press0=g["meta/vel_press0"].copy())]
    if name == "md_nhc_mtk_bthermo_nanocell":
        bt = NHCThermostat(T, timecon=float(g["meta/timecon_baro_thermo"]), chainlength=3,
                           chain_vel0=g["meta/baro_chain_vel0"].copy())
        return [nhc, MTKBarostat(ff, T, press, timecon=tb, baro_thermo=bt, vel_press0=g["meta/vel_press0"].copy())]
    if name == "md_nhc_bbaro_nanocell":
        return [nhc, BerendsenBarostat(ff, T, press, timecon=tb)]
    if name == "md_nhc_bbaro_iso_nanocell":
        return [nhc, BerendsenBarostat(ff, T, press, timecon=tb, anisotropic=False)]
    if name == "md_nhc_bbaro_volc_nanocell":
        return [nhc, BerendsenBarostat(ff, T, press, timecon=tb, vol_constraint=True)]
    if name == "md_nhc_lbaro_volc_nanocell":
        return [nhc, LangevinBarostat(ff, T, press, timecon=tb, vol_constraint=True, vel_press0=g["vel_press0"],
                                      replay_noise=g["baro_noise"])]
    if name == "md_nhc_lbaro_nanocell":
        return [nhc, LangevinBarostat(ff, T, press, timecon=tb, vel_press0=g["vel_press0"],
                                      replay_noise=g["baro_noise"])]
    raise KeyError(name)


NAMES = ["md_langevin_nanocell", "md_nhc_nanocell", "md_mtk_nanocell", "md_nhc_mtk_nanocell",
         "md_langevin_mtk_nanocell", "md_berendsen_nanocell", "md_csvr_nanocell", "md_berendsen_mtk_nanocell",
         "md_nhc_bbaro_nanocell", "md_lbaro_nanocell", "md_nhc_lbaro_nanocell", "md_gle_nanocell",
         "md_andersen_nanocell", "md_mtk_iso_nanocell", "md_nhc_mtk_volc_nanocell", "md_nhc_mtk_bthermo_nanocell",
         "md_nhc_bbaro_iso_nanocell", "md_nhc_bbaro_volc_nanocell", "md_lbaro_iso_nanocell", "md_nhc_lbaro_volc_nanocell"]


@pytest.mark.parametrize("name", NAMES)
def test_host_hooks_match_reference(name):
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g = load_golden(name)
    s, ff = _oracle_ff(g)
    rows = Rows()
    n = len(g["records"]) - 1
    hooks = hooks_for(name, g, ff)
    if "meta/np_random_seed" in g.files:  # draws from np.random, seeded as the reference run was
        np.random.seed(int(g["meta/np_random_seed"]))
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=hooks + [rows.hook], vel0=g["vel0"].copy(),
                          device=False)
    vi.run(n)
    ref = g["records"][: n + 1]
    got = np.array(rows.rows)
    assert got.shape[0] == n + 1
    for col in (1, 2, 3):  # epot, ekin, econs
        assert np.abs(got[:, col] - ref[:, col]).max() <= 1e-9 * np.abs(ref[:, col]).max()
    assert np.abs(got[:, 4:13] - ref[:, 6:15]).max() <= 1e-9 * np.abs(ref[:, 6:15]).max()  # virial
    assert np.abs(got[:, 13:22] - ref[:, 24:33]).max() <= 1e-12 * np.abs(ref[:, 24:33]).max()  # domain
