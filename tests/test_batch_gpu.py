"""Batched persistent kernel: reference trajectories, relaxation, precision, autotuning, graphs."""
import numpy as np
import pytest

from conftest import load_golden, make_system, system_dict

pytestmark = pytest.mark.gpu


def _golden_batch(name, copies=1, precision="fp64"):
    from micmec_gb300.batch import BatchSystems

    g = load_golden(name)
    systems = [make_system(system_dict(g, "sys/")) for _ in range(copies)]
    return g, BatchSystems(systems, model=str(g["model"]), precision=precision)


def _check(g, rec, n, rtol):
    from micmec_gb300.batch import REC

    ref = g["records"][1: n + 1]
    econs = rec[:, REC["epot"]] + rec[:, REC["ekin"]] + rec[:, REC["ecorr"]]
    for got, col in ((rec[:, REC["epot"]], 1), (rec[:, REC["ekin"]], 2), (econs, 3)):
        assert np.abs(got - ref[:, col]).max() <= rtol * np.abs(ref[:, col]).max(), col
    vt = rec[:, REC["vtens"]]
    assert np.abs(vt - ref[:, 6:15]).max() <= rtol * np.abs(ref[:, 6:15]).max()
    vol = rec[:, REC["volume"]]
    assert np.abs(vol - ref[:, -1]).max() <= rtol * ref[:, -1].max()


def test_batch_nve_matches_reference_in_every_copy():
    g, b = _golden_batch("md_nve_nanocell", copies=3)
    b.setup_md(vel=[g["vel0"]] * 3, thermostat=None)
    rec = b.md(1000, timestep=float(g["timestep"]), record=True, use_graph=False)
    for i in range(3):
        _check(g, rec[i], 1000, 1e-8)
    pos, vel, _ = b.get_state()
    assert np.abs(pos[1] - g["pos_1000"]).max() < 1e-6


def test_batch_langevin_replay_matches_reference():
    g, b = _golden_batch("md_langevin_nanocell")
    b.setup_md(vel=[g["vel0"]], thermostat="langevin", temp=float(g["meta/temp"]))
    noise = g["noise"].reshape(200, 2, -1, 3)
    rec = b.md(200, timestep=float(g["timestep"]), thermostat="langevin", temp=float(g["meta/temp"]),
               timecon=float(g["meta/timecon"]), noise=noise, record=True)
    _check(g, rec[0], 200, 1e-8)


def test_batch_nhc_matches_reference():
    g, b = _golden_batch("md_nhc_nanocell")
    T, tau = float(g["meta/temp"]), float(g["meta/timecon"])
    b.setup_md(vel=[g["vel0"]], thermostat="nhc", temp=T, timecon=tau, chain_vel0=[g["meta/chain_vel0"]])
    rec = b.md(200, timestep=float(g["timestep"]), thermostat="nhc", temp=T, timecon=tau, record=True)
    _check(g, rec[0], 200, 1e-8)
    from micmec_gb300.batch import CTL

    assert np.allclose(b.control()[0, CTL["chain_pos"]], g["chain_pos_end"], rtol=1e-7, atol=1e-12)


@pytest.mark.parametrize("name", ["md_mtk_nanocell", "md_nhc_mtk_nanocell", "md_langevin_mtk_nanocell"])
def test_batch_mtk_matches_reference(name):
    g, b = _golden_batch(name)
    T, P = float(g["meta/temp"]), float(g["meta/press"])
    n = len(g["records"]) - 1
    if name == "md_mtk_nanocell":
        thermo, tt, tb = None, 100.0, float(g["meta/timecon"])
    else:
        thermo = "nhc" if "nhc" in name else "langevin"
        tt, tb = float(g["meta/timecon_thermo"]), float(g["meta/timecon_baro"])
    chain0 = [g["meta/chain_vel0"]] if thermo == "nhc" else None
    b.setup_md(vel=[g["vel0"]], thermostat=thermo, temp=T, timecon=tt, chain_vel0=chain0, barostat="mtk",
               baro_timecon=tb, vel_press0=[g["meta/vel_press0"]])
    noise = g["noise"].reshape(n, 2, -1, 3) if thermo == "langevin" else None
    rec = b.md(n, timestep=float(g["timestep"]), thermostat=thermo, temp=T, timecon=tt, barostat="mtk", press=P,
               noise=noise, record=True)
    _check(g, rec[0], n, 1e-7)
    _, _, rv = b.get_state()
    assert np.allclose(rv[0], g["rvecs_end"], rtol=1e-9)


@pytest.mark.parametrize("name", ["md_mtk_iso_nanocell", "md_nhc_mtk_volc_nanocell", "md_nhc_mtk_bthermo_nanocell"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_mtk_options_match_reference(name, precision):
    """setup_md / md with the MTK barostat's options, in two copies of the system."""
    from micmec_gb300.batch import CTL

    g, b = _golden_batch(name, copies=2, precision=precision)
    rtol = 1e-7 if precision == "fp64" else 2e-5
    T, P = float(g["meta/temp"]), float(g["meta/press"])
    n = len(g["records"]) - 1
    opts = {}
    if name == "md_mtk_iso_nanocell":
        thermo, tt, tb, chain0 = None, 100.0, float(g["meta/timecon"]), None
        opts["anisotropic"] = False
        vp0 = float(g["meta/vel_press0"])
    else:
        thermo, tt, tb = "nhc", float(g["meta/timecon_thermo"]), float(g["meta/timecon_baro"])
        chain0 = [g["meta/chain_vel0"]] * 2
        vp0 = g["meta/vel_press0"]
        if "volc" in name:
            opts["vol_constraint"] = True
        else:
            opts.update(baro_chainlength=3, baro_chain_timecon=float(g["meta/timecon_baro_thermo"]),
                        baro_chain_vel0=g["meta/baro_chain_vel0"])
    b.setup_md(vel=[g["vel0"]] * 2, thermostat=thermo, temp=T, timecon=tt, chain_vel0=chain0, barostat="mtk",
               baro_timecon=tb, vel_press0=vp0, **opts)
    rec = b.md(n, timestep=float(g["timestep"]), thermostat=thermo, temp=T, timecon=tt,
               barostat=b.hooks["barostat"], press=P, record=True)
    for i in range(2):
        _check(g, rec[i], n, rtol)
    _, _, rv = b.get_state()
    assert np.abs(rv[1] - g["rvecs_end"]).max() <= (1e-9 if precision == "fp64" else 1e-7) * np.abs(g["rvecs_end"]).max()
    c = b.control()[1]
    vp = c[CTL["vel_press"]]
    vtol = 1e-6 if precision == "fp64" else 1e-3  # the barostat velocity integrates the FP32 virial
    if "iso" in name:
        assert np.allclose(vp[0], g["vel_press_end"], rtol=vtol) and not vp[1:].any()
    else:
        ref = g["vel_press_end"]
        assert np.abs(vp.reshape(3, 3) - ref).max() <= vtol * np.abs(ref).max()
    if "bthermo" in name:
        assert np.allclose(c[CTL["bchain_pos"]], g["baro_chain_pos_end"], rtol=vtol, atol=1e-12)


@pytest.mark.parametrize("name", ["md_nhc_bbaro_iso_nanocell", "md_nhc_bbaro_volc_nanocell", "md_lbaro_iso_nanocell",
                                  "md_nhc_lbaro_volc_nanocell"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_berendsen_langevin_barostat_options_match_reference(name, precision):
    """setup_md / md with the Berendsen and Langevin barostats isotropic or volume-constrained."""
    from micmec_gb300.batch import HOOK_NOISE_LEN

    g, b = _golden_batch(name, precision=precision)
    T, P = float(g["meta/temp"]), float(g["meta/press"])
    n = len(g["records"]) - 1
    baro = "berendsen" if "bbaro" in name else "langevin"
    thermo = "nhc" if "nhc" in name else None
    tt = float(g["meta/timecon_thermo"]) if thermo else 100.0
    tb = float(g["meta/timecon_baro"]) if thermo else float(g["meta/timecon"])
    opts = {"anisotropic": False} if "iso" in name else {"vol_constraint": True}
    vp0 = None
    if baro == "langevin":
        vp0 = g["vel_press0"] if "volc" in name else float(g["vel_press0"])
    chain0 = [g["meta/chain_vel0"]] if thermo else None
    b.setup_md(vel=[g["vel0"]], thermostat=thermo, temp=T, timecon=tt, chain_vel0=chain0, barostat=baro,
               baro_timecon=tb, vel_press0=vp0, **opts)
    hook = None
    if baro == "langevin":
        hook = np.zeros((n, 1, HOOK_NOISE_LEN))
        hook[:, 0, 2:26] = g["baro_noise"][:n].reshape(n, 24)
    rec = b.md(n, timestep=float(g["timestep"]), thermostat=thermo, temp=T, timecon=tt,
               barostat=b.hooks["barostat"], press=P, hook_noise=hook, record=True)
    _check(g, rec[0], n, 1e-7 if precision == "fp64" else 2e-5)
    _, _, rv = b.get_state()
    ref = g["rvecs_end"]
    assert np.abs(rv[0] - ref).max() <= (1e-9 if precision == "fp64" else 1e-7) * np.abs(ref).max()


@pytest.mark.parametrize("name", ["md_berendsen_nanocell", "md_csvr_nanocell", "md_berendsen_mtk_nanocell",
                                  "md_nhc_bbaro_nanocell", "md_lbaro_nanocell", "md_nhc_lbaro_nanocell"])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_hooks_match_reference(name, precision):
    """Berendsen / CSVR thermostats, Berendsen / Langevin barostats through the batch API
    (hook constants from setup_md, replayed draws as hook noise)."""
    from micmec_gb300.batch import HOOK_NOISE_LEN

    g, b = _golden_batch(name, precision=precision)
    T = float(g["meta/temp"])
    n = len(g["records"]) - 1
    tag = name[3:-9]
    thermo = {"berendsen": "berendsen", "csvr": "csvr", "berendsen_mtk": "berendsen", "nhc_bbaro": "nhc",
              "lbaro": None, "nhc_lbaro": "nhc"}[tag]
    baro = {"berendsen": None, "csvr": None, "berendsen_mtk": "mtk", "nhc_bbaro": "berendsen", "lbaro": "langevin",
            "nhc_lbaro": "langevin"}[tag]
    tt = float(g["meta/timecon_thermo"]) if "meta/timecon_thermo" in g.files else float(g["meta/timecon"])
    tb = float(g["meta/timecon_baro"]) if "meta/timecon_baro" in g.files else float(g["meta/timecon"])
    P = float(g["meta/press"]) if baro else 0.0
    vp0 = None
    if baro == "mtk":
        vp0 = [g["meta/vel_press0"]]
    elif baro == "langevin":
        vp0 = [g["vel_press0"]]
    chain0 = [g["meta/chain_vel0"]] if thermo == "nhc" else None
    b.setup_md(vel=[g["vel0"]], thermostat=thermo, temp=T, timecon=tt, chain_vel0=chain0, barostat=baro,
               baro_timecon=tb, vel_press0=vp0)
    hook = None
    if thermo == "csvr" or baro == "langevin":
        hook = np.zeros((n, 1, HOOK_NOISE_LEN))
        if thermo == "csvr":
            hook[:, 0, 0:2] = g["csvr_noise"][:n]
        if baro == "langevin":
            hook[:, 0, 2:26] = g["baro_noise"][:n].reshape(n, 24)
    rec = b.md(n, timestep=float(g["timestep"]), thermostat=thermo, temp=T, timecon=tt, barostat=baro, press=P,
               hook_noise=hook, record=True)
    _check(g, rec[0], n, 1e-7 if precision == "fp64" else 2e-5)
    _, _, rv = b.get_state()
    ref = g["rvecs_end"]
    assert np.abs(rv[0] - ref).max() <= (1e-9 if precision == "fp64" else 1e-7) * np.abs(ref).max()


def _mixed_batch(ns, precision, seed=0, sigma=0.1, strains=None):
    from micmec_gb300 import lattices, units
    from micmec_gb300.batch import BatchSystems
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    systems = []
    for i, n in enumerate(ns):
        d = lattices.make_lattice(lattices.defect_grid(n, 0.2, rng), nstates=2)
        if strains is not None:
            F = np.eye(3)
            F[0, 0] += strains[i]
            d["pos"] = d["pos"] @ F
            d["rvecs"] = d["rvecs"] @ F
        d["pos"] = lattices.displace(d["pos"], sigma * units.angstrom, rng)
        systems.append(System.from_dict(d))
    return systems, BatchSystems(systems, model="nanocell", precision=precision)


def test_batch_relax_reaches_tolerance_and_matches_single_system_forces():
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    systems, b = _mixed_batch([3, 4, 5, 6], "fp64", strains=[0.0, 0.01, 0.02, 0.03])
    e0 = [MicMecForceField(s, [ForcePartMechanical(s)]).compute() for s in systems]
    gmax, iters = b.relax(max_iter=3000, gtol=1e-7)
    assert (gmax < 1e-7).all(), (gmax, iters)
    pos, _, rv = b.get_state()
    e_batch = b.energies()
    for i, s in enumerate(systems):
        s.pos[:] = pos[i]
        ff = MicMecForceField(s, [ForcePartMechanical(s)])
        gp = np.zeros((s.nnodes, 3))
        e = ff.compute(gp)
        assert e < e0[i]
        assert abs(e - e_batch[i]) <= 1e-10 * abs(e)
        assert np.sqrt((gp**2).sum(axis=1)).max() < 1e-7


def test_batch_fp32_tracks_fp64_with_replayed_noise():
    from micmec_gb300.batch import REC

    recs = {}
    ns = [3, 5, 7, 4]
    for prec in ("fp64", "fp32"):
        systems, b = _mixed_batch(ns, prec, seed=3)
        N = int(b.offsets[-1])
        noise = np.random.default_rng(5).normal(size=(50, 2, N, 3))
        b.setup_md(temp=300.0, thermostat="langevin", seed=11)
        recs[prec] = b.md(50, thermostat="langevin", temp=300.0, noise=noise, record=True)
    a, f = recs["fp64"], recs["fp32"]
    for i in range(len(ns)):
        for col in (REC["epot"], REC["ekin"]):
            assert np.abs(a[i, :, col] - f[i, :, col]).max() <= 1e-5 * np.abs(a[i, :, col]).max()


def test_autotune_and_graph_replay_keep_results():
    from micmec_gb300.batch import REC

    systems, b = _mixed_batch([3, 6, 4, 8, 5, 3, 7], "fp32", seed=4)
    b.setup_md(temp=300.0, thermostat=None, seed=2)
    pos0, vel0, rv0 = b.get_state()
    ref = b.md(20, record=True, use_graph=False)
    cfg = b.autotune(probe_steps=3)
    assert cfg["cta_threads"] in (128, 256) and cfg["ctas"] >= 1
    for use_graph in (True, True, False):
        b.set_state(pos0, vel0, rv0)
        got = b.md(20, record=True, use_graph=use_graph)
        for col in (REC["epot"], REC["ekin"]):
            assert np.abs(got[:, :, col] - ref[:, :, col]).max() <= 1e-6 * np.abs(ref[:, :, col]).max()


@pytest.mark.parametrize("kind", ["strain", "full"])
def test_batch_cell_relax_reaches_reference_minimum(kind):
    """Positions and domain relaxed together (StrainCellDOF / FullCellDOF) reach the minimum
    the reference's QNOptimizer found from the same start (energy, domain metric, stress)."""
    g, b = _golden_batch("opt_cell_%s_nanocell" % kind, copies=2)
    d = system_dict(g, "sys/")
    b.set_state([d["pos"]] * 2, None, [d["rvecs"]] * 2)
    gmax, iters = b.relax(max_iter=3000, gtol=1e-7, cell=kind, stress_tol=1e-11)
    assert (gmax < 1e-7).all() and (b.residual_stress() < 1e-11).all(), (gmax, iters)
    E = b.energies()
    assert np.abs(E - float(g["epot_end"])).max() <= 1e-10 * abs(float(g["epot_end"]))
    _, _, rv = b.get_state()
    ref = g["rvecs_end"]
    for r in rv:
        if kind == "strain":
            assert np.abs(r - ref).max() <= 1e-6 * np.abs(ref).max()
        else:  # a rigid rotation of the domain is a zero mode: compare the metric
            assert np.abs(r @ r.T - ref @ ref.T).max() <= 2e-6 * np.abs(ref @ ref.T).max()


def test_batch_cell_relax_under_pressure_and_fp32():
    """At 1 GPa the relaxed domain shrinks and the residual stress vtens / V + P I vanishes;
    FP32 cells reach the FP64 minimum to the FP32 force resolution."""
    from micmec_gb300 import units
    from micmec_gb300.batch import CTL

    P = 1e9 * units.pascal
    out = {}
    for prec in ("fp64", "fp32"):
        systems, b = _mixed_batch([3, 4, 5], prec, seed=8, sigma=0.05)
        vol0 = b.control()[:, CTL["volume"]].copy()
        gmax, iters = b.relax(max_iter=4000, gtol=1e-6 if prec == "fp64" else 1e-4, cell="strain", press=P,
                              stress_tol=1e-10 if prec == "fp64" else 1e-8)
        c = b.control()
        out[prec] = (c[:, CTL["epot"]] + P * c[:, CTL["volume"]], c[:, CTL["volume"]])
        if prec == "fp64":
            assert (gmax < 1e-6).all(), (gmax, iters)
            assert (b.residual_stress() < 1e-10).all()
            assert (c[:, CTL["volume"]] < vol0).all()
            for i in range(len(systems)):
                vt = c[i, CTL["vtens"]].reshape(3, 3) / c[i, CTL["volume"]] + P * np.eye(3)
                assert np.abs(vt).max() < 1e-10
    h64, v64 = out["fp64"]
    h32, v32 = out["fp32"]
    assert np.abs(h32 - h64).max() <= 1e-5 * np.abs(h64).max()
    assert np.abs(v32 / v64 - 1).max() < 1e-4


def test_batch_set_params_matches_single_system_with_the_same_parameters():
    """mm_batch_set_params: a batch evaluated with replaced tables gives the energy and
    stress of a single-system handle carrying the same parameters (mm_set_params)."""
    import torch

    from micmec_gb300.autograd import MicMecParameters
    from micmec_gb300.batch import BatchSystems
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    systems, _ = _mixed_batch([4], "fp64", seed=9, sigma=0.05)
    s = systems[0]
    part = ForcePartMechanical(s, model="nanocell", precision="fp64")
    ff = MicMecForceField(s, [part])
    params = MicMecParameters(part)
    with torch.no_grad():
        params.c21.mul_(1.1)
        params.h0.mul_(1.002)
        params.free_energy.add_(1e-4)
    params.upload(*params.tensors())
    vt = np.zeros((3, 3))
    e_part = ff.compute(None, vt)
    b = BatchSystems([s], model="nanocell", precision="fp64")
    C, H, D = params.native_tables(*params.tensors())
    b.set_params(H, C, D, params.temp, params.nstates)
    b.set_state([s.pos], None, [s.domain.rvecs])
    b.relax(max_iter=0, gtol=1e-3)  # one force evaluation, no step
    assert abs(b.energies()[0] - e_part) <= 1e-11 * abs(e_part)
    assert np.abs(b.stress()[0] - vt / s.domain.volume).max() <= 1e-10 * np.abs(vt / s.domain.volume).max()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
def test_batch_original_model_matches_single_system_path(precision, tol):
    """The averaged-matrix model (the one the reference's mmff.py imports) in the batch kernel:
    energy and stress of uneven systems equal those of ForcePartMechanical(model="original")."""
    from micmec_gb300.batch import BatchSystems
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    systems, _ = _mixed_batch([3, 5, 9, 4], "fp64", seed=12)
    b = BatchSystems(systems, model="original", precision=precision)
    b.relax(max_iter=0, gtol=1e-3)  # one force evaluation, no step
    E, W = b.energies(), b.stress()
    for i, s in enumerate(systems):
        vt = np.zeros((3, 3))
        e = MicMecForceField(s, [ForcePartMechanical(s, model="original", precision="fp64")]).compute(None, vt)
        assert abs(E[i] - e) <= tol * abs(e)
        ref = vt / s.domain.volume
        assert np.abs(W[i] - ref).max() <= tol * np.abs(ref).max()
