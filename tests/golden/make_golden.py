"""Generate the golden fixtures by running the unmodified reference implementation.

Run in the build container (where the reference source is mounted):

    python tests/golden/make_golden.py

It imports the reference package through ``oracle/build_ref.py`` (which compiles
the reference's Cython ``Domain`` extension into ``oracle/_ref/``) together with
the molmod/h5py stand-ins under ``tests/golden/standin/``, runs the reference's
own ``System``, ``ForcePartMechanical``, ``VerletIntegrator``, thermostats,
barostat, builder and ``QNOptimizer`` on small seeded inputs, and writes the
inputs and outputs as compressed ``.npz`` files next to this script. The tests
read only those files; they never touch the reference at run time.

Random draws the reference makes with ``np.random.normal`` (Langevin noise, the CSVR
thermostat's scalars, the Langevin barostat's random tensors) are recorded into the
fixtures so the GPU path can replay them.
"""

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.build_ref import import_reference  # noqa: E402

import_reference()

import micmec.pes.mmff as rmmff  # noqa: E402
import micmec.pes.nanocell as r_nc  # noqa: E402
import micmec.pes.nanocell_original as r_no  # noqa: E402
from micmec.system import System  # noqa: E402
from micmec.pes.mmff import MicMecForceField, ForcePartMechanical  # noqa: E402
from micmec.sampling.verlet import VerletIntegrator  # noqa: E402
from micmec.sampling.iterative import Hook  # noqa: E402
from micmec.sampling.nvt import (  # noqa: E402
    AndersenThermostat, BerendsenThermostat, CSVRThermostat, GLEThermostat, LangevinThermostat, NHCThermostat,
)
from micmec.sampling.npt import BerendsenBarostat, LangevinBarostat, MTKBarostat, TBCombination  # noqa: E402
from micmec.sampling.dof import CartesianDOF, FullCellDOF, StrainCellDOF  # noqa: E402
from micmec.sampling.opt import QNOptimizer  # noqa: E402
from micmec import utils as rutils  # noqa: E402

from micmec_gb300 import units  # noqa: E402
from micmec_gb300 import lattices  # noqa: E402

DATA = os.path.join(os.environ.get("MICMEC_REFERENCE", "/root/reference"), "data")
NUMERIC_PARAM_FIELDS = ("cell", "elasticity", "free_energy", "effective_temp", "mass")


def set_model(model):
    src = r_nc if model == "nanocell" else r_no
    rmmff.elastic_energy_nanocell = src.elastic_energy_nanocell
    rmmff.grad_elastic_energy_nanocell = src.grad_elastic_energy_nanocell


def system_arrays(s, prefix=""):
    out = {
        prefix + "pos": np.array(s.pos, dtype=np.float64),
        prefix + "masses": np.array(s.masses, dtype=np.float64),
        prefix + "rvecs": np.array(s.domain.rvecs, dtype=np.float64).reshape(-1, 3),
        prefix + "surrounding_cells": np.array(s.surrounding_cells, dtype=np.int64),
        prefix + "surrounding_nodes": np.array(s.surrounding_nodes, dtype=np.int64),
        prefix + "grid": np.array(s.grid, dtype=np.int64),
        prefix + "types": np.array(s.types, dtype=np.int64),
    }
    for key, value in s.params.items():
        if key.split("/")[-1] in NUMERIC_PARAM_FIELDS:
            out[prefix + "param:" + key] = np.array(value, dtype=np.float64)
    return out


def save(name, **arrays):
    fn = os.path.join(HERE, name + ".npz")
    np.savez_compressed(fn, **arrays)
    print("wrote", fn, os.path.getsize(fn), "bytes")


def system_from_dict(d):
    kw = dict(d)
    params = {k: v for k, v in kw.items() if "/" in k}
    for k in params:
        kw.pop(k)
    for k in ("pbc",):
        kw.pop(k, None)
    kw["params"] = params
    kw["surrounding_cells"] = np.asarray(kw["surrounding_cells"])
    kw["surrounding_nodes"] = np.asarray(kw["surrounding_nodes"])
    kw["types"] = np.asarray(kw["types"])
    kw["boundary_nodes"] = np.asarray(kw["boundary_nodes"])
    return System(**kw)


def synthetic_system(n, nstates, seed, sigma_angstrom, defect_fraction=0.0, pbc=True, vacancies=0):
    """Reference ``build_system`` on the standard fcu/reo types."""
    rng = np.random.default_rng(seed)
    grid = lattices.defect_grid(n, defect_fraction, rng)
    if vacancies:
        flat = grid.reshape(-1)
        flat[rng.permutation(flat.size)[:vacancies]] = 0
    data = lattices.standard_types(nstates=nstates, with_reo=bool((grid == 2).any()))
    if not (grid == 2).any():
        data = {1: data[1]}
    d = rutils.build_system(data, grid, pbc=pbc)
    s = system_from_dict(d)
    s.pos[:] = lattices.displace(s.pos, sigma_angstrom * units.angstrom, rng)
    return s


def compute_all(s, model):
    set_model(model)
    fp = ForcePartMechanical(s)
    ff = MicMecForceField(s, [fp])
    gpos = np.zeros((s.nnodes, 3))
    vtens = np.zeros((3, 3))
    e = ff.compute(gpos, vtens)
    return e, gpos, vtens, fp.epot_cells, fp.gpos_cells


# ------------------------------------------------------------------ forces


def make_force_fixtures():
    arrays = {}
    cases = []
    chk_names = [
        "2x2x2_fcu_micmec", "2x2x2_fcu_hollow_micmec", "3x3x3_test_micmec",
        "3x3x3_conf0_micmec", "3x3x3_fcu_hollow_micmec", "4x4x4_fcu_hollow_micmec",
        "5x5x5_fcu_hollow_micmec",
    ]
    for i, name in enumerate(chk_names):
        s = System.from_file(os.path.join(DATA, name + ".chk"))
        rng = np.random.default_rng(100 + i)
        s.pos[:] += rng.normal(0.0, 0.2 * units.angstrom, s.pos.shape)
        cases.append((name, s))
    cases.append(("synth_4x4x4_2types_2states", synthetic_system(4, 2, 7, 0.1, 0.25)))
    # Non-periodic systems are not included: the reference's deformation() reads
    # rvecs[0] unconditionally (micmec/pes/mmff.py:349) and raises IndexError
    # when the domain has no vectors.
    cases.append(("synth_5x4x3_vacancies_periodic", synthetic_system((5, 4, 3), 2, 9, 0.1, 0.2, pbc=True, vacancies=7)))
    names = []
    for name, s in cases:
        for model in ("original", "nanocell"):
            key = f"{name}/{model}/"
            e, gpos, vtens, ecells, gcells = compute_all(s, model)
            arrays[key + "energy"] = np.array(e)
            arrays[key + "gpos"] = gpos
            arrays[key + "vtens"] = vtens
            arrays[key + "epot_cells"] = np.asarray(ecells)
            arrays[key + "gpos_cells"] = np.asarray(gcells)
        arrays.update(system_arrays(s, prefix=name + "/sys/"))
        names.append(name)
    arrays["cases"] = np.array(names)
    save("forces", **arrays)


# ------------------------------------------------------------------ builder


def make_builder_fixture():
    arrays = {}
    rng = np.random.default_rng(11)
    for pbc in (True, False):
        grid = rng.integers(0, 3, size=(4, 3, 5))
        grid[0, 0, 0] = 1
        data = lattices.standard_types(nstates=2)
        d = rutils.build_system(data, grid, pbc=pbc)
        tag = "pbc" if pbc else "nopbc"
        for k in ("pos", "rvecs", "surrounding_cells", "surrounding_nodes", "boundary_nodes", "masses", "types"):
            arrays[f"{tag}/{k}"] = np.asarray(d[k])
        arrays[f"{tag}/grid"] = grid
    save("builder", **arrays)


# ------------------------------------------------------------------ MD


class Recorder(Hook):
    def __init__(self, every_pos=1):
        Hook.__init__(self, 0, 1)
        self.rows = []
        self.snap = {}
        self.every_pos = every_pos

    def __call__(self, it):
        self.rows.append(
            [it.counter, it.epot, it.ekin, it.econs, it.temp, getattr(it, "press", 0.0)]
            + list(np.asarray(it.vtens).ravel())
            + list(np.asarray(getattr(it, "ptens", np.zeros((3, 3)))).ravel())
            + list(np.asarray(it.mmf.system.domain.rvecs).ravel())
            + [it.mmf.system.domain.volume]
        )
        if it.counter % self.every_pos == 0:
            self.snap[f"pos_{it.counter}"] = it.pos.copy()
            self.snap[f"vel_{it.counter}"] = it.vel.copy()


class NoiseLog(object):
    """Wraps ``numpy.random.normal`` to record every draw the reference makes."""

    def __enter__(self):
        self.orig = np.random.normal
        self.draws = []

        def normal(*args, **kwargs):
            out = self.orig(*args, **kwargs)
            self.draws.append(np.array(out, dtype=np.float64))
            return out

        np.random.normal = normal
        return self

    def __exit__(self, *exc):
        np.random.normal = self.orig


def md_system(seed=1):
    """Config-1 lattice: 3x3x3 fcu, one state, sigma = 0.05 A, MB velocities at 300 K."""
    s = synthetic_system(3, 1, seed, 0.05)
    rng = np.random.default_rng(seed + 1000)
    kT = units.boltzmann * 300.0
    vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(kT / s.masses)[:, None]
    vel -= (s.masses @ vel) / s.masses.sum()
    return s, vel


def run_md(tag, model, nsteps, hooks_fn, every_pos, seed=1, dt_fs=1.0, record_noise=False, extra=None):
    set_model(model)
    s, vel0 = md_system(seed)
    arrays = system_arrays(s, prefix="sys/")
    ff = MicMecForceField(s, [ForcePartMechanical(s)])
    rec = Recorder(every_pos)
    hooks, meta = hooks_fn(ff)
    np.random.seed(seed + 2000)
    with NoiseLog() as nl:
        vi = VerletIntegrator(ff, dt_fs * units.femtosecond, hooks=hooks + [rec], vel0=vel0.copy())
        vi.run(nsteps)
    arrays["vel0"] = vel0
    arrays["timestep"] = np.array(dt_fs * units.femtosecond)
    arrays["records"] = np.array(rec.rows)
    arrays["model"] = np.array(model)
    arrays["ndof"] = np.array(vi.ndof)
    for k, v in rec.snap.items():
        arrays[k] = v
    for k, v in meta.items():
        arrays["meta/" + k] = np.asarray(v)
    if record_noise:
        arrays["noise"] = np.array([d for d in nl.draws if d.shape == s.pos.shape])
    if extra:
        vi.noise_draws = nl.draws
        extra(arrays, vi)
    save("md_" + tag, **arrays)


def make_md_fixtures():
    T = 300.0 * units.kelvin
    fs = units.femtosecond

    if "md-fast" not in sys.argv:
        run_md("nve_original", "original", 1000, lambda ff: ([], {}), 100)
        run_md("nve_nanocell", "nanocell", 1000, lambda ff: ([], {}), 100)

    def langevin(ff):
        return [LangevinThermostat(T, timecon=100 * fs)], {"temp": T, "timecon": 100 * fs}

    run_md("langevin_nanocell", "nanocell", 200, langevin, 50, record_noise=True)

    rng = np.random.default_rng(5)
    chain_vel0 = rng.normal(0, 1e-5, 3)

    def nhc(ff):
        return (
            [NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())],
            {"temp": T, "timecon": 100 * fs, "chain_vel0": chain_vel0},
        )

    def nhc_extra(arrays, vi):
        hook = [h for h in vi.hooks if isinstance(h, NHCThermostat)][0]
        arrays["chain_pos_end"] = hook.chain.pos
        arrays["chain_vel_end"] = hook.chain.vel

    run_md("nhc_nanocell", "nanocell", 200, nhc, 50, extra=nhc_extra)

    vp = rng.normal(0, 1e-6, (3, 3))
    vp = 0.5 * (vp + vp.T)
    press = 100e6 * units.pascal

    def mtk(ff):
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, vel_press0=vp.copy())
        return [b], {"temp": T, "press": press, "timecon": 1000 * fs, "vel_press0": vp}

    def mtk_extra(arrays, vi):
        hook = [h for h in vi.hooks if isinstance(h, MTKBarostat) or h.name == "TBCombination"][0]
        baro = hook if isinstance(hook, MTKBarostat) else hook.barostat
        arrays["vel_press_end"] = baro.vel_press
        arrays["rvecs_end"] = vi.mmf.system.domain.rvecs
        if hook.name == "TBCombination" and hasattr(hook.thermostat, "chain"):
            arrays["chain_pos_end"] = hook.thermostat.chain.pos
            arrays["chain_vel_end"] = hook.thermostat.chain.vel

    run_md("mtk_nanocell", "nanocell", 100, mtk, 25, extra=mtk_extra)

    def nhc_mtk(ff):
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, vel_press0=vp.copy())
        t = NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())
        return [t, b], {"temp": T, "press": press, "timecon_baro": 1000 * fs,
                        "timecon_thermo": 100 * fs, "vel_press0": vp, "chain_vel0": chain_vel0}

    run_md("nhc_mtk_nanocell", "nanocell", 100, nhc_mtk, 25, extra=mtk_extra)

    def lang_mtk(ff):
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, vel_press0=vp.copy())
        t = LangevinThermostat(T, timecon=100 * fs)
        return [t, b], {"temp": T, "press": press, "timecon_baro": 1000 * fs,
                        "timecon_thermo": 100 * fs, "vel_press0": vp}

    run_md("langevin_mtk_nanocell", "nanocell", 50, lang_mtk, 25, record_noise=True, extra=mtk_extra)


def _hook_end_state(arrays, vi):
    """End state of a hook run: domain, barostat velocity, chain state, and the recorded draws
    of the Langevin barostat (its initial velocity and four unit-normal tensors per step) and
    of the CSVR thermostat."""
    tril = [(i, j) for i in range(3) for j in range(i + 1)]
    hook = [h for h in vi.hooks if h.name in ("TBCombination", "Langevin", "Berendsen", "MTTK", "CSVR")][0]
    baro = getattr(hook, "barostat", hook if getattr(hook, "method", "") == "barostat" else None)
    thermo = getattr(hook, "thermostat", hook if getattr(hook, "method", "") == "thermostat" else None)
    arrays["rvecs_end"] = vi.mmf.system.domain.rvecs
    if baro is not None and getattr(baro, "vel_press", None) is not None:
        arrays["vel_press_end"] = np.asarray(baro.vel_press)
    if thermo is not None and hasattr(thermo, "chain"):
        arrays["chain_pos_end"] = thermo.chain.pos
        arrays["chain_vel_end"] = thermo.chain.vel
    draws = vi.noise_draws
    if isinstance(baro, LangevinBarostat):
        # first (3, 3) draw: the initial barostat velocity (get_random_vel_press); then
        # four unit-normal tensors per step (getR, lower triangle used)
        mats = [d for d in draws if d.shape == (3, 3)]
        arrays["vel_press0"] = baro.vel_press0
        arrays["baro_noise"] = np.array([[m[i, j] for (i, j) in tril] for m in mats[1:]]).reshape(-1, 4, 6)
    if isinstance(thermo, CSVRThermostat):
        R = [float(d) for d in draws if d.shape == ()]
        S = [float((d ** 2).sum()) for d in draws if d.ndim == 1]
        arrays["csvr_noise"] = np.array([R, S]).T


class _LB(LangevinBarostat):
    """The Langevin barostat, keeping its initial velocity (drawn by its init)."""

    def init(self, iterative):
        LangevinBarostat.init(self, iterative)
        self.vel_press0 = np.array(self.vel_press, dtype=float).copy()


def make_hook_fixtures():
    """The rest of the hook set TBCombination accepts (npt.py:163-177) and the CSVR thermostat."""
    T = 300.0 * units.kelvin
    fs = units.femtosecond
    press = 100e6 * units.pascal
    rng = np.random.default_rng(6)
    chain_vel0 = rng.normal(0, 1e-5, 3)
    vp = rng.normal(0, 1e-6, (3, 3))
    vp = 0.5 * (vp + vp.T)
    end_state = _hook_end_state
    LB = _LB

    def berendsen(ff):
        return [BerendsenThermostat(2 * T, timecon=50 * fs)], {"temp": 2 * T, "timecon": 50 * fs}

    run_md("berendsen_nanocell", "nanocell", 200, berendsen, 50, extra=end_state)

    def csvr(ff):
        return [CSVRThermostat(2 * T, timecon=50 * fs)], {"temp": 2 * T, "timecon": 50 * fs}

    run_md("csvr_nanocell", "nanocell", 200, csvr, 50, extra=end_state)

    def berendsen_mtk(ff):
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, vel_press0=vp.copy())
        t = BerendsenThermostat(T, timecon=100 * fs)
        return [TBCombination(t, b)], {"temp": T, "press": press, "timecon_baro": 1000 * fs,
                                       "timecon_thermo": 100 * fs, "vel_press0": vp}

    run_md("berendsen_mtk_nanocell", "nanocell", 100, berendsen_mtk, 25, extra=end_state)

    def nhc_bbaro(ff):
        b = BerendsenBarostat(ff, T, press, timecon=1000 * fs)
        t = NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())
        return [TBCombination(t, b)], {"temp": T, "press": press, "timecon_baro": 1000 * fs,
                                       "timecon_thermo": 100 * fs, "chain_vel0": chain_vel0}

    run_md("nhc_bbaro_nanocell", "nanocell", 100, nhc_bbaro, 25, extra=end_state)

    def lbaro(ff):
        return [LB(ff, T, press, timecon=1000 * fs)], {"temp": T, "press": press, "timecon": 1000 * fs}

    run_md("lbaro_nanocell", "nanocell", 100, lbaro, 25, extra=end_state)

    def nhc_lbaro(ff):
        b = LB(ff, T, press, timecon=1000 * fs)
        t = NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())
        return [TBCombination(t, b)], {"temp": T, "press": press, "timecon_baro": 1000 * fs,
                                       "timecon_thermo": 100 * fs, "chain_vel0": chain_vel0}

    run_md("nhc_lbaro_nanocell", "nanocell", 100, nhc_lbaro, 25, extra=end_state)


def make_gle_fixture():
    """The coloured-noise (GLE) thermostat with two auxiliary momenta (nvt.py:277-358)."""
    T = 300.0 * units.kelvin
    fs = units.femtosecond
    a_p = np.array([[1.0, 0.5, 0.2], [-0.5, 2.0, 0.0], [-0.2, 0.0, 3.0]]) / (100 * fs)

    def gle(ff):
        return [GLEThermostat(T, a_p)], {"temp": T, "a_p": a_p}

    def draws(arrays, vi):
        d = vi.noise_draws
        n3 = vi.pos.size
        arrays["gle_s0"] = [x for x in d if x.shape == (2, n3)][0]
        arrays["gle_noise"] = np.array([x for x in d if x.shape == (3, n3)])

    run_md("gle_nanocell", "nanocell", 40, gle, 20, extra=draws)

    def andersen(ff):
        # velocities redrawn every 5 steps for half of the nodes, with annealing; the draws
        # come from np.random seeded as run_md seeds it (seed + 2000)
        return ([AndersenThermostat(2 * T, step=5, select=np.arange(0, 27, 2), annealing=0.99)],
                {"temp": 2 * T, "step": 5, "annealing": 0.99, "np_random_seed": 2001})

    run_md("andersen_nanocell", "nanocell", 50, andersen, 25)


# ------------------------------------------------------------------ optimiser


def make_opt_fixture():
    set_model("nanocell")
    s = synthetic_system(3, 2, 21, 0.1, 0.3)
    arrays = system_arrays(s, prefix="sys/")
    ff = MicMecForceField(s, [ForcePartMechanical(s)])
    energies = []

    class E(Hook):
        def __call__(self, it):
            energies.append(it.epot)

    dof = CartesianDOF(ff, gpos_rms=1e-6, dpos_rms=1e-4)
    opt = QNOptimizer(dof, hooks=[E()])
    opt.run(60)
    arrays["energies"] = np.array(energies)
    arrays["pos_end"] = s.pos.copy()
    save("opt_qn_nanocell", **arrays)


def make_cell_opt_fixtures():
    """Relaxation of positions and domain (StrainCellDOF / FullCellDOF with QNOptimizer,
    opt.py:258-443, dof.py:199-697) to a tight tolerance: the minimum a device relaxation
    must reach."""
    set_model("nanocell")
    for tag, cls in (("strain", StrainCellDOF), ("full", FullCellDOF)):
        s = synthetic_system(3, 2, 23, 0.1, 0.3)
        arrays = system_arrays(s, prefix="sys/")
        ff = MicMecForceField(s, [ForcePartMechanical(s)])
        dof = cls(ff, gpos_rms=1e-8, dpos_rms=1e-6, grvecs_rms=1e-8, drvecs_rms=1e-6)
        opt = QNOptimizer(dof)
        opt.run(2000)
        gpos = np.zeros(s.pos.shape)
        vtens = np.zeros((3, 3))
        arrays["epot_end"] = np.array(ff.compute(gpos, vtens))
        arrays["vtens_end"] = vtens
        arrays["gpos_end"] = gpos
        arrays["pos_end"] = s.pos.copy()
        arrays["rvecs_end"] = s.domain.rvecs.copy()
        arrays["converged"] = np.array(bool(dof.converged))
        arrays["iterations"] = np.array(opt.counter)
        arrays["model"] = np.array("nanocell")
        save("opt_cell_%s_nanocell" % tag, **arrays)


def make_mtk_variant_fixtures():
    """The MTK barostat's other options (npt.py:513-757): isotropic domain fluctuations, a volume
    constraint, and its own Nose-Hoover chain on the barostat velocity (baro_thermo)."""
    T = 300.0 * units.kelvin
    fs = units.femtosecond
    press = 100e6 * units.pascal
    rng = np.random.default_rng(8)
    chain_vel0 = rng.normal(0, 1e-5, 3)
    baro_chain_vel0 = rng.normal(0, 1e-5, 3)
    vp = rng.normal(0, 1e-6, (3, 3))
    vp = 0.5 * (vp + vp.T)

    def extra(arrays, vi):
        hook = [h for h in vi.hooks if isinstance(h, MTKBarostat) or h.name == "TBCombination"][0]
        baro = hook if isinstance(hook, MTKBarostat) else hook.barostat
        arrays["vel_press_end"] = np.asarray(baro.vel_press)
        arrays["rvecs_end"] = vi.mmf.system.domain.rvecs
        if hook.name == "TBCombination" and hasattr(hook.thermostat, "chain"):
            arrays["chain_pos_end"] = hook.thermostat.chain.pos
            arrays["chain_vel_end"] = hook.thermostat.chain.vel
        if baro.baro_thermo is not None:
            arrays["baro_chain_pos_end"] = baro.baro_thermo.chain.pos
            arrays["baro_chain_vel_end"] = baro.baro_thermo.chain.vel

    def iso(ff):
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, anisotropic=False, vel_press0=2e-6)
        return [b], {"temp": T, "press": press, "timecon": 1000 * fs, "vel_press0": 2e-6}

    run_md("mtk_iso_nanocell", "nanocell", 100, iso, 25, extra=extra)

    def volc(ff):
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, vol_constraint=True, vel_press0=vp.copy())
        t = NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())
        return [t, b], {"temp": T, "press": press, "timecon_baro": 1000 * fs, "timecon_thermo": 100 * fs,
                        "vel_press0": vp, "chain_vel0": chain_vel0}

    run_md("nhc_mtk_volc_nanocell", "nanocell", 100, volc, 25, extra=extra)

    def bthermo(ff):
        bt = NHCThermostat(T, timecon=500 * fs, chainlength=3, chain_vel0=baro_chain_vel0.copy())
        b = MTKBarostat(ff, T, press, timecon=1000 * fs, baro_thermo=bt, vel_press0=vp.copy())
        t = NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())
        return [t, b], {"temp": T, "press": press, "timecon_baro": 1000 * fs, "timecon_thermo": 100 * fs,
                        "timecon_baro_thermo": 500 * fs, "vel_press0": vp, "chain_vel0": chain_vel0,
                        "baro_chain_vel0": baro_chain_vel0}

    run_md("nhc_mtk_bthermo_nanocell", "nanocell", 100, bthermo, 25, extra=extra)


def make_baro_variant_fixtures():
    """The Berendsen and Langevin barostats isotropic and under a volume constraint
    (npt.py:180-510), alone or with a Nose-Hoover chain."""
    T = 300.0 * units.kelvin
    fs = units.femtosecond
    press = 100e6 * units.pascal
    rng = np.random.default_rng(9)
    chain_vel0 = rng.normal(0, 1e-5, 3)

    def nhc():
        return NHCThermostat(T, timecon=100 * fs, chainlength=3, chain_vel0=chain_vel0.copy())

    meta = {"temp": T, "press": press, "timecon_baro": 1000 * fs, "timecon_thermo": 100 * fs,
            "chain_vel0": chain_vel0}

    def bbaro_iso(ff):
        return [TBCombination(nhc(), BerendsenBarostat(ff, T, press, timecon=1000 * fs, anisotropic=False))], meta

    run_md("nhc_bbaro_iso_nanocell", "nanocell", 100, bbaro_iso, 25, extra=_hook_end_state)

    def bbaro_volc(ff):
        return [TBCombination(nhc(), BerendsenBarostat(ff, T, press, timecon=1000 * fs, vol_constraint=True))], meta

    run_md("nhc_bbaro_volc_nanocell", "nanocell", 100, bbaro_volc, 25, extra=_hook_end_state)

    def lbaro_iso(ff):
        # a slower barostat: with 1,000 fs the reference's isotropic Langevin barostat runs away
        # on this 27-cell system (exp overflow at npt.py:448)
        return [_LB(ff, T, press, timecon=5000 * fs, anisotropic=False)], {"temp": T, "press": press,
                                                                           "timecon": 5000 * fs}

    run_md("lbaro_iso_nanocell", "nanocell", 100, lbaro_iso, 25, extra=_hook_end_state)

    def lbaro_volc(ff):
        return [TBCombination(nhc(), _LB(ff, T, press, timecon=1000 * fs, vol_constraint=True))], meta

    run_md("nhc_lbaro_volc_nanocell", "nanocell", 100, lbaro_volc, 25, extra=_hook_end_state)


# ------------------------------------------------------------------ units and sampling utilities


def make_units_fixture():
    """Numbers of the reference's data that pin the atomic mass unit: the 'fcu' type mass
    (data/type_1x1x1_fcu_atomic.pickle) and the element counts of the atomic structure
    (data/1x1x1_fcu_atomic.chk) whose atomic weights it sums."""
    import pickle

    from molmod.io.chk import load_chk

    with open(os.path.join(DATA, "type_1x1x1_fcu_atomic.pickle"), "rb") as f:
        fcu = pickle.load(f)
    numbers = np.asarray(load_chk(os.path.join(DATA, "1x1x1_fcu_atomic.chk"))["numbers"])
    z, counts = np.unique(numbers, return_counts=True)
    save("units_pin", fcu_mass=np.array(float(np.asarray(fcu["mass"]))), numbers=z, counts=counts)


class _FakeFF(object):
    """The three members of a force field that domain_symmetrize uses."""

    def __init__(self, pos, rvecs):
        from micmec.pes.ext import Domain

        self.system = type("S", (), {})()
        self.system.pos = np.array(pos)
        self.system.domain = Domain(np.ascontiguousarray(rvecs))

    def update_rvecs(self, rvecs):
        self.system.domain.update_rvecs(np.ascontiguousarray(rvecs))

    def update_pos(self, pos):
        self.system.pos[:] = pos


def make_sampling_utils_fixture():
    """The reference's initial-velocity, momentum-removal, dof and symmetrisation routines
    (micmec/sampling/utils.py) on seeded inputs; np.random seeds are recorded."""
    from micmec.pes.ext import Domain
    from micmec.sampling import utils as su

    arrays = {}
    rng = np.random.default_rng(5)
    masses = rng.uniform(0.5, 1.5, 50) * lattices.FCU_MASS
    arrays["masses"] = masses
    cases = [(300.0, True, None), (300.0, False, None), (600.0, True, np.array([1, 5, 7, 30])), (0.0, True, None)]
    for i, (temp, scale, select) in enumerate(cases):
        np.random.seed(100 + i)
        arrays["vel%d" % i] = su.get_random_vel(temp, scale, masses, select=select)
    arrays["vel_seeds"] = 100 + np.arange(len(cases))
    baro_mass = (3 * 50 + 9) * units.boltzmann * 300.0 / (2 * np.pi / (1000 * units.femtosecond)) ** 2
    np.random.seed(200)
    arrays["vel_press"] = su.get_random_vel_press(baro_mass, 300.0)
    arrays["baro_mass"] = np.array(baro_mass)
    pos = rng.normal(size=(50, 3)) * 50.0
    vel = rng.normal(size=(50, 3)) * 1e-4
    arrays["clean_pos0"], arrays["clean_vel0"] = pos, vel
    for tag, rvecs in (("pbc", np.eye(3) * 100.0), ("iso", np.zeros((0, 3)))):
        p, v = pos.copy(), vel.copy()
        su.clean_momenta(p, v, masses, Domain(np.ascontiguousarray(rvecs)))
        arrays["clean_%s_pos" % tag], arrays["clean_%s_vel" % tag] = p, v
    arrays["ndof_internal"] = np.array([su.get_ndof_internal_md(57, n) for n in (0, 1, 2, 3)])
    arrays["ndof_baro"] = np.array([su.get_ndof_baro(3, a, c) for a, c in ((True, False), (True, True), (False, False))])
    rv = np.array([[40.0, 1.5, -0.7], [0.9, 41.0, 2.1], [-1.2, 0.3, 39.0]])
    ff = _FakeFF(pos, rv)
    vecs, tens = su.domain_symmetrize(ff, vector_lst=[vel[:3].copy()], tensor_lst=[np.outer(vel[0], vel[1])])
    arrays["sym_rvecs0"] = rv
    arrays["sym_rvecs"] = np.array(ff.system.domain.rvecs)
    arrays["sym_pos"] = np.array(ff.system.pos)
    arrays["sym_vec"] = vecs[0]
    arrays["sym_tens"] = tens[0]
    save("sampling_utils", **arrays)


if __name__ == "__main__":
    which = sys.argv[1:] or ["forces", "builder", "md", "hooks", "gle", "opt", "cellopt", "units", "sutils",
                             "mtkvar", "barovar"]
    if "forces" in which:
        make_force_fixtures()
    if "builder" in which:
        make_builder_fixture()
    if "md" in which:
        make_md_fixtures()
    if "hooks" in which:
        make_hook_fixtures()
    if "gle" in which:
        make_gle_fixture()
    if "opt" in which:
        make_opt_fixture()
    if "cellopt" in which:
        make_cell_opt_fixtures()
    if "units" in which:
        make_units_fixture()
    if "sutils" in which:
        make_sampling_utils_fixture()
    if "mtkvar" in which:
        make_mtk_variant_fixtures()
    if "barovar" in which:
        make_baro_variant_fixtures()
