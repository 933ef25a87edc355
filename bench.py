"""Benchmark: nanocell-steps/s of Langevin MD on a 64^3 two-type, two-state lattice.

Workload (one "step" = one velocity-Verlet step with the Langevin thermostat
applied before and after it, over the whole lattice):
  periodic 64 x 64 x 64 lattice, 262,144 cells and nodes; 90% fcu and 10% reo
  cells (seeded permutation); 2 metastable states per type (h0 x (1 +/- 0.015),
  free energies 0 and 2 kJ/mol, effective temperature 300 K); eight-corner-matrix
  ("nanocell") energy model with FP32 per-cell arithmetic, FP64 state and
  reductions; Langevin 300 K, timecon 100 fs, dt 1 fs.
  Synthetic inputs: Gaussian node displacements (0.05 A) and Maxwell-Boltzmann
  velocities at 300 K from a fixed seed.

Timing: W untimed warm-up steps; then K steps, each bracketed by CUDA events
on the launching stream, with a 256 MiB buffer overwritten before every step
(outside the events) so that no step starts from a warm L2. ``value`` is
cells x K / (summed event time). ``e2e`` is the same metric through the
host-buffer C-ABI step (mm_md_step_host): per step pos, vel and gpos are copied
in from pinned host memory and back out, plus the step record.

``--impl reference`` times the CPU restatement of the reference's force
evaluation and Langevin step (the oracle, NumPy FP64) on a bounded sample of the
same lattice with all host cores (one process per core, spawn), reported in the
same unit.

Multi-GPU: the path is run as independent replicas, one per rank
(torchrun); ``value`` sums the cells of all ranks over the slowest rank's time.
"""

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "cell-steps/s"
UNIT = "nanocell-steps/s"
N_SIDE = 64
DEFECT = 0.10
SEED = 1234
FLUSH_BYTES = 256 << 20

# algorithmic figures (per cell, per evaluation / step)
STEP_BYTES = 97          # pos r/w 24+24, vel r/w 24+24, cell type 1 (FP64 SoA state)
CELL_KERNEL_BYTES = 109  # displacement read 12 (FP32 xyz), type 1, corner gradients written 96 (24 x FP32)
FLOP_PER_STATE = 2400    # 8 corner matrices x ~300 flop (strain, stress, energy, gradient), general h0 / C
FLOP_PER_STATE_CUBIC = 1450  # the same with diagonal h0 and cubic C (reduced 3x3 / 6x6 products)
FLOP_LSE = 20


def config(nstates=2):
    return {
        "workload": "lattice64_langevin_nvt",
        "lattice": [N_SIDE] * 3,
        "cells": N_SIDE**3,
        "types": {"fcu": 1 - DEFECT, "reo": DEFECT},
        "states_per_type": nstates,
        "model": "nanocell (8 corner matrices)",
        "cell_precision": "fp32",
        "state_precision": "fp64",
        "thermostat": "langevin 300 K, timecon 100 fs",
        "timestep_fs": 1.0,
        "l2": "flushed before every timed step (256 MiB overwrite)",
        "parallelism": "replicas",
    }


def build_workload(nstates=2):
    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    rng = np.random.default_rng(SEED)
    grid = lattices.defect_grid(N_SIDE, DEFECT, rng)
    d = lattices.make_lattice(grid, nstates=nstates)
    d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
    s = System.from_dict(d)
    kT = units.boltzmann * 300.0
    vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(kT / s.masses)[:, None]
    vel -= (s.masses @ vel) / s.masses.sum()
    return s, d, vel


def peaks():
    fn = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(fn):
        with open(fn) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler(object):
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.proc = None
        self.index = index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out = ""
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[3:7]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": float(max(smax)) if smax else None,
            "samples": len(sm),
            "reasons": sorted(reasons),
        }


def max_over_ranks(x, dist, device):
    """Largest value of x over all ranks of the default process group (the step time
    that the whole job waited for)."""
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---------------------------------------------------------------- reference (CPU) arm


def cpu_langevin_steps(d, vel, nsteps, nproc, model="nanocell"):
    """Oracle Langevin steps (force evaluation split over nproc processes); returns seconds."""
    import multiprocessing as mp

    from oracle import md as omd

    ctx = mp.get_context("spawn")
    pool = ctx.Pool(nproc) if nproc > 1 else None
    try:
        state = omd.LangevinState(d, vel.copy(), model=model, temp=300.0, timecon_fs=100.0, dt_fs=1.0, seed=SEED,
                                  pool=pool, nproc=nproc)
        t0 = time.perf_counter()
        for _ in range(nsteps):
            state.step()
        return time.perf_counter() - t0
    finally:
        if pool is not None:
            pool.close()
            pool.join()


def run_reference(args):
    """CPU arm: the oracle's Langevin step with all host cores, on bounded samples of the lattice."""
    import multiprocessing as mp

    from oracle import md as omd

    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    s, d, vel = build_workload()
    nproc = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(nproc)
    try:
        state = omd.LangevinState(d, vel.copy(), model="nanocell", temp=300.0, timecon_fs=100.0, dt_fs=1.0,
                                  seed=SEED, pool=pool, nproc=nproc)
        M = s.ncells
        t0 = time.perf_counter()
        state.step()  # one full-lattice step to size the samples
        t_full = time.perf_counter() - t0
        budget = float(os.environ.get("MICMEC_REF_BUDGET_S", "90"))
        per_step = budget / max(1, args.steps + args.warmup)
        ncells = int(max(nproc * 64, min(M, M * per_step / t_full)))
        for _ in range(args.warmup):
            state.step(ncells)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            state.step(ncells)
            times.append(time.perf_counter() - t0)
    finally:
        pool.close()
        pool.join()
    tot = float(np.sum(times))
    value = ncells * args.steps / tot
    sample = ("Langevin step of the 64^3 lattice with the force evaluation restricted to the first %d cells "
              "(full-lattice step: %.2f s), NumPy FP64 oracle split over %d spawned processes" % (ncells, t_full, nproc))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config(),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nproc, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- GPU arm


def general_form(d):
    """Copy of a system dict whose types have a slightly anisotropic C and sheared h0.

    The standard fcu/reo types have diagonal rest matrices and cubic elasticity, for
    which the cell kernel uses reduced strain/stress products; this variant takes the
    general 3x3 / 6x6 products and is timed beside the main line.
    """
    g = dict(d)
    for k in list(d):
        if k.endswith("/elasticity"):
            C = np.array(d[k], dtype=float)
            C[..., 0, 0, 0, 0] *= 1.001
            g[k] = C
        elif k.endswith("/cell"):
            h = np.array(d[k], dtype=float)
            h[..., 0, 1] += 1e-4 * h[..., 0, 0]
            h[..., 1, 0] += 1e-4 * h[..., 0, 0]
            g[k] = h
    return g


def measure_lattice(s, vel, nsteps, flush, precision="fp64"):
    """The same session API on the same lattice at another cell precision."""
    import torch

    from micmec_gb300 import _native as nat, units
    from micmec_gb300.pes.mmff import ForcePartMechanical

    L = nat.lib()
    dev = flush.device
    fp = ForcePartMechanical(s, model="nanocell", precision=precision)
    stream = torch.cuda.current_stream().cuda_stream
    pos_d = torch.from_numpy(np.ascontiguousarray(s.pos)).to(dev)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
    dt, tau = 1.0 * units.femtosecond, 100.0 * units.femtosecond
    nat.check(L.mm_md_begin(fp.handle, pos_d.data_ptr(), vel_d.data_ptr(), dt, 1, 300.0, tau, SEED, None, 0, stream),
              "mm_md_begin")
    for _ in range(3):
        nat.check(L.mm_md_advance(fp.handle, 1, None, 0, stream), "mm_md_advance")
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
    for i in range(nsteps):
        flush.fill_(i & 0xFF)
        ev[i][0].record()
        nat.check(L.mm_md_advance(fp.handle, 1, None, 0, stream), "mm_md_advance")
        ev[i][1].record()
    torch.cuda.synchronize()
    ms = float(sum(a.elapsed_time(b) for a, b in ev))
    nat.check(L.mm_md_advance(fp.handle, 1, None, 1, stream), "mm_md_advance")
    torch.cuda.synchronize()
    return s.ncells * nsteps / (ms * 1e-3), ms / nsteps


def batch_workload(nsys=512, seed=77, nstates=2):
    """512 periodic systems, n ~ U{3..12}, defect fraction ~ U[0, 0.3], uniaxial strain 0..5% in 0.25% steps."""
    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    systems, strains = [], []
    for i in range(nsys):
        n = int(rng.integers(3, 13))
        frac = float(rng.uniform(0.0, 0.3))
        strain = 0.0025 * (i % 21)
        d = lattices.make_lattice(lattices.defect_grid(n, frac, rng), nstates=nstates)
        F = np.eye(3)
        F[0, 0] += strain
        d["pos"] = d["pos"] @ F
        d["rvecs"] = d["rvecs"] @ F
        d["pos"] = lattices.displace(d["pos"], 0.02 * units.angstrom, rng)
        systems.append(System.from_dict(d))
        strains.append(strain)
    return systems, np.array(strains)


def measure_batch(systems, strains, precision, md_steps, relax_iters, drift=False):
    """Config 3 on the batch kernel: batched CG relaxation of every strained system, then
    md_steps NHC + MTK steps (300 K, 0 MPa) of all systems in one launch replayed from a CUDA
    graph after autotuning. drift: a further untimed md_steps-step run with per-step records
    gives each system's conserved quantity (epot + ekin + the hooks' corrections)."""
    import torch

    from micmec_gb300 import units
    from micmec_gb300.batch import REC, BatchSystems

    fs = units.femtosecond
    b = BatchSystems(systems, model="nanocell", precision=precision)
    gtol = 1e-4 * units.electronvolt / units.angstrom
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    gmax, iters = b.relax(max_iter=relax_iters, gtol=gtol)
    torch.cuda.synchronize()
    t_relax = time.perf_counter() - t0
    stress = b.stress()[:, 0, 0] / units.gigapascal
    b.setup_md(temp=300.0, thermostat="nhc", barostat="mtk", timecon=100 * fs, baro_timecon=1000 * fs, seed=5)
    kw = dict(thermostat="nhc", temp=300.0, barostat="mtk", press=0.0)
    cfg = b.autotune(probe_steps=3, **kw)
    b.md(1, use_graph=True, **kw)  # capture
    b.md(md_steps, use_graph=True, step0=1, **kw)  # capture of the timed launch's key (nsteps, step0)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.md(md_steps, use_graph=True, step0=1, **kw)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = float(np.sum(b.sizes))
    out = {
        "systems": len(systems), "cells": int(cells), "precision": precision, "md_steps": md_steps,
        "md_ms": ms, "systems_steps_per_s": len(systems) * md_steps / (ms * 1e-3),
        "cell_steps_per_s": cells * md_steps / (ms * 1e-3),
        "force_evals_per_step": 3, "relax_s": t_relax, "relax_converged": int(np.sum(gmax < gtol)),
        "relax_max_iters": int(np.max(iters)), "autotune": cfg,
        "stress_xx_gpa_by_strain": {f"{s:.4f}": float(np.mean(stress[np.isclose(strains, s)])) for s in
                                     np.unique(strains)[:: 5]},
    }
    if drift:
        rec = b.md(md_steps, use_graph=False, step0=1 + md_steps, record=True, **kw)
        econs = rec[:, :, REC["epot"]] + rec[:, :, REC["ekin"]] + rec[:, :, REC["ecorr"]]
        etot = np.abs(rec[:, :, REC["epot"]] + rec[:, :, REC["ekin"]]).mean(axis=1)
        per1000 = np.abs(econs[:, -1] - econs[:, 0]) / etot * (1000.0 / (md_steps - 1))
        fluct = (econs.max(axis=1) - econs.min(axis=1)) / etot
        thermal = 0.5 * (3.0 * b.sizes - 3.0) * units.boltzmann * 300.0  # ndof kT / 2 of each system
        per1000_th = np.abs(econs[:, -1] - econs[:, 0]) / thermal * (1000.0 / (md_steps - 1))
        out["conserved_quantity"] = {
            "steps": md_steps, "timestep_fs": 1.0,
            "change_per_1000_steps_rel_median": float(np.median(per1000)),
            "change_per_1000_steps_rel_max": float(per1000.max()),
            "change_per_1000_steps_over_thermal_energy_median": float(np.median(per1000_th)),
            "change_per_1000_steps_over_thermal_energy_max": float(per1000_th.max()),
            "fluctuation_rel_median": float(np.median(fluct)), "fluctuation_rel_max": float(fluct.max()),
            "note": "epot + ekin + NHC and MTK corrections per system, relative to |epot + ekin| and to the "
                    "system's thermal energy (3N - 3) kT / 2; the strained systems relax under GPa-level stress "
                    "at 0 MPa, and the MTK splitting error of that volume motion dominates",
        }
    return out


def measure_plain_per_system(systems, nsteps, device):
    """The plain FP64 GPU path for the same hooks, one System at a time through VerletIntegrator
    with NHC + MTK. device=True: the hooks run on the device (the integrator hands each system
    to the persistent kernel as a one-system batch); device=False: host hooks, every force
    evaluation on the GPU (three round trips per step)."""
    import torch

    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.npt import MTKBarostat
    from micmec_gb300.sampling.nvt import NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator

    fs = units.femtosecond
    t = 0.0
    steps = 0
    for s in systems:
        ff = MicMecForceField(s, [ForcePartMechanical(s, model="nanocell", precision="fp64")])
        hooks = [NHCThermostat(300.0, timecon=100 * fs), MTKBarostat(ff, 300.0, 0.0, timecon=1000 * fs)]
        vi = VerletIntegrator(ff, 1.0 * fs, hooks=hooks, temp0=300.0, device=device)
        if device:
            vi.run(2)  # first run: the one-system batch is created
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vi.run(nsteps)
        torch.cuda.synchronize()
        t += time.perf_counter() - t0
        steps += nsteps
    return {"systems": len(systems), "steps_each": nsteps, "hooks_on_device": bool(device),
            "systems_steps_per_s": steps / t, "cell_steps_per_s": sum(s.ncells for s in systems) * nsteps / t,
            "system_sizes": [int(s.ncells) for s in systems]}


def measure_large_mtk(n=256, nsteps=1000, cmp_steps=100):
    """Config 5: a large single system (periodic n^3 lattice, 20% clustered defects, two
    states per type) under NHC + MTK NPT at 300 K and 100 MPa, dt = 2 fs, through
    VerletIntegrator (device=True routes it to the lattice engine). FP64 and FP32 cells run
    the same cmp_steps steps from the same state (conserved quantity and energy compared at
    the end); the FP32 run then continues for nsteps timed steps, with the conserved quantity
    recorded before and after them."""
    import torch

    from micmec_gb300 import lattices, units
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField
    from micmec_gb300.sampling.iterative import Hook
    from micmec_gb300.sampling.npt import MTKBarostat
    from micmec_gb300.sampling.nvt import NHCThermostat
    from micmec_gb300.sampling.verlet import VerletIntegrator
    from micmec_gb300.system import System

    rng = np.random.default_rng(SEED + 5)
    t0 = time.perf_counter()
    d = lattices.make_lattice(lattices.defect_grid(n, 0.2, rng, clustered=True), nstates=2, device=True)
    d["pos"] = lattices.displace(d["pos"], 0.02 * units.angstrom, rng)
    t_setup = time.perf_counter() - t0
    kT = units.boltzmann * 300.0
    out = {"lattice": [n] * 3, "cells": n ** 3, "hooks": "NHC + MTK, 300 K, 100 MPa", "timestep_fs": 2.0,
           "host_setup_s": t_setup}

    class Econs(Hook):
        # fires only where it is scheduled (a per-step host hook would bring the state back
        # to the host every step)
        def __init__(self):
            Hook.__init__(self, 2, cmp_steps)
            self.rows = []

        def __call__(self, it):
            self.rows.append((it.counter, it.econs, it.epot, it.ekin))

    vel = None
    end = {}
    for prec in ("fp64", "fp32"):
        s = System.from_dict(d)
        if vel is None:
            vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(kT / s.masses)[:, None]
            vel -= (s.masses @ vel) / s.masses.sum()
        ff = MicMecForceField(s, [ForcePartMechanical(s, precision=prec)])
        rec = Econs()
        # fixed initial chain and barostat velocities (drawn at random by default): both
        # precisions start from the same extended state
        hooks = [NHCThermostat(300.0, timecon=100 * units.femtosecond, chain_vel0=np.zeros(3)),
                 MTKBarostat(ff, 300.0, 100e6 * units.pascal, timecon=1000 * units.femtosecond,
                             vel_press0=np.zeros((3, 3))), rec]
        vi = VerletIntegrator(ff, 2.0 * units.femtosecond, hooks=hooks, vel0=vel.copy(), device=True)
        vi.run(2)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        vi.run(cmp_steps)
        torch.cuda.synchronize()
        t_cmp = time.perf_counter() - t0
        (c0, e0, p0, k0), (c1, e1, p1, k1) = rec.rows[-2], rec.rows[-1]
        end[prec] = (e1, p1, k1)
        res = {"econs_change_over_cmp_steps": e1 - e0, "epot": p1, "ekin": k1,
               "cmp_s": t_cmp, "cmp_cell_steps_per_s": n ** 3 * cmp_steps / t_cmp}
        if prec == "fp32":
            rec.start, rec.step = 2 + cmp_steps + nsteps, 1  # one call, after the timed run
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            vi.run(nsteps)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            c2, e2, p2, k2 = rec.rows[-1]
            res.update({"steps": nsteps, "s": dt, "cell_steps_per_s": n ** 3 * nsteps / dt,
                        "econs_change_over_steps_rel": (e2 - e1) / abs(p2 + k2),
                        "epot_change_over_steps_rel": (p2 - p1) / abs(p2 + k2)})
        out[prec] = res
        del vi, ff, s
        torch.cuda.empty_cache()
    out["cmp_steps"] = cmp_steps
    etot = abs(end["fp64"][1] + end["fp64"][2])
    out["fp32_minus_fp64_after_cmp_steps_rel"] = {
        "econs": float((end["fp32"][0] - end["fp64"][0]) / etot),
        "epot": float((end["fp32"][1] - end["fp64"][1]) / etot),
        "ekin": float((end["fp32"][2] - end["fp64"][2]) / etot)}
    return out


def lattice_md_rate(s, vel, model, precision, nsteps, flush):
    """Langevin NVT steps (300 K, 100 fs, dt 1 fs) of a lattice through the MD session API:
    per-step CUDA events with L2 flushed before every step, and the per-kernel event times
    (cells, nodes) from mm_md_time_kernels. Returns (cell-steps/s, ms/step, cell ms, node ms)."""
    import torch

    from micmec_gb300 import _native as nat, units
    from micmec_gb300.pes.mmff import ForcePartMechanical

    L = nat.lib()
    dev = flush.device
    fp = ForcePartMechanical(s, model=model, precision=precision)
    stream = torch.cuda.current_stream().cuda_stream
    pos_d = torch.from_numpy(np.ascontiguousarray(s.pos)).to(dev)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
    dt, tau = 1.0 * units.femtosecond, 100.0 * units.femtosecond
    nat.check(L.mm_md_begin(fp.handle, pos_d.data_ptr(), vel_d.data_ptr(), dt, 1, 300.0, tau, SEED, None, 0, stream),
              "mm_md_begin")
    for _ in range(3):
        nat.check(L.mm_md_advance(fp.handle, 1, None, 0, stream), "mm_md_advance")
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
    for i in range(nsteps):
        flush.fill_(i & 0xFF)
        ev[i][0].record()
        nat.check(L.mm_md_advance(fp.handle, 1, None, 0, stream), "mm_md_advance")
        ev[i][1].record()
    torch.cuda.synchronize()
    ms = float(sum(a.elapsed_time(b) for a, b in ev))
    mc, mn = nat.c_double(), nat.c_double()
    nat.check(L.mm_md_time_kernels(fp.handle, nsteps, flush.data_ptr(), FLUSH_BYTES, nat.ctypes.byref(mc),
                                   nat.ctypes.byref(mn), stream), "mm_md_time_kernels")
    nat.check(L.mm_md_advance(fp.handle, 1, None, 1, stream), "mm_md_advance")
    torch.cuda.synchronize()
    del fp
    return s.ncells * nsteps / (ms * 1e-3), ms / nsteps, mc.value / nsteps, mn.value / nsteps


def measure_models(flush, sizes=(64, 256)):
    """The averaged-matrix model the reference's mmff.py imports (nanocell_original.py) beside
    the eight-corner-matrix model, FP32 cells, Langevin NVT, on the two-type two-state lattice
    (10% defects) at each size: step rate, per-kernel times and the HBM fraction of the step's
    97 algorithmic bytes per cell-step and of the cell kernel's 109 bytes per cell."""
    import torch

    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    hbm, kind = peaks()
    out = {"peak_gbs": hbm, "peak_kind": kind}
    for n in sizes:
        rng = np.random.default_rng(SEED + n)
        d = lattices.make_lattice(lattices.defect_grid(n, DEFECT, rng), nstates=2, device=n > 128)
        d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
        s = System.from_dict(d)
        vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(units.boltzmann * 300.0 / s.masses)[:, None]
        vel -= (s.masses @ vel) / s.masses.sum()
        for model in ("original", "nanocell"):
            steps = 20 if n <= 64 else 10
            v, ms, cms, nms = lattice_md_rate(s, vel, model, "fp32", steps, flush)
            M = s.ncells
            out["%s_%d" % (model, n)] = {
                "cell_steps_per_s": v, "ms_per_step": ms, "cells_ms": cms, "nodes_ms": nms,
                "step_hbm_gbs": STEP_BYTES * M / (ms * 1e-3) / 1e9,
                "step_hbm_frac": STEP_BYTES * M / (ms * 1e-3) / 1e9 / hbm,
                "cell_kernel_hbm_gbs": CELL_KERNEL_BYTES * M / (cms * 1e-3) / 1e9,
                "cell_kernel_hbm_frac": CELL_KERNEL_BYTES * M / (cms * 1e-3) / 1e9 / hbm}
        del s, d
        torch.cuda.empty_cache()
    return out


def measure_drift_nve(s, vel, nsteps=1000):
    """Energy conservation of the 64^3 workload lattice under plain velocity Verlet (NVE,
    dt = 1 fs) for FP64 and FP32 cells: change and spread of epot + ekin over nsteps steps
    relative to |epot + ekin| (the records of the device MD loop, one per step)."""
    import torch

    from micmec_gb300 import _native as nat, units
    from micmec_gb300.pes.mmff import ForcePartMechanical

    L = nat.lib()
    out = {"lattice": [N_SIDE] * 3, "steps": nsteps, "timestep_fs": 1.0, "ensemble": "NVE"}
    dev = torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream().cuda_stream
    for prec in ("fp64", "fp32"):
        fp = ForcePartMechanical(s, model="nanocell", precision=prec)
        e0 = fp.compute()
        ek0 = 0.5 * float(np.sum(s.masses[:, None] * vel ** 2))
        pos_d = torch.from_numpy(np.ascontiguousarray(s.pos)).to(dev)
        vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
        rec = torch.zeros((nsteps, nat.MM_REC_LEN), dtype=torch.float64, device=dev)
        nat.check(L.mm_md_run(fp.handle, pos_d.data_ptr(), vel_d.data_ptr(), nsteps, 1.0 * units.femtosecond, 0, 0.0,
                              1.0, SEED, None, rec.data_ptr(), 0, stream), "mm_md_run")
        r = rec.cpu().numpy()
        econs = np.concatenate([[e0 + ek0], r[:, 0] + r[:, 1]])
        ref = abs(econs[0])
        slope = np.polyfit(np.arange(nsteps + 1), econs, 1)[0]
        out[prec] = {"econs_change_rel": float((econs[-1] - econs[0]) / ref),
                     "econs_trend_per_1000_steps_rel": float(slope * 1000 / ref),
                     "econs_spread_rel": float((econs.max() - econs.min()) / ref),
                     "ekin_mean_over_initial": float(r[:, 1].mean() / ek0)}
        del fp
    return out


def _error_text(exc):
    """The exception and the innermost frame that raised it (file:line), for the JSON line."""
    import traceback

    tb = traceback.extract_tb(exc.__traceback__)
    where = "%s:%d" % (os.path.basename(tb[-1].filename), tb[-1].lineno) if tb else "?"
    return ("%r at %s" % (exc, where))[:300]


def measure_builder(n_cmp=128, n_large=256):
    """System construction: the device builder (mm_build_topology, tables copied back to host
    arrays) against the vectorised host builder on the same grid, and the device builder alone
    at 256^3 (20% clustered defects, two types, periodic)."""
    import torch

    from micmec_gb300 import lattices
    from micmec_gb300.utils import build_system

    rng = np.random.default_rng(5)
    data = lattices.standard_types(nstates=2)
    build_system(data, lattices.defect_grid(8, 0.2, rng), pbc=True, device=True)  # warm-up
    grid = lattices.defect_grid(n_cmp, 0.2, rng, clustered=True)
    t0 = time.perf_counter()
    host = build_system(data, grid, pbc=True)
    t_host = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dev = build_system(data, grid, pbc=True, device=True)
    t_dev = time.perf_counter() - t0
    same = all(np.array_equal(np.asarray(host[k]), np.asarray(dev[k]))
               for k in ("surrounding_cells", "surrounding_nodes", "boundary_nodes", "types", "masses", "pos"))
    del host, dev
    grid = lattices.defect_grid(n_large, 0.2, rng, clustered=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    big = build_system(data, grid, pbc=True, device=True)
    t_big = time.perf_counter() - t0
    ncells = len(big["types"])
    del big
    return {"lattice_cmp": [n_cmp] * 3, "host_s": t_host, "device_s": t_dev, "identical": bool(same),
            "lattice_large": [n_large] * 3, "device_large_s": t_big, "large_cells": ncells,
            "note": "wall time of build_system, device tables copied back into host arrays"}


def measure_config4(n=16, npts=11, nsteps=200, every=20):
    """The differentiation workload end to end: a 16^3 two-type two-state lattice; loss =
    MSE of the relaxed stress over 11 uniaxial strain points (0 .. 2.5%) + MSE of the mean
    node forces over a 200-step Verlet trajectory (dt 1 fs, checkpoint every 20 steps)
    against targets from a hidden parameter set (C per Voigt component x (1 + U[-0.2, 0.2]),
    h0 x (1 + U[-0.01, 0.01])). The strain points are relaxed together by the batched device
    relaxer (FP64, max |gradient| < 1e-9 Ha/bohr) for every parameter value; gradients with
    respect to the 21 Voigt C components and h0 per type and state and the free energies come
    from the adjoint (implicit differentiation through the relaxations, checkpointed
    recomputation through the trajectory) and are checked against central differences
    (h = 1e-4 relative) of the whole loss for three parameters."""
    import torch

    from micmec_gb300 import lattices, units
    from micmec_gb300.autograd import MicMecParameters, relaxed_stress, verlet_trajectory
    from micmec_gb300.batch import BatchSystems
    from micmec_gb300.pes.mmff import ForcePartMechanical
    from micmec_gb300.system import System

    t_start = time.perf_counter()
    rng = np.random.default_rng(41)
    d = lattices.make_lattice(lattices.defect_grid(n, 0.2, rng), nstates=2)
    s = System.from_dict(d)
    part = ForcePartMechanical(s, model="nanocell", precision="fp64")
    params = MicMecParameters(part)
    base_rv = np.array(s.domain.rvecs)
    pos0 = np.array(s.pos)
    Fs = []
    for e in np.linspace(0.0, 0.025, npts):
        F = np.eye(3)
        F[0, 0] += e
        Fs.append(F)
    batch = BatchSystems([System.from_dict(d) for _ in Fs], model="nanocell", precision="fp64")
    dev = torch.device("cuda")
    kT = units.boltzmann * 300.0
    vel0 = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(kT / s.masses)[:, None]
    vel0 -= (s.masses @ vel0) / s.masses.sum()
    x0 = torch.tensor(pos0, dtype=torch.float64, device=dev)
    v0 = torch.tensor(vel0, dtype=torch.float64, device=dev)
    m = torch.tensor(np.asarray(s.masses), dtype=torch.float64, device=dev)
    dt = 1.0 * units.femtosecond
    tensors = list(params.tensors())
    relax_iters = []

    def relax_all():
        C, H, D = params.native_tables(*tensors)
        batch.set_params(H, C, D, params.temp, params.nstates)
        batch.set_state([pos0 @ F for F in Fs], None, [base_rv @ F for F in Fs])
        gmax, iters = batch.relax(max_iter=50000, gtol=1e-9)
        relax_iters.append(int(iters.max()))
        if not (gmax < 1e-9).all():
            raise RuntimeError("relaxation did not converge: %g" % float(gmax.max()))
        return batch.get_state()[0]

    def set_domain(rv):
        s.domain.update_rvecs(rv)
        part.update_rvecs(rv)

    def evaluate(targets=None, grad=False):
        """(loss, gradients or None, stresses, mean forces)."""
        positions = relax_all()
        total, sigmas = 0.0, []
        grads = [torch.zeros_like(t) for t in tensors] if grad else None
        for i, F in enumerate(Fs):
            set_domain(base_rv @ F)
            x = torch.tensor(positions[i], dtype=torch.float64, device=dev)
            with torch.set_grad_enabled(grad):
                sig = relaxed_stress(x, params)
                sigmas.append(sig.detach())
                if targets is not None:
                    loss = ((sig - targets[0][i]) ** 2).sum()
                    total += float(loss.detach())
                    if grad:
                        for acc, gr in zip(grads, torch.autograd.grad(loss, tensors)):
                            acc += gr
        set_domain(base_rv)
        with torch.set_grad_enabled(grad):
            gl, _, _ = verlet_trajectory(x0, v0, m, params, dt, nsteps, checkpoint_every=every)
            fbar = -torch.stack(gl[1:]).mean(0)
            if targets is not None:
                loss = ((fbar - targets[1]) ** 2).mean()
                total += float(loss.detach())
                if grad:
                    for acc, gr in zip(grads, torch.autograd.grad(loss, tensors)):
                        acc += gr
        return total, grads, sigmas, fbar.detach()

    # targets from the hidden parameter set
    hidden = np.random.default_rng(4242)
    saved = [t.detach().clone() for t in tensors]
    with torch.no_grad():
        tensors[0].mul_(torch.tensor(1 + hidden.uniform(-0.2, 0.2, tuple(tensors[0].shape)), device=tensors[0].device))
        tensors[1].mul_(torch.tensor(1 + hidden.uniform(-0.01, 0.01, tuple(tensors[1].shape)),
                                     device=tensors[1].device))
    _, _, sig_t, f_t = evaluate()
    with torch.no_grad():
        for t, v in zip(tensors, saved):
            t.copy_(v)
    t_setup = time.perf_counter() - t_start
    # one untimed evaluation of each kind, then the median of `reps` timed ones
    reps = 3
    evaluate((sig_t, f_t), grad=True)
    evaluate((sig_t, f_t))
    t_grads, t_losses = [], []
    for _ in range(reps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        loss0, grads, _, _ = evaluate((sig_t, f_t), grad=True)
        torch.cuda.synchronize()
        t_grads.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        evaluate((sig_t, f_t))
        torch.cuda.synchronize()
        t_losses.append(time.perf_counter() - t0)
    t_grad, t_loss = float(np.median(t_grads)), float(np.median(t_losses))

    def central(which, idx, hrel):
        t = tensors[which]
        base = float(t.detach()[idx])
        h = hrel * abs(base)
        vals = []
        for sgn in (1, -1):
            with torch.no_grad():
                t[idx] = base + sgn * h
            vals.append(evaluate((sig_t, f_t))[0])
        with torch.no_grad():
            t[idx] = base
        return (vals[0] - vals[1]) / (2 * h)

    errs = []
    picks = [(0, (0, 0, 0)), (0, (1, 0, 1)), (1, (0, 0, 1, 1))]
    for which, idx in picks:
        fd = central(which, idx, 1e-4)
        errs.append(abs(float(grads[which][idx]) - fd) / max(abs(fd), 1e-300))
    # the h0 component: central differences over a range of steps and their Richardson
    # extrapolation (D(h) - D(2h)) / 3 + D(h), which removes the O(h^2) truncation term
    which, idx = picks[2]
    g_adj = float(grads[which][idx])
    sweep = {}
    prev = None
    for hrel in (4e-4, 2e-4, 1e-4, 5e-5, 2.5e-5, 1e-5):
        fd = central(which, idx, hrel)
        entry = {"fd_rel_err": abs(g_adj - fd) / abs(fd)}
        if prev is not None and abs(prev[0] / hrel - 2.0) < 1e-9:
            rich = fd + (fd - prev[1]) / 3.0
            entry["richardson_rel_err"] = abs(g_adj - rich) / abs(rich)
        sweep["%g" % hrel] = entry
        prev = (hrel, fd)
    return {"lattice": [n] * 3, "strain_points": npts, "trajectory_steps": nsteps, "checkpoint_every": every,
            "loss": loss0, "loss_s": t_loss, "loss_and_gradient_s": t_grad,
            "grad_over_fwd": t_grad / t_loss, "timing": "median of %d after one untimed evaluation of each" % reps,
            "loss_s_all": t_losses, "loss_and_gradient_s_all": t_grads, "setup_s": t_setup,
            "relax_iterations_max": max(relax_iters), "fd_rel_err": errs, "fd_h": "1e-4 relative",
            "fd_params": ["C11 type 0 state 0", "C12 type 1 state 0", "h0_yy type 0 state 0"],
            "h0_yy_step_sweep": sweep}


def measure_grad_over_fwd(n=16, reps=5):
    """Cost of the adjoint (backward of a force loss) relative to the forward force evaluation, 16^3 FP64."""
    import torch

    from micmec_gb300 import lattices, units
    from micmec_gb300.autograd import MicMecParameters, energy_and_gradient
    from micmec_gb300.pes.mmff import ForcePartMechanical
    from micmec_gb300.system import System

    rng = np.random.default_rng(3)
    d = lattices.make_lattice(lattices.defect_grid(n, 0.2, rng), nstates=2)
    d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
    s = System.from_dict(d)
    part = ForcePartMechanical(s, model="nanocell", precision="fp64")
    params = MicMecParameters(part)
    pos = torch.tensor(s.pos, dtype=torch.float64, device="cuda")
    w = torch.tensor(rng.normal(size=(s.nnodes, 3)), dtype=torch.float64, device="cuda")
    fwd, bwd = [], []
    for _ in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        E, g = energy_and_gradient(pos, params)
        loss = (w * g).sum()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        torch.autograd.grad(loss, [params.c21, params.h0, params.free_energy])
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        fwd.append(t1 - t0)
        bwd.append(t2 - t1)
    f, b = float(np.median(fwd[1:])), float(np.median(bwd[1:]))
    # central differences (h = 1e-4 relative) of the same loss for three parameters
    gc, gh, gd = torch.autograd.grad((w * energy_and_gradient(pos, params)[1]).sum(),
                                     [params.c21, params.h0, params.free_energy])
    errs = []
    # C11 of type 0 and C12 of type 1 in state 0, a diagonal entry of h0 (all nonzero; the
    # lattice sits near state 0's rest cell, where the other states' weights are below rounding)
    for tensor, grad, idx in ((params.c21, gc, (0, 0, 0)), (params.c21, gc, (1, 0, 1)), (params.h0, gh, (0, 0, 1, 1))):
        base = float(tensor.detach()[idx])
        if base == 0.0:
            raise ValueError("finite-difference probe on a zero parameter")
        h = 1e-4 * abs(base)
        vals = []
        for sgn in (1, -1):
            with torch.no_grad():
                tensor[idx] = base + sgn * h
                vals.append(float((w * energy_and_gradient(pos, params)[1]).sum()))
        with torch.no_grad():
            tensor[idx] = base
        fd = (vals[0] - vals[1]) / (2 * h)
        errs.append(abs(float(grad[idx]) - fd) / abs(fd))
    return {"lattice": [n] * 3, "forward_ms": 1e3 * f, "backward_ms": 1e3 * b, "grad_over_fwd": b / f,
            "fd_rel_err_max": max(errs), "fd_h": "1e-4 relative"}


def force_error_fp32(s):
    """Relative force and energy error of the FP32-cell path against the FP64 path (itself
    equal to the reference's forces to 1e-10) at the same positions."""
    from micmec_gb300.pes.mmff import ForcePartMechanical

    out = {}
    res = {}
    for prec in ("fp64", "fp32"):
        fp = ForcePartMechanical(s, model="nanocell", precision=prec)
        g = np.zeros((s.nnodes, 3))
        v = np.zeros((3, 3))
        e = fp.compute(g, v)
        res[prec] = (e, g, v)
    (e64, g64, v64), (e32, g32, v32) = res["fp64"], res["fp32"]
    out["force_rel_err"] = float(np.abs(g32 - g64).max() / np.abs(g64).max())
    out["energy_rel_err"] = float(abs(e32 - e64) / abs(e64))
    out["virial_rel_err"] = float(np.abs(v32 - v64).max() / np.abs(v64).max())
    return out


def host_link_rates(pinned, dev, reps=5):
    """Pinned host <-> device copy rates (GB/s) for the three arrays of the e2e step,
    copied as 1 stream per array (x3) and as 2 halves per array on 6 streams (x6), and
    for one array alone (x1)."""
    import torch

    n = pinned.numel()
    h = [pinned.clone().reshape(-1).pin_memory() for _ in range(3)]
    d = [torch.empty(n, dtype=pinned.dtype, device=dev) for _ in range(3)]
    streams = [torch.cuda.Stream(dev) for _ in range(6)]
    out = {}
    for name in ("h2d", "d2h"):
        for k in (1, 3, 6):
            pieces = []
            if k == 1:
                pieces = [(0, 0, n)]
            elif k == 3:
                pieces = [(i, 0, n) for i in range(3)]
            else:
                pieces = [(i, j * (n // 2), (j + 1) * (n // 2) if j == 0 else n) for i in range(3) for j in range(2)]
            best = None
            for _ in range(reps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                for sidx, (i, lo, hi) in enumerate(pieces):
                    with torch.cuda.stream(streams[sidx]):
                        if name == "h2d":
                            d[i][lo:hi].copy_(h[i][lo:hi], non_blocking=True)
                        else:
                            h[i][lo:hi].copy_(d[i][lo:hi], non_blocking=True)
                torch.cuda.synchronize()
                dt = time.perf_counter() - t0
                best = dt if best is None else min(best, dt)
            nbytes = sum(hi - lo for _, lo, hi in pieces) * pinned.element_size()
            out["%s_gbs_x%d" % (name, k)] = nbytes / best / 1e9
    return out


def run_gpu(args):
    import torch

    from micmec_gb300 import _native as nat
    from micmec_gb300.pes.mmff import ForcePartMechanical

    rank, world, local = dist_env()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA GPU")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
        pg = dist

    s, d, vel = build_workload()
    M = s.ncells
    fp = ForcePartMechanical(s, model="nanocell", precision="fp32")
    L = nat.lib()
    stream = torch.cuda.current_stream().cuda_stream
    pos_d = torch.from_numpy(np.ascontiguousarray(s.pos)).to(dev)
    vel_d = torch.from_numpy(np.ascontiguousarray(vel)).to(dev)
    from micmec_gb300 import units

    dt, temp, tau = 1.0 * units.femtosecond, 300.0, 100.0 * units.femtosecond
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    rec = torch.empty((max(args.steps, 1), nat.MM_REC_LEN), dtype=torch.float64, device=dev)

    nat.check(L.mm_md_begin(fp.handle, pos_d.data_ptr(), vel_d.data_ptr(), dt, 1, temp, tau, SEED, None, 0, stream),
              "mm_md_begin")
    for _ in range(args.warmup):
        nat.check(L.mm_md_advance(fp.handle, 1, None, 0, stream), "mm_md_advance")
    torch.cuda.synchronize()

    # ---- timed region
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if pg is not None:
        pg.barrier()
    torch.cuda.synchronize()
    clocks.start()
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record()
        nat.check(L.mm_md_advance(fp.handle, 1, rec[i].data_ptr(), 0, stream), "mm_md_advance")
        ev[i][1].record()
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    if pg is not None:
        pg.barrier()
    # keep sampling a moment so short regions still have clock samples
    time.sleep(0.3)
    clk = clocks.stop()
    ms = float(sum(a.elapsed_time(b) for a, b in ev))
    if pg is not None:
        ms = max_over_ranks(ms, pg, dev)
    recs = rec.cpu().numpy()
    finite = bool(np.isfinite(recs[: args.steps, :2]).all())
    value = world * M * args.steps / (ms * 1e-3)

    # ---- per-kernel timing for the roofline (same session, same flush)
    nk = max(20, min(200, args.steps))
    mc, mn = nat.c_double(), nat.c_double()
    nat.check(L.mm_md_time_kernels(fp.handle, nk, flush.data_ptr(), FLUSH_BYTES, nat.ctypes.byref(mc),
                                   nat.ctypes.byref(mn), stream), "mm_md_time_kernels")
    cell_ms, node_ms = mc.value / nk, mn.value / nk
    nat.check(L.mm_md_advance(fp.handle, 1, None, 1, stream), "mm_md_advance")
    torch.cuda.synchronize()

    # ---- e2e through the host-buffer C-ABI step
    pos_h = torch.from_numpy(np.ascontiguousarray(s.pos)).pin_memory()
    vel_h = torch.from_numpy(np.ascontiguousarray(vel)).pin_memory()
    gpos_h = torch.zeros((s.nnodes, 3), dtype=torch.float64).pin_memory()
    rec_h = torch.zeros(nat.MM_REC_LEN, dtype=torch.float64).pin_memory()
    e_steps = max(3, min(args.steps, 50))
    fp.compute_device(pos_d.copy_(pos_h), None, None)  # warm
    for i in range(2 + e_steps):
        if i == 2:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
        nat.check(L.mm_md_step_host(fp.handle, pos_h.data_ptr(), vel_h.data_ptr(), gpos_h.data_ptr(),
                                    rec_h.data_ptr(), dt, 1, temp, tau, SEED, 10**6 + i), "mm_md_step_host")
    e2e_s = time.perf_counter() - t0
    e2e_value = world * M * e_steps / e2e_s
    link = host_link_rates(pos_h, dev)

    # ---- roofline of the dominant kernel (cells)
    hbm, kind = peaks()
    achieved = CELL_KERNEL_BYTES * M / (cell_ms * 1e-3) / 1e9
    # the standard fcu/reo types have diagonal h0 and cubic C: the kernel runs the reduced products
    flops = (FLOP_PER_STATE_CUBIC * 2 + FLOP_LSE) * M / (cell_ms * 1e-3) / 1e12
    # the reference's maths (general h0 / C products per corner and state) as the algorithmic count
    flops_ref = (FLOP_PER_STATE * 2 + FLOP_LSE) * M / (cell_ms * 1e-3) / 1e12
    # DRAM bytes of one launch of the same kernel on the same workload come from an ncu capture
    # (no in-process counter exists); the file names the kernel it was measured on
    traffic, traffic_src = None, None
    tfile = os.path.join(ROOT, "profiles", "cells_fp32_nanocell_traffic.json")
    if os.path.exists(tfile):
        with open(tfile) as f:
            tj = json.load(f)
        traffic = tj.get("bytes_per_launch_64cubed")
        traffic_src = "%s, %s: %s" % (tj.get("kernel"), tj.get("workload"), tj.get("source"))
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32-cell/f64-state", "data": "synthetic", "config": config(),
        "wall_s_timed_region": t_wall, "finite": finite,
        "kernel_ms": {"cells": cell_ms, "nodes": node_ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": traffic, "traffic_source": traffic_src, "peak_kind": kind,
                     "note": "cell kernel (one thread per cell) is FP32-pipe and latency bound; algorithmic bytes "
                             "per cell %d; per-step HBM fraction in step_hbm_gbs" % CELL_KERNEL_BYTES,
                     "compute": {"achieved_tflops_fp32": flops, "nominal_peak_tflops_fp32": fp32_peak,
                                 "frac_of_nominal": flops / fp32_peak,
                                 "achieved_tflops_fp32_reference_maths": flops_ref,
                                 "frac_of_nominal_reference_maths": flops_ref / fp32_peak,
                                 "note": "first pair: reduced cubic products as executed; second pair: the "
                                         "reference's general per-corner maths (2,400 flop per cell and state)"},
                     "step_hbm_gbs": STEP_BYTES * M * args.steps / (ms * 1e-3) / 1e9},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 3 * 24 * s.nnodes,
                "d2h_bytes_per_step": 3 * 24 * s.nnodes + 8 * nat.MM_REC_LEN, "host_link": link},
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
    }
    if rank == 0 and not args.no_extra:
        try:
            v64, ms64 = measure_lattice(s, vel, max(5, min(args.steps, 30)), flush, "fp64")
            line["fp64_lattice"] = {"value": v64, "unit": UNIT, "ms_per_step": ms64,
                                    "fp32_over_fp64": value / world / v64}
            line["fp32_error_vs_fp64"] = force_error_fp32(s)
            from micmec_gb300.system import System

            sg = System.from_dict(general_form(d))
            vg, msg = measure_lattice(sg, vel, max(5, min(args.steps, 30)), flush, "fp32")
            line["general_params_fp32"] = {"value": vg, "unit": UNIT, "ms_per_step": msg,
                                           "note": "anisotropic C, sheared h0: full 3x3/6x6 products"}
            systems, strains = batch_workload()
            bf = measure_batch(systems, strains, "fp32", 2000, 400, drift=True)
            bd = measure_batch(systems, strains, "fp64", 100, 100)
            # the plain FP64 GPU path, one system at a time: a sample across the size range
            sample = sorted(systems, key=lambda s: s.ncells)[:: max(1, len(systems) // 8)][:8]
            plain_dev = measure_plain_per_system(sample, 50, device=True)
            plain_host = measure_plain_per_system(sample[:4], 5, device=False)
            sx32 = np.array(list(bf["stress_xx_gpa_by_strain"].values()))
            sx64 = np.array(list(bd["stress_xx_gpa_by_strain"].values()))
            bf["stress_rel_err_vs_fp64"] = float(np.abs(sx32 - sx64).max() / np.abs(sx64).max())
            line["batched"] = {
                "fp32": bf, "fp64": bd, "plain_fp64_per_system_device_hooks": plain_dev,
                "plain_fp64_per_system_host_hooks": plain_host,
                "batched_fp32_over_batched_fp64_systems_per_s": bf["systems_steps_per_s"] / bd["systems_steps_per_s"],
                "batched_fp32_over_plain_fp64_device_systems_per_s":
                    bf["systems_steps_per_s"] / plain_dev["systems_steps_per_s"],
                "batched_fp32_over_plain_fp64_host_hooks_systems_per_s":
                    bf["systems_steps_per_s"] / plain_host["systems_steps_per_s"]}
        except Exception as exc:  # extra measurements never block the main line
            line["extra_error"] = _error_text(exc)
        for key, fn in (("drift_nve_64", lambda: measure_drift_nve(s, vel)),
                        ("models_fp32", lambda: measure_models(flush)),
                        ("builder", measure_builder), ("adjoint", measure_grad_over_fwd),
                        ("differentiation_16cubed", measure_config4), ("large_mtk", measure_large_mtk)):
            try:
                line[key] = fn()
            except Exception as exc:
                line[key] = {"error": _error_text(exc)}
    if rank == 0 and not args.no_cpu_baseline:
        nproc = 1
        sample_steps = 1
        tcpu = cpu_langevin_steps(d, vel, sample_steps, nproc)
        line["cpu_baseline"] = {"value": M * sample_steps / tcpu, "unit": UNIT, "cores": nproc, "kind": "port",
                                "sample": "%d full 64^3 Langevin step, NumPy FP64 oracle, 1 process" % sample_steps}
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the FP64 / batched / adjoint side measurements")
    ap.add_argument("--large-only", type=int, default=0, metavar="N",
                    help="only the large single-system NHC + MTK run (lattice engine) on an N^3 lattice")
    ap.add_argument("--config4", action="store_true",
                    help="only the differentiation workload (16^3, 11 relaxed strain points + 200-step trajectory)")
    ap.add_argument("--builder-only", type=int, default=0, metavar="N",
                    help="only the device system builder on an N^3 lattice with 20%% clustered defects, built "
                         "--warmup + --steps times (for kernel profiles)")
    ap.add_argument("--lattice-only", type=int, default=0, metavar="N",
                    help="only the Langevin step rate of an N^3 two-type two-state lattice with --model and "
                         "FP32 cells, --steps timed steps after --warmup (for kernel profiles)")
    ap.add_argument("--model", default="nanocell", choices=["nanocell", "original"])
    ap.add_argument("--batch-only", action="store_true",
                    help="only the batched workload (512 systems, NHC + MTK, FP32 cells): one warm-up launch of "
                         "--warmup steps and one launch of --steps steps, no autotuning or graph (for kernel profiles)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.batch_only:
        return run_batch_only(args)
    if args.lattice_only:
        return run_lattice_only(args)
    if args.large_only:
        print(json.dumps(measure_large_mtk(n=args.large_only, nsteps=args.steps)), flush=True)
        return 0
    if args.builder_only:
        return run_builder_only(args)
    if args.config4:
        print(json.dumps(measure_config4()), flush=True)
        return 0
    return run_gpu(args)


def run_lattice_only(args):
    import torch

    from micmec_gb300 import lattices, units
    from micmec_gb300.system import System

    n = args.lattice_only
    rng = np.random.default_rng(SEED + n)
    d = lattices.make_lattice(lattices.defect_grid(n, DEFECT, rng), nstates=2, device=n > 128)
    d["pos"] = lattices.displace(d["pos"], 0.05 * units.angstrom, rng)
    s = System.from_dict(d)
    vel = rng.normal(0.0, 1.0, s.pos.shape) * np.sqrt(units.boltzmann * 300.0 / s.masses)[:, None]
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    v, ms, cms, nms = lattice_md_rate(s, vel, args.model, "fp32", args.steps, flush)
    print(json.dumps({"lattice": [n] * 3, "model": args.model, "cell_steps_per_s": v, "ms_per_step": ms,
                      "cells_ms": cms, "nodes_ms": nms}), flush=True)
    return 0


def run_builder_only(args):
    import torch

    from micmec_gb300 import lattices
    from micmec_gb300.utils import build_system

    n = args.builder_only
    grid = lattices.defect_grid(n, 0.2, np.random.default_rng(5), clustered=True)
    data = lattices.standard_types(nstates=2)
    times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d = build_system(data, grid, pbc=True, device=True)
        times.append(time.perf_counter() - t0)
    print(json.dumps({"builder_lattice": [n] * 3, "cells": len(d["types"]), "nodes": len(d["masses"]),
                      "wall_s_median": float(np.median(times[args.warmup:]))}), flush=True)
    return 0


def run_batch_only(args):
    import torch

    from micmec_gb300 import units
    from micmec_gb300.batch import BatchSystems

    systems, _ = batch_workload()
    b = BatchSystems(systems, model="nanocell", precision="fp32")
    fs = units.femtosecond
    b.setup_md(temp=300.0, thermostat="nhc", barostat="mtk", timecon=100 * fs, baro_timecon=1000 * fs, seed=5)
    kw = dict(thermostat="nhc", temp=300.0, barostat="mtk", press=0.0, use_graph=False)
    b.md(args.warmup, **kw)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.md(args.steps, step0=args.warmup, **kw)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = float(np.sum(b.sizes))
    print(json.dumps({"workload": "batched 512 systems, NHC + MTK, FP32 cells", "steps": args.steps, "ms": ms,
                      "systems_steps_per_s": len(systems) * args.steps / (ms * 1e-3),
                      "cell_steps_per_s": cells * args.steps / (ms * 1e-3)}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
