"""Velocity-Verlet integrator with the Verlet-hook protocol.

Interface of micmec/sampling/verlet.py:49-374 (``VerletIntegrator``,
``VerletHook``, ``VerletScreenLog``, ``ConsErrTracker``).

Two execution paths with the same results:

* device path (used by ``run`` when the force field is a single
  ``ForcePartMechanical`` and the only Verlet hook is absent or a
  ``LangevinThermostat``): the whole step loop runs on the GPU
  (``mm_md_run``: one cell kernel and one fused gather/kick/thermostat/drift
  kernel per step); positions and velocities stay in device memory and are
  copied back only where a regular hook expects a call;
* host path (any other combination, e.g. NHC thermostats and the MTK
  barostat): the reference's step order on the host, with every force
  evaluation on the GPU.
"""

import time

import numpy as np

from micmec_gb300.units import boltzmann, kelvin
from micmec_gb300.sampling.iterative import (
    Iterative, Hook, AttributeStateItem, PosStateItem, TemperatureStateItem, VolumeStateItem, DomainStateItem,
)
from micmec_gb300.sampling.utils import get_random_vel, clean_momenta

__all__ = ["VerletIntegrator", "VerletHook", "VerletScreenLog", "ConsErrTracker"]


class VerletIntegrator(Iterative):
    default_state = [
        AttributeStateItem("counter"), AttributeStateItem("time"), AttributeStateItem("epot"), PosStateItem(),
        AttributeStateItem("vel"), AttributeStateItem("rmsd_delta"), AttributeStateItem("rmsd_gpos"),
        AttributeStateItem("ekin"), TemperatureStateItem(), AttributeStateItem("etot"), AttributeStateItem("econs"),
        AttributeStateItem("cons_err"), AttributeStateItem("ptens"), AttributeStateItem("vtens"),
        AttributeStateItem("press"), VolumeStateItem(), DomainStateItem(),
    ]
    log_name = "VERLET"

    def __init__(self, mmf, timestep=None, state=None, hooks=None, vel0=None, temp0=300 * kelvin, scalevel0=True,
                 time0=None, ndof=None, counter0=None, device=True, chunk=1000):
        self.ndof = ndof
        self.hooks = hooks
        self.device = device
        self.chunk = int(chunk)
        self.pos = mmf.system.pos.copy()
        self.rvecs = mmf.system.domain.rvecs.copy()
        self.masses = mmf.system.masses.copy()
        self.timestep = timestep
        self.time = 0.0 if time0 is None else time0
        self._verify_hooks()
        if vel0 is None:
            self.vel = get_random_vel(temp0, scalevel0, self.masses)
            clean_momenta(self.pos, self.vel, self.masses, mmf.system.domain)
        else:
            self.vel = vel0.copy()
        self.gpos = np.zeros(self.pos.shape, float)
        self.delta = np.zeros(self.pos.shape, float)
        self.vtens = np.zeros((3, 3), float)
        self._cons_err_tracker = ConsErrTracker()
        Iterative.__init__(self, mmf, state, self.hooks, 0 if counter0 is None else counter0)

    # ------------------------------------------------------------ reference step
    def initialize(self):
        self.gpos[:] = 0.0
        self.delta[:] = 0.0
        self.mmf.update_pos(self.pos)
        self.epot = self.mmf.compute(self.gpos)
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.posold = self.pos.copy()
        self.call_verlet_hooks("init")
        if self.ndof is None:
            self.ndof = np.size(self.pos)
        self.compute_properties()
        Iterative.initialize(self)

    def propagate(self):
        self.call_verlet_hooks("pre")
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.vel += 0.5 * self.acc * self.timestep
        self.pos += self.timestep * self.vel
        self.mmf.update_pos(self.pos)
        self.gpos[:] = 0.0
        self.vtens[:] = 0.0
        self.epot = self.mmf.compute(self.gpos, self.vtens)
        self.acc = -self.gpos / self.masses.reshape(-1, 1)
        self.vel += 0.5 * self.acc * self.timestep
        self.ekin = self._compute_ekin()
        self.call_verlet_hooks("post")
        self.posnew = self.pos.copy()
        self.delta[:] = self.posnew - self.posold
        self.posold[:] = self.posnew
        self.time += self.timestep
        self.compute_properties()
        Iterative.propagate(self)

    def _compute_ekin(self):
        return np.sum(0.5 * (self.vel**2.0 * self.masses.reshape(-1, 1)))

    def compute_properties(self):
        self.rmsd_gpos = np.sqrt(np.mean(self.gpos**2))
        self.rmsd_delta = np.sqrt(np.mean(self.delta**2))
        self.ekin = self._compute_ekin()
        self._finish_properties()

    def _finish_properties(self, ktens=None):
        self.temp = (self.ekin / self.ndof) * (2.0 / boltzmann)
        self.etot = self.ekin + self.epot
        self.econs = self.etot
        for hook in self.hooks:
            if isinstance(hook, VerletHook):
                self.econs += hook.econs_correction
        self._cons_err_tracker.update(self.ekin, self.econs)
        self.cons_err = self._cons_err_tracker.get()
        if self.mmf.system.domain.nvec > 0:
            if ktens is None:
                ktens = np.dot(self.vel.T * self.masses, self.vel)
            self.ptens = (ktens - self.vtens) / self.mmf.system.domain.volume
            self.press = np.trace(self.ptens) / 3.0

    def call_verlet_hooks(self, kind):
        for hook in self.hooks:
            if isinstance(hook, VerletHook) and hook.expects_call(self.counter):
                if kind == "init":
                    hook.init(self)
                elif kind == "pre":
                    hook.pre(self)
                elif kind == "post":
                    hook.post(self)
                else:
                    raise NotImplementedError

    def _add_default_hooks(self):
        if not any(isinstance(hook, VerletScreenLog) for hook in self.hooks):
            self.hooks.append(VerletScreenLog())

    def _verify_hooks(self):
        """Merge a separate thermostat and barostat into a TBCombination (verlet.py:216-272)."""
        if self.hooks is None:
            return
        hooks = self.hooks if hasattr(self.hooks, "__len__") else [self.hooks]
        thermo = [h for h in hooks if getattr(h, "method", None) == "thermostat"]
        baro = [h for h in hooks if getattr(h, "method", None) == "barostat"]
        if thermo and baro:
            from micmec_gb300.sampling.npt import TBCombination

            t, b = thermo[-1], baro[-1]
            rest = [h for h in hooks if h is not t and h is not b]
            rest.append(TBCombination(t, b))
            if hasattr(self.hooks, "__len__"):
                self.hooks[:] = rest
            else:
                self.hooks = rest

    # ------------------------------------------------------------ device path
    def _device_plan(self):
        """(thermostat or None) if the device path applies, else False."""
        if not self.device:
            return False
        from micmec_gb300.pes.mmff import ForcePartMechanical
        from micmec_gb300.sampling.nvt import LangevinThermostat

        parts = getattr(self.mmf, "parts", None)
        if not parts or len(parts) != 1 or not isinstance(parts[0], ForcePartMechanical):
            return False
        vhooks = [h for h in self.hooks if isinstance(h, VerletHook)]
        if not vhooks:
            return None
        if len(vhooks) == 1 and type(vhooks[0]) is LangevinThermostat and vhooks[0].start == 0 and vhooks[0].step == 1:
            return vhooks[0]
        return False

    def run(self, nsteps=None):
        plan = self._device_plan() if nsteps is not None else False
        if plan is False:
            return Iterative.run(self, nsteps)
        self._run_device(int(nsteps), plan)
        self.finalize()

    def _next_hook_gap(self, remaining):
        gap = remaining
        for hook in self.hooks:
            if isinstance(hook, VerletHook) or (isinstance(hook, VerletScreenLog) and not hook.verbose):
                continue
            c = self.counter + 1
            if c < hook.start:
                c = hook.start
            else:
                c = c + (-(c - hook.start)) % hook.step
            gap = min(gap, c - self.counter)
        return max(1, min(gap, self.chunk))

    def _run_device(self, nsteps, thermo):
        import torch

        from micmec_gb300 import _native as nat

        fp = self.mmf.parts[0]
        dev = fp.device
        pos_d = torch.from_numpy(np.ascontiguousarray(self.pos)).to(dev)
        vel_d = torch.from_numpy(np.ascontiguousarray(self.vel)).to(dev)
        kind, temp, timecon = 0, 0.0, 1.0
        if thermo is not None:
            kind, temp, timecon = 1, float(thermo.temp), float(thermo.timecon)
        stream = torch.cuda.current_stream().cuda_stream
        remaining = nsteps
        while remaining > 0:
            k = self._next_hook_gap(remaining)
            rec = torch.empty((k, nat.MM_REC_LEN), dtype=torch.float64, device=dev)
            noise = None
            if thermo is not None and thermo.replay_noise is not None:
                i0 = 2 * (self.counter - thermo.replay_offset)
                noise = torch.from_numpy(np.ascontiguousarray(thermo.replay_noise[i0:i0 + 2 * k])).to(dev)
                if noise.shape[0] != 2 * k:
                    raise ValueError("replay_noise is too short for this run")
            seed = 0 if thermo is None else thermo.seed
            st = nat.lib().mm_md_run(fp.handle, pos_d.data_ptr(), vel_d.data_ptr(), k, float(self.timestep), kind,
                                     temp, timecon, seed, nat.ptr(noise), rec.data_ptr(), int(self.counter), stream)
            nat.check(st, "mm_md_run")
            recs = rec.cpu().numpy()
            if not np.isfinite(recs[:, :3]).all():
                raise ValueError("The energy is not-a-number (``nan``).")
            self.pos[:] = pos_d.cpu().numpy()
            self.vel[:] = vel_d.cpu().numpy()
            for i in range(k):
                r = recs[i]
                self.counter += 1
                self.time += self.timestep
                self.epot = r[nat.REC["epot"]]
                self.ekin = r[nat.REC["ekin"]]
                if thermo is not None:
                    thermo.econs_correction += r[nat.REC["decons"]]
                self.vtens = r[nat.REC["vtens"]].reshape(3, 3).copy()
                self._finish_properties(ktens=r[nat.REC["ktens"]].reshape(3, 3))
            self.mmf.update_pos(self.pos)
            self.delta[:] = self.pos - self.posold
            self.posold[:] = self.pos
            self.rmsd_delta = np.sqrt(np.mean(self.delta**2))
            remaining -= k
            self.call_hooks()


class ConsErrTracker(object):
    """Running variances of ekin and econs (Welford; verlet.py:275-307)."""

    def __init__(self):
        self.counter = 0
        self.ekin_m = self.ekin_s = self.econs_m = self.econs_s = 0.0

    def update(self, ekin, econs):
        if self.counter == 0:
            self.ekin_m = ekin
            self.econs_m = econs
        else:
            d = ekin - self.ekin_m
            self.ekin_m += d / (self.counter + 1)
            self.ekin_s += d * (ekin - self.ekin_m)
            d = econs - self.econs_m
            self.econs_m += d / (self.counter + 1)
            self.econs_s += d * (econs - self.econs_m)
        self.counter += 1

    def get(self):
        if self.counter > 1 and self.ekin_s > 0:
            return np.sqrt(self.econs_s / self.ekin_s)
        return 0.0


class VerletHook(Hook):
    """Hook with init/pre/post calls around each Verlet step (thermostats, barostats)."""

    def __init__(self, start=0, step=1):
        self.econs_correction = 0.0
        Hook.__init__(self, start=start, step=step)

    def __call__(self, iterative):
        pass

    def init(self, iterative):
        raise NotImplementedError

    def pre(self, iterative):
        raise NotImplementedError

    def post(self, iterative):
        raise NotImplementedError


class VerletScreenLog(Hook):
    """Screen logger (silent unless ``verbose``)."""

    def __init__(self, start=0, step=1, verbose=False):
        Hook.__init__(self, start, step)
        self.time0 = None
        self.verbose = verbose

    def __call__(self, iterative):
        if not self.verbose:
            return
        if self.time0 is None:
            self.time0 = time.time()
            print("counter  Cons.Err.       Temp     d-RMSD     g-RMSD   Walltime")
        print("%7i %10.5f %10.2f %10.3e %10.3e %10.1f" % (
            iterative.counter, iterative.cons_err, iterative.temp, iterative.rmsd_delta, iterative.rmsd_gpos,
            time.time() - self.time0))
