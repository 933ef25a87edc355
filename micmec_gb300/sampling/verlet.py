"""Velocity-Verlet integrator with the Verlet-hook protocol.

Interface of micmec/sampling/verlet.py:49-374 (``VerletIntegrator``,
``VerletHook``, ``VerletScreenLog``, ``ConsErrTracker``).

Two execution paths with the same results:

* device paths (used by ``run`` when the force field is a single
  ``ForcePartMechanical``): with no Verlet hook or a ``LangevinThermostat`` the whole
  step loop runs on the GPU (``mm_md_run``: one cell kernel and one fused
  gather/kick/thermostat/drift kernel per step); with a Nose-Hoover-chain, Berendsen or
  CSVR thermostat and/or an anisotropic MTK, Berendsen or Langevin barostat (alone or in
  a ``TBCombination``) the hooks run on the GPU too: in the one-CTA persistent batch
  kernel for systems up to ``batch_max_cells`` cells, else in the grid-wide lattice
  engine (``mm_md_engine``). Positions and velocities stay in device memory and are
  copied back only where a regular hook expects a call;
* host path (any other combination): the reference's step order on the host, with
  every force evaluation on the GPU.
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
        spec = self._batch_spec(vhooks, parts[0])
        if spec is not None:
            return ("batch", spec)
        return False

    # systems up to this many cells run the thermostat / barostat hooks in the one-CTA batch kernel
    batch_max_cells = 32768

    def _batch_spec(self, vhooks, part):
        """Hook set the persistent kernels run: a thermostat (NHC, Langevin, Berendsen, CSVR) and/or a
        barostat (MTK, Berendsen, Langevin, each anisotropic, isotropic or volume-constrained; the MTK
        barostat with a chain of its own), alone or in a TBCombination."""
        from micmec_gb300.sampling.npt import BerendsenBarostat, LangevinBarostat, MTKBarostat, TBCombination
        from micmec_gb300.sampling.nvt import BerendsenThermostat, CSVRThermostat, LangevinThermostat, NHCThermostat

        if len(vhooks) != 1 or not part.handle:
            return None
        h = vhooks[0]
        if h.start != 0 or h.step != 1:
            return None
        thermo, baro = None, None
        if isinstance(h, TBCombination):
            thermo, baro = h.thermostat, h.barostat
            if thermo.step != 1 or baro.step != 1 or thermo.start != 0 or baro.start != 0:
                return None
        elif type(h) in (NHCThermostat, BerendsenThermostat, CSVRThermostat):
            thermo = h
        elif type(h) in (MTKBarostat, BerendsenBarostat, LangevinBarostat):
            baro = h
        else:
            return None
        if thermo is not None and type(thermo) not in (NHCThermostat, LangevinThermostat, BerendsenThermostat,
                                                       CSVRThermostat):
            return None
        if type(thermo) is CSVRThermostat and baro is not None:
            return None
        if baro is not None:
            if type(baro) not in (MTKBarostat, BerendsenBarostat, LangevinBarostat):
                return None
            if not baro.anisotropic and baro.vol_constraint:
                return None
            bt = getattr(baro, "baro_thermo", None)
            if bt is not None and (type(bt) is not NHCThermostat or not 1 <= bt.chain.length <= 3):
                return None
            if not part.pbc:
                return None
        if type(thermo) is NHCThermostat and thermo.chain.length != 3:
            return None
        s = self.mmf.system
        grid = np.asarray(s.grid)
        small = (part.pbc and not (grid == 0).any() and s.nnodes == grid.size and s.ncells <= self.batch_max_cells)
        return dict(hook=h, thermo=thermo, baro=baro, engine="batch" if small else "lattice")

    def _hook_control(self, thermo, baro):
        """Control block (layout of the batch/engine kernels) and kernel arguments from the
        initialised hooks: (ctl, thermostat kind, barostat code, temp, timecon, seed)."""
        from micmec_gb300.batch import CTL, CTL_LEN, baro_code
        from micmec_gb300.sampling.npt import BerendsenBarostat, LangevinBarostat, MTKBarostat
        from micmec_gb300.sampling.nvt import BerendsenThermostat, CSVRThermostat, LangevinThermostat, NHCThermostat

        c = np.zeros(CTL_LEN)
        c[CTL["ndof"]] = self.ndof
        kind, bkind, temp, timecon, seed = None, None, 0.0, 1.0, 0
        if thermo is not None:
            kind = {NHCThermostat: "nhc", LangevinThermostat: "langevin", BerendsenThermostat: "berendsen",
                    CSVRThermostat: "csvr"}[type(thermo)]
            temp = thermo.temp
            timecon = thermo.chain.timecon if kind == "nhc" else thermo.timecon
            c[CTL["econs_thermo"]] = thermo.econs_correction
            seed = getattr(thermo, "seed", 0)
        if type(thermo) is NHCThermostat:
            c[CTL["chain_pos"]] = thermo.chain.pos
            c[CTL["chain_vel"]] = thermo.chain.vel
            c[CTL["chain_mass"]] = thermo.chain.masses
            c[CTL["chain_ndof"]] = thermo.chain.ndof
        if baro is not None:
            bkind = {MTKBarostat: "mtk", BerendsenBarostat: "berendsen", LangevinBarostat: "langevin"}[type(baro)]
            vp = getattr(baro, "vel_press", None)
            if vp is not None:
                if baro.anisotropic:
                    c[CTL["vel_press"]] = np.asarray(vp).ravel()
                else:  # the isotropic MTK barostat's scalar velocity
                    c[CTL["vel_press"].start] = float(vp)
            bt = getattr(baro, "baro_thermo", None)
            if bt is not None:
                n = bt.chain.length
                c[CTL["bchain_pos"].start:CTL["bchain_pos"].start + n] = bt.chain.pos
                c[CTL["bchain_vel"].start:CTL["bchain_vel"].start + n] = bt.chain.vel
                c[CTL["bchain_mass"].start:CTL["bchain_mass"].start + n] = bt.chain.masses
                c[CTL["bchain_temp"]] = bt.chain.temp
            c[CTL["mass_press"]] = baro.mass_press
            c[CTL["baro_ndof"]] = baro.baro_ndof
            c[CTL["econs_baro"]] = baro.econs_correction
            if bkind == "langevin":
                c[CTL["timecon_press"]] = baro.timecon
                c[CTL["temp_press"]] = baro.temp
                if kind not in ("langevin", "csvr"):
                    seed = baro.seed
            if thermo is None:
                temp = baro.temp
            bkind = baro_code(bkind, baro.anisotropic, baro.vol_constraint, 0 if bt is None else bt.chain.length)
        return c, kind, bkind, temp, timecon, seed

    def _replays(self, thermo, baro, nsteps):
        """Replayed draws of the stochastic hooks for the next nsteps steps: (Langevin thermostat
        normals (2 nsteps, N, 3) or None, hook draws (nsteps, HOOK_NOISE_LEN) or None)."""
        from micmec_gb300.batch import HOOK_NOISE_LEN
        from micmec_gb300.sampling.npt import LangevinBarostat
        from micmec_gb300.sampling.nvt import CSVRThermostat, LangevinThermostat

        noise, hook = None, None
        if type(thermo) is LangevinThermostat and thermo.replay_noise is not None:
            i0 = 2 * (self.counter - thermo.replay_offset)
            noise = np.ascontiguousarray(thermo.replay_noise[i0:i0 + 2 * nsteps])
            if noise.shape[0] != 2 * nsteps:
                raise ValueError("replay_noise is too short for this run")
        sources = []
        if type(thermo) is CSVRThermostat and thermo.replay_noise is not None:
            sources.append((thermo, slice(0, 2), 2))
        if type(baro) is LangevinBarostat and baro.replay_noise is not None:
            sources.append((baro, slice(2, 26), 24))
        stochastic = int(type(thermo) is CSVRThermostat) + int(type(baro) is LangevinBarostat)
        if sources:
            if len(sources) != stochastic:
                raise ValueError("replay draws for some stochastic hooks but not for others")
            hook = np.zeros((nsteps, HOOK_NOISE_LEN))
            for h, cols, n in sources:
                i0 = self.counter - h.replay_offset
                rows = np.asarray(h.replay_noise[i0:i0 + nsteps]).reshape(-1, n)
                if rows.shape[0] != nsteps:
                    raise ValueError("replay_noise is too short for this run")
                hook[:, cols] = rows
        return noise, hook

    def _hook_back(self, thermo, baro, c):
        """Hook state after a device run, from the returned control block."""
        from micmec_gb300.batch import CTL
        from micmec_gb300.sampling.nvt import NHCThermostat

        if type(thermo) is NHCThermostat:
            thermo.chain.pos[:] = c[CTL["chain_pos"]]
            thermo.chain.vel[:] = c[CTL["chain_vel"]]
        if baro is not None and getattr(baro, "vel_press", None) is not None:
            if baro.anisotropic:
                baro.vel_press = c[CTL["vel_press"]].reshape(3, 3).copy()
            else:
                baro.vel_press = float(c[CTL["vel_press"].start])
        bt = getattr(baro, "baro_thermo", None)
        if bt is not None:
            n = bt.chain.length
            bt.chain.pos[:] = c[CTL["bchain_pos"].start:CTL["bchain_pos"].start + n]
            bt.chain.vel[:] = c[CTL["bchain_vel"].start:CTL["bchain_vel"].start + n]

    def _run_batch(self, nsteps, spec):
        """Thermostat / barostat hooks on the device: the system as a one-element batch (one persistent CTA)."""
        from micmec_gb300.batch import CTL, BatchSystems

        part = self.mmf.parts[0]
        thermo, baro, hook = spec["thermo"], spec["baro"], spec["hook"]
        b = getattr(self, "_batch", None)
        if b is None:
            b = self._batch = BatchSystems([self.mmf.system], model=part.model, precision=part.precision)
        b.set_state([self.pos], [self.vel], [self.mmf.system.domain.rvecs])
        c, kind, bkind, temp, timecon, seed = self._hook_control(thermo, baro)
        c0 = b.control()[0]
        for key in ("L", "rvecs", "volume"):  # lattice matrix and domain as set_state left them
            c[CTL[key]] = c0[CTL[key]]
        c[CTL["epot"]] = self.epot
        c[CTL["vtens"]] = self.vtens.ravel()
        b.set_control(c[None, :])
        noise, hook_noise = self._replays(thermo, baro, nsteps)
        if noise is not None:
            noise = noise.reshape(nsteps, 2, -1, 3)
        if hook_noise is not None:
            hook_noise = hook_noise[:, None, :]
        rec = b.md(nsteps, timestep=self.timestep, thermostat=kind, temp=temp, timecon=timecon, barostat=bkind,
                   press=0.0 if baro is None else baro.press, seed=seed, step0=self.counter, noise=noise,
                   hook_noise=hook_noise, record=True, use_graph=False)[0]
        if not np.isfinite(rec[:, :3]).all():
            raise ValueError("The energy is not-a-number (``nan``).")
        pos, vel, rv = b.get_state()
        c = b.control()[0]
        self._hook_back(thermo, baro, c)
        return rec, pos[0], vel[0], rv[0], c, (thermo, baro, hook)

    def _run_engine(self, nsteps, spec):
        """Thermostat / barostat hooks on the device for a system spread over the whole GPU (mm_md_engine)."""
        import torch

        from micmec_gb300 import _native as nat
        from micmec_gb300.batch import CTL, REC_LEN, _THERMO, baro_code

        part = self.mmf.parts[0]
        thermo, baro, hook = spec["thermo"], spec["baro"], spec["hook"]
        c, kind, bkind, temp, timecon, seed = self._hook_control(thermo, baro)
        c[CTL["epot"]] = self.epot
        c[CTL["vtens"]] = self.vtens.ravel()
        dev = part.device
        pos_d = torch.from_numpy(np.ascontiguousarray(self.pos)).to(dev)
        vel_d = torch.from_numpy(np.ascontiguousarray(self.vel)).to(dev)
        rec = torch.zeros((nsteps, REC_LEN), dtype=torch.float64, device=dev)
        noise, hook_noise = self._replays(thermo, baro, nsteps)
        noise = None if noise is None else torch.from_numpy(noise).to(dev)
        hook_noise = None if hook_noise is None else torch.from_numpy(np.ascontiguousarray(hook_noise)).to(dev)
        st = nat.lib().mm_md_engine(part.handle, pos_d.data_ptr(), vel_d.data_ptr(), int(nsteps), float(self.timestep),
                                    _THERMO[kind], float(temp), float(timecon), baro_code(bkind),
                                    0.0 if baro is None else float(baro.press), 3, int(seed), nat.ptr(noise),
                                    nat.ptr(hook_noise), c.ctypes.data, rec.data_ptr(), int(self.counter),
                                    torch.cuda.current_stream().cuda_stream)
        nat.check(st, "mm_md_engine")
        rec = rec.cpu().numpy()
        if not np.isfinite(rec[:, :3]).all():
            raise ValueError("The energy is not-a-number (``nan``).")
        self._hook_back(thermo, baro, c)
        rv = c[CTL["rvecs"]].reshape(3, 3).copy()
        return rec, pos_d.cpu().numpy(), vel_d.cpu().numpy(), rv, c, (thermo, baro, hook)

    def _finish_batch_chunk(self, rec, pos, vel, rv, ctl, hooks):
        from micmec_gb300.batch import CTL, REC

        thermo, baro, hook = hooks
        for r in rec:
            self.counter += 1
            self.time += self.timestep
            self.epot = r[REC["epot"]]
            self.ekin = r[REC["ekin"]]
            hook.econs_correction = r[REC["ecorr"]]
            self.vtens = r[REC["vtens"]].reshape(3, 3).copy()
            if baro is not None:
                self.mmf.system.domain.update_rvecs(r[REC["rvecs"]].reshape(3, 3))
            self._finish_properties(ktens=r[REC["ktens"]].reshape(3, 3))
        if thermo is not None and thermo is not hook:
            thermo.econs_correction = ctl[CTL["econs_thermo"]]
        if baro is not None and baro is not hook:
            baro.econs_correction = ctl[CTL["econs_baro"]]
        self.pos[:] = pos
        self.vel[:] = vel
        if baro is not None:
            self.rvecs[:] = rv
            self.mmf.update_rvecs(rv)
        self.mmf.update_pos(self.pos)
        self.delta[:] = self.pos - self.posold
        self.posold[:] = self.pos
        self.rmsd_delta = np.sqrt(np.mean(self.delta**2))

    def run(self, nsteps=None):
        plan = self._device_plan() if nsteps is not None else False
        if plan is False:
            return Iterative.run(self, nsteps)
        if isinstance(plan, tuple) and plan[0] == "batch":
            remaining = int(nsteps)
            while remaining > 0:
                k = self._next_hook_gap(remaining)
                if plan[1]["engine"] == "batch":
                    out = self._run_batch(k, plan[1])
                else:
                    out = self._run_engine(k, plan[1])
                self._finish_batch_chunk(*out)
                remaining -= k
                self.call_hooks()
        else:
            self._run_device(int(nsteps), plan)
        self.finalize()

    def _next_hook_gap(self, remaining, counter=None):
        counter = self.counter if counter is None else counter
        gap = remaining
        for hook in self.hooks:
            if isinstance(hook, VerletHook) or (isinstance(hook, VerletScreenLog) and not hook.verbose):
                continue
            c = counter + 1
            if c < hook.start:
                c = hook.start
            else:
                c = c + (-(c - hook.start)) % hook.step
            gap = min(gap, c - counter)
        return max(1, min(gap, self.chunk))

    def _hooks_read_only(self, counter):
        """True when every hook due at ``counter`` only reads the state."""
        return all(isinstance(h, VerletHook) or not h.modifies_state or not h.expects_call(counter)
                   for h in self.hooks)

    def _run_device(self, nsteps, thermo):
        """NVE / Langevin steps in ``mm_md_run`` chunks that end where a regular hook is due.

        The state stays on the device. After each chunk the positions, velocities and
        per-step records are copied into pinned host buffers (two slots, alternating); when
        every hook due at the chunk's end only reads the state (writers, logs), the next
        chunk is launched before the host processes the records and runs the hooks on the
        snapshot, so the GPU keeps stepping while they write. A hook that may change the
        state runs before the next launch, and its changes to ``pos`` / ``vel`` are uploaded.
        """
        import torch

        from micmec_gb300 import _native as nat

        fp = self.mmf.parts[0]
        dev = fp.device
        pos_d = torch.from_numpy(np.ascontiguousarray(self.pos)).to(dev)
        vel_d = torch.from_numpy(np.ascontiguousarray(self.vel)).to(dev)
        kind, temp, timecon = 0, 0.0, 1.0
        if thermo is not None:
            kind, temp, timecon = 1, float(thermo.temp), float(thermo.timecon)
        seed = 0 if thermo is None else thermo.seed
        stream = torch.cuda.current_stream()
        chunks, c, rem = [], self.counter, nsteps
        while rem > 0:
            k = self._next_hook_gap(rem, c)
            chunks.append((c, k))
            c += k
            rem -= k
        kmax = max(k for _, k in chunks)
        slots = [dict(rec_d=torch.empty((kmax, nat.MM_REC_LEN), dtype=torch.float64, device=dev),
                      rec=torch.empty((kmax, nat.MM_REC_LEN), dtype=torch.float64).pin_memory(),
                      pos=torch.empty(pos_d.shape, dtype=torch.float64).pin_memory(),
                      vel=torch.empty(vel_d.shape, dtype=torch.float64).pin_memory(),
                      ev=torch.cuda.Event()) for _ in range(2)]
        pending = None
        for i, (c0, k) in enumerate(chunks):
            sl = slots[i % 2]
            noise = None
            if thermo is not None and thermo.replay_noise is not None:
                i0 = 2 * (c0 - thermo.replay_offset)
                noise = torch.from_numpy(np.ascontiguousarray(thermo.replay_noise[i0:i0 + 2 * k])).to(dev)
                if noise.shape[0] != 2 * k:
                    raise ValueError("replay_noise is too short for this run")
            st = nat.lib().mm_md_run(fp.handle, pos_d.data_ptr(), vel_d.data_ptr(), k, float(self.timestep), kind,
                                     temp, timecon, seed, nat.ptr(noise), sl["rec_d"].data_ptr(), int(c0),
                                     stream.cuda_stream)
            nat.check(st, "mm_md_run")
            sl["rec"][:k].copy_(sl["rec_d"][:k], non_blocking=True)
            sl["pos"].copy_(pos_d, non_blocking=True)
            sl["vel"].copy_(vel_d, non_blocking=True)
            sl["ev"].record(stream)
            if pending is not None:  # the previous chunk's hooks run while this chunk steps
                self._finish_device_chunk(*pending, thermo)
            pending = (sl, k)
            if not self._hooks_read_only(c0 + k):
                self._finish_device_chunk(sl, k, thermo)
                pending = None
                pos_d.copy_(torch.from_numpy(np.ascontiguousarray(self.pos)))
                vel_d.copy_(torch.from_numpy(np.ascontiguousarray(self.vel)))
        if pending is not None:
            self._finish_device_chunk(*pending, thermo)

    def _finish_device_chunk(self, sl, k, thermo):
        from micmec_gb300 import _native as nat

        sl["ev"].synchronize()
        recs = sl["rec"][:k].numpy()
        if not np.isfinite(recs[:, :3]).all():
            raise ValueError("The energy is not-a-number (``nan``).")
        self.pos[:] = sl["pos"].numpy()
        self.vel[:] = sl["vel"].numpy()
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
        # The reference accepts start and step but calls every Verlet hook at every step
        # from step 0 (its VerletHook passes start=0, step=1 to Hook, verlet.py:316-327);
        # trajectories are kept identical to the reference's, so this does the same.
        self.econs_correction = 0.0
        Hook.__init__(self, start=0, step=1)

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

    modifies_state = False

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
