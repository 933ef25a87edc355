"""CPU oracle for the Langevin/NVE velocity-Verlet step (test and baseline infrastructure).

Restates micmec/sampling/verlet.py:140-166 (half kick, drift, force evaluation,
half kick) with the Langevin thermostat of micmec/sampling/nvt.py:196-218
applied before and after each step, on top of the NumPy force oracle in
``oracle/mmff.py``. The force evaluation can be split by cells over a pool of
worker processes (start the pool with the 'spawn' method).
"""

import numpy as np

from oracle import mmff as om

_W = {}


def _init_worker(static):
    _W.clear()
    _W.update(static)


def _work(args):
    pos, rvecs, lo, hi = args
    cells = np.arange(lo, hi)
    e, g, _ = om.deformation(pos, rvecs, _W["grid"], _W["sn"], _W["types"], _W["params"], _W["model"],
                             cells=cells, shifts=_W["shifts"])
    return lo, e, g


class LangevinState(object):
    """State and stepper of a Langevin (or NVE with temp=None) MD run on the oracle forces."""

    def __init__(self, d, vel, model="nanocell", temp=300.0, timecon_fs=100.0, dt_fs=1.0, seed=0, pool=None,
                 nproc=1):
        self.d = d
        self.model = model
        self.pos = np.array(d["pos"], dtype=np.float64)
        self.vel = np.array(vel, dtype=np.float64)
        self.masses = np.asarray(d["masses"], dtype=np.float64)
        self.rvecs = np.asarray(d["rvecs"], dtype=np.float64).reshape(-1, 3)
        fs = 1e-15 / 2.418884326500e-17
        self.dt = dt_fs * fs
        self.temp = temp
        self.tau = timecon_fs * fs
        self.rng = np.random.default_rng(seed)
        self.params = {k: v for k, v in d.items() if "/" in k} if "params" not in d else d["params"]
        self.sn = np.asarray(d["surrounding_nodes"])
        self.sc = np.asarray(d["surrounding_cells"])
        self.grid = np.asarray(d["grid"])
        self.types = np.asarray(d["types"])
        self.shifts = om.cell_shifts(self.grid, self.sn, self.rvecs.shape[0] == 3)
        self.pool = pool
        self.nproc = nproc
        if pool is not None:
            static = dict(grid=self.grid, sn=self.sn, types=self.types, params=self.params, model=model,
                          shifts=self.shifts)
            pool.map(_init_worker, [static] * nproc)
        self.epot, self.gpos = self.forces()

    def forces(self, ncells=None):
        """Energy and gradient; with ``ncells`` only the first ncells cells contribute (a bounded sample)."""
        M = len(self.sn) if ncells is None else int(ncells)
        if self.pool is None:
            e, g, _ = om.deformation(self.pos, self.rvecs, self.grid, self.sn, self.types, self.params, self.model,
                                     shifts=self.shifts, cells=None if ncells is None else np.arange(M))
            if ncells is not None:
                gfull = np.zeros((len(self.sn), 8, 3))
                gfull[:M] = g
                g = gfull
        else:
            bounds = np.linspace(0, M, 4 * self.nproc + 1).astype(int)
            parts = self.pool.map(_work, [(self.pos, self.rvecs, lo, hi) for lo, hi in zip(bounds[:-1], bounds[1:])])
            e = np.zeros(M)
            g = np.zeros((len(self.sn), 8, 3))
            for lo, ee, gg in parts:
                e[lo:lo + len(ee)] = ee
                g[lo:lo + len(ee)] = gg
        return float(np.sum(e)), om.gather_gpos(g, self.sc)

    def thermo(self):
        if self.temp is None:
            return
        c1 = np.exp(-self.dt / self.tau / 2)
        c2 = np.sqrt((1.0 - c1**2) * self.temp * om.BOLTZMANN / self.masses).reshape(-1, 1)
        self.vel = c1 * self.vel + c2 * self.rng.normal(0, 1, self.vel.shape)

    def step(self, ncells=None):
        """One step; ``ncells`` restricts the force evaluation to a sample of the cells."""
        self.thermo()
        self.vel += 0.5 * (-self.gpos / self.masses[:, None]) * self.dt
        self.pos += self.dt * self.vel
        self.epot, self.gpos = self.forces(ncells)
        self.vel += 0.5 * (-self.gpos / self.masses[:, None]) * self.dt
        self.thermo()
        return self.epot
