"""CPU oracle for the Langevin/NVE velocity-Verlet step (test and baseline infrastructure).

Restates micmec/sampling/verlet.py:140-166 (half kick, drift, force evaluation,
half kick) with the Langevin thermostat of micmec/sampling/nvt.py:196-218
applied before and after each step, on top of the NumPy force oracle in
``oracle/mmff.py``. The force evaluation can be split by cells over a pool of
worker processes (start the pool with the 'spawn' method); every task carries the
data of its cells, so the workers hold no state.
"""

import numpy as np

from oracle import mmff as om


def chunk_deformation(job):
    """Energies and corner gradients of one chunk of cells (a worker-process task).

    The job carries everything the chunk needs, so workers keep no state: the corner
    positions of its cells (m, 8, 3), rvecs, cell types, image shifts, parameters and
    model. Returns (per-cell energies, corner gradients, vertices).
    """
    corner_pos, rvecs, types, shifts, params, model = job
    m = len(types)
    sn = np.arange(8 * m, dtype=np.int64).reshape(m, 8)
    return om.deformation(corner_pos.reshape(-1, 3), rvecs, None, sn, types, params, model, pbc=True,
                          shifts=shifts)


def pooled_deformation(pool, nproc, pos, rvecs, sn, types, shifts, params, model, ncells=None):
    """om.deformation over the first ``ncells`` cells (all by default), split over a process pool."""
    M = len(sn) if ncells is None else int(ncells)
    bounds = np.linspace(0, M, 4 * nproc + 1).astype(int)
    jobs = [(pos[sn[lo:hi]], rvecs, types[lo:hi], shifts[lo:hi], params, model)
            for lo, hi in zip(bounds[:-1], bounds[1:])]
    parts = pool.map(chunk_deformation, jobs)
    return (np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts]),
            np.concatenate([p[2] for p in parts]))


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
        fs = 1e-15 / 2.418884326505e-17
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
        self.epot, self.gpos = self.forces()

    def forces(self, ncells=None):
        """Energy and gradient; with ``ncells`` only the first ncells cells contribute (a bounded sample)."""
        M = len(self.sn) if ncells is None else int(ncells)
        if self.pool is None:
            e, g, _ = om.deformation(self.pos, self.rvecs, self.grid, self.sn, self.types, self.params, self.model,
                                     shifts=self.shifts, cells=None if ncells is None else np.arange(M))
        else:
            e, g, _ = pooled_deformation(self.pool, self.nproc, self.pos, self.rvecs, self.sn, self.types,
                                         self.shifts, self.params, self.model, ncells)
        if ncells is not None:
            gfull = np.zeros((len(self.sn), 8, 3))
            gfull[:M] = g
            g = gfull
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
