"""Thermostats (interface of micmec/sampling/nvt.py:48-557).

``LangevinThermostat`` and ``NHCThermostat`` are the thermostats of the hot
path; Berendsen, Andersen and CSVR complete the set ``TBCombination`` accepts.
On the host path each is applied exactly as the reference does; the Langevin
thermostat additionally runs fused into the GPU step kernel (see
``VerletIntegrator``), where its noise comes from a counter-based Philox
generator keyed by (seed, node, step, pre/post).
"""

import numpy as np

from micmec_gb300.units import boltzmann, femtosecond
from micmec_gb300.sampling.iterative import StateItem
from micmec_gb300.sampling.utils import get_random_vel, clean_momenta, get_ndof_internal_md, stabilized_cholesky_decomp
from micmec_gb300.sampling.verlet import VerletHook

__all__ = [
    "AndersenThermostat", "BerendsenThermostat", "LangevinThermostat", "CSVRThermostat", "GLEThermostat",
    "NHCThermostat", "NHChain", "NHCAttributeStateItem",
]


class AndersenThermostat(VerletHook):
    """Andersen: redraw velocities every ``step`` steps (nvt.py:48-107)."""

    name = "Andersen"
    kind = "stochastic"
    method = "thermostat"

    def __init__(self, temp, start=0, step=1, select=None, annealing=1.0):
        self.temp = temp
        self.select = select
        self.annealing = annealing
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)

    def pre(self, iterative, G1_add=None):
        ekin_before = iterative._compute_ekin()
        if self.select is None:
            iterative.vel[:] = get_random_vel(self.temp, False, iterative.masses)
        else:
            iterative.vel[self.select] = get_random_vel(self.temp, False, iterative.masses, self.select)
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        self.econs_correction += ekin_before - iterative._compute_ekin()
        self.temp *= self.annealing

    def post(self, iterative, G1_add=None):
        pass


class BerendsenThermostat(VerletHook):
    """Berendsen velocity rescaling (nvt.py:110-162)."""

    name = "Berendsen"
    kind = "deterministic"
    method = "thermostat"

    def __init__(self, temp, start=0, timecon=100 * femtosecond, restart=False):
        self.temp = temp
        self.timecon = timecon
        self.restart = restart
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.mmf.system.domain.nvec)

    def pre(self, iterative, G1_add=None):
        ekin = iterative.ekin
        temp_inst = 2.0 * iterative.ekin / (boltzmann * iterative.ndof)
        c = np.sqrt(1 + iterative.timestep / self.timecon * (self.temp / temp_inst - 1))
        iterative.vel[:] = c * iterative.vel
        iterative.ekin = iterative._compute_ekin()
        self.econs_correction += (1 - c**2) * ekin

    def post(self, iterative, G1_add=None):
        pass


class LangevinThermostat(VerletHook):
    """Langevin thermostat (Bussi and Parrinello, Phys. Rev. E 75, 056707 (2007)); nvt.py:165-218.

    Every call applies v <- c1 v + sqrt((1 - c1^2) kT / m) xi with c1 = exp(-dt / (2 timecon)),
    before and after each Verlet step, and adds the kinetic-energy change to the
    conserved-quantity correction.

    Extra, for validation: ``seed`` keys the device noise generator; ``replay_noise``
    (shape (2 * nsteps, N, 3), draw order pre/post of each step, first draw for step
    ``replay_offset + 1``) makes both execution paths use given standard normals.
    """

    name = "Langevin"
    kind = "stochastic"
    method = "thermostat"

    def __init__(self, temp, start=0, timecon=100 * femtosecond, seed=None, replay_noise=None, replay_offset=0):
        self.temp = temp
        self.timecon = timecon
        self.seed = int(np.random.randint(0, 2**62)) if seed is None else int(seed)
        self.replay_noise = replay_noise
        self.replay_offset = replay_offset
        self._draw = 0
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)

    def pre(self, iterative, G1_add=None):
        ekin0 = iterative.ekin
        self.thermo(iterative, 0)
        self.econs_correction += ekin0 - iterative.ekin

    def post(self, iterative, G1_add=None):
        ekin0 = iterative.ekin
        self.thermo(iterative, 1)
        self.econs_correction += ekin0 - iterative.ekin

    def _noise(self, iterative, call):
        if self.replay_noise is not None:
            # pre of step s is draw 2 (s - 1 - offset); post is the next one
            step = iterative.counter + 1 if call == 0 else iterative.counter + 1
            idx = 2 * (step - 1 - self.replay_offset) + call
            return self.replay_noise[idx]
        return np.random.normal(0, 1, iterative.vel.shape)

    def thermo(self, iterative, call=0):
        c1 = np.exp(-iterative.timestep / self.timecon / 2)
        c2 = np.sqrt((1.0 - c1**2) * self.temp * boltzmann / iterative.masses).reshape(-1, 1)
        iterative.vel[:] = c1 * iterative.vel + c2 * self._noise(iterative, call)
        iterative.ekin = iterative._compute_ekin()


class CSVRThermostat(VerletHook):
    """Canonical sampling through velocity rescaling (Bussi, Donadio, Parrinello, J. Chem. Phys.
    126, 014101 (2007)); nvt.py:221-274.

    Before every step the velocities are scaled by alpha with
    alpha^2 = c + (S + R^2) f + 2 R sqrt(c f), c = exp(-dt / timecon),
    f = (1 - c) K / (ndof ekin), K = ndof kT / 2, R a standard normal and S a chi-squared
    variate with ndof - 1 degrees of freedom; the kinetic-energy change goes into the
    conserved-quantity correction.

    Extra, for validation: ``seed`` keys the device generator; ``replay_noise`` (shape
    (nsteps, 2): R and S of each step, first row for step ``replay_offset + 1``) makes both
    execution paths use given draws.
    """

    name = "CSVR"
    kind = "stochastic"
    method = "thermostat"

    def __init__(self, temp, start=0, timecon=100 * femtosecond, seed=None, replay_noise=None, replay_offset=0):
        self.temp = temp
        self.timecon = timecon
        self.seed = int(np.random.randint(0, 2**62)) if seed is None else int(seed)
        self.replay_noise = None if replay_noise is None else np.asarray(replay_noise, dtype=float)
        self.replay_offset = replay_offset
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.mmf.system.domain.nvec)
        self.kin = 0.5 * iterative.ndof * boltzmann * self.temp

    def _draws(self, iterative):
        if self.replay_noise is not None:
            r = self.replay_noise[iterative.counter - self.replay_offset]
            return float(r[0]), float(r[1])
        R = np.random.normal(0, 1)
        S = (np.random.normal(0, 1, iterative.ndof - 1) ** 2).sum()
        return R, S

    def pre(self, iterative, G1_add=None):
        c = np.exp(-iterative.timestep / self.timecon)
        R, S = self._draws(iterative)
        iterative.ekin = iterative._compute_ekin()
        fact = (1 - c) * self.kin / iterative.ndof / iterative.ekin
        alpha = np.sign(R + np.sqrt(c / fact)) * np.sqrt(c + (S + R**2) * fact + 2 * R * np.sqrt(c * fact))
        iterative.vel[:] = alpha * iterative.vel
        ekin_new = alpha**2 * iterative.ekin
        self.econs_correction += (1 - alpha**2) * iterative.ekin
        iterative.ekin = ekin_new

    def post(self, iterative, G1_add=None):
        pass


class GLEThermostat(VerletHook):
    """Generalised Langevin (coloured-noise) thermostat (Ceriotti, Bussi, Parrinello, J. Chem.
    Theory Comput. 6, 1170 (2010)); nvt.py:277-358.

    ns auxiliary momenta per degree of freedom; before and after every step the extended
    vector (sqrt(m) v, s) is propagated by T = exp(-A dt / 2) and noise S xi with
    S S^T = C - T C T^T (C = kT I unless given); the kinetic-energy change goes into the
    conserved-quantity correction. A host hook (the step's forces still run on the GPU).

    Extra, for validation: ``replay_noise`` (a list: the (ns, 3N) draw of ``init``, then one
    (ns + 1, 3N) draw per call) makes the run use given standard normals.
    """

    name = "GLE"
    kind = "stochastic"
    method = "thermostat"

    def __init__(self, temp, a_p, c_p=None, start=0, replay_noise=None):
        self.temp = temp
        self.ns = int(a_p.shape[0] - 1)
        self.a_p = np.asarray(a_p, dtype=float)
        self.c_p = boltzmann * self.temp * np.eye(self.ns + 1) if c_p is None else np.asarray(c_p, dtype=float)
        self.replay_noise = None if replay_noise is None else list(replay_noise)
        VerletHook.__init__(self, start, 1)

    def _normal(self, shape):
        if self.replay_noise is not None:
            z = np.asarray(self.replay_noise.pop(0), dtype=float)
            if z.shape != tuple(shape):
                raise ValueError("replayed draw of shape %s, expected %s" % (z.shape, tuple(shape)))
            return z
        return np.random.normal(size=shape)

    def init(self, iterative):
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        self.s = 0.5 * boltzmann * self.temp * self._normal((self.ns, iterative.pos.size))
        eigval, eigvec = np.linalg.eig(-self.a_p * iterative.timestep / 2)
        self.t = np.dot(eigvec * np.exp(eigval), np.linalg.inv(eigvec)).real
        self.S = stabilized_cholesky_decomp(self.c_p - np.dot(np.dot(self.t, self.c_p), self.t.T)).real
        self.n_atoms = iterative.pos.shape[0]

    def pre(self, iterative, G1_add=None):
        self.thermo(iterative)

    def post(self, iterative, G1_add=None):
        self.thermo(iterative)

    def thermo(self, iterative):
        ekin0 = iterative.ekin
        sq = np.sqrt(iterative.masses)[:, None]
        p = (sq * iterative.vel).reshape(-1)
        s_old = np.vstack([p, self.s])
        s_new = np.dot(self.t, s_old) + np.dot(self.S, self._normal((self.ns + 1, 3 * self.n_atoms)))
        iterative.vel[:] = np.sqrt(1.0 / iterative.masses)[:, None] * s_new[0, :].reshape((self.n_atoms, 3))
        self.s[:] = s_new[1:, :]
        iterative.ekin = iterative._compute_ekin()
        self.econs_correction += ekin0 - iterative.ekin


class NHChain(object):
    """Nose-Hoover chain of ``length`` beads (Martyna, Tuckerman, Tobias, Klein, Mol. Phys. 87, 1117 (1996));
    the Trotter splitting of nvt.py:361-458."""

    def __init__(self, length, timestep, temp, ndof, pos0, vel0, timecon=100 * femtosecond):
        self.length = length
        self.timestep = timestep
        self.temp = temp
        self.timecon = timecon
        self.restart_pos = pos0 is not None
        self.restart_vel = vel0 is not None
        self.pos = np.array(pos0, dtype=float).copy() if self.restart_pos else np.zeros(length)
        self.vel = np.array(vel0, dtype=float).copy() if self.restart_vel else np.zeros(length)
        if ndof > 0:
            self.set_ndof(ndof)

    def set_ndof(self, ndof):
        self.ndof = ndof
        afreq = 2 * np.pi / self.timecon
        self.masses = np.ones(self.length) * (boltzmann * self.temp / afreq**2)
        self.masses[0] *= ndof
        if not self.restart_vel:
            self.vel = self.get_random_vel_therm()

    def get_random_vel_therm(self):
        return np.random.normal(0, np.sqrt(self.masses * boltzmann * self.temp), self.length) / self.masses

    def _bead(self, k, ekin, G1_add):
        if k == 0:
            g = 2 * ekin - self.ndof * self.temp * boltzmann
            if G1_add is not None:
                g += G1_add
        else:
            g = self.masses[k - 1] * self.vel[k - 1] ** 2 - self.temp * boltzmann
        g /= self.masses[k]
        if k == self.length - 1:
            self.vel[k] += g * self.timestep / 4
        else:
            self.vel[k] *= np.exp(-self.vel[k + 1] * self.timestep / 8)
            self.vel[k] += g * self.timestep / 4
            self.vel[k] *= np.exp(-self.vel[k + 1] * self.timestep / 8)

    def __call__(self, ekin, vel, G1_add):
        for k in range(self.length - 1, -1, -1):
            self._bead(k, ekin, G1_add)
        self.pos += self.vel * self.timestep / 2
        factor = np.exp(-self.vel[0] * self.timestep / 2)
        vel *= factor
        ekin *= factor**2
        for k in range(self.length):
            self._bead(k, ekin, G1_add)
        return vel, ekin

    def get_econs_correction(self):
        kt = boltzmann * self.temp
        return 0.5 * (self.vel**2 * self.masses).sum() + kt * (self.ndof * self.pos[0] + self.pos[1:].sum())


class NHCThermostat(VerletHook):
    """Nose-Hoover chain thermostat (nvt.py:461-532)."""

    name = "NHC"
    kind = "deterministic"
    method = "thermostat"

    def __init__(self, temp, start=0, timecon=100 * femtosecond, chainlength=3, chain_pos0=None, chain_vel0=None,
                 restart=False):
        self.temp = temp
        self.restart = restart
        self.chain = NHChain(chainlength, 0.0, temp, 0, chain_pos0, chain_vel0, timecon)
        VerletHook.__init__(self, start, 1)

    def init(self, iterative):
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.mmf.system.domain.nvec)
        self.chain.timestep = iterative.timestep
        self.chain.set_ndof(iterative.ndof)

    def pre(self, iterative, G1_add=None):
        velnew, iterative.ekin = self.chain(iterative.ekin, iterative.vel, G1_add)
        iterative.vel[:] = velnew

    def post(self, iterative, G1_add=None):
        velnew, iterative.ekin = self.chain(iterative.ekin, iterative.vel, G1_add)
        iterative.vel[:] = velnew
        self.econs_correction = self.chain.get_econs_correction()


def find_hook(iterative, cls, role):
    """The hook of type ``cls`` among the iterative's hooks, also when it sits inside a
    TBCombination under the attribute ``role`` ("thermostat" / "barostat"); None if absent."""
    for hook in iterative.hooks:
        for candidate in (hook, getattr(hook, role, None)):
            if isinstance(candidate, cls):
                return candidate
    return None


class NHCAttributeStateItem(StateItem):
    """Recorded Nose-Hoover chain variable (``attr`` "pos", "vel", "masses", ...) under the key
    thermo_<attr>, for trajectories of NHC runs."""

    def __init__(self, attr):
        self.attr = attr
        StateItem.__init__(self, "thermo_" + attr)

    def get_value(self, iterative):
        thermo = find_hook(iterative, NHCThermostat, "thermostat")
        if thermo is None:
            raise TypeError("No NHCThermostat among the iterative's hooks: thermo_%s cannot be recorded." % self.attr)
        return getattr(thermo.chain, self.attr)
