"""Barostats and thermostat-barostat coupling (interface of micmec/sampling/npt.py:52-787).

``BerendsenBarostat`` (npt.py:180-292) and ``LangevinBarostat`` (npt.py:295-510) complete
the set ``TBCombination`` accepts; the Langevin barostat shares the MTK scaling half step.

``MTKBarostat`` is the Martyna-Tobias-Klein barostat (J. Chem. Phys. 101, 4177
(1994)) with the symplectic splitting of Martyna, Tuckerman, Tobias and Klein
(Mol. Phys. 87, 1117 (1996)), as used by the reference (npt.py:513-757): the
barostat velocity tensor v_g is propagated from the internal pressure
(sum m v (x) v - vtens), positions and domain are scaled with exp(v_g dt/2),
the forces are re-evaluated, and velocities are scaled with
exp(-(v_g + tr(v_g)/ndof) dt/2). Every force evaluation runs on the GPU.
"""

import numpy as np

from micmec_gb300.units import bar, boltzmann, femtosecond
from micmec_gb300.sampling.iterative import StateItem
from micmec_gb300.sampling.utils import (
    domain_symmetrize, get_random_vel_press, get_ndof_internal_md, clean_momenta, get_ndof_baro,
)
from micmec_gb300.sampling.verlet import VerletHook
from micmec_gb300.sampling.nvt import NHCThermostat, LangevinThermostat, BerendsenThermostat, find_hook

__all__ = ["TBCombination", "BerendsenBarostat", "LangevinBarostat", "MTKBarostat", "MTKAttributeStateItem"]


class TBCombination(VerletHook):
    """Thermostat + barostat called in the right order, with NHC/MTK coupling (npt.py:52-177)."""

    name = "TBCombination"

    def __init__(self, thermostat, barostat, start=0):
        self.thermostat = thermostat
        self.barostat = barostat
        self.start = start
        if not self.verify():
            self.barostat, self.thermostat = thermostat, barostat
            if not self.verify():
                raise TypeError("The Thermostat or Barostat instance is not supported (yet).")
        self.step_thermo = self.thermostat.step
        self.step_baro = self.barostat.step
        VerletHook.__init__(self, start, min(self.step_thermo, self.step_baro))

    def init(self, iterative):
        set_ndof = iterative.ndof is not None
        self.thermostat.init(iterative)
        self.barostat.init(iterative)
        p_cm_fluct = isinstance(self.thermostat, LangevinThermostat) or isinstance(self.barostat, LangevinBarostat)
        if (not set_ndof) and p_cm_fluct:
            iterative.ndof = iterative.pos.size
        self.chainvel0 = None
        self.G1_add = None

    def pre(self, iterative):
        if self.expectscall(iterative, "baro"):
            if isinstance(self.thermostat, NHCThermostat):
                self.chainvel0 = self.thermostat.chain.vel[0]
            self.barostat.pre(iterative, self.chainvel0)
        if self.expectscall(iterative, "thermo"):
            if isinstance(self.barostat, MTKBarostat):
                self.G1_add = self.barostat.add_press_cont()
            self.thermostat.pre(iterative, self.G1_add)

    def post(self, iterative):
        if self.expectscall(iterative, "thermo"):
            if isinstance(self.barostat, MTKBarostat):
                self.G1_add = self.barostat.add_press_cont()
            self.thermostat.post(iterative, self.G1_add)
        if self.expectscall(iterative, "baro"):
            if isinstance(self.thermostat, NHCThermostat):
                self.chainvel0 = self.thermostat.chain.vel[0]
            self.barostat.post(iterative, self.chainvel0)
        self.econs_correction = self.thermostat.econs_correction + self.barostat.econs_correction
        if isinstance(self.thermostat, NHCThermostat):
            if not (isinstance(self.barostat, MTKBarostat) and self.barostat.baro_thermo is not None):
                kt = boltzmann * self.thermostat.temp
                self.econs_correction += self.barostat.baro_ndof * kt * self.thermostat.chain.pos[0]

    def expectscall(self, iterative, kind):
        step = self.step_thermo if kind == "thermo" else self.step_baro
        return iterative.counter >= self.start and (iterative.counter - self.start) % step == 0

    def verify(self):
        thermo_ok = isinstance(self.thermostat, (NHCThermostat, LangevinThermostat, BerendsenThermostat))
        baro_ok = isinstance(self.barostat, (BerendsenBarostat, LangevinBarostat, MTKBarostat))
        return thermo_ok and baro_ok


def _scaling_half_step(iterative, vel_press, dt, anisotropic, vol_constraint):
    """Positions and domain scaled by exp(v_g dt/2), forces re-evaluated, velocities scaled by
    exp(-(v_g + tr(v_g)/ndof) dt/2), kinetic energy updated: the middle of the MTK and
    Langevin barostat half steps (npt.py:446-486 and 686-731)."""
    if anisotropic:
        Dr, Qg = np.linalg.eigh(vel_press)
        rot_mat = np.dot(Qg * np.exp(Dr * dt / 2), Qg.T)
        pos_new = np.dot(iterative.pos, rot_mat)
        rvecs_new = np.dot(iterative.rvecs, rot_mat)
    else:
        c = np.exp(vel_press * dt / 2)
        pos_new = c * iterative.pos
        rvecs_new = c * iterative.rvecs
    iterative.mmf.update_pos(pos_new)
    iterative.pos[:] = pos_new
    iterative.mmf.update_rvecs(rvecs_new)
    iterative.rvecs[:] = rvecs_new
    iterative.gpos[:] = 0.0
    iterative.vtens[:] = 0.0
    iterative.epot = iterative.mmf.compute(iterative.gpos, iterative.vtens)
    if anisotropic:
        if vol_constraint:
            Dg, Eg = np.linalg.eigh(vel_press)
        else:
            Dg, Eg = np.linalg.eigh(vel_press + (np.trace(vel_press) / iterative.ndof) * np.eye(3))
        rot_mat = np.dot(Eg * np.exp(-Dg * dt / 2), Eg.T)
        vel_new = np.dot(iterative.vel, rot_mat)
    else:
        vel_new = np.exp(-((1.0 + 3.0 / iterative.ndof) * vel_press) * dt / 2) * iterative.vel
    iterative.vel[:] = vel_new
    iterative.ekin = iterative._compute_ekin()


class BerendsenBarostat(VerletHook):
    """Berendsen barostat (Berendsen, Postma, van Gunsteren, DiNola, Haak, J. Chem. Phys. 81,
    3684 (1984)); npt.py:180-292.

    After every step, positions and domain are multiplied by mu = sym(I - dt/W (P I - ptens)),
    ptens = (sum m v (x) v - vtens) / V, W = 3 timecon / beta * sqrt(ndof); the forces are
    re-evaluated and the energy change goes into the conserved-quantity correction.
    """

    name = "Berendsen"
    kind = "deterministic"
    method = "barostat"

    def __init__(self, mmf, temp, press, start=0, step=1, timecon=1000 * femtosecond, beta=4.57e-5 / bar,
                 anisotropic=True, vol_constraint=False, restart=False):
        self.temp = temp
        self.press = press
        self.timecon_press = timecon
        self.beta = beta
        self.mass_press = 3.0 * timecon / beta
        self.anisotropic = anisotropic
        self.vol_constraint = vol_constraint
        self.dim = mmf.system.domain.nvec
        self.baro_ndof = get_ndof_baro(self.dim, self.anisotropic, self.vol_constraint)
        if self.anisotropic:
            domain_symmetrize(mmf)
        self.domain = mmf.system.domain.rvecs.copy()
        self.restart = restart
        self.vel_press = None
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        self.timestep_press = iterative.timestep
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.mmf.compute(iterative.gpos, iterative.vtens)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.pos.shape[0], iterative.mmf.system.domain.nvec)
        self.mass_press *= np.sqrt(iterative.ndof)

    def pre(self, iterative, chainvel0=None):
        pass

    def mu(self, iterative):
        """The scaling matrix of one post call."""
        ptens = (np.dot(iterative.vel.T * iterative.masses, iterative.vel) - iterative.vtens) \
            / iterative.mmf.system.domain.volume
        dmu = self.timestep_press / self.mass_press * (self.press * np.eye(3) - ptens)
        if self.vol_constraint:
            dmu -= np.trace(dmu) / self.dim * np.eye(self.dim)
        mu = np.eye(3) - dmu
        mu = 0.5 * (mu + mu.T)
        if not self.anisotropic:
            mu = ((np.trace(mu) / 3.0) ** (1.0 / 3.0)) * np.eye(3)
        return mu

    def post(self, iterative, chainvel0=None):
        epot0 = iterative.epot
        mu = self.mu(iterative)
        pos_new = np.dot(iterative.pos, mu)
        rvecs_new = np.dot(iterative.rvecs, mu)
        iterative.mmf.update_pos(pos_new)
        iterative.pos[:] = pos_new
        iterative.mmf.update_rvecs(rvecs_new)
        iterative.rvecs[:] = rvecs_new
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.mmf.compute(iterative.gpos, iterative.vtens)
        self.econs_correction += epot0 - iterative.epot


class LangevinBarostat(VerletHook):
    """Langevin barostat (Feller, Zhang, Pastor, Brooks, J. Chem. Phys. 103, 4613 (1995));
    npt.py:295-510.

    The MTK half steps with a friction exp(-dt / (8 timecon)) on the barostat velocity
    around each of its updates and a random symmetric force tensor R (variance
    2 W kT / (dt timecon)) in them; W = (ndof + 3) / 3 kT (timecon / 2 pi)^2. Pre and post
    add the change of epot + ekin to the conserved-quantity correction.

    Extra, for validation: ``vel_press0`` replaces the random initial barostat velocity;
    ``seed`` keys the device generator; ``replay_noise`` (shape (nsteps, 4, 6): the lower
    triangles (00, 10, 11, 20, 21, 22) of the four unit-normal tensors of each step, in call
    order, first row for step ``replay_offset + 1``) makes both execution paths use given draws.
    """

    name = "Langevin"
    kind = "stochastic"
    method = "barostat"

    _TRIL = ((0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2))

    def __init__(self, mmf, temp, press, start=0, step=1, timecon=1000 * femtosecond, anisotropic=True,
                 vol_constraint=False, vel_press0=None, seed=None, replay_noise=None, replay_offset=0):
        self.temp = temp
        self.press = press
        self.timecon = timecon
        self.anisotropic = anisotropic
        self.vol_constraint = vol_constraint
        self.dim = mmf.system.domain.nvec
        self.baro_ndof = get_ndof_baro(self.dim, self.anisotropic, self.vol_constraint)
        if self.anisotropic:
            domain_symmetrize(mmf)
        self.domain = mmf.system.domain.rvecs.copy()
        self.vel_press0 = None if vel_press0 is None else np.array(vel_press0, dtype=float).copy()
        self.seed = int(np.random.randint(0, 2**62)) if seed is None else int(seed)
        self.replay_noise = None if replay_noise is None else np.asarray(replay_noise, dtype=float)
        self.replay_offset = replay_offset
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        self.timestep_press = iterative.timestep
        clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        if iterative.ndof is None:
            iterative.ndof = iterative.pos.size
        self.mass_press = (iterative.ndof + 3) / 3 * boltzmann * self.temp * (self.timecon / (2 * np.pi)) ** 2
        if self.vel_press0 is not None:
            self.vel_press = np.array(self.vel_press0, dtype=float).copy()
        else:
            self.vel_press = get_random_vel_press(self.mass_press, self.temp)
        if self.vol_constraint:
            self.vel_press -= np.trace(self.vel_press) / 3 * np.eye(3)
        if not self.anisotropic and np.ndim(self.vel_press) == 2:  # (vel_press0 may be the scalar already)
            self.vel_press = self.vel_press[0][0]
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.mmf.compute(iterative.gpos, iterative.vtens)

    def pre(self, iterative, chainvel0=None):
        e0 = iterative.epot + iterative.ekin
        self.baro(iterative, chainvel0, 0)
        self.econs_correction += e0 - iterative.epot - iterative.ekin

    def post(self, iterative, chainvel0=None):
        e0 = iterative.epot + iterative.ekin
        self.baro(iterative, chainvel0, 2)
        self.econs_correction += e0 - iterative.epot - iterative.ekin

    def getR(self, iterative, call):
        """Random symmetric force tensor of one barostat-velocity update."""
        if self.replay_noise is not None:
            z = self.replay_noise[iterative.counter - self.replay_offset, call]
            rand = np.zeros((3, 3))
            for k, (i, j) in enumerate(self._TRIL):
                rand[i, j] = z[k]
        else:
            rand = np.random.normal(0, 1, (3, 3))
        rand = rand * np.sqrt(2 * self.mass_press * boltzmann * self.temp / (self.timestep_press * self.timecon))
        return np.tril(rand) + np.tril(rand, -1).T

    def _update_baro_vel(self, iterative, chainvel0, call):
        dt = self.timestep_press
        self.vel_press *= np.exp(-dt / (8 * self.timecon))
        if chainvel0 is not None:
            self.vel_press *= np.exp(-dt * chainvel0 / 8)
        ptens_vol = np.dot(iterative.vel.T * iterative.masses, iterative.vel) - iterative.vtens
        ptens_vol = 0.5 * (ptens_vol.T + ptens_vol)
        G = (ptens_vol + (2.0 * iterative.ekin / iterative.ndof - self.press * iterative.mmf.system.domain.volume)
             * np.eye(3)) / self.mass_press
        R = self.getR(iterative, call)
        if self.vol_constraint:
            G -= np.trace(G) / self.dim * np.eye(self.dim)
            R -= np.trace(R) / self.dim * np.eye(self.dim)
        if not self.anisotropic:
            G = np.trace(G)
            R = R[0][0]
        self.vel_press += (G - R / self.mass_press) * dt / 4
        self.vel_press *= np.exp(-dt / (8 * self.timecon))
        if chainvel0 is not None:
            self.vel_press *= np.exp(-dt * chainvel0 / 8)

    def baro(self, iterative, chainvel0, call0=0):
        self._update_baro_vel(iterative, chainvel0, call0)
        _scaling_half_step(iterative, self.vel_press, self.timestep_press, self.anisotropic, self.vol_constraint)
        self._update_baro_vel(iterative, chainvel0, call0 + 1)


class MTKBarostat(VerletHook):
    """Martyna-Tobias-Klein barostat (npt.py:513-757)."""

    name = "MTTK"
    kind = "deterministic"
    method = "barostat"

    def __init__(self, mmf, temp, press, start=0, step=1, timecon=1000 * femtosecond, anisotropic=True,
                 vol_constraint=False, baro_thermo=None, vel_press0=None, restart=False):
        self.temp = temp
        self.press = press
        self.timecon_press = timecon
        self.anisotropic = anisotropic
        self.vol_constraint = vol_constraint
        self.baro_thermo = baro_thermo
        self.dim = mmf.system.domain.nvec
        self.restart = restart
        self.baro_ndof = get_ndof_baro(self.dim, self.anisotropic, self.vol_constraint)
        if self.anisotropic and not self.restart:
            domain_symmetrize(mmf)
        self.domain = mmf.system.domain.rvecs.copy()
        self.vel_press = None if vel_press0 is None else np.array(vel_press0, dtype=float).copy()
        VerletHook.__init__(self, start, step)

    def init(self, iterative):
        self.timestep_press = iterative.timestep
        if not self.restart:
            clean_momenta(iterative.pos, iterative.vel, iterative.masses, iterative.mmf.system.domain)
        if iterative.ndof is None:
            iterative.ndof = get_ndof_internal_md(iterative.mmf.system.nnodes, iterative.mmf.system.domain.nvec)
        angfreq = 2 * np.pi / self.timecon_press
        self.mass_press = (iterative.ndof + self.dim**2) * boltzmann * self.temp / angfreq**2
        if self.vel_press is None:
            self.vel_press = get_random_vel_press(self.mass_press, self.temp)
            if not self.anisotropic:
                self.vel_press = self.vel_press[0][0]
        if self.baro_thermo is not None:
            self.baro_thermo.chain.timestep = iterative.timestep
            self.baro_thermo.chain.set_ndof(self.baro_ndof)
        if self.vol_constraint:
            self.vel_press -= np.trace(self.vel_press) / 3 * np.eye(3)
        iterative.gpos[:] = 0.0
        iterative.vtens[:] = 0.0
        iterative.epot = iterative.mmf.compute(iterative.gpos, iterative.vtens)

    def pre(self, iterative, chainvel0=None):
        if self.baro_thermo is not None:
            chainvel0 = self.baro_thermo.chain.vel[0]
        self.baro(iterative, chainvel0)
        if self.baro_thermo is not None:
            self.baro_thermo.chain(self._compute_ekin_baro(), np.array(self.vel_press, dtype=float), 0)

    def post(self, iterative, chainvel0=None):
        if self.baro_thermo is not None:
            self.baro_thermo.chain(self._compute_ekin_baro(), np.array(self.vel_press, dtype=float), 0)
            chainvel0 = self.baro_thermo.chain.vel[0]
        self.baro(iterative, chainvel0)
        self.econs_correction = self._compute_ekin_baro()
        if not self.vol_constraint:
            self.econs_correction += self.press * iterative.mmf.system.domain.volume
        if self.baro_thermo is not None:
            self.econs_correction += self.baro_thermo.chain.get_econs_correction()

    def _update_baro_vel(self, iterative, chainvel0):
        dt = self.timestep_press
        if chainvel0 is not None:
            self.vel_press *= np.exp(-dt * chainvel0 / 8)
        ptens_vol = np.dot(iterative.vel.T * iterative.masses, iterative.vel) - iterative.vtens
        ptens_vol = 0.5 * (ptens_vol.T + ptens_vol)
        G = (ptens_vol + (2.0 * iterative.ekin / iterative.ndof - self.press * iterative.mmf.system.domain.volume)
             * np.eye(3)) / self.mass_press
        if not self.anisotropic:
            G = np.trace(G)
        if self.vol_constraint:
            G -= np.trace(G) / self.dim * np.eye(self.dim)
        self.vel_press += G * dt / 4
        if chainvel0 is not None:
            self.vel_press *= np.exp(-dt * chainvel0 / 8)

    def baro(self, iterative, chainvel0):
        self._update_baro_vel(iterative, chainvel0)
        _scaling_half_step(iterative, self.vel_press, self.timestep_press, self.anisotropic, self.vol_constraint)
        self._update_baro_vel(iterative, chainvel0)

    def add_press_cont(self):
        kt = self.temp * boltzmann
        if self.baro_thermo is None:
            return 2 * self._compute_ekin_baro() - self.baro_ndof * kt
        return 0

    def _compute_ekin_baro(self):
        if self.anisotropic:
            return 0.5 * self.mass_press * np.trace(np.dot(self.vel_press.T, self.vel_press))
        return 0.5 * self.mass_press * self.vel_press**2


class MTKAttributeStateItem(StateItem):
    """Recorded MTK barostat variable under the key baro_<attr>: an attribute of the barostat
    ("vel_press", "mass_press", ...) or, for attr "chain_<name>", the variable <name> of the
    barostat's own Nose-Hoover chain (0 when it has none)."""

    def __init__(self, attr):
        self.attr = attr
        StateItem.__init__(self, "baro_" + attr)

    def get_value(self, iterative):
        baro = find_hook(iterative, MTKBarostat, "barostat")
        if baro is None:
            raise TypeError("No MTKBarostat among the iterative's hooks: baro_%s cannot be recorded." % self.attr)
        if self.attr.startswith("chain_"):
            chain_attr = self.attr[len("chain_"):]
            return 0 if baro.baro_thermo is None else getattr(baro.baro_thermo.chain, chain_attr)
        return getattr(baro, self.attr)
