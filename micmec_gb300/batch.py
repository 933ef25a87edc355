"""Batches of independent periodic systems on one GPU (one persistent launch).

``BatchSystems`` packs hundreds of fully periodic lattices of uneven size
(defect configurations, strain-scan points, replicas) into one device batch.
``md`` runs velocity-Verlet steps of every system with the reference's hooks
(none / Langevin / Nose-Hoover chain / Berendsen / CSVR thermostat, and the MTK,
Berendsen or Langevin barostat, anisotropic, isotropic or volume-constrained) in one persistent kernel (optionally replayed from a CUDA graph);
``relax`` minimises every system's energy over node positions with nonlinear
conjugate gradients. By default every system is its own CTA (launched longest
first); ``autotune`` picks the CTA size (128 or 256 threads) and the number of
CTAs (1, 2 or 4 per SM, or one per system) by timing.

The hook constants are set up the way the reference's hook ``init`` methods set
them (micmec/sampling/nvt.py:393-400, 507-523; npt.py:82-97, 579-614):
degrees of freedom, Nose-Hoover chain masses, barostat mass and the initial
momentum removal.
"""

import ctypes

import numpy as np

from micmec_gb300 import _native as nat
from micmec_gb300.units import bar, boltzmann, femtosecond

__all__ = ["BatchSystems", "CTL", "REC", "HOOK_NOISE_LEN", "baro_code"]

CTL = dict(L=slice(0, 9), rvecs=slice(9, 18), volume=18, epot=19, ekin=20, vtens=slice(21, 30), ktens=slice(30, 39),
           vel_press=slice(39, 48), chain_pos=slice(48, 51), chain_vel=slice(51, 54), chain_mass=slice(54, 57),
           ndof=57, mass_press=58, baro_ndof=59, econs_thermo=60, econs_baro=61, gmax=62, iters=63, alpha=64,
           chain_ndof=65, timecon_press=66, temp_press=67, stress_res=69, bchain_pos=slice(70, 73),
           bchain_vel=slice(73, 76), bchain_mass=slice(76, 79), bchain_temp=79)
CTL_LEN = 80
# barostat options in the barostat code (kind | options | MTK chain length << 8)
BARO_ISO, BARO_VOLC, MTK_CHAIN = 0x10, 0x20, 0x40
REC = dict(epot=0, ekin=1, ecorr=2, volume=3, vtens=slice(4, 13), ktens=slice(13, 22), rvecs=slice(22, 31))
REC_LEN = 31
_THERMO = {None: 0, "langevin": 1, "nhc": 2, "berendsen": 3, "csvr": 4}
_BARO = {None: 0, "mtk": 1, "berendsen": 2, "langevin": 3}


def baro_code(barostat, anisotropic=True, vol_constraint=False, chainlength=0):
    """Barostat argument of the kernels: the kind and its options (isotropic, volume constraint;
    for the MTK barostat also a Nose-Hoover chain of ``chainlength`` beads of its own)."""
    if barostat is None or isinstance(barostat, (int, np.integer)):
        return int(barostat or 0)
    code = _BARO[barostat]
    if chainlength and barostat != "mtk":
        raise ValueError("a chain of the barostat's own is an MTK barostat option")
    if not anisotropic and vol_constraint:
        raise ValueError("an isotropic barostat under a volume constraint has no degree of freedom left")
    if not anisotropic:
        code |= BARO_ISO
    if vol_constraint:
        code |= BARO_VOLC
    if chainlength:
        code |= MTK_CHAIN | (int(chainlength) << 8)
    return code
HOOK_NOISE_LEN = 26  # per system and step: CSVR R, S; Langevin barostat 4 x 6 unit normals


def _declare(L):
    if getattr(L, "_batch_declared", False):
        return
    P = ctypes.c_void_p
    L.mm_batch_create.argtypes = [ctypes.c_int, P, P, ctypes.c_int, P, P, P, P, P, P, ctypes.c_int, ctypes.c_int,
                                  ctypes.POINTER(ctypes.c_void_p)]
    L.mm_batch_destroy.argtypes = [P]
    L.mm_batch_set_state.argtypes = [P, P, P, P]
    L.mm_batch_get_state.argtypes = [P, P, P, P]
    L.mm_batch_control.argtypes = [P, P, ctypes.c_int]
    L.mm_batch_md.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                              ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_uint64, ctypes.c_int64, P, P, P,
                              ctypes.c_int, P]
    L.mm_batch_relax.argtypes = [P, ctypes.c_int, ctypes.c_double, P]
    L.mm_batch_set_params.argtypes = [P, P, P, P, P, P]
    L.mm_batch_relax_cell.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_int, P]
    L.mm_batch_autotune.argtypes = [P, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_int, P]
    L.mm_batch_config.argtypes = [P, P, P]
    for n in ("mm_batch_create", "mm_batch_destroy", "mm_batch_set_state", "mm_batch_get_state", "mm_batch_control",
              "mm_batch_md", "mm_batch_relax", "mm_batch_relax_cell", "mm_batch_autotune", "mm_batch_config",
              "mm_batch_set_params"):
        getattr(L, n).restype = ctypes.c_int
    L._batch_declared = True


class BatchSystems(object):
    """A batch of fully periodic ``System`` objects sharing one parameter table.

    Every system's grid must be fully occupied (defects are other cell types) and its
    ``surrounding_*`` tables must follow the lattice (as ``build_system`` makes them).
    """

    def __init__(self, systems, model="nanocell", precision="fp32"):
        import torch

        from micmec_gb300.pes.mmff import type_parameters

        if not torch.cuda.is_available():
            raise nat.MMError("BatchSystems needs a CUDA device")
        self.torch = torch
        self.systems = list(systems)
        self.model = model
        self.precision = precision
        L = nat.lib()
        _declare(L)
        self.L = L
        ids = sorted(set(int(t) for s in self.systems for t in np.asarray(s.types)))
        index = {k: i for i, k in enumerate(ids)}
        params = {}
        for s in self.systems:
            params.update(s.params)
        shapes, ctype, masses = [], [], []
        for s in self.systems:
            grid = np.asarray(s.grid)
            if (grid == 0).any() or np.asarray(s.domain.rvecs).shape != (3, 3):
                raise ValueError("BatchSystems takes fully occupied, 3-D periodic lattices")
            if s.nnodes != grid.size or s.ncells != grid.size:
                raise ValueError("node/cell count does not match the grid")
            shapes.append(grid.shape)
            ctype.append([index[int(t)] for t in np.asarray(s.types)])
            masses.append(np.asarray(s.masses, dtype=np.float64))
        self.sizes = np.array([s.ncells for s in self.systems])
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)])
        nstates, h0, C, df, temp = type_parameters(params, ids)
        self._keep = [np.ascontiguousarray(np.array(shapes, dtype=np.int32)),
                      np.ascontiguousarray(np.concatenate(ctype).astype(np.int32)), nstates, h0, C, df, temp,
                      np.ascontiguousarray(np.concatenate(masses))]
        h = ctypes.c_void_p()
        st = L.mm_batch_create(len(self.systems), *(k.ctypes.data for k in self._keep[:2]), len(ids),
                               *(k.ctypes.data for k in self._keep[2:]), {"original": 0, "nanocell": 1}[model],
                               {"fp64": 0, "fp32": 1}[precision], ctypes.byref(h))
        nat.check(st, "mm_batch_create")
        self._h = h
        self.masses = self._keep[-1]
        self.set_state([s.pos for s in self.systems], None, [s.domain.rvecs for s in self.systems])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None:
            try:
                self.L.mm_batch_destroy(h)
            except Exception:
                pass
            self._h = None

    def __len__(self):
        return len(self.systems)

    # ------------------------------------------------------------ state
    def set_state(self, pos, vel=None, rvecs=None):
        pos = np.ascontiguousarray(np.concatenate([np.asarray(p, dtype=np.float64) for p in pos]))
        v = None if vel is None else np.ascontiguousarray(np.concatenate([np.asarray(x, dtype=np.float64) for x in vel]))
        if rvecs is None:
            rvecs = self.get_state()[2]
        rv = np.ascontiguousarray(np.array([np.asarray(r, dtype=np.float64).reshape(3, 3) for r in rvecs]))
        nat.check(self.L.mm_batch_set_state(self._h, pos.ctypes.data, nat.ptr(v), rv.ctypes.data), "set_state")

    def get_state(self):
        N = int(self.offsets[-1])
        pos = np.zeros((N, 3))
        vel = np.zeros((N, 3))
        rv = np.zeros((len(self), 3, 3))
        nat.check(self.L.mm_batch_get_state(self._h, pos.ctypes.data, vel.ctypes.data, rv.ctypes.data), "get_state")
        split = lambda a: [a[self.offsets[i]:self.offsets[i + 1]] for i in range(len(self))]
        return split(pos), split(vel), list(rv)

    def set_params(self, h0, C, free_energy, temp_eff, nstates):
        """Replace the parameter tables: h0 (types*4, 9), C (types*4, 81), free energies (types*4,),
        effective temperatures (types,), states per type (types,) -- the layout of
        ``type_parameters`` and ``MicMecParameters.native_tables`` (types in increasing id order)."""
        arrs = [np.ascontiguousarray(nstates, dtype=np.int32), np.ascontiguousarray(h0, dtype=np.float64),
                np.ascontiguousarray(C, dtype=np.float64), np.ascontiguousarray(free_energy, dtype=np.float64),
                np.ascontiguousarray(temp_eff, dtype=np.float64)]
        nat.check(self.L.mm_batch_set_params(self._h, *[a.ctypes.data for a in arrs]), "mm_batch_set_params")

    def control(self):
        c = np.zeros((len(self), CTL_LEN))
        nat.check(self.L.mm_batch_control(self._h, c.ctypes.data, 0), "control")
        return c

    def set_control(self, c):
        c = np.ascontiguousarray(c, dtype=np.float64)
        nat.check(self.L.mm_batch_control(self._h, c.ctypes.data, 1), "control")

    # ------------------------------------------------------------ hooks set-up
    def setup_md(self, vel=None, temp=300.0, thermostat=None, timecon=100 * femtosecond, chainlength=3,
                 chain_vel0=None, barostat=None, baro_timecon=1000 * femtosecond, vel_press0=None, ndof=None,
                 seed=0, clean=True, beta=4.57e-5 / bar, anisotropic=True, vol_constraint=False, baro_chainlength=0,
                 baro_chain_timecon=100 * femtosecond, baro_chain_temp=None, baro_chain_vel0=None):
        """Initial velocities and hook constants for every system (as the hooks' init does).
        beta: the Berendsen barostat's compressibility. ``anisotropic`` False (a scalar barostat
        velocity, or an isotropic Berendsen scaling) and ``vol_constraint`` (a traceless velocity
        or scaling increment) for every barostat, and for the MTK barostat ``baro_chainlength`` > 0
        for a Nose-Hoover chain of its own (time constant, temperature and initial velocities
        ``baro_chain_*``), as the barostats' init sets them up (npt.py:180-611)."""
        code = baro_code(barostat, anisotropic, vol_constraint, baro_chainlength)
        bndof = (6 if anisotropic else 1) - (1 if vol_constraint else 0)
        rng = np.random.default_rng(seed)
        pos, _, rvecs = self.get_state()
        vels = []
        c = self.control()
        for i, s in enumerate(self.systems):
            m = np.asarray(s.masses)
            if vel is None:
                v = rng.normal(0.0, 1.0, (s.nnodes, 3)) * np.sqrt(boltzmann * temp / m)[:, None]
            else:
                v = np.array(vel[i], dtype=np.float64)
            if clean and (thermostat is not None or barostat is not None):
                v -= (m @ v) / m.sum()
            vels.append(v)
            n3 = 3 * s.nnodes
            nd = ndof
            if nd is None:
                if barostat == "langevin":
                    # the hook that initialises first sets ndof: NHC / Berendsen the internal
                    # count, else the Langevin barostat the full one (npt.py:349-351)
                    nd = n3 - 3 if thermostat in ("nhc", "berendsen") else n3
                else:
                    nd = n3 if (thermostat in (None, "langevin") and barostat is None) else n3 - 3
            chain_nd = nd
            if barostat in ("mtk", "langevin") and not anisotropic:  # scalar velocity in the first slot
                vp = np.zeros((3, 3))
                if vel_press0 is not None:
                    vp[0, 0] = vel_press0[i] if np.ndim(vel_press0) == 1 else vel_press0
            else:
                vp = np.zeros((3, 3)) if vel_press0 is None else np.array(vel_press0[i] if np.ndim(vel_press0) == 3
                                                                          else vel_press0, dtype=np.float64)
            if barostat == "mtk":
                angfreq = 2 * np.pi / baro_timecon
                c[i, CTL["mass_press"]] = (nd + 9) * boltzmann * temp / angfreq**2
                if vol_constraint:
                    vp -= np.trace(vp) / 3 * np.eye(3)
                c[i, CTL["vel_press"]] = vp.ravel()
                if baro_chainlength:
                    bt = temp if baro_chain_temp is None else baro_chain_temp
                    bm = np.zeros(3)
                    bm[:baro_chainlength] = boltzmann * bt / (2 * np.pi / baro_chain_timecon) ** 2
                    bm[0] *= bndof
                    bv = np.zeros(3)
                    if baro_chain_vel0 is not None:
                        bv[:baro_chainlength] = np.asarray(baro_chain_vel0[i] if np.ndim(baro_chain_vel0) == 2
                                                           else baro_chain_vel0)
                    c[i, CTL["bchain_mass"]] = bm
                    c[i, CTL["bchain_vel"]] = bv
                    c[i, CTL["bchain_pos"]] = 0.0
                    c[i, CTL["bchain_temp"]] = bt
            elif barostat == "berendsen":
                c[i, CTL["mass_press"]] = 3.0 * baro_timecon / beta * np.sqrt(nd)
            elif barostat == "langevin":
                c[i, CTL["mass_press"]] = (nd + 3) / 3 * boltzmann * temp * (baro_timecon / (2 * np.pi)) ** 2
                if vol_constraint:
                    vp -= np.trace(vp) / 3 * np.eye(3)
                c[i, CTL["vel_press"]] = vp.ravel()
                c[i, CTL["timecon_press"]] = baro_timecon
                c[i, CTL["temp_press"]] = temp
            if barostat is not None:
                c[i, CTL["baro_ndof"]] = bndof
                if ndof is None and (thermostat == "langevin" or barostat == "langevin"):
                    nd = n3  # TBCombination: the centre of mass fluctuates (npt.py:86-90)
            if thermostat == "nhc":
                afreq = 2 * np.pi / timecon
                cm = np.ones(3) * (boltzmann * temp / afreq**2)
                cm[0] *= chain_nd
                c[i, CTL["chain_mass"]] = cm
                cv = np.zeros(3) if chain_vel0 is None else np.asarray(chain_vel0[i] if np.ndim(chain_vel0) == 2
                                                                        else chain_vel0)
                c[i, CTL["chain_vel"]] = cv
                c[i, CTL["chain_pos"]] = 0.0
                c[i, CTL["chain_ndof"]] = chain_nd
            c[i, CTL["ndof"]] = nd
            c[i, CTL["econs_thermo"]] = 0.0
            c[i, CTL["econs_baro"]] = 0.0
        self.set_state(pos, vels, rvecs)
        # set_state rewrote the lattice part; merge the hook constants back in
        c2 = self.control()
        keep = [CTL["L"], CTL["rvecs"], CTL["volume"]]
        for sl in keep:
            c[:, sl] = c2[:, sl]
        self.set_control(c)
        self.hooks = dict(thermostat=thermostat, barostat=code if code & ~0xF else barostat, temp=temp,
                          timecon=timecon, chain=chainlength)

    # ------------------------------------------------------------ kernels
    def md(self, nsteps, timestep=1.0 * femtosecond, thermostat=None, temp=300.0, timecon=100 * femtosecond,
           barostat=None, press=0.0, chainlength=3, seed=1, step0=0, noise=None, hook_noise=None, record=False,
           use_graph=True):
        """nsteps MD steps of every system. thermostat: None, "langevin", "nhc", "berendsen", "csvr";
        barostat: None, "mtk", "berendsen", "langevin" (anisotropic), or a ``baro_code`` (with the
        barostat's options; ``setup_md`` stores the one it set up in ``hooks["barostat"]``). The control block holds the
        hook state (``control`` / ``set_control``). noise: (nsteps, 2, sum N, 3) Langevin normals;
        hook_noise: (nsteps, nsys, HOOK_NOISE_LEN) CSVR / Langevin-barostat draws."""
        torch = self.torch
        dev = torch.device("cuda", torch.cuda.current_device())
        rec = None
        if record:
            rec = torch.zeros((len(self), nsteps, REC_LEN), dtype=torch.float64, device=dev)
        nz = None
        if noise is not None:
            nz = torch.from_numpy(np.ascontiguousarray(noise, dtype=np.float64)).to(dev)
        hz = None
        if hook_noise is not None:
            hook_noise = np.ascontiguousarray(hook_noise, dtype=np.float64)
            if hook_noise.shape != (nsteps, len(self), HOOK_NOISE_LEN):
                raise ValueError("hook_noise must have shape (nsteps, nsys, %d)" % HOOK_NOISE_LEN)
            hz = torch.from_numpy(hook_noise).to(dev)
        st = self.L.mm_batch_md(self._h, int(nsteps), float(timestep), _THERMO[thermostat], float(temp),
                                float(timecon), baro_code(barostat), float(press), int(chainlength),
                                int(seed), int(step0), nat.ptr(nz), nat.ptr(hz), nat.ptr(rec), int(bool(use_graph)),
                                torch.cuda.current_stream().cuda_stream)
        nat.check(st, "mm_batch_md")
        if record:
            return rec.cpu().numpy()
        return None

    def relax(self, max_iter=2000, gtol=1e-6, cell=None, press=0.0, stress_tol=1e-9):
        """CG relaxation of every system; returns (largest gradient norm, iterations) per system.

        cell=None: node positions only (the domain is fixed). cell="strain" / "full": positions
        and domain together, as StrainCellDOF / FullCellDOF (dof.py:492-697), at external
        pressure ``press`` (E + P V); converged when max |gpos| < gtol and the largest residual
        stress component |vtens / V + P I| < stress_tol (atomic units)."""
        torch = self.torch
        stream = torch.cuda.current_stream().cuda_stream
        if cell is None:
            nat.check(self.L.mm_batch_relax(self._h, int(max_iter), float(gtol), stream), "mm_batch_relax")
        else:
            full = {"strain": 0, "full": 1}[cell]
            nat.check(self.L.mm_batch_relax_cell(self._h, int(max_iter), float(gtol), float(stress_tol), float(press),
                                                 full, stream), "mm_batch_relax_cell")
        c = self.control()
        return c[:, CTL["gmax"]], c[:, CTL["iters"]]

    def residual_stress(self):
        """Largest residual stress component of the last cell relaxation, per system."""
        return self.control()[:, CTL["stress_res"]]

    def autotune(self, probe_steps=5, timestep=1.0 * femtosecond, thermostat=None, temp=300.0,
                 timecon=100 * femtosecond, barostat=None, press=0.0, chainlength=3):
        best = ctypes.c_double()
        nat.check(self.L.mm_batch_autotune(self._h, int(probe_steps), float(timestep), _THERMO[thermostat], float(temp),
                                           float(timecon), baro_code(barostat), float(press),
                                           int(chainlength), ctypes.byref(best)), "mm_batch_autotune")
        bt, nc = ctypes.c_int(), ctypes.c_int()
        nat.check(self.L.mm_batch_config(self._h, ctypes.byref(bt), ctypes.byref(nc)), "mm_batch_config")
        return {"cta_threads": bt.value, "ctas": nc.value, "probe_ms": best.value}

    # ------------------------------------------------------------ observables
    def energies(self):
        return self.control()[:, CTL["epot"]]

    def stress(self):
        """Static stress vtens / V per system (3x3), from the last force evaluation
        (the convention of the reference's stress-strain script, simulations/stress_strain.py:88-90)."""
        c = self.control()
        return np.array([c[i, CTL["vtens"]].reshape(3, 3) / c[i, CTL["volume"]] for i in range(len(self))])
