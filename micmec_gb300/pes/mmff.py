"""Micromechanical force field: ``ForcePart``, ``MicMecForceField``,
``ForcePartMechanical`` and ``ForcePartPressure``.

The classes keep the reference's interface (micmec/pes/mmff.py:39-323):
``compute(gpos=None, vtens=None)`` takes optional Fortran-style output arrays,
**adds** the part's gradient and virial to them and returns the energy; a NaN
in energy, gradient or virial raises ``ValueError`` (mmff.py:135-148).

``ForcePartMechanical`` is backed by the native library: system topology and
parameters are uploaded once, and each ``compute`` runs the per-cell and per-node
CUDA kernels. There is no CPU code path; a missing library or GPU raises.
"""

import numpy as np

from micmec_gb300 import _native as nat
from micmec_gb300.utils import Grid

__all__ = ["MicMecForceField", "ForcePart", "ForcePartMechanical", "ForcePartPressure", "type_parameters"]

_MODELS = {"original": 0, "nanocell": 1}
_PRECISIONS = {"fp64": 0, "fp32": 1}
_CORNERS = np.array([(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)])


class ForcePart(object):
    """Base class of the parts of a micromechanical force field (mmff.py:39-149)."""

    def __init__(self, name, system):
        self.name = name
        self.energy = 0.0
        self.gpos = np.zeros((system.nnodes, 3), float)
        self.vtens = np.zeros((3, 3), float)
        self.clear()

    def clear(self):
        """Mark the cached results as invalid (NaN)."""
        self.energy = np.nan
        self.gpos[:] = np.nan
        self.vtens[:] = np.nan

    def update_rvecs(self, rvecs):
        self.clear()

    def update_pos(self, pos):
        self.clear()

    def compute(self, gpos=None, vtens=None):
        """Energy of this part; gradient and virial are ADDED to ``gpos`` and ``vtens`` if given."""
        mmf_gpos = None
        if gpos is not None:
            mmf_gpos = self.gpos
            mmf_gpos[:] = 0.0
        mmf_vtens = None
        if vtens is not None:
            mmf_vtens = self.vtens
            mmf_vtens[:] = 0.0
        self.energy = self._internal_compute(mmf_gpos, mmf_vtens)
        if np.isnan(self.energy):
            raise ValueError("The energy is not-a-number (``nan``).")
        if gpos is not None:
            if np.isnan(mmf_gpos).any():
                raise ValueError("Some ``gpos`` element(s) is/are not-a-number (``nan``).")
            gpos += mmf_gpos
        if vtens is not None:
            if np.isnan(mmf_vtens).any():
                raise ValueError("Some ``vtens`` element(s) is/are not-a-number (``nan``).")
            vtens += mmf_vtens
        return self.energy

    def _internal_compute(self, gpos, vtens):
        raise NotImplementedError


class MicMecForceField(ForcePart):
    """A complete micromechanical force field: the sum of its parts (mmff.py:156-201)."""

    def __init__(self, system, parts):
        ForcePart.__init__(self, "all", system)
        self.system = system
        self.parts = []
        for part in parts:
            self.add_part(part)

    def add_part(self, part):
        self.parts.append(part)
        name = "part_%s" % part.name
        if name in self.__dict__:
            raise ValueError("The part %s occurs twice in the micromechanical force field." % name)
        self.__dict__[name] = part

    def update_rvecs(self, rvecs):
        ForcePart.update_rvecs(self, rvecs)
        self.system.domain.update_rvecs(rvecs)
        for part in self.parts:
            part.update_rvecs(rvecs)

    def update_pos(self, pos):
        ForcePart.update_pos(self, pos)
        self.system.pos[:] = pos
        for part in self.parts:
            part.update_pos(pos)

    def _internal_compute(self, gpos, vtens):
        return sum([part.compute(gpos, vtens) for part in self.parts])


def type_parameters(params, type_ids):
    """Pack ``type{k}/...`` parameters into the arrays the C ABI takes.

    Returns (nstates[T], h0[T*4,9], C[T*4,81], free_energy[T*4], temp_eff[T]) for the
    type ids in ``type_ids`` (in that order), as parsed by micmec/pes/mmff.py:218-242.
    """
    T = len(type_ids)
    nstates = np.zeros(T, dtype=np.int32)
    h0 = np.zeros((T * 4, 9))
    C = np.zeros((T * 4, 81))
    df = np.zeros(T * 4)
    temp = np.zeros(T)
    for t, k in enumerate(type_ids):
        cells = params[f"type{k}/cell"]
        elast = params[f"type{k}/elasticity"]
        efree = params.get(f"type{k}/free_energy", [0.0] * len(cells))
        ns = len(cells)
        if ns < 1 or ns > 4:
            raise ValueError("type %d has %d states; 1 to 4 are supported" % (k, ns))
        nstates[t] = ns
        for s in range(ns):
            h0[4 * t + s] = np.asarray(cells[s], dtype=np.float64).reshape(9)
            C[4 * t + s] = np.asarray(elast[s], dtype=np.float64).reshape(81)
            df[4 * t + s] = float(np.atleast_1d(efree)[s])
        temp[t] = float(params.get(f"type{k}/effective_temp", 300.0))
    return nstates, h0, C, df, temp


class ForcePartMechanical(ForcePart):
    """The micromechanical part of the force field (mmff.py:204-323), on the GPU.

    Parameters
    ----------
    system : micmec_gb300.system.System
    model : {"nanocell", "original"}
        "nanocell": eight corner matrices per cell (micmec/pes/nanocell.py);
        "original": one averaged matrix per cell (micmec/pes/nanocell_original.py,
        what the reference's mmff.py imports).
    precision : {"fp64", "fp32"}
        Arithmetic of the per-cell strain/energy/gradient. Reductions, the
        log-sum-exp shift and all node state stay FP64.
    """

    def __init__(self, system, model="nanocell", precision="fp64"):
        ForcePart.__init__(self, "micmec", system)
        import torch

        if not torch.cuda.is_available():
            raise nat.MMError("ForcePartMechanical needs a CUDA device")
        self.system = system
        self.model = model
        self.precision = precision
        self.torch = torch
        self.device = torch.device("cuda", torch.cuda.current_device())
        self._handle = None
        self._create()
        self.epot_cells_dev = None

    # ---------------------------------------------------------------- setup
    def _topology(self):
        s = self.system
        rvecs = np.asarray(s.domain.rvecs).reshape(-1, 3)
        nper = rvecs.shape[0]
        if nper not in (0, 3):
            raise ValueError(
                "Attribute `rvecs` only supports finite systems or 3D periodic systems, not %dD periodic systems." % nper
            )
        pbc = nper == 3
        if s.grid is None:
            raise ValueError("ForcePartMechanical needs system.grid")
        g = Grid(np.asarray(s.grid).astype(np.int64), pbc=pbc)
        node_coords = g.node_coords
        cell_coords = g.cell_coords
        sn = np.asarray(s.surrounding_nodes, dtype=np.int64)
        sc = np.asarray(s.surrounding_cells, dtype=np.int64)
        nn = np.array(g.shape_nodes)
        if len(node_coords) != s.nnodes or len(cell_coords) != s.ncells:
            raise ValueError("system.grid does not match the number of nodes/cells")
        expect = (cell_coords[:, None, :] + _CORNERS[None]) % nn
        if not np.array_equal(node_coords[sn], expect):
            raise ValueError("surrounding_nodes does not follow the grid's lattice")
        return pbc, node_coords, sn, sc, nn

    def _create(self):
        torch = self.torch
        s = self.system
        L = nat.lib()
        pbc, node_coords, sn, sc, nn = self._topology()
        self.pbc = pbc
        self.node_coords = node_coords
        self.lattice_shape = nn
        types = np.asarray(s.types).astype(np.int64)
        type_ids = sorted(set(int(t) for t in types))
        index = {k: i for i, k in enumerate(type_ids)}
        self.type_ids = type_ids
        cell_type = np.array([index[int(t)] for t in types], dtype=np.int32)
        nstates, h0, C, df, temp = type_parameters(s.params, type_ids)
        arrays = dict(
            node_coords=np.ascontiguousarray(node_coords, dtype=np.int32),
            cell_nodes=np.ascontiguousarray(sn, dtype=np.int32),
            node_cells=np.ascontiguousarray(sc, dtype=np.int32),
            cell_type=cell_type,
            shape=np.ascontiguousarray(nn, dtype=np.int32),
            nstates=nstates,
            h0=np.ascontiguousarray(h0),
            C=np.ascontiguousarray(C),
            df=np.ascontiguousarray(df),
            temp=np.ascontiguousarray(temp),
            masses=np.ascontiguousarray(s.masses, dtype=np.float64),
        )
        self._arrays = arrays  # keep alive during the call
        h = nat.c_void_p()
        st = L.mm_create(
            s.nnodes, s.ncells, nat.ptr(arrays["node_coords"]), nat.ptr(arrays["cell_nodes"]),
            nat.ptr(arrays["node_cells"]), nat.ptr(arrays["cell_type"]), nat.ptr(arrays["shape"]), int(pbc),
            len(type_ids), nat.ptr(arrays["nstates"]), nat.ptr(arrays["h0"]), nat.ptr(arrays["C"]),
            nat.ptr(arrays["df"]), nat.ptr(arrays["temp"]), nat.ptr(arrays["masses"]), _MODELS[self.model],
            _PRECISIONS[self.precision], nat.ctypes.byref(h),
        )
        nat.check(st, "mm_create")
        self._handle = h
        dev = self.device
        self._pos = torch.zeros((s.nnodes, 3), dtype=torch.float64, device=dev)
        self._gpos = torch.zeros((s.nnodes, 3), dtype=torch.float64, device=dev)
        self._out = torch.zeros(10, dtype=torch.float64, device=dev)
        self._flag = torch.zeros(1, dtype=torch.int32, device=dev)
        self._lattice = None
        if not pbc:
            # isolated: node spacing = mean edge vector along each lattice direction
            pos = np.asarray(s.pos)
            Lm = np.zeros((3, 3))
            for d in range(3):
                lo = [k for k in range(8) if _CORNERS[k][d] == 0]
                hi = [k for k in range(8) if _CORNERS[k][d] == 1]
                edges = [pos[sn[:, h]] - pos[sn[:, l]] for l, h in zip(lo, hi)]
                Lm[d] = np.mean(np.concatenate(edges), axis=0)
            self._lattice = np.ascontiguousarray(Lm)
        self._push_domain()

    def _push_domain(self):
        rv = np.asarray(self.system.domain.rvecs, dtype=np.float64).reshape(-1, 3)
        rv = np.ascontiguousarray(rv) if self.pbc else None
        nat.check(nat.lib().mm_set_domain(self._handle, nat.ptr(rv), nat.ptr(self._lattice)), "mm_set_domain")

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None and nat._lib is not None:
            try:
                nat._lib.mm_destroy(h)
            except Exception:
                pass
            self._handle = None

    @property
    def handle(self):
        return self._handle

    def lattice_matrix(self):
        """Rows L_d: the lattice translation between neighbouring nodes along d (rvecs_d / n_d
        for a periodic domain, the mean edge vector for an isolated one)."""
        if self._lattice is not None:
            return np.array(self._lattice)
        rv = np.asarray(self.system.domain.rvecs, dtype=np.float64).reshape(3, 3)
        return rv / np.asarray(self.lattice_shape, dtype=np.float64)[:, None]

    # ---------------------------------------------------------------- API
    def update_rvecs(self, rvecs):
        ForcePart.update_rvecs(self, rvecs)
        self._push_domain()

    def compute_device(self, pos, gpos=None, vtens=None, energy=None, flag=None, stream=None):
        """Enqueue a compute on device tensors: pos (N,3); gpos (N,3) and vtens (3,3) are added to.

        ``energy`` is a device double tensor that receives the energy. Nothing is synchronised.
        """
        torch = self.torch
        if energy is None:
            energy = self._out[:1]
        if stream is None:
            stream = torch.cuda.current_stream().cuda_stream
        st = nat.lib().mm_compute(self._handle, nat.ptr(pos), nat.ptr(gpos), nat.ptr(vtens), nat.ptr(energy),
                                  nat.ptr(flag), stream)
        nat.check(st, "mm_compute")
        return energy

    def _internal_compute(self, gpos, vtens):
        torch = self.torch
        self._pos.copy_(torch.from_numpy(np.ascontiguousarray(self.system.pos, dtype=np.float64)))
        self._out.zero_()
        self._flag.zero_()
        gp = None
        if gpos is not None:
            self._gpos.zero_()
            gp = self._gpos
        vt = self._out[1:] if vtens is not None else None
        self.compute_device(self._pos, gp, vt, self._out[:1], self._flag)
        out = self._out.cpu().numpy()
        if gpos is not None:
            gpos[:] = self._gpos.cpu().numpy()
        if vtens is not None:
            vtens[:] = out[1:].reshape(3, 3)
        if int(self._flag.item()) != 0 and not np.isnan(out[0]):
            # a NaN in the gradient with a finite energy: report through gpos
            if gpos is not None:
                gpos[:] = np.nan
        return float(out[0])

    # per-cell results of the last compute (mmff.py:209-214 keeps them as attributes)
    @property
    def epot_cells(self):
        torch = self.torch
        out = torch.empty(self.system.ncells, dtype=torch.float64, device=self.device)
        nat.check(nat.lib().mm_cell_results(self._handle, nat.ptr(out), None,
                                            torch.cuda.current_stream().cuda_stream), "mm_cell_results")
        return out.cpu().numpy()

    @property
    def gpos_cells(self):
        torch = self.torch
        out = torch.empty((self.system.ncells, 8, 3), dtype=torch.float64, device=self.device)
        nat.check(nat.lib().mm_cell_results(self._handle, None, nat.ptr(out),
                                            torch.cuda.current_stream().cuda_stream), "mm_cell_results")
        return out.cpu().numpy()

    @property
    def verts_cells(self):
        s = self.system
        pos = np.asarray(s.pos)
        sn = np.asarray(s.surrounding_nodes)
        r0 = pos[sn[:, 0]]
        d = pos[sn] - r0[:, None, :]
        if self.pbc:
            g = Grid(np.asarray(s.grid).astype(np.int64), pbc=True)
            wrap = (g.cell_coords[:, None, :] + _CORNERS[None]) >= np.array(g.shape_nodes)
            rv = np.asarray(s.domain.rvecs)
            d = d + wrap.astype(float) @ rv
        return r0[:, None, :] + d


class ForcePartPressure(ForcePart):
    """External-pressure term E = P V of the domain, with virial P V I.

    Not present in the reference; it follows the usual definition of this part
    in Yaff-style force fields (energy pext * volume; the virial adds
    pext * volume to the diagonal). The part has no node gradient.
    """

    def __init__(self, system, pext):
        ForcePart.__init__(self, "press", system)
        self.system = system
        self.pext = float(pext)

    def _internal_compute(self, gpos, vtens):
        volume = self.system.domain.volume
        if vtens is not None:
            vtens.ravel()[::4] += self.pext * volume
        return self.pext * volume
