"""Reference-side binding: the file a MicMec maintainer adds as ``micmec/pes/mmff_gb300.py``.

It is written against the reference's own modules (``micmec.pes.mmff.ForcePart``,
``micmec.utils.Grid``) and calls the C ABI of ``libmicmec_gb300.so`` through ctypes,
with host buffers (``mm_compute_host``). ``ForcePartMechanicalGPU(system)`` takes the
same ``System`` that ``ForcePartMechanical(system)`` takes (micmec/pes/mmff.py:204-245)
and gives the same ``compute(gpos, vtens)`` results (mmff.py:87-149, 288-323):
``ForcePart.compute`` zeroes the part's own buffers and adds them to the caller's, so
the add-into semantics of ``mm_compute_host`` reproduce the reference's behaviour,
and a NaN status becomes the reference's ``ValueError``. Periodic (three domain
vectors) and isolated (none) systems are both accepted, as the reference's part does.

The library path comes from the environment variable ``MICMEC_GB300_LIB``; without it
the in-tree build of this package is used. The tests run this file unchanged on a
namespace that maps ``micmec.pes.mmff`` and ``micmec.utils`` to this package's mirrors.
"""
import ctypes
import os

import numpy as np
from micmec.pes.mmff import ForcePart
from micmec.utils import Grid

_DEFAULT = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "lib", "libmicmec_gb300.so")
_lib = ctypes.CDLL(os.environ.get("MICMEC_GB300_LIB", _DEFAULT))
_P = ctypes.c_void_p
_lib.mm_create.argtypes = ([ctypes.c_int, ctypes.c_int] + [_P] * 5 + [ctypes.c_int, ctypes.c_int] + [_P] * 6
                           + [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)])
_lib.mm_create.restype = ctypes.c_int
_lib.mm_destroy.argtypes = [_P]
_lib.mm_destroy.restype = ctypes.c_int
_lib.mm_set_domain.argtypes = [_P, _P, _P]
_lib.mm_set_domain.restype = ctypes.c_int
_lib.mm_compute_host.argtypes = [_P, _P, _P, _P, _P]
_lib.mm_compute_host.restype = ctypes.c_int
_lib.mm_last_error.restype = ctypes.c_char_p

MM_OK, MM_ERR_NAN = 0, 1
MODELS = {"original": 0, "nanocell": 1}
PRECISIONS = {"fp64": 0, "fp32": 1}


def _check(status, what):
    if status != MM_OK:
        raise RuntimeError("%s failed (status %d): %s" % (what, status, _lib.mm_last_error().decode(errors="replace")))


class ForcePartMechanicalGPU(ForcePart):
    """Drop-in for ForcePartMechanical (micmec/pes/mmff.py:204-323): same inputs, GPU compute."""

    def __init__(self, system, model="nanocell", precision="fp64"):
        ForcePart.__init__(self, "micmec", system)
        self.system = system
        rvecs = np.asarray(system.domain.rvecs, dtype=float).reshape(-1, 3)
        self.pbc = rvecs.shape[0] == 3
        if rvecs.shape[0] not in (0, 3):
            raise ValueError("only isolated or 3D periodic systems are supported")
        g = Grid(np.asarray(system.grid), pbc=self.pbc)
        nodes = np.ascontiguousarray(g.nodes, dtype=np.int32)
        types = sorted(set(int(t) for t in system.types))
        tidx = np.array([types.index(int(t)) for t in system.types], dtype=np.int32)
        nst = np.array([len(system.params["type%d/cell" % k]) for k in types], dtype=np.int32)
        h0 = np.zeros((len(types) * 4, 9))
        C = np.zeros((len(types) * 4, 81))
        df = np.zeros(len(types) * 4)
        temp = np.array([float(system.params.get("type%d/effective_temp" % k, 300.0)) for k in types])
        for t, k in enumerate(types):
            efree = np.atleast_1d(system.params.get("type%d/free_energy" % k, np.zeros(nst[t])))
            for s in range(nst[t]):
                h0[4 * t + s] = np.ravel(system.params["type%d/cell" % k][s])
                C[4 * t + s] = np.ravel(system.params["type%d/elasticity" % k][s])
                df[4 * t + s] = float(efree[s])
        sn = np.ascontiguousarray(system.surrounding_nodes, dtype=np.int32)
        sc = np.ascontiguousarray(system.surrounding_cells, dtype=np.int32)
        shape = np.array([g.nx_nodes, g.ny_nodes, g.nz_nodes], dtype=np.int32)
        masses = np.ascontiguousarray(system.masses, dtype=float)
        self._keep = (nodes, tidx, nst, h0, C, df, temp, sn, sc, shape, masses)
        self._h = ctypes.c_void_p()
        _check(_lib.mm_create(system.nnodes, system.ncells, nodes.ctypes.data, sn.ctypes.data, sc.ctypes.data,
                              tidx.ctypes.data, shape.ctypes.data, int(self.pbc), len(types), nst.ctypes.data,
                              h0.ctypes.data, C.ctypes.data, df.ctypes.data, temp.ctypes.data, masses.ctypes.data,
                              MODELS[model], PRECISIONS[precision], ctypes.byref(self._h)), "mm_create")
        self._lattice = None
        if not self.pbc:
            # isolated: the lattice matrix is the mean edge vector along each lattice direction
            corners = np.array([(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1),
                                (1, 1, 1)])
            pos = np.asarray(system.pos)
            lat = np.zeros((3, 3))
            for d in range(3):
                lo = [k for k in range(8) if corners[k][d] == 0]
                hi = [k for k in range(8) if corners[k][d] == 1]
                lat[d] = np.mean(np.concatenate([pos[sn[:, b]] - pos[sn[:, a]] for a, b in zip(lo, hi)]), axis=0)
            self._lattice = np.ascontiguousarray(lat)
        self.update_rvecs(rvecs)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.mm_destroy(h)
            self._h = None

    def update_rvecs(self, rvecs):
        ForcePart.update_rvecs(self, rvecs)
        rv = np.ascontiguousarray(np.asarray(rvecs, dtype=float).reshape(-1, 3))
        lat = None if self._lattice is None else self._lattice.ctypes.data
        _check(_lib.mm_set_domain(self._h, rv.ctypes.data if self.pbc else None, lat), "mm_set_domain")

    def _internal_compute(self, gpos, vtens):
        pos = np.ascontiguousarray(self.system.pos, dtype=float)
        e = np.zeros(1)
        st = _lib.mm_compute_host(self._h, pos.ctypes.data, None if gpos is None else gpos.ctypes.data,
                                  None if vtens is None else vtens.ctypes.data, e.ctypes.data)
        if st == MM_ERR_NAN:
            raise ValueError("The energy is not-a-number (``nan``).")
        _check(st, "mm_compute_host")
        return float(e[0])
