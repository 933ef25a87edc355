"""``Domain``: the periodic simulation domain (rvecs, gvecs, volume, nvec).

Host-side equivalent of the reference's Cython/C ``Domain`` (micmec/pes/ext.pyx:36-123,
micmec/pes/domain.c:13-72): the same properties and the same SVD-based
completion of the domain matrix and reciprocal vectors (ext.pyx:52-72). It is a
few 3x3 operations per update; the device copy of the lattice lives in the
native handle of each force part.
"""

import numpy as np

__all__ = ["Domain"]


class Domain(object):
    """Representation of periodic boundary conditions."""

    def __init__(self, rvecs):
        self.update_rvecs(rvecs)

    def update_rvecs(self, rvecs):
        if rvecs is None or np.size(rvecs) == 0:
            mod_rvecs = np.identity(3, float)
            gvecs = mod_rvecs
            nvec = 0
        else:
            rvecs = np.asarray(rvecs, dtype=np.float64)
            if rvecs.ndim != 2 or rvecs.shape[0] > 3 or rvecs.shape[1] != 3:
                raise TypeError("rvecs must be a C-contiguous array with three columns and at most three rows.")
            nvec = len(rvecs)
            Up, Sp, Vt = np.linalg.svd(rvecs, full_matrices=True)
            S = np.ones(3, float)
            S[:nvec] = Sp
            U = np.identity(3, float)
            U[:nvec, :nvec] = Up
            mod_rvecs = np.dot(U * S, Vt)
            mod_rvecs[:nvec] = rvecs
            gvecs = np.dot(U / S, Vt)
        self._nvec = nvec
        self._rvecs = np.array(mod_rvecs, dtype=np.float64)
        self._gvecs = np.array(gvecs, dtype=np.float64)
        r = self._rvecs
        if nvec == 0:
            self._volume = 0.0
        elif nvec == 1:
            self._volume = float(np.sqrt(np.dot(r[0], r[0])))
        elif nvec == 2:
            tmp = np.dot(r[0], r[1])
            tmp = np.dot(r[0], r[0]) * np.dot(r[1], r[1]) - tmp * tmp
            self._volume = float(np.sqrt(tmp)) if tmp > 0 else 0.0
        else:
            self._volume = float(abs(
                r[0, 0] * (r[1, 1] * r[2, 2] - r[1, 2] * r[2, 1])
                + r[0, 1] * (r[1, 2] * r[2, 0] - r[1, 0] * r[2, 2])
                + r[0, 2] * (r[1, 0] * r[2, 1] - r[1, 1] * r[2, 0])
            ))

    @property
    def nvec(self):
        return self._nvec

    @property
    def volume(self):
        return self._volume

    def _get_rvecs(self, full=False):
        out = self._rvecs.copy() if full else self._rvecs[: self._nvec].copy()
        out.setflags(write=False)
        return out

    rvecs = property(_get_rvecs)

    def _get_gvecs(self, full=False):
        out = self._gvecs.copy() if full else self._gvecs[: self._nvec].copy()
        out.setflags(write=False)
        return out

    gvecs = property(_get_gvecs)

    @property
    def parameters(self):
        rvecs = self._get_rvecs()
        tmp = np.dot(rvecs, rvecs.T)
        lengths = np.sqrt(np.diag(tmp))
        tmp = tmp / lengths
        tmp = tmp / lengths.reshape((-1, 1))
        if len(rvecs) < 2:
            cosines = np.array([])
        elif len(rvecs) == 2:
            cosines = np.array([tmp[0, 1]])
        else:
            cosines = np.array([tmp[1, 2], tmp[2, 0], tmp[0, 1]])
        angles = np.arccos(np.clip(cosines, -1, 1))
        return lengths, angles
