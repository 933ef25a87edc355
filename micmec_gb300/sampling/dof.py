"""Degrees of freedom for geometry and domain optimisation (interface of micmec/sampling/dof.py:32-697).

``CartesianDOF``: node positions. ``FullCellDOF``: the 9 scaled domain-vector
components plus fractional coordinates. ``StrainCellDOF``: a symmetric
deformation of the initial domain (6 parameters, no rotations) plus fractional
coordinates. The cell gradient comes from the virial, grvecs = gvecs . vtens
(dof.py:353-385). Every energy/gradient evaluation is one GPU force call.
"""

import numpy as np

__all__ = ["DOF", "CartesianDOF", "BaseCellDOF", "FullCellDOF", "StrainCellDOF"]


class DOF(object):
    def __init__(self, mmf):
        self.mmf = mmf
        self.x0 = None
        self._init_initial()
        self._gx = np.zeros(self.ndof, float)

    def _init_initial(self):
        raise NotImplementedError

    ndof = property(lambda self: len(self.x0))

    def _update(self, x):
        raise NotImplementedError

    def reset(self):
        self._update(self.x0)

    def check_delta(self, x=None, eps=1e-4, zero=None, ntest=20, rng=None):
        """Finite-difference test of the gradient (replaces molmod.minimizer.check_delta).

        Returns the largest relative deviation between the analytic and the central-difference
        directional derivative over ``ntest`` random directions.
        """
        x = self.x0.copy() if x is None else np.array(x, dtype=float)
        rng = np.random.default_rng(0) if rng is None else rng
        _, g = self.fun(x, True)
        worst = 0.0
        for _ in range(ntest):
            dx = rng.uniform(-eps, eps, len(x))
            if zero is not None:
                dx[zero] = 0.0
            fp = self.fun(x + dx)
            fm = self.fun(x - dx)
            num = fp - fm
            ana = 2 * np.dot(g, dx)
            worst = max(worst, abs(num - ana) / max(abs(ana), 1e-300))
        self._update(x)
        return worst

    def log(self):
        pass


def _conv(pairs):
    vals = [(v, n) for v, n in pairs if v is not None]
    if not vals:
        raise RuntimeError("At least one convergence criterion must be present.")
    conv_val, conv_worst = max(vals)
    return conv_val, conv_worst, sum(int(v >= 1) for v, _ in vals)


class CartesianDOF(DOF):
    """Cartesian node coordinates (dof.py:75-193)."""

    def __init__(self, mmf, gpos_rms=1e-5, dpos_rms=1e-3, select=None):
        self.th_gpos_rms = gpos_rms
        self.th_dpos_rms = dpos_rms
        self.select = select
        DOF.__init__(self, mmf)
        self._last_pos = None

    def _init_initial(self):
        pos = self.mmf.system.pos
        self.x0 = (pos if self.select is None else pos[self.select]).ravel().copy()
        self._pos = pos.copy()
        self._dpos = np.zeros(pos.shape, float)
        self._gpos = np.zeros(pos.shape, float)

    def _update(self, x):
        if self.select is None:
            self._pos[:] = x.reshape(-1, 3)
        else:
            self._pos[self.select] = x.reshape(-1, 3)
        self.mmf.update_pos(self._pos[:])

    def fun(self, x, do_gradient=False):
        self._update(x)
        if do_gradient:
            self._gpos[:] = 0.0
            v = self.mmf.compute(self._gpos)
            g = self._gpos if self.select is None else self._gpos[self.select]
            self._gx[:] = g.ravel()
            return v, self._gx.copy()
        return self.mmf.compute()

    def check_convergence(self):
        if self._last_pos is None:
            self._last_pos = self._pos.copy()
            self.converged = False
            self.conv_val = 2
            self.conv_worst = "first_step"
            self.conv_count = -1
            return
        sel = slice(None) if self.select is None else self.select
        gpossq = (self._gpos[sel] ** 2).sum(axis=1)
        self.gpos_max = np.sqrt(gpossq.max())
        self.gpos_rms = np.sqrt(gpossq.mean())
        self._dpos[:] = self._pos - self._last_pos
        dpossq = (self._dpos[sel] ** 2).sum(axis=1)
        self.dpos_max = np.sqrt(dpossq.max())
        self.dpos_rms = np.sqrt(dpossq.mean())
        pairs = []
        if self.th_gpos_rms is not None:
            pairs += [(self.gpos_rms / self.th_gpos_rms, "gpos_rms"), (self.gpos_max / (self.th_gpos_rms * 3), "gpos_max")]
        if self.th_dpos_rms is not None:
            pairs += [(self.dpos_rms / self.th_dpos_rms, "dpos_rms"), (self.dpos_max / (self.th_dpos_rms * 3), "dpos_max")]
        self.conv_val, self.conv_worst, self.conv_count = _conv(pairs)
        self.converged = self.conv_count == 0
        self._last_pos[:] = self._pos


class BaseCellDOF(DOF):
    """Cell variables (a subclass defines them) plus fractional coordinates (dof.py:199-478)."""

    def __init__(self, mmf, gpos_rms=1e-5, dpos_rms=1e-3, grvecs_rms=1e-5, drvecs_rms=1e-3, do_frozen=False,
                 freemask=None):
        if freemask is not None:
            if not (isinstance(freemask, np.ndarray) and freemask.dtype == bool and freemask.ndim == 1
                    and freemask.sum() > 0):
                raise TypeError("When given, freemask must be a vector of booleans.")
        self.th_gpos_rms = gpos_rms
        self.th_dpos_rms = dpos_rms
        self.th_grvecs_rms = grvecs_rms
        self.th_drvecs_rms = drvecs_rms
        self.do_frozen = do_frozen
        self.freemask = freemask
        DOF.__init__(self, mmf)
        self._last_pos = None
        self._last_rvecs = None

    ncellvar = property(lambda self: len(self.domainvars0))
    ncelldof = property(lambda self: len(self.domainvars0) if self.freemask is None else int(self.freemask.sum()))

    def _reduce_cellvars(self, cellvars):
        return cellvars if self.freemask is None else cellvars[self.freemask]

    def _expand_celldofs(self, celldofs):
        if self.freemask is None:
            return celldofs
        cellvars = self.domainvars0.copy()
        cellvars[self.freemask] = celldofs
        return cellvars

    def _isfree(self, i):
        return True if self.freemask is None else bool(self.freemask[i])

    def _init_initial(self):
        self.domainvars0 = self._get_initial_cellvars()
        if self.freemask is not None and len(self.freemask) != self.ncellvar:
            raise TypeError("The length of the freemask vector does not match the number of cellvars.")
        celldofs0 = self._reduce_cellvars(self.domainvars0)
        gvecs_full = self.mmf.system.domain._get_gvecs(full=True)
        frac = np.dot(self.mmf.system.pos, gvecs_full.T)
        if self.do_frozen:
            self.x0 = celldofs0
            self._frac0 = frac
        else:
            self.x0 = np.concatenate([celldofs0, frac.ravel()])
        self._pos = self.mmf.system.pos.copy()
        self._dpos = np.zeros(self._pos.shape, float)
        self._gpos = np.zeros(self._pos.shape, float)
        self._rvecs = self.mmf.system.domain.rvecs.copy()
        self._dcell = np.zeros(self._rvecs.shape, float)
        self._vtens = np.zeros((3, 3), float)
        self._grvecs = np.zeros(self._rvecs.shape, float)

    def _update(self, x):
        self._rvecs = self._cellvars_to_rvecs(self._expand_celldofs(x[: self.ncelldof]))
        self.mmf.update_rvecs(self._rvecs[:])
        rvecs_full = self.mmf.system.domain._get_rvecs(full=True)
        frac = self._frac0 if self.do_frozen else x[self.ncelldof:].reshape(-1, 3)
        self._pos[:] = np.dot(frac, rvecs_full)
        self.mmf.update_pos(self._pos[:])

    def fun(self, x, do_gradient=False):
        self._update(x)
        if not do_gradient:
            return self.mmf.compute()
        self._gpos[:] = 0.0
        self._vtens[:] = 0.0
        v = self.mmf.compute(self._gpos, self._vtens)
        self._grvecs[:] = np.dot(self.mmf.system.domain.gvecs, self._vtens)
        jac = self._get_celldofs_jacobian(x[: self.ncelldof])
        self._gx[: self.ncelldof] = np.dot(self._grvecs.ravel(), jac)
        U, S, Vt = np.linalg.svd(jac, full_matrices=False)
        self._grvecs[:] = np.dot(U, np.dot(U.T, self._grvecs.ravel())).reshape(-1, 3)
        if not self.do_frozen:
            self._gx[self.ncelldof:] = np.dot(self._gpos, self._rvecs.T).ravel()
        return v, self._gx.copy()

    def check_convergence(self):
        if self._last_pos is None:
            self._last_pos = self._pos.copy()
            self._last_rvecs = self._rvecs.copy()
            self.converged = False
            self.conv_val = 2
            self.conv_worst = "first_step"
            self.conv_count = -1
            return
        pairs = []
        if not self.do_frozen:
            gpossq = (self._gpos**2).sum(axis=1)
            self.gpos_max = np.sqrt(gpossq.max())
            self.gpos_rms = np.sqrt(gpossq.mean())
            self._dpos[:] = self._pos - self._last_pos
            if self.th_gpos_rms is not None:
                pairs += [(self.gpos_rms / self.th_gpos_rms, "gpos_rms"),
                          (self.gpos_max / (self.th_gpos_rms * 3), "gpos_max")]
        dpossq = (self._dpos**2).sum(axis=1)
        self.dpos_max = np.sqrt(dpossq.max())
        self.dpos_rms = np.sqrt(dpossq.mean())
        grvecssq = (self._grvecs**2).sum(axis=1)
        self.grvecs_max = np.sqrt(grvecssq.max())
        self.grvecs_rms = np.sqrt(grvecssq.mean())
        self._dcell[:] = self._rvecs - self._last_rvecs
        dcellsq = (self._dcell**2).sum(axis=1)
        self.drvecs_max = np.sqrt(dcellsq.max())
        self.drvecs_rms = np.sqrt(dcellsq.mean())
        if self.th_dpos_rms is not None:
            pairs += [(self.dpos_rms / self.th_dpos_rms, "dpos_rms"), (self.dpos_max / (self.th_dpos_rms * 3), "dpos_max")]
        if self.th_grvecs_rms is not None:
            pairs += [(self.grvecs_rms / self.th_grvecs_rms, "grvecs_rms"),
                      (self.grvecs_max / (self.th_grvecs_rms * 3), "grvecs_max")]
        if self.th_drvecs_rms is not None:
            pairs += [(self.drvecs_rms / self.th_drvecs_rms, "drvecs_rms"),
                      (self.drvecs_max / (self.th_drvecs_rms * 3), "drvecs_max")]
        self.conv_val, self.conv_worst, self.conv_count = _conv(pairs)
        self.converged = self.conv_count == 0
        self._last_pos[:] = self._pos
        self._last_rvecs[:] = self._rvecs

    def _get_initial_cellvars(self):
        raise NotImplementedError

    def _cellvars_to_rvecs(self, cellvars):
        raise NotImplementedError

    def _get_celldofs_jacobian(self, x):
        raise NotImplementedError


class FullCellDOF(BaseCellDOF):
    """All domain-vector components, scaled by volume^(1/nvec) (dof.py:482-513)."""

    def _get_initial_cellvars(self):
        cell = self.mmf.system.domain
        if cell.nvec == 0:
            raise ValueError("A cell optimization requires a system that is periodic.")
        self._rvecs_scale = cell.volume ** (1.0 / cell.nvec)
        return cell.rvecs.ravel() / self._rvecs_scale

    def _cellvars_to_rvecs(self, cellvars):
        return cellvars.reshape(-1, 3) * self._rvecs_scale

    def _get_celldofs_jacobian(self, x):
        result = np.identity(self.ncellvar) * self._rvecs_scale
        return result if self.freemask is None else result[:, self.freemask]


class StrainCellDOF(BaseCellDOF):
    """Symmetric deformation A of the initial domain, rvecs = A . rvecs0 (dof.py:516-697).

    3-D parameters: [A_00, A_11, A_22, 2 A_12, 2 A_20, 2 A_01].
    """

    _PAIRS = {3: [(0, 0), (1, 1), (2, 2), (1, 2), (2, 0), (0, 1)], 2: [(0, 0), (1, 1), (0, 1)], 1: [(0, 0)]}

    def _get_initial_cellvars(self):
        cell = self.mmf.system.domain
        if cell.nvec == 0:
            raise ValueError("A cell optimization requires a system that is periodic.")
        self.rvecs0 = cell.rvecs.copy()
        n = cell.nvec
        return np.array([1.0] * n + [0.0] * (n * (n + 1) // 2 - n))

    def _basis(self, k):
        n = self.mmf.system.domain.nvec
        i, j = self._PAIRS[n][k]
        E = np.zeros((n, n))
        if i == j:
            E[i, i] = 1.0
        else:
            E[i, j] = E[j, i] = 0.5
        return E

    def _cellvars_to_rvecs(self, x):
        n = self.mmf.system.domain.nvec
        deform = sum(x[k] * self._basis(k) for k in range(n * (n + 1) // 2))
        return np.dot(deform, self.rvecs0)

    def _get_celldofs_jacobian(self, x):
        n = self.mmf.system.domain.nvec
        cols = [np.dot(self._basis(k), self.rvecs0).ravel() for k in range(n * (n + 1) // 2) if self._isfree(k)]
        return np.array(cols).T
