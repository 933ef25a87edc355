"""Optimisation variables ("degrees of freedom") for geometry and domain relaxation.

A DOF object turns a flat vector x into a configuration of the force field, returns the
energy (and dE/dx), and judges convergence from how much the configuration moved and how
large the gradient is between two calls of ``check_convergence``.

* ``CartesianDOF``: x = node positions, or those of a selection of nodes
  (micmec/sampling/dof.py:75-193).
* ``FullCellDOF``: x = [the nine domain-vector components divided by V^(1/3), the
  fractional node coordinates] (dof.py:482-513).
* ``StrainCellDOF``: x = [a symmetric deformation A of the initial domain in the order
  A_00, A_11, A_22, 2 A_12, 2 A_20, 2 A_01, the fractional node coordinates]; rvecs =
  A rvecs_0, so rigid rotations are excluded (dof.py:516-697).

Domain gradients come from the virial, dE/d(rvecs) = gvecs . vtens (dof.py:353-385),
chained with the Jacobian of rvecs with respect to the cell variables; node gradients in
fractional coordinates are gpos . rvecs^T. Convergence criteria (each optional) are rms
values against a threshold t and maxima against 3 t; the run has converged when every
ratio is below one (dof.py:155-193, 387-478). Every evaluation is one GPU force call.
"""

import numpy as np

__all__ = ["DOF", "CartesianDOF", "BaseCellDOF", "FullCellDOF", "StrainCellDOF"]


def _norms(vectors):
    """(rms, max) of the row norms of an (n, 3) array."""
    sq = (np.asarray(vectors) ** 2).sum(axis=1)
    return np.sqrt(sq.mean()), np.sqrt(sq.max())


class _Verdict(object):
    """Ratios of measured sizes to thresholds; the worst one and how many are >= 1."""

    def __init__(self):
        self.ratios = []

    def add(self, name, rms, maximum, threshold):
        if threshold is None:
            return
        self.ratios.append((rms / threshold, name + "_rms"))
        self.ratios.append((maximum / (3.0 * threshold), name + "_max"))

    def apply(self, dof):
        if not self.ratios:
            raise RuntimeError("No convergence criterion is set: give at least one threshold.")
        dof.conv_val, dof.conv_worst = max(self.ratios)
        dof.conv_count = sum(1 for ratio, _ in self.ratios if ratio >= 1.0)
        dof.converged = dof.conv_count == 0


class DOF(object):
    """Base: subclasses define ``_initial_vector``, ``_apply`` (x -> force field) and
    ``_gradient_vector`` (dE/dx after a compute with gradient), plus ``_measure`` for convergence."""

    def __init__(self, mmf):
        self.mmf = mmf
        self.x0 = self._initial_vector()
        self._gx = np.zeros(len(self.x0))
        self._reference = None  # configuration at the last convergence check
        self.converged = False

    @property
    def ndof(self):
        return len(self.x0)

    def _update(self, x):
        self._apply(np.asarray(x, dtype=float))

    def reset(self):
        self._update(self.x0)

    def fun(self, x, do_gradient=False):
        """Energy at x; with do_gradient also dE/dx (a copy)."""
        self._update(x)
        if not do_gradient:
            return self.mmf.compute()
        energy = self._compute_with_gradient()
        self._gx[:] = self._gradient_vector(x)
        return energy, self._gx.copy()

    def check_convergence(self):
        """Compare with the configuration of the previous call. The first call only records it."""
        now = self._snapshot()
        if self._reference is None:
            self._reference = now
            self.converged = False
            self.conv_val = np.inf
            self.conv_worst = "first_step"
            self.conv_count = -1
            return
        verdict = _Verdict()
        self._measure(now, self._reference, verdict)
        verdict.apply(self)
        self._reference = now

    def check_delta(self, x=None, eps=1e-4, zero=None, ntest=20, rng=None):
        """Largest relative difference between dE/dx . dx and a central difference E(x + dx) -
        E(x - dx) over ``ntest`` random steps dx of size ``eps`` (entries ``zero`` kept at 0).
        Serves the purpose of molmod.minimizer.check_delta, which the reference calls."""
        x = np.array(self.x0 if x is None else x, dtype=float)
        rng = np.random.default_rng(0) if rng is None else rng
        _, grad = self.fun(x, True)
        worst = 0.0
        for _ in range(ntest):
            step = rng.uniform(-eps, eps, len(x))
            if zero is not None:
                step[zero] = 0.0
            numeric = self.fun(x + step) - self.fun(x - step)
            analytic = 2.0 * grad @ step
            worst = max(worst, abs(numeric - analytic) / max(abs(analytic), 1e-300))
        self._update(x)
        return worst

    def log(self):
        pass


class CartesianDOF(DOF):
    """Cartesian node coordinates (micmec/sampling/dof.py:75-193); ``select``: a subset of nodes."""

    def __init__(self, mmf, gpos_rms=1e-5, dpos_rms=1e-3, select=None):
        self.th_gpos_rms = gpos_rms
        self.th_dpos_rms = dpos_rms
        self.select = select
        self._rows = slice(None) if select is None else select
        DOF.__init__(self, mmf)

    def _initial_vector(self):
        self._pos = np.array(self.mmf.system.pos, dtype=float)
        self._gpos = np.zeros_like(self._pos)
        return self._pos[self._rows].ravel().copy()

    def _apply(self, x):
        self._pos[self._rows] = x.reshape(-1, 3)
        self.mmf.update_pos(self._pos)

    def _compute_with_gradient(self):
        self._gpos[:] = 0.0
        return self.mmf.compute(self._gpos)

    def _gradient_vector(self, x):
        return self._gpos[self._rows].ravel()

    def _snapshot(self):
        return self._pos.copy()

    def _measure(self, pos, last, verdict):
        self.gpos_rms, self.gpos_max = _norms(self._gpos[self._rows])
        self.dpos_rms, self.dpos_max = _norms((pos - last)[self._rows])
        verdict.add("gpos", self.gpos_rms, self.gpos_max, self.th_gpos_rms)
        verdict.add("dpos", self.dpos_rms, self.dpos_max, self.th_dpos_rms)


class BaseCellDOF(DOF):
    """Domain variables (defined by a subclass) plus fractional node coordinates (dof.py:199-478).

    ``do_frozen``: keep the fractional coordinates fixed (only the domain moves).
    ``freemask``: boolean vector over the cell variables; False entries stay at their
    initial values and are not part of x.
    """

    def __init__(self, mmf, gpos_rms=1e-5, dpos_rms=1e-3, grvecs_rms=1e-5, drvecs_rms=1e-3, do_frozen=False,
                 freemask=None):
        if freemask is not None:
            ok = isinstance(freemask, np.ndarray) and freemask.dtype == bool and freemask.ndim == 1
            if not ok or not freemask.any():
                raise TypeError("freemask must be a 1-D boolean array with at least one True entry.")
        self.th_gpos_rms = gpos_rms
        self.th_dpos_rms = dpos_rms
        self.th_grvecs_rms = grvecs_rms
        self.th_drvecs_rms = drvecs_rms
        self.do_frozen = do_frozen
        self.freemask = freemask
        DOF.__init__(self, mmf)

    # ------------------------------------------------------------ the cell variables
    @property
    def ncellvar(self):
        return len(self.domainvars0)

    @property
    def ncelldof(self):
        return self.ncellvar if self.freemask is None else int(self.freemask.sum())

    def _free(self):
        return np.ones(self.ncellvar, bool) if self.freemask is None else self.freemask

    def _cellvars_from_x(self, x):
        cellvars = self.domainvars0.copy()
        cellvars[self._free()] = x[: self.ncelldof]
        return cellvars

    def _get_initial_cellvars(self):
        raise NotImplementedError

    def _cellvars_to_rvecs(self, cellvars):
        raise NotImplementedError

    def _rvecs_jacobian(self, cellvars):
        """d(rvecs.ravel())/d(cellvars), one column per cell variable."""
        raise NotImplementedError

    def _get_celldofs_jacobian(self, x):
        """d(rvecs.ravel())/d(free cell variables)."""
        return self._rvecs_jacobian(self._cellvars_from_x(x))[:, self._free()]

    # ------------------------------------------------------------ DOF interface
    def _initial_vector(self):
        domain = self.mmf.system.domain
        if domain.nvec == 0:
            raise ValueError("Domain relaxation needs a periodic system (it has no domain vectors).")
        self.domainvars0 = np.asarray(self._get_initial_cellvars(), dtype=float)
        if self.freemask is not None and len(self.freemask) != self.ncellvar:
            raise TypeError("freemask has %d entries for %d cell variables." % (len(self.freemask), self.ncellvar))
        self._pos = np.array(self.mmf.system.pos, dtype=float)
        self._gpos = np.zeros_like(self._pos)
        self._vtens = np.zeros((3, 3))
        self._grvecs = np.zeros_like(np.asarray(domain.rvecs))
        self._rvecs = np.array(domain.rvecs, dtype=float)
        frac = self._pos @ domain._get_gvecs(full=True).T
        celldofs = self.domainvars0[self._free()]
        if self.do_frozen:
            self._frac0 = frac
            return celldofs.copy()
        return np.concatenate([celldofs, frac.ravel()])

    def _apply(self, x):
        self._rvecs = self._cellvars_to_rvecs(self._cellvars_from_x(x))
        self.mmf.update_rvecs(self._rvecs)
        frac = self._frac0 if self.do_frozen else x[self.ncelldof:].reshape(-1, 3)
        self._pos[:] = frac @ self.mmf.system.domain._get_rvecs(full=True)
        self.mmf.update_pos(self._pos)

    def _compute_with_gradient(self):
        self._gpos[:] = 0.0
        self._vtens[:] = 0.0
        return self.mmf.compute(self._gpos, self._vtens)

    def _gradient_vector(self, x):
        jac = self._get_celldofs_jacobian(x)
        grvecs = self.mmf.system.domain.gvecs @ self._vtens
        g = np.empty(self.ndof)
        g[: self.ncelldof] = grvecs.ravel() @ jac
        # the part of dE/d(rvecs) the cell variables can move along (for the convergence test)
        self._grvecs[:] = (jac @ (np.linalg.pinv(jac) @ grvecs.ravel())).reshape(self._grvecs.shape)
        if not self.do_frozen:
            g[self.ncelldof:] = (self._gpos @ self._rvecs.T).ravel()
        return g

    def _snapshot(self):
        return self._pos.copy(), self._rvecs.copy()

    def _measure(self, now, last, verdict):
        (pos, rvecs), (pos0, rvecs0) = now, last
        if not self.do_frozen:
            self.gpos_rms, self.gpos_max = _norms(self._gpos)
            verdict.add("gpos", self.gpos_rms, self.gpos_max, self.th_gpos_rms)
        self.dpos_rms, self.dpos_max = _norms(pos - pos0)
        verdict.add("dpos", self.dpos_rms, self.dpos_max, self.th_dpos_rms)
        self.grvecs_rms, self.grvecs_max = _norms(self._grvecs)
        verdict.add("grvecs", self.grvecs_rms, self.grvecs_max, self.th_grvecs_rms)
        self.drvecs_rms, self.drvecs_max = _norms(rvecs - rvecs0)
        verdict.add("drvecs", self.drvecs_rms, self.drvecs_max, self.th_drvecs_rms)


class FullCellDOF(BaseCellDOF):
    """All domain-vector components, divided by s = V^(1/nvec) to make them dimensionless."""

    def _get_initial_cellvars(self):
        domain = self.mmf.system.domain
        self._rvecs_scale = domain.volume ** (1.0 / domain.nvec)
        return np.asarray(domain.rvecs).ravel() / self._rvecs_scale

    def _cellvars_to_rvecs(self, cellvars):
        return cellvars.reshape(-1, 3) * self._rvecs_scale

    def _rvecs_jacobian(self, cellvars):
        return self._rvecs_scale * np.eye(self.ncellvar)


# (row, column) of the deformation entry that cell variable k sets, per number of domain vectors
_STRAIN_ENTRIES = {3: [(0, 0), (1, 1), (2, 2), (1, 2), (2, 0), (0, 1)], 2: [(0, 0), (1, 1), (0, 1)], 1: [(0, 0)]}


class StrainCellDOF(BaseCellDOF):
    """Symmetric deformation A of the initial domain: rvecs = A . rvecs_0.

    Cell variable k sets A[i, j] for diagonal entries and A[i, j] = A[j, i] = x_k / 2 for
    off-diagonal ones, (i, j) = (0,0), (1,1), (2,2), (1,2), (2,0), (0,1) in 3-D.
    """

    def _get_initial_cellvars(self):
        domain = self.mmf.system.domain
        self.rvecs0 = np.array(domain.rvecs, dtype=float)
        return np.array([1.0 if i == j else 0.0 for i, j in _STRAIN_ENTRIES[domain.nvec]])

    def _generator(self, k):
        """dA/dx_k."""
        n = self.rvecs0.shape[0]
        i, j = _STRAIN_ENTRIES[n][k]
        E = np.zeros((n, n))
        E[i, j] += 0.5
        E[j, i] += 0.5
        return E

    def _cellvars_to_rvecs(self, cellvars):
        A = sum(v * self._generator(k) for k, v in enumerate(cellvars))
        return A @ self.rvecs0

    def _rvecs_jacobian(self, cellvars):
        return np.stack([(self._generator(k) @ self.rvecs0).ravel() for k in range(self.ncellvar)], axis=1)
