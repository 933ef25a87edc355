"""Geometry and domain optimisers (interface of micmec/sampling/opt.py:52-443).

``QNOptimizer`` restates the reference's self-contained quasi-Newton method:
SR1 Hessian updates with a trust radius and a ridge-regularised step in the
Hessian eigenbasis (opt.py:258-443). ``CGOptimizer`` is a nonlinear conjugate
gradient (Polak-Ribiere+, restarted when the direction is not a descent
direction) with a secant (Newton-on-the-derivative) line search; the reference
delegates the same method to the third-party ``molmod.minimizer`` (molmod 1.4.8,
not available here), so its iterates are not bit-comparable to the reference's.
Every energy/gradient evaluation is one GPU force call.
"""

import time

import numpy as np
from numpy.linalg import eigh

from micmec_gb300.sampling.iterative import (
    Iterative, AttributeStateItem, PosStateItem, VolumeStateItem, DomainStateItem, EPotContribStateItem, Hook,
)

__all__ = ["OptScreenLog", "BaseOptimizer", "CGOptimizer", "BFGSHessianModel", "SR1HessianModel", "QNOptimizer",
           "solve_trust_radius"]


class OptScreenLog(Hook):
    def __init__(self, start=0, step=1, verbose=False):
        Hook.__init__(self, start, step)
        self.time0 = None
        self.verbose = verbose

    def __call__(self, iterative):
        if not self.verbose:
            return
        if self.time0 is None:
            self.time0 = time.time()
            print("counter  Conv.val.  N           Worst     Energy   Walltime")
        print("%7i % 10.3e %2i %15s % 14.8e %10.1f" % (
            iterative.counter, iterative.dof.conv_val, iterative.dof.conv_count, iterative.dof.conv_worst,
            iterative.epot, time.time() - self.time0))


class BaseOptimizer(Iterative):
    default_state = [AttributeStateItem("counter"), AttributeStateItem("epot"), PosStateItem(), VolumeStateItem(),
                     DomainStateItem(), EPotContribStateItem()]
    log_name = "XXOPT"

    def __init__(self, dof, state=None, hooks=None, counter0=0):
        self.dof = dof
        Iterative.__init__(self, dof.mmf, state, hooks, counter0)

    def _add_default_hooks(self):
        if not any(isinstance(hook, OptScreenLog) for hook in self.hooks):
            self.hooks.append(OptScreenLog())

    def fun(self, x, do_gradient=False):
        if do_gradient:
            self.epot, gx = self.dof.fun(x, True)
            return self.epot, gx
        self.epot = self.dof.fun(x, False)
        return self.epot

    def initialize(self):
        self.dof.check_convergence()
        Iterative.initialize(self)

    def propagate(self):
        self.dof.check_convergence()
        Iterative.propagate(self)
        return self.dof.converged


class CGOptimizer(BaseOptimizer):
    """Nonlinear conjugate gradient with a secant line search."""

    log_name = "CGOPT"

    def __init__(self, dof, state=None, hooks=None, counter0=0, max_line=8, device=False):
        self.max_line = max_line
        self.device = device
        BaseOptimizer.__init__(self, dof, state, hooks, counter0)

    # ------------------------------------------------------------ device route
    def _device_kind(self):
        """None (positions), "strain" or "full" when the batched device relaxation applies, else False.

        It applies to a force field of one ``ForcePartMechanical`` (plus optionally one
        ``ForcePartPressure``) on a full periodic lattice, with a CartesianDOF without
        selection, or a StrainCellDOF / FullCellDOF without freemask or frozen positions."""
        from micmec_gb300.pes.mmff import ForcePartMechanical, ForcePartPressure
        from micmec_gb300.sampling.dof import CartesianDOF, FullCellDOF, StrainCellDOF

        if not self.device:
            return False
        parts = getattr(self.mmf, "parts", [])
        mech = [p for p in parts if isinstance(p, ForcePartMechanical)]
        if len(mech) != 1 or any(not isinstance(p, (ForcePartMechanical, ForcePartPressure)) for p in parts):
            return False
        if sum(isinstance(p, ForcePartPressure) for p in parts) > 1:
            return False
        s, part = self.mmf.system, mech[0]
        grid = np.asarray(s.grid)
        if not part.pbc or (grid == 0).any() or s.nnodes != grid.size:
            return False
        dof = self.dof
        if type(dof) is CartesianDOF and dof.select is None:
            return None
        if type(dof) in (StrainCellDOF, FullCellDOF) and dof.freemask is None and not dof.do_frozen:
            return "strain" if type(dof) is StrainCellDOF else "full"
        return False

    def run(self, nsteps=None):
        kind = self._device_kind() if nsteps is not None else False
        if kind is False:
            return BaseOptimizer.run(self, nsteps)
        return self._run_device(int(nsteps), kind)

    def _run_device(self, nsteps, kind):
        """All iterations in the batched CG kernel (mm_batch_relax / mm_batch_relax_cell). The
        convergence test is the kernel's: max |gpos| below 3 gpos_rms (the DOF's gpos_max
        criterion, dof.py:155-193) and, for cell DOFs, the residual stress below the stress
        that the grvecs_rms threshold allows on this domain."""
        from micmec_gb300.batch import BatchSystems
        from micmec_gb300.pes.mmff import ForcePartMechanical, ForcePartPressure

        s = self.mmf.system
        part = [p for p in self.mmf.parts if isinstance(p, ForcePartMechanical)][0]
        press = sum(p.pext for p in self.mmf.parts if isinstance(p, ForcePartPressure))
        b = BatchSystems([s], model=part.model, precision=part.precision)
        b.set_state([s.pos], None, [s.domain.rvecs])
        gtol = 3.0 * self.dof.th_gpos_rms
        if kind is None:
            gmax, iters = b.relax(max_iter=nsteps, gtol=gtol)
        else:
            rv = np.asarray(s.domain.rvecs)
            stol = self.dof.th_grvecs_rms * np.linalg.norm(rv, axis=1).max() / s.domain.volume
            gmax, iters = b.relax(max_iter=nsteps, gtol=gtol, cell=kind, press=press, stress_tol=stol)
        pos, _, rvecs = b.get_state()
        if kind is not None:
            self.mmf.update_rvecs(rvecs[0])
        self.mmf.update_pos(pos[0])
        self.counter += int(iters[0])
        self.epot = self.mmf.compute()
        self.dof.converged = bool(iters[0] < nsteps)
        self.call_hooks()
        self.finalize()
        return self.dof.converged

    def initialize(self):
        self.x = self.dof.x0.copy()
        self.f, self.g = self.fun(self.x, True)
        self.d = -self.g
        self.alpha = None
        BaseOptimizer.initialize(self)

    def _line_search(self):
        d = self.d
        s0 = float(np.dot(self.g, d))
        if s0 >= 0:
            d = self.d = -self.g
            s0 = float(np.dot(self.g, d))
        dn = np.linalg.norm(d)
        alpha = self.alpha if self.alpha else min(1.0, 0.1 / max(dn, 1e-300)) * 1.0
        best = None
        for _ in range(self.max_line):
            x1 = self.x + alpha * d
            f1, g1 = self.fun(x1, True)
            s1 = float(np.dot(g1, d))
            if f1 <= self.f + 1e-4 * alpha * s0 and (best is None or f1 < best[1]):
                best = (x1, f1, g1, alpha)
            denom = s1 - s0
            if denom > 0:  # the directional derivative grew: secant root of phi'
                a_new = alpha * (-s0) / denom
                if best is not None and abs(s1) <= 0.1 * abs(s0):
                    break
                alpha = min(max(a_new, 0.1 * alpha), 10.0 * alpha)
            else:
                if best is not None:
                    break
                alpha *= 0.5 if f1 > self.f else 2.0
        if best is None:
            return False
        self.x, f_new, g_new, self.alpha = best
        g_old = self.g
        self.f, self.g = f_new, g_new
        beta = max(0.0, float(np.dot(g_new, g_new - g_old)) / max(float(np.dot(g_old, g_old)), 1e-300))
        self.d = -g_new + beta * self.d
        # leave the force field at the accepted point
        self.fun(self.x, True)
        return True

    def propagate(self):
        if not self._line_search():
            return True
        return BaseOptimizer.propagate(self)


class HessianModel(object):
    def __init__(self, ndof, hessian0=None):
        self.ndof = ndof
        if hessian0 is None:
            self.hessian = np.identity(ndof, float)
        else:
            self.hessian = hessian0.copy()
            if self.hessian.shape != (ndof, ndof):
                raise TypeError("Incorrect shape of the initial hessian in quasi-newton method.")

    def get_spectrum(self):
        return eigh(self.hessian)


class BFGSHessianModel(HessianModel):
    def update(self, dx, dg):
        tmp = np.dot(self.hessian, dx)
        hmax = abs(self.hessian).max()
        denom1 = np.dot(dx, tmp)
        if hmax * denom1 <= 1e-5 * abs(tmp).max() ** 2:
            return False
        denom2 = np.dot(dg, dx)
        if hmax * denom2 <= 1e-5 * abs(dg).max() ** 2:
            return False
        self.hessian -= np.outer(tmp, tmp) / denom1
        self.hessian += np.outer(dg, dg) / denom2
        return True


class SR1HessianModel(HessianModel):
    def update(self, dx, dg):
        tmp = dg - np.dot(self.hessian, dx)
        denom = np.dot(tmp, dx)
        if abs(denom) > 1e-5 * np.linalg.norm(dx) * np.linalg.norm(tmp):
            self.hessian += np.outer(tmp, tmp) / denom
            return True
        return False


class QNOptimizer(BaseOptimizer):
    """Quasi-Newton optimiser with SR1 updates and a trust radius (opt.py:258-393)."""

    log_name = "QNOPT"

    def __init__(self, dof, state=None, hooks=None, counter0=0, trust_radius=1.0, small_radius=1e-5,
                 too_small_radius=1e-10, hessian0=None):
        self.x_old = dof.x0
        self.hessian = SR1HessianModel(len(dof.x0), hessian0)
        self.trust_radius = trust_radius
        self.initial_trust_radius = trust_radius
        self.small_radius = small_radius
        self.too_small_radius = too_small_radius
        BaseOptimizer.__init__(self, dof, state, hooks, counter0)

    def initialize(self):
        self.f_old, self.g_old = self.fun(self.dof.x0, True)
        self.x, self.f, self.g = self.make_step()
        BaseOptimizer.initialize(self)

    def propagate(self):
        if not self.hessian.update(self.x - self.x_old, self.g - self.g_old):
            self.hessian = SR1HessianModel(len(self.x))
            self.trust_radius = self.initial_trust_radius
        self.x_old, self.f_old, self.g_old = self.x, self.f, self.g
        self.x, self.f, self.g = self.make_step()
        return BaseOptimizer.propagate(self)

    def make_step(self):
        evals, evecs = self.hessian.get_spectrum()
        grad_eigen = np.dot(evecs.T, self.g_old)
        while True:
            delta_eigen = solve_trust_radius(grad_eigen, evals, self.trust_radius)
            radius = np.linalg.norm(delta_eigen)
            x = self.x_old + np.dot(evecs, delta_eigen)
            f, g = self.fun(x, True)
            must_shrink = f - self.f_old > 0
            if self.trust_radius < self.small_radius and np.linalg.norm(g) - np.linalg.norm(self.g_old) > 0:
                must_shrink = True
            if must_shrink:
                self.trust_radius *= 0.5
                while self.trust_radius >= radius:
                    self.trust_radius *= 0.5
                if self.trust_radius < self.too_small_radius:
                    raise RuntimeError("The trust radius becomes too small. Is the potential energy surface smooth?")
            else:
                if self.trust_radius < self.initial_trust_radius:
                    self.trust_radius *= 2.0
                return x, f, g


def solve_trust_radius(grad, evals, radius, threshold=1e-5):
    """Step in the Hessian eigenbasis with norm ``radius`` (opt.py:396-443)."""
    if evals.min() > 0:
        step = -grad / evals
        if np.linalg.norm(step) <= radius:
            return step

    def compute_step(ridge):
        return -grad / (evals + ridge)

    def compute_error(ridge):
        return np.linalg.norm(compute_step(ridge)) - radius

    ridge_min = -evals.min()

    def find_edge(alpha, sign):
        while True:
            ridge = ridge_min + alpha
            error = compute_error(ridge)
            if sign * error < 0:
                return ridge, error
            alpha = alpha * 2 if sign > 0 else alpha / 2

    a = find_edge(min(1e1, abs(evals.max())), -1)
    b = find_edge(max(1e-5, abs(ridge_min)), 1)
    error = np.inf
    c = a
    while abs(error) > radius * threshold:
        ridge = (a[1] * a[0] - b[1] * b[0]) / (a[1] - b[1])
        error = compute_error(ridge)
        c = ridge, error
        if error > 0 and a[1] > 0:
            a = c
        else:
            b = c
    return compute_step(c[0])
