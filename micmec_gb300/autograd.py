"""Differentiation: gradients with respect to the model parameters, through forces and trajectories.

``MicMecParameters`` holds differentiable per-(type, state) parameters as torch
tensors: the 21 independent Voigt components of each elasticity tensor, the 3x3
rest matrix h0 and the state free energy. ``energy_and_gradient(pos, params)`` is
a ``torch.autograd.Function``: forward runs the GPU force evaluation, backward runs
the hand-written FP64 adjoint kernel (``mm_adjoint``) once, with the incoming
gradient of the forces as tangent direction. That gives, in one pass,
dL/dpos = gE dE/dx + H lam and dL/dtheta = gE dE/dtheta + d/dtheta (lam . dE/dx),
with lam = dL/d(dE/dx), so losses on energies, forces and trajectories built from
them differentiate exactly (to FP64 rounding).

``verlet_trajectory`` integrates velocity Verlet with torch operations on top of
that Function, recomputing segments of ``checkpoint_every`` steps in the backward
pass (torch.utils.checkpoint) instead of storing every step.

``relaxed_stress`` gives the stress at relaxed positions, differentiable in the
parameters through the relaxation (implicit differentiation: one Hessian solve by
conjugate gradients on adjoint Hessian-vector products per backward pass), for losses
on relaxed stress-strain curves.

Elasticity in Voigt notation C_v (6x6, symmetric, order 00,11,22,12,02,01, as
micmec/analysis/tensor.py:96-149 with mode="elasticity"); the kernel's stress map is
A = C_v diag(1,1,1,2,2,2).
"""

import numpy as np
import torch

from micmec_gb300 import _native as nat

__all__ = ["MicMecParameters", "energy_and_gradient", "verlet_trajectory", "voigt21_to_tensor", "stress",
           "relaxed_stress", "relaxed_stress_gradient"]

_IU = np.triu_indices(6)
_VPAIRS = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]


def _voigt_index():
    idx = np.zeros((3, 3), dtype=np.int64)
    for p, (i, j) in enumerate(_VPAIRS):
        idx[i, j] = idx[j, i] = p
    return idx


_VIDX = _voigt_index()


def voigt21_to_matrix(c21):
    """(..., 21) upper-triangle Voigt components -> (..., 6, 6) symmetric matrix."""
    shape = c21.shape[:-1]
    m = torch.zeros(shape + (6, 6), dtype=c21.dtype, device=c21.device)
    iu = torch.as_tensor(_IU[0]), torch.as_tensor(_IU[1])
    m[..., iu[0], iu[1]] = c21
    m[..., iu[1], iu[0]] = c21
    return m


def voigt21_to_tensor(c21):
    """(..., 21) -> (..., 3, 3, 3, 3) elasticity tensor (voigt_inv, mode="elasticity")."""
    m = voigt21_to_matrix(c21)
    v = torch.as_tensor(_VIDX)
    return m[..., v[:, :, None, None], v[None, None, :, :]]


class MicMecParameters(object):
    """Differentiable parameters of the cell types of one ``ForcePartMechanical``."""

    def __init__(self, part):
        from micmec_gb300.pes.mmff import type_parameters

        self.part = part
        nstates, h0, C, df, temp = type_parameters(part.system.params, part.type_ids)
        self.nstates = nstates
        self.temp = np.ascontiguousarray(temp)
        T = len(part.type_ids)
        c21 = np.zeros((T, 4, 21))
        for t in range(T):
            for s in range(nstates[t]):
                Ct = C[4 * t + s].reshape(3, 3, 3, 3)
                M = np.array([[Ct[_VPAIRS[p] + _VPAIRS[q]] for q in range(6)] for p in range(6)])
                c21[t, s] = M[_IU]
        self.c21 = torch.tensor(c21, dtype=torch.float64, requires_grad=True)
        self.h0 = torch.tensor(h0.reshape(T, 4, 3, 3), dtype=torch.float64, requires_grad=True)
        self.free_energy = torch.tensor(df.reshape(T, 4), dtype=torch.float64, requires_grad=True)

    def tensors(self):
        return self.c21, self.h0, self.free_energy

    def native_tables(self, c21, h0, df):
        """(C (T*4, 81), h0 (T*4, 9), free energies (T*4,)) in the layout of the C ABI's
        parameter tables; unused state slots repeat state 0."""
        T = c21.shape[0]
        C = voigt21_to_tensor(c21.detach()).cpu().numpy().reshape(T * 4, 81).copy()
        H = h0.detach().cpu().numpy().reshape(T * 4, 9).copy()
        D = df.detach().cpu().numpy().reshape(T * 4).copy()
        for t in range(T):
            for s in range(self.nstates[t], 4):
                C[4 * t + s] = C[4 * t]
                H[4 * t + s] = H[4 * t]
                D[4 * t + s] = D[4 * t]
        return tuple(np.ascontiguousarray(a) for a in (C, H, D))

    def upload(self, c21, h0, df):
        """Push parameter values into the native handle (skipped when the handle already holds
        exactly these tables, as along a trajectory whose steps all use the same values)."""
        C, H, D = self.native_tables(c21, h0, df)
        last = getattr(self, "_uploaded", None)
        if last is not None and last[0] == self.part.handle.value and all(
                np.array_equal(a, b) for a, b in zip(last[1:], (C, H, D))):
            return
        nat.check(nat.lib().mm_set_params(self.part.handle, H.ctypes.data, C.ctypes.data, D.ctypes.data,
                                          self.temp.ctypes.data), "mm_set_params")
        self._uploaded = (self.part.handle.value, C, H, D)


def _adjoint(part, pos, lam, dlattice=None, with_virial=False):
    dev = pos.device
    N = pos.shape[0]
    T = len(part.type_ids)
    energy = torch.zeros(2, dtype=torch.float64, device=dev)
    gpos = torch.zeros((N, 3), dtype=torch.float64, device=dev)
    hvp = torch.zeros((N, 3), dtype=torch.float64, device=dev) if lam is not None else None
    vt = torch.zeros(18, dtype=torch.float64, device=dev)
    pg = torch.zeros((T, 4, 46, 2), dtype=torch.float64, device=dev)
    dl = None if dlattice is None else np.ascontiguousarray(dlattice, dtype=np.float64)
    lam_c = None if lam is None else lam.contiguous()
    st = nat.lib().mm_adjoint(part.handle, pos.contiguous().data_ptr(), nat.ptr(lam_c), nat.ptr(dl),
                              energy.data_ptr(), gpos.data_ptr(), nat.ptr(hvp), vt.data_ptr(), pg.data_ptr(),
                              torch.cuda.current_stream().cuda_stream)
    nat.check(st, "mm_adjoint")
    if with_virial:
        return energy, gpos, hvp, pg, vt
    return energy, gpos, hvp, pg


def _hvp(part, pos, lam):
    """H lam (H = d2E/dx2 at pos) by one adjoint evaluation that forms nothing else: no
    gradient, virial or parameter derivatives are written. The result lives in a buffer
    kept with the part and is overwritten by the next call."""
    buf = getattr(part, "_hvp_buf", None)
    if buf is None or buf[1].shape != pos.shape or buf[1].device != pos.device:
        buf = (torch.zeros(2, dtype=torch.float64, device=pos.device), torch.empty_like(pos))
        part._hvp_buf = buf
    energy, hvp = buf
    st = nat.lib().mm_adjoint(part.handle, pos.contiguous().data_ptr(), lam.contiguous().data_ptr(), None,
                              energy.data_ptr(), None, hvp.data_ptr(), None, None,
                              torch.cuda.current_stream().cuda_stream)
    nat.check(st, "mm_adjoint")
    return hvp


def _slots_to_params(slot, params, device):
    """dL/d(raw slot) (T, 4, 46): [dE/dA (36), dE/dh0 (9), dE/dF (1)] -> (c21, h0, free energy),
    formed on the slot tensor's device (no host round trip)."""
    sdev = slot.device
    dA = slot[..., :36].reshape(slot.shape[:2] + (6, 6))
    w = torch.tensor([1.0, 1.0, 1.0, 2.0, 2.0, 2.0], dtype=torch.float64, device=sdev)
    dCv = dA * w  # A = C_v diag(w)  ->  dL/dC_v[p, q] = dL/dA[p, q] w_q
    i0, i1 = torch.as_tensor(_IU[0], device=sdev), torch.as_tensor(_IU[1], device=sdev)
    dC21 = dCv[..., i0, i1] + torch.where(i0 != i1, dCv[..., i1, i0], torch.zeros_like(dCv[..., i0, i1]))
    dh0 = slot[..., 36:45].reshape(slot.shape[:2] + (3, 3))
    ddf = slot[..., 45]
    mask = torch.zeros(slot.shape[:2], dtype=torch.float64)
    for t, n in enumerate(params.nstates):
        mask[t, :n] = 1.0
    mask = mask.to(sdev)
    return (dC21 * mask[..., None]).to(device), (dh0 * mask[..., None, None]).to(device), (ddf * mask).to(device)


class _EnergyGrad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pos, c21, h0, df, params):
        params.upload(c21, h0, df)
        energy, gpos, _, _ = _adjoint(params.part, pos.detach(), None)
        ctx.params = params
        ctx.save_for_backward(pos.detach(), c21.detach(), h0.detach(), df.detach())
        return energy[0].clone(), gpos

    @staticmethod
    def backward(ctx, gE, gG):
        pos, c21, h0, df = ctx.saved_tensors
        params = ctx.params
        params.upload(c21, h0, df)
        lam = gG if gG is not None else torch.zeros_like(pos)
        gE = gE if gE is not None else torch.zeros((), dtype=torch.float64, device=pos.device)
        energy, gpos, hvp, pg = _adjoint(params.part, pos, lam)
        grad_pos = gE * gpos + hvp
        # dL/dtheta per slot: gE * value + tangent, kept on the device
        slot = gE * pg[..., 0] + pg[..., 1]  # (T, 4, 46)
        dC21, dh0, ddf = _slots_to_params(slot, params, c21.device)
        return grad_pos, dC21, dh0, ddf, None


def _hessian_solve(part, pos, rhs, tol=1e-11, maxiter=5000):
    """mu with H mu = rhs (H = d2E/dx2 at pos, FP64 adjoint products) by conjugate
    gradients on the translation-free subspace (rhs and iterates have zero mean)."""

    def H(p):
        return _hvp(part, pos, p)

    b = rhs - rhs.mean(dim=0)
    x = torch.zeros_like(b)
    r = b.clone()
    p = r.clone()
    rr = (r * r).sum()
    b2 = float((b * b).sum())
    if b2 == 0.0:
        return x
    # the scalars stay device tensors; convergence is read back every `check` iterations only
    check = 8
    for it in range(maxiter):
        Ap = H(p)
        Ap = Ap - Ap.mean(dim=0)
        alpha = rr / (p * Ap).sum()
        x = x + alpha * p
        r = r - alpha * Ap
        rr_new = (r * r).sum()
        if it % check == check - 1 and float(rr_new) <= tol * tol * b2:
            break
        p = r + (rr_new / rr) * p
        rr = rr_new
    return x


def stress(pos, params):
    """Stress tensor sigma = vtens / V (3x3, FP64) at device positions pos."""
    part = params.part
    params.upload(params.c21, params.h0, params.free_energy)
    vt = _adjoint(part, pos.detach(), None, with_virial=True)[4]
    return vt[:9].reshape(3, 3) / float(part.system.domain.volume)


def relaxed_stress_gradient(pos, params, w, tol=1e-11):
    """Stress at relaxed positions and the total parameter derivative of s = sum(w * sigma).

    pos: device (N, 3) positions at an energy minimum for the current parameters (the
    caller relaxes them); w: (3, 3) weights (e.g. dLoss/dsigma). The relaxed positions
    move with the parameters, x*(theta) with g(x*, theta) = 0, so
    ds/dtheta = ds/dtheta|_x - mu . dg/dtheta with H mu = ds/dx (implicit differentiation).
    The homogeneous deformation pos -> pos (I + eps), L -> L (I + eps) with eps = w^T is the
    tangent whose energy derivative is sum(w * vtens); in the kernel's variables
    (u = pos - X(L), L) it is (u eps, L eps). One adjoint evaluation along that tangent
    gives V ds/dtheta|_x and the Hessian part of V ds/dx; conjugate gradients with
    adjoint Hessian products give mu; a last adjoint evaluation with lam = mu gives
    mu . dg/dtheta. Returns (sigma (3, 3) tensor, d/dc21, d/dh0, d/dfree_energy).
    """
    part = params.part
    params.upload(params.c21, params.h0, params.free_energy)
    dev = pos.device
    V = float(part.system.domain.volume)
    L = part.lattice_matrix()
    eps = np.asarray(w, dtype=np.float64).T
    D = L @ eps
    nc = torch.tensor(np.asarray(part.node_coords, dtype=np.float64), device=dev)
    epst = torch.tensor(eps, device=dev)
    pos = pos.detach()
    lam = pos @ epst - nc @ torch.tensor(D, device=dev)
    _, g, hvp, pg, vt = _adjoint(part, pos, lam, D, with_virial=True)
    sigma = vt[:9].reshape(3, 3) / V
    q = (hvp + g @ epst.T) / V  # ds/dx: Hessian-tangent part + derivative of the tangent u eps
    mu = _hessian_solve(part, pos, q, tol=tol)
    pg_mu = _adjoint(part, pos, mu)[3]
    slot = pg[..., 1] / V - pg_mu[..., 1]
    dC21, dh0, ddf = _slots_to_params(slot, params, params.c21.device)
    return sigma, dC21, dh0, ddf


class _RelaxedStress(torch.autograd.Function):
    @staticmethod
    def forward(ctx, c21, h0, df, params, pos):
        params.upload(c21, h0, df)
        vt = _adjoint(params.part, pos.detach(), None, with_virial=True)[4]
        ctx.params = params
        ctx.save_for_backward(pos.detach())
        return vt[:9].reshape(3, 3) / float(params.part.system.domain.volume)

    @staticmethod
    def backward(ctx, gs):
        pos, = ctx.saved_tensors
        _, dC21, dh0, ddf = relaxed_stress_gradient(pos, ctx.params, gs.detach().cpu().numpy())
        return dC21, dh0, ddf, None, None


def relaxed_stress(pos, params):
    """Stress (3, 3) at relaxed device positions ``pos``, differentiable in the parameters
    through the relaxation (the caller relaxes ``pos`` for the current parameters)."""
    c21, h0, df = params.tensors()
    return _RelaxedStress.apply(c21, h0, df, params, pos)


def energy_and_gradient(pos, params):
    """(E, dE/dx) at device positions ``pos`` (N,3) for ``params`` (differentiable in both)."""
    c21, h0, df = params.tensors()
    return _EnergyGrad.apply(pos, c21, h0, df, params)


def verlet_trajectory(pos0, vel0, masses, params, timestep, nsteps, checkpoint_every=20):
    """Velocity-Verlet trajectory (micmec/sampling/verlet.py:140-166) as torch operations.

    Returns the list of gradients dE/dx at every step (index 0 = initial positions) and
    the final (pos, vel). Segments of ``checkpoint_every`` steps are recomputed in the
    backward pass.
    """
    from torch.utils.checkpoint import checkpoint

    inv_m = (1.0 / masses).reshape(-1, 1)
    dt = float(timestep)

    def segment(x, v, g, k):
        grads = []
        for _ in range(k):
            v = v - 0.5 * dt * g * inv_m
            x = x + dt * v
            _, g = energy_and_gradient(x, params)
            v = v - 0.5 * dt * g * inv_m
            grads.append(g)
        return (x, v, g) + tuple(grads)

    _, g = energy_and_gradient(pos0, params)
    x, v = pos0, vel0
    out = [g]
    done = 0
    while done < nsteps:
        k = min(checkpoint_every, nsteps - done)
        res = checkpoint(segment, x, v, g, k, use_reentrant=False)
        x, v, g = res[0], res[1], res[2]
        out.extend(res[3:])
        done += k
    return out, x, v
