"""Differentiable FP64 PyTorch restatement of the force evaluation (test infrastructure only).

Same mathematics as ``oracle/mmff.py`` (which follows micmec/pes/mmff.py:326-403,
nanocell.py:40-132, nanocell_original.py:46-132), written with torch operations so
that autograd gives exact first and second derivatives with respect to positions,
elasticity (21 Voigt components per type and state), rest matrices and free
energies. Used by the tests as the FP64 reference gradient for the adjoint kernel.
"""

import numpy as np
import torch

from oracle.mmff import BOLTZMANN, MULT, cell_shifts

_VPAIRS = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]


def _voigt_tensor(c21):
    iu = np.triu_indices(6)
    m = torch.zeros(c21.shape[:-1] + (6, 6), dtype=c21.dtype)
    m[..., iu[0], iu[1]] = c21
    m[..., iu[1], iu[0]] = c21
    idx = np.zeros((3, 3), dtype=np.int64)
    for p, (i, j) in enumerate(_VPAIRS):
        idx[i, j] = idx[j, i] = p
    v = torch.as_tensor(idx)
    return m[..., v[:, :, None, None], v[None, None, :, :]]


def energy(pos, rvecs, grid, surrounding_nodes, types, type_ids, nstates, c21, h0, df, temp, model="nanocell"):
    """Total energy as a differentiable torch scalar.

    pos (N,3) torch; c21 (T,4,21), h0 (T,4,3,3), df (T,4) torch; types: cell types (ids);
    type_ids: sorted ids defining the T axis; temp: effective temperatures (T,).
    """
    sn = np.asarray(surrounding_nodes, dtype=np.int64)
    shifts = torch.as_tensor(cell_shifts(grid, sn, True), dtype=torch.float64)
    rv = torch.as_tensor(np.asarray(rvecs), dtype=torch.float64)
    r0 = pos[sn[:, 0]]
    verts = r0[:, None, :] + (pos[sn] - r0[:, None, :] + shifts @ rv)
    mult = torch.as_tensor(MULT, dtype=torch.float64)
    mats = torch.einsum("adn,cnj->cadj", mult, verts)
    C = _voigt_tensor(c21)
    types = np.asarray(types).astype(np.int64)
    total = torch.zeros((), dtype=torch.float64)
    for t, k in enumerate(type_ids):
        sel = np.nonzero(types == k)[0]
        if len(sel) == 0:
            continue
        Es = []
        for s in range(int(nstates[t])):
            hinv = torch.linalg.inv(h0[t, s])
            det = torch.linalg.det(h0[t, s])
            m = mats[sel]
            if model == "original":
                mat = 0.125 * m.sum(dim=1)
                F = torch.einsum("cji,kj->cik", mat, hinv)
                eps = 0.5 * (torch.einsum("cji,cjk->cik", F, F) - torch.eye(3, dtype=torch.float64))
                E = 0.5 * torch.einsum("cij,ijkl,ckl->c", eps, C[t, s], eps) * det
            else:
                F = torch.einsum("caji,kj->caik", m, hinv)
                eps = 0.5 * (torch.einsum("caji,cajk->caik", F, F) - torch.eye(3, dtype=torch.float64))
                E = 0.125 * 0.5 * torch.einsum("caij,ijkl,cakl->c", eps, C[t, s], eps) * det
            Es.append(E + df[t, s])
        Es = torch.stack(Es)
        kT = BOLTZMANN * float(temp[t])
        total = total + (-kT * torch.logsumexp(-Es / kT, dim=0)).sum()
    return total
