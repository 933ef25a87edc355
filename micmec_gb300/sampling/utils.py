"""Initial velocities, momentum removal and degree-of-freedom counting.

Host-side restatements of micmec/sampling/utils.py:28-501 (Maxwell-Boltzmann
velocities, centre-of-mass and angular momentum removal, internal degrees of
freedom, domain symmetrisation, barostat velocities).
"""

import numpy as np

from micmec_gb300.units import boltzmann

__all__ = [
    "get_random_vel", "remove_com_moment", "remove_angular_moment", "clean_momenta", "inertia_tensor",
    "angular_moment", "angular_velocity", "rigid_body_angular_velocities", "get_ndof_internal_md",
    "domain_symmetrize", "get_random_vel_press", "get_ndof_baro", "stabilized_cholesky_decomp",
]


def get_random_vel(temp0, scalevel0, masses, select=None):
    """Maxwell-Boltzmann velocities at temp0, optionally rescaled to exactly temp0 (utils.py:28-65)."""
    if select is not None:
        masses = masses[select]
    vel0 = np.random.normal(0, 1, (len(masses), 3)) * np.sqrt(boltzmann * temp0 / masses).reshape(-1, 1)
    if scalevel0 and temp0 > 0:
        temp = np.mean(vel0**2 * masses.reshape(-1, 1)) / boltzmann
        vel0 *= np.sqrt(temp0 / temp)
    return vel0


def remove_com_moment(vel, masses):
    """Subtract the centre-of-mass velocity in place (utils.py:68-94)."""
    vel[:] -= np.dot(masses, vel) / np.sum(masses)


def inertia_tensor(pos, masses):
    """Inertia tensor of point masses about the origin."""
    r2 = (pos**2).sum(axis=1)
    itens = np.eye(3) * np.dot(masses, r2) - np.einsum("i,ij,ik->jk", masses, pos, pos)
    return itens


def angular_moment(pos, vel, masses):
    return np.einsum("i,ij->j", masses, np.cross(pos, vel))


def angular_velocity(amom, itens, epsilon=1e-10):
    """Solve I w = L on the eigenvectors of I whose eigenvalue exceeds epsilon (a pseudo-inverse
    for linear bodies; utils.py:229-270)."""
    evals, evecs = np.linalg.eigh(itens)
    keep = evals > epsilon
    return evecs[:, keep] @ ((evecs[:, keep].T @ amom) / evals[keep])


def rigid_body_angular_velocities(pos, avel):
    return np.cross(avel, pos)


def remove_angular_moment(pos, vel, masses):
    """Subtract the rigid rotation about the centre of mass in place (utils.py:97-139)."""
    pos = pos.copy()
    pos -= np.dot(masses, pos) / np.sum(masses)
    avel = angular_velocity(angular_moment(pos, vel, masses), inertia_tensor(pos, masses))
    vel[:] -= rigid_body_angular_velocities(pos, avel)


def clean_momenta(pos, vel, masses, domain):
    """Remove the external momenta that the boundary conditions allow (utils.py:142-174)."""
    remove_com_moment(vel, masses)
    if domain.nvec == 0:
        remove_angular_moment(pos, vel, masses)
    elif domain.nvec == 1:
        raise NotImplementedError


def get_ndof_internal_md(nnodes, nper):
    """3N - 6 (isolated), 3N - 4 (1-D periodic) or 3N - 3 (utils.py:322-343)."""
    if nper == 0:
        return 3 * nnodes - 6
    if nper == 1:
        return 3 * nnodes - 4
    return 3 * nnodes - 3


def domain_symmetrize(mmf, vector_lst=None, tensor_lst=None):
    """Rotate domain and positions so that the domain matrix is symmetric (utils.py:346-383)."""
    domain = mmf.system.domain.rvecs.copy()
    U, s, Vt = np.linalg.svd(domain)
    rot_mat = np.dot(Vt.T, U.T)
    mmf.update_rvecs(np.dot(domain, rot_mat))
    mmf.update_pos(np.dot(mmf.system.pos, rot_mat))
    new_vectors = [np.dot(v, rot_mat) for v in (vector_lst or [])]
    new_tensors = [np.dot(np.dot(rot_mat.T, t), rot_mat) for t in (tensor_lst or [])]
    return new_vectors, new_tensors


def get_random_vel_press(mass, temp):
    """Symmetric random barostat velocity tensor (utils.py:450-475)."""
    rand = np.random.normal(0, np.sqrt(mass * boltzmann * temp), (3, 3)) / mass
    vel_press = np.tril(rand) + np.tril(rand, -1).T
    off = ~np.eye(3, dtype=bool)
    vel_press[off] /= np.sqrt(2)
    return vel_press


def get_ndof_baro(dim, anisotropic, vol_constraint):
    """Degrees of freedom of the domain fluctuations (utils.py:478-501)."""
    ndof = dim * (dim + 1) // 2 if anisotropic else 1
    if vol_constraint:
        ndof -= 1
    if ndof == 0:
        raise AssertionError("Isotropic barostat called with a volume constraint.")
    return ndof


def stabilized_cholesky_decomp(mat):
    """L with L L^T = mat for symmetric mat, negative pivots clipped to zero (utils.py:504-528)."""
    if np.all(np.linalg.eigvals(mat) > 0):
        return np.linalg.cholesky(mat)
    n = mat.shape[0]
    D = np.zeros(n)
    L = np.eye(n)
    for i in range(n):
        for j in range(i):
            val = mat[i, j] - np.sum(L[i, :j] * L[j, :j] * D[:j])
            L[i, j] = val / D[j] if abs(D[j]) > 1e-12 else 0.0
        D[i] = mat[i, i] - np.sum(L[i, :i] ** 2 * D[:i])
    return L * np.sqrt(D.clip(min=0))
