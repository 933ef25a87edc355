"""Seeded synthetic lattices with the shapes of the standard MicMec workloads.

Two cell types modelled on the UiO-66 'fcu' crystal and its 'reo' defect phase:

* fcu: cubic rest cell h0 = 20.7 A * I, cubic elasticity C11/C12/C44 =
  60/30/15 GPa, cell mass 6656 amu;
* reo: h0 = 20.3 A * I, elasticity 0.6 x fcu, mass 0.6832 x fcu (the reo/fcu
  mass ratio of the reference's data/type_1x1x1_{reo,fcu}_atomic.pickle).

With ``nstates=2`` each type gets two metastable states whose rest cells are
h0 * (1 + 0.015) with free energy 0 and h0 * (1 - 0.015) with free energy
2 kJ/mol, combined at an effective temperature of 300 K.

Elasticity tensors are built from Voigt matrices with ``voigt_inv(...,
mode="elasticity")`` as the reference's tools do (micmec/analysis/tensor.py:152-202).
"""

import numpy as np

from micmec_gb300 import units
from micmec_gb300.utils import build_system, build_type, voigt_inv

__all__ = [
    "cubic_elasticity", "standard_types", "defect_grid", "make_lattice",
    "displace", "FCU_MASS", "REO_MASS",
]

FCU_MASS = 6656.0 * units.amu
REO_MASS = FCU_MASS * (8289953.673067445 / 12133589.4468533)
FCU_H0 = 20.7 * units.angstrom
REO_H0 = 20.3 * units.angstrom


def cubic_elasticity(c11, c12, c44):
    m = np.zeros((6, 6))
    m[:3, :3] = c12
    m[0, 0] = m[1, 1] = m[2, 2] = c11
    m[3, 3] = m[4, 4] = m[5, 5] = c44
    return voigt_inv(m, mode="elasticity")


def _type(name, mass, a, C, nstates):
    if nstates == 1:
        cells = [a * np.eye(3)]
        efree = [0.0]
    elif nstates == 2:
        cells = [a * (1.0 + 0.015) * np.eye(3), a * (1.0 - 0.015) * np.eye(3)]
        efree = [0.0, 2.0 * units.kjmol]
    else:
        raise ValueError("nstates must be 1 or 2")
    return build_type(
        name, mass, cells, [C.copy() for _ in cells], free_energy=efree,
        effective_temp=300.0 * units.kelvin, topology=name,
    )


def standard_types(nstates=1, with_reo=True):
    gpa = units.gigapascal
    C = cubic_elasticity(60.0 * gpa, 30.0 * gpa, 15.0 * gpa)
    data = {1: _type("fcu", FCU_MASS, FCU_H0, C, nstates)}
    if with_reo:
        data[2] = _type("reo", REO_MASS, REO_H0, 0.6 * C, nstates)
    return data


def defect_grid(n, fraction, rng, clustered=False):
    """(n, n, n) grid of types: 1 (fcu) with round(fraction * n^3) cells set to 2 (reo).

    Uniform: the defect cells are a random subset drawn with ``rng.permutation``.
    Clustered: face-connected clusters of 1-8 cells, each grown by a random walk of
    ``size - 1`` face steps from a random seed cell (size ~ U{1..8}), until the defect
    count is reached. Clusters are grown in rounds of many walkers at once (vectorised);
    the last round is trimmed to the exact count.
    """
    shape = (n, n, n) if np.isscalar(n) else tuple(n)
    total = int(np.prod(shape))
    ndef = int(round(fraction * total))
    grid = np.ones(total, dtype=np.int64)
    if not clustered:
        grid[rng.permutation(total)[:ndef]] = 2
        return grid.reshape(shape)
    shp = np.array(shape)
    steps = np.array([(1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)])
    flat = grid
    placed = 0
    while placed < ndef:
        nwalk = max(1, (ndef - placed) // 4)
        size = rng.integers(1, 9, nwalk)
        cur = rng.integers(0, shp, size=(nwalk, 3))
        cells = []
        for k in range(8):
            alive = size > k
            idx = np.ravel_multi_index(cur[alive].T, shape)
            cells.append(np.stack([np.nonzero(alive)[0], np.full(alive.sum(), k), idx], axis=1))
            cur = (cur + steps[rng.integers(0, 6, nwalk)]) % shp
        order = np.concatenate(cells)
        order = order[np.lexsort((order[:, 1], order[:, 0]))]  # walker by walker, step by step
        idx = order[:, 2]
        new = idx[flat[idx] != 2]
        _, first = np.unique(new, return_index=True)
        new = new[np.sort(first)][: ndef - placed]
        flat[new] = 2
        placed += len(new)
    return grid.reshape(shape)


def make_lattice(grid, nstates=1, pbc=True, device=False):
    """System dict (as ``build_system``) for a type grid with the standard types
    (``device=True``: topology built on the GPU)."""
    grid = np.asarray(grid)
    data = standard_types(nstates=nstates, with_reo=bool((grid == 2).any()))
    if 2 not in data:
        data = {1: data[1]}
    return build_system(data, grid, pbc=pbc, device=device)


def displace(pos, sigma, rng):
    """Gaussian node displacements with standard deviation ``sigma`` (bohr)."""
    return pos + rng.normal(0.0, sigma, pos.shape)
