"""CPU oracle for the MicMec force evaluation (test infrastructure only).

A vectorised FP64 NumPy restatement of the reference's per-cell loop. It is
imported only by ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py``; the product never calls it.

It follows, step by step:

* cell vertices with the minimum-image shift, micmec/pes/mmff.py:334-371
  (``delta``: ``pos[j] - pos[i]`` then ``+ rvecs . mic``, then ``r0 + delta``);
* the topological minimum image of ``get_mic``, micmec/pes/mmff.py:258-286,
  restated as "corner offset o_d of a cell at grid index k_d wraps when
  k_d + o_d == n_d" (equivalent for lattices with n_d >= 2 nodes per
  periodic direction; the dense (N, N, 3) table is never built);
* corner matrices from the multiplicator, micmec/pes/nanocell_utils.py:32-75,
  whose row d of corner a is the edge along d that touches corner a,
  v[a | bit d] - v[a & ~bit d], with corners numbered as micmec/utils.py:43-52;
* the "original" single averaged matrix model, micmec/pes/nanocell_original.py:46-132,
  and the eight-representation model, micmec/pes/nanocell.py:40-132;
* the stress as ``C_ijkl eps_kl`` contracted with the symmetric strain
  derivative, exactly as the reference's analytic gradient does
  (nanocell.py:124-130), so that slightly asymmetric elasticity tensors read
  from CHK files give the reference's numbers;
* the multi-state -kT log-sum-exp combination, micmec/pes/mmff.py:377-398;
* the per-node gather in corner order, micmec/pes/mmff.py:303-318, and the
  virial ``einsum('ijk,ijl->kl', gpos_cells, verts_cells)``, mmff.py:320-323.
"""

import numpy as np

BOLTZMANN = 1.3806505e-23 / 4.35974381e-18  # Hartree per kelvin (molmod value)

# corner offsets (micmec/utils.py:43-52)
CORNERS = np.array(
    [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)],
    dtype=np.int64,
)


def _corner_index(o):
    for i, c in enumerate(CORNERS):
        if tuple(c) == tuple(o):
            return i
    raise KeyError(o)


def make_multiplicator():
    """(8, 3, 8) integer table: row d of corner matrix a as a combination of the 8 vertices."""
    mult = np.zeros((8, 3, 8), dtype=np.int64)
    for a in range(8):
        for d in range(3):
            hi = CORNERS[a].copy()
            lo = CORNERS[a].copy()
            hi[d] = 1
            lo[d] = 0
            mult[a, d, _corner_index(hi)] += 1
            mult[a, d, _corner_index(lo)] -= 1
    return mult


MULT = make_multiplicator()
MULT_AVG = MULT.mean(axis=0)  # (3, 8): derivative of the averaged matrix, 1/8 sum_a


# ---------------------------------------------------------------- topology


def grid_nodes(grid, pbc=True):
    """Node lattice coordinates in the reference's order (micmec/utils.py:113-136)."""
    grid = np.asarray(grid)
    nx, ny, nz = grid.shape
    p = np.array([pbc] * 3 if isinstance(pbc, (bool, np.bool_)) else pbc, dtype=bool)
    nn = np.array([nx, ny, nz]) + 1 - p.astype(int)
    kk, ll, mm = np.meshgrid(np.arange(nn[0]), np.arange(nn[1]), np.arange(nn[2]), indexing="ij")
    coords = np.stack([kk.ravel(), ll.ravel(), mm.ravel()], axis=1)
    keep = np.zeros(len(coords), dtype=bool)
    for c in CORNERS:
        cell = coords - c
        ok = np.ones(len(coords), dtype=bool)
        for d, n in enumerate((nx, ny, nz)):
            if p[d]:
                cell[:, d] %= n
            else:
                ok &= (cell[:, d] >= 0) & (cell[:, d] < n)
        cl = np.where(ok[:, None], cell, 0)
        keep |= ok & (grid[cl[:, 0], cl[:, 1], cl[:, 2]] != 0)
    return coords[keep], nn


def grid_cells(grid):
    """Cell lattice coordinates and types in the reference's order (micmec/utils.py:149-161)."""
    grid = np.asarray(grid)
    idx = np.argwhere(grid != 0)
    return idx, grid[idx[:, 0], idx[:, 1], idx[:, 2]]


def cell_shifts(grid, surrounding_nodes, pbc=True):
    """Integer image shifts (M, 8, 3) of each cell corner relative to corner 0."""
    cells, _ = grid_cells(grid)
    nodes, nn = grid_nodes(grid, pbc)
    sn = np.asarray(surrounding_nodes)
    # consistency check of the tables against the lattice
    expect = (cells[:, None, :] + CORNERS[None, :, :]) % nn
    if sn.shape != (len(cells), 8) or not np.array_equal(nodes[sn], expect):
        raise ValueError("surrounding_nodes does not match the grid's lattice")
    wrap = (cells[:, None, :] + CORNERS[None, :, :]) >= nn
    if not pbc:
        wrap[:] = False
    return wrap.astype(np.int64)


# ---------------------------------------------------------------- parameters


def type_tables(params):
    """Per type: (effective_temp, [free energies], [h0], [C]) from ``type{k}/...`` keys.

    Mirrors the parameter filter of micmec/pes/mmff.py:218-242.
    """
    out = {}
    for key, item in params.items():
        head, _, field = key.partition("/")
        if not head.startswith("type"):
            continue
        k = int(head[4:])
        entry = out.setdefault(k, {})
        entry[field] = item
    tables = {}
    for k, e in out.items():
        if "cell" not in e:
            continue
        tables[k] = (
            float(e.get("effective_temp", 300.0)),
            [float(x) for x in np.atleast_1d(e["free_energy"])],
            [np.asarray(h, dtype=np.float64) for h in e["cell"]],
            [np.asarray(c, dtype=np.float64) for c in e["elasticity"]],
        )
    return tables


# ---------------------------------------------------------------- per state


def _state_energy_grad(mats, h0, C0, model):
    """Energy (M,) and corner-matrix gradient of one state for a batch of cells.

    ``mats`` is (M, 8, 3, 3): the eight corner matrices of every cell.
    Returns (E, dE/dmats) with dE/dmats shaped like ``mats``.
    """
    h0inv = np.linalg.inv(h0)
    h0det = np.linalg.det(h0)
    eye = np.eye(3)
    if model == "original":
        mat = 0.125 * mats.sum(axis=1)  # (M,3,3)
        F = np.einsum("cji,kj->cik", mat, h0inv)
        eps = 0.5 * (np.einsum("cji,cjk->cik", F, F) - eye)
        sig = np.einsum("ijkl,ckl->cij", C0, eps)
        ssym = 0.5 * (sig + np.swapaxes(sig, 1, 2))
        E = 0.5 * np.einsum("cij,cij->c", eps, sig) * h0det
        GF = np.einsum("cik,ckl->cil", F, ssym) * h0det  # dE/dF (reference form)
        GM = np.einsum("cik,kj->cji", GF, h0inv)  # dE/dM[j, i]
        return E, np.repeat(0.125 * GM[:, None], 8, axis=1)
    F = np.einsum("caji,kj->caik", mats, h0inv)
    eps = 0.5 * (np.einsum("caji,cajk->caik", F, F) - eye)
    sig = np.einsum("ijkl,cakl->caij", C0, eps)
    ssym = 0.5 * (sig + np.swapaxes(sig, 2, 3))
    E = 0.125 * 0.5 * np.einsum("caij,caij->c", eps, sig) * h0det
    GF = 0.125 * np.einsum("caik,cakl->cail", F, ssym) * h0det
    GM = np.einsum("caik,kj->caji", GF, h0inv)
    return E, GM


def deformation(pos, rvecs, grid, surrounding_nodes, types, params, model="original", pbc=None, cells=None,
                shifts=None):
    """Per-cell energies (M,), corner gradients (M, 8, 3) and vertices (M, 8, 3).

    ``cells`` (optional index array) restricts the evaluation to those cells;
    ``shifts`` (optional, from ``cell_shifts``) skips recomputing the image shifts.
    """
    pos = np.asarray(pos, dtype=np.float64)
    rvecs = np.asarray(rvecs, dtype=np.float64).reshape(-1, 3)
    if pbc is None:
        pbc = rvecs.shape[0] == 3
    sn = np.asarray(surrounding_nodes, dtype=np.int64)
    types = np.asarray(types).astype(np.int64)
    if shifts is None:
        shifts = cell_shifts(grid, sn, pbc)
    if cells is not None:
        sn, types, shifts = sn[cells], types[cells], shifts[cells]
    r0 = pos[sn[:, 0]]
    dvec = pos[sn] - r0[:, None, :]
    if pbc:
        dvec = dvec + (
            rvecs[0] * shifts[..., 0:1] + rvecs[1] * shifts[..., 1:2] + rvecs[2] * shifts[..., 2:3]
        )
    verts = r0[:, None, :] + dvec
    mats = np.einsum("adn,cnj->cadj", MULT.astype(np.float64), verts)  # (M,8,3,3)

    tables = type_tables(params)
    M = len(sn)
    epot = np.zeros(M)
    gcells = np.zeros((M, 8, 3))
    for t in np.unique(types):
        sel = np.nonzero(types == t)[0]
        temp, efree, h0s, C0s = tables[int(t)]
        Es, Gs = [], []
        for s in range(len(h0s)):
            E, GM = _state_energy_grad(mats[sel], h0s[s], C0s[s], model)
            Es.append(E + efree[s])
            # corner gradient: sum over reps a and rows d of mult[a,d,n] * GM[a,d,:]
            Gs.append(np.einsum("adn,cadj->cnj", MULT.astype(np.float64), GM))
        Es = np.array(Es)  # (S, m)
        Emin = Es.min(axis=0)
        w = np.exp(-(Es - Emin) / (BOLTZMANN * temp))
        wsum = w.sum(axis=0)
        epot[sel] = Emin - temp * BOLTZMANN * np.log(wsum)
        wn = w / wsum
        g = np.zeros((len(sel), 8, 3))
        for s in range(len(h0s)):
            g += wn[s][:, None, None] * Gs[s]
        gcells[sel] = g
    return epot, gcells, verts


def gather_gpos(gcells, surrounding_cells):
    """Per-node gradient: sum over incident cells in corner order, skipping -1."""
    sc = np.asarray(surrounding_cells, dtype=np.int64)
    gpos = np.zeros((len(sc), 3))
    for k in range(8):
        ok = sc[:, k] >= 0
        gpos[ok] += gcells[sc[ok, k], k]
    return gpos


def compute(system, model="original"):
    """Energy, gpos (N, 3) and vtens (3, 3) for a dict-like system description.

    ``system`` needs keys pos, rvecs, grid, surrounding_nodes, surrounding_cells,
    types and params (the ``type{k}/...`` entries).
    """
    epot_cells, gcells, verts = deformation(
        system["pos"], system["rvecs"], system["grid"], system["surrounding_nodes"],
        system["types"], system["params"], model,
    )
    gpos = gather_gpos(gcells, system["surrounding_cells"])
    vtens = np.einsum("ijk,ijl->kl", gcells, verts)
    return float(np.sum(epot_cells)), gpos, vtens
