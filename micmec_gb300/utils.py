"""System construction: lattice topology, cell types and Voigt helpers.

Host-side restatement of micmec/utils.py (``neighbor_cells``, ``neighbor_nodes``,
``Grid``, ``build_system``, ``build_type``) and of the Voigt maps of
micmec/analysis/tensor.py:74-227. The reference builds the topology with a
node search inside a per-cell loop (utils.py:202-218, O(cells x nodes));
here every table is built with array operations, so 256^3 lattices build in
seconds. Orderings and accumulation orders are kept: nodes and cells are
enumerated lexicographically with the last grid index fastest, corner k of a
cell is ``neighbor_nodes[k]``, and each node's mass sums 1/8 of its cells'
type masses in increasing cell order (utils.py:217).
"""

import numpy as np

from micmec_gb300.units import kelvin

__all__ = [
    "build_system", "build_type", "neighbor_cells", "neighbor_nodes", "Grid",
    "voigt", "voigt_inv", "VOIGT",
]

# Each node has at most eight neighboring cells (micmec/utils.py:32-41).
neighbor_cells = [
    (0, 0, 0), (-1, 0, 0), (0, -1, 0), (0, 0, -1),
    (-1, -1, 0), (-1, 0, -1), (0, -1, -1), (-1, -1, -1),
]
# Each cell always has eight neighboring nodes (micmec/utils.py:43-52).
neighbor_nodes = [
    (0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1),
    (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1),
]
_CORNERS = np.array(neighbor_nodes, dtype=np.int64)

VOIGT = {0: (0, 0), 1: (1, 1), 2: (2, 2), 3: (1, 2), 4: (0, 2), 5: (0, 1)}


def _pbc_list(pbc):
    if pbc is None or pbc is True:
        return [True, True, True]
    if pbc is False:
        return [False, False, False]
    return [bool(p) for p in pbc]


class Grid(object):
    """Lattice bookkeeping for a 3-D grid of cell types (0 = vacancy).

    Same properties as micmec/utils.py:55-161: ``nodes``, ``nnodes``,
    ``boundary_nodes``, ``cells``, ``ncells``, ``types``; plus array forms
    ``node_coords`` (nnodes, 3) and ``cell_coords`` (ncells, 3).
    """

    def __init__(self, grid, pbc=None):
        self.grid = np.asarray(grid)
        self.pbc = _pbc_list(pbc)
        self.nx, self.ny, self.nz = self.grid.shape
        self.nx_nodes = self.nx + 1 - self.pbc[0]
        self.ny_nodes = self.ny + 1 - self.pbc[1]
        self.nz_nodes = self.nz + 1 - self.pbc[2]
        self._node_coords = None
        self._cell_coords = None

    @property
    def shape_nodes(self):
        return (self.nx_nodes, self.ny_nodes, self.nz_nodes)

    @property
    def node_coords(self):
        if self._node_coords is None:
            nn = np.array(self.shape_nodes)
            kk, ll, mm = np.meshgrid(*(np.arange(n) for n in nn), indexing="ij")
            coords = np.stack([kk.ravel(), ll.ravel(), mm.ravel()], axis=1)
            keep = np.zeros(len(coords), dtype=bool)
            shape = np.array(self.grid.shape)
            occupied = self.grid != 0
            for c in neighbor_cells:
                cell = coords + np.array(c)
                ok = np.ones(len(coords), dtype=bool)
                for d in range(3):
                    if self.pbc[d]:
                        cell[:, d] %= shape[d]
                    else:
                        ok &= (cell[:, d] >= 0) & (cell[:, d] < shape[d])
                cl = np.where(ok[:, None], cell, 0)
                keep |= ok & occupied[cl[:, 0], cl[:, 1], cl[:, 2]]
            self._node_coords = coords[keep]
        return self._node_coords

    @property
    def nodes(self):
        return [tuple(int(v) for v in row) for row in self.node_coords]

    @property
    def nnodes(self):
        return len(self.node_coords)

    @property
    def boundary_nodes(self):
        c = self.node_coords
        nn = np.array(self.shape_nodes)
        b = ((c == 0) | (c == nn - 1)).any(axis=1)
        return list(np.nonzero(b)[0])

    @property
    def cell_coords(self):
        if self._cell_coords is None:
            self._cell_coords = np.argwhere(self.grid != 0)
        return self._cell_coords

    @property
    def cells(self):
        return [tuple(int(v) for v in row) for row in self.cell_coords]

    @property
    def ncells(self):
        return len(self.cell_coords)

    @property
    def types(self):
        c = self.cell_coords
        return list(self.grid[c[:, 0], c[:, 1], c[:, 2]])

    def node_index(self):
        """Dense (nx_nodes, ny_nodes, nz_nodes) map from node coordinates to index (-1 = absent)."""
        idx = -np.ones(self.shape_nodes, dtype=np.int64)
        c = self.node_coords
        idx[c[:, 0], c[:, 1], c[:, 2]] = np.arange(len(c))
        return idx


def build_system(data, grid, pbc=None, device=False):
    """Micromechanical system as a ``dict`` ready for ``dump_chk`` (micmec/utils.py:164-263).

    ``device=True`` builds the topology, masses and positions on the GPU
    (``mm_build_topology``; the same tables, bit for bit) and copies them back."""
    grid = np.asarray(grid)
    if device:
        return _build_system_device(data, grid, pbc)
    g = Grid(grid, pbc=pbc)
    nodes = g.node_coords
    cells = g.cell_coords
    nn = np.array(g.shape_nodes)
    node_idx = g.node_index()

    corner_nodes = (cells[:, None, :] + _CORNERS[None, :, :]) % nn  # (M, 8, 3)
    surrounding_nodes = node_idx[corner_nodes[..., 0], corner_nodes[..., 1], corner_nodes[..., 2]]
    if (surrounding_nodes < 0).any():
        raise ValueError("Inconsistent grid: a cell corner has no node.")
    ncells = len(cells)
    surrounding_cells = -np.ones((len(nodes), 8), dtype=np.int64)
    corner_id = np.broadcast_to(np.arange(8), surrounding_nodes.shape)
    cell_id = np.broadcast_to(np.arange(ncells)[:, None], surrounding_nodes.shape)
    surrounding_cells[surrounding_nodes.ravel(), corner_id.ravel()] = cell_id.ravel()

    types = grid[cells[:, 0], cells[:, 1], cells[:, 2]]
    type_mass = {k: float(v["mass"]) for k, v in data.items()}
    cell_mass = np.array([0.125 * type_mass[int(t)] for t in types], dtype=np.float64)
    masses = np.zeros(len(nodes))
    # cell-major order: each node accumulates in increasing cell index
    np.add.at(masses, surrounding_nodes.ravel(), np.repeat(cell_mass, 8))

    dx, dy, dz = _majority_cell_size(data, grid)
    pos = nodes.astype(np.float64) * np.array([dx, dy, dz])

    rvecs = []
    if g.pbc[0]:
        rvecs.append([g.nx * dx, 0.0, 0.0])
    if g.pbc[1]:
        rvecs.append([0.0, g.ny * dy, 0.0])
    if g.pbc[2]:
        rvecs.append([0.0, 0.0, g.nz * dz])
    rvecs = np.array(rvecs, dtype=np.float64).reshape(-1, 3)

    output = {
        "pos": pos,
        "rvecs": rvecs,
        "types": types,
        "grid": grid,
        "pbc": g.pbc,
        "surrounding_cells": surrounding_cells,
        "surrounding_nodes": surrounding_nodes,
        "boundary_nodes": g.boundary_nodes,
        "masses": masses,
    }
    for type_idx, type_data in data.items():
        for key, value in type_data.items():
            output[f"type{type_idx}/{key}"] = value
    return output


def _majority_cell_size(data, grid):
    counts = np.bincount(np.array(grid.ravel(), dtype=np.int64))[1:]
    maj = int(np.argmax(counts)) + 1
    return np.diag(np.asarray(data[maj]["cell"][0])).astype(np.float64)


def _build_system_device(data, grid, pbc):
    import torch

    from micmec_gb300 import _native as nat

    if grid.ndim != 3 or grid.min() < 0:
        raise ValueError("grid must be a 3-D array of type ids >= 0")
    nx, ny, nz = grid.shape
    flags = _pbc_list(pbc)
    nn = [n + 1 - int(p) for n, p in zip(grid.shape, flags)]
    ncg, nng = nx * ny * nz, nn[0] * nn[1] * nn[2]
    ntype_ids = int(grid.max()) + 1
    type_mass = np.zeros(ntype_ids)
    for k, v in data.items():
        if int(k) < ntype_ids:
            type_mass[int(k)] = float(v["mass"])
    dx, dy, dz = _majority_cell_size(data, grid)
    dev = torch.device("cuda", torch.cuda.current_device())
    g_d = torch.from_numpy(np.ascontiguousarray(grid, dtype=np.int32)).to(dev)
    snodes = torch.empty((ncg, 8), dtype=torch.int64, device=dev)
    scells = torch.empty((nng, 8), dtype=torch.int64, device=dev)
    masses = torch.empty(nng, dtype=torch.float64, device=dev)
    pos = torch.empty((nng, 3), dtype=torch.float64, device=dev)
    types = torch.empty(ncg, dtype=torch.int32, device=dev)
    boundary = torch.empty(nng, dtype=torch.uint8, device=dev)
    counts = np.zeros(2, dtype=np.int64)
    pbc_a = np.array(flags, dtype=np.int32)
    size = np.array([dx, dy, dz], dtype=np.float64)
    nat.check(nat.lib().mm_build_topology(g_d.data_ptr(), nx, ny, nz, pbc_a.ctypes.data, type_mass.ctypes.data,
                                          ntype_ids, size.ctypes.data, snodes.data_ptr(), scells.data_ptr(),
                                          masses.data_ptr(), pos.data_ptr(), types.data_ptr(), boundary.data_ptr(),
                                          counts.ctypes.data, torch.cuda.current_stream().cuda_stream),
              "mm_build_topology")
    M, N = int(counts[0]), int(counts[1])
    rvecs = []
    if flags[0]:
        rvecs.append([nx * dx, 0.0, 0.0])
    if flags[1]:
        rvecs.append([0.0, ny * dy, 0.0])
    if flags[2]:
        rvecs.append([0.0, 0.0, nz * dz])
    output = {
        "pos": pos[:N].cpu().numpy(),
        "rvecs": np.array(rvecs, dtype=np.float64).reshape(-1, 3),
        "types": types[:M].cpu().numpy().astype(grid.dtype),
        "grid": grid,
        "pbc": flags,
        "surrounding_cells": scells[:N].cpu().numpy(),
        "surrounding_nodes": snodes[:M].cpu().numpy(),
        "boundary_nodes": list(np.nonzero(boundary[:N].cpu().numpy())[0]),
        "masses": masses[:N].cpu().numpy(),
    }
    for type_idx, type_data in data.items():
        for key, value in type_data.items():
            output[f"type{type_idx}/{key}"] = value
    return output


def build_type(material, mass, cell0, elasticity0, free_energy=None, effective_temp=None, topology=None):
    """A cell type ``dict`` (micmec/utils.py:266-329)."""
    if type(cell0) is not list:
        cell0 = [cell0]
    if type(elasticity0) is not list:
        elasticity0 = [elasticity0]
    if topology is None:
        topology = "UNKNOWN"
    if effective_temp is None:
        effective_temp = 300 * kelvin
    if free_energy is None:
        free_energy = [0.0] * len(cell0)
    if type(free_energy) is not list:
        free_energy = [free_energy]
    output = {
        "material": material,
        "topology": topology,
        "mass": mass,
        "cell": cell0,
        "elasticity": elasticity0,
        "free_energy": free_energy,
        "effective_temp": effective_temp,
    }
    if len(cell0) == len(elasticity0) and len(cell0) == len(free_energy):
        return output
    raise ValueError("Inconsistent number of metastable states.")


def voigt(tensor, mode=None):
    """(3,3,3,3) -> (6,6) or (3,3) -> (6,) in Voigt order 00,11,22,12,02,01 (tensor.py:96-149)."""
    tensor = np.asarray(tensor)
    if tensor.shape == (3, 3, 3, 3):
        m = np.zeros((6, 6))
        for p in range(6):
            for q in range(6):
                m[p, q] = tensor[VOIGT[p] + VOIGT[q]]
                if mode is None or mode == "compliance":
                    m[p, q] *= (2.0 if p >= 3 else 1.0) * (2.0 if q >= 3 else 1.0)
                elif mode != "elasticity":
                    raise ValueError("Method `voigt` did not receive valid input for keyword `mode`.")
        return m
    if tensor.shape == (3, 3):
        col = np.array([tensor[VOIGT[p]] for p in range(6)], dtype=np.float64)
        if mode is None or mode == "strain":
            col[3:] *= 2.0
        elif mode != "stress":
            raise ValueError("Method `voigt` did not receive valid input for keyword `mode`.")
        return col
    raise ValueError("Method `voigt` did not receive valid input for `tensor`.")


def _vidx(i, j):
    a, b = sorted((i, j))
    for k, v in VOIGT.items():
        if v == (a, b):
            return k


def voigt_inv(matrix, mode=None):
    """(6,6) -> (3,3,3,3) or (6,) -> (3,3) (tensor.py:152-227)."""
    matrix = np.asarray(matrix, dtype=np.float64)
    if matrix.shape == (6, 6):
        t = np.zeros((3, 3, 3, 3))
        for idx in np.ndindex(3, 3, 3, 3):
            p = _vidx(idx[0], idx[1])
            q = _vidx(idx[2], idx[3])
            t[idx] = matrix[p, q]
            if mode is None or mode == "compliance":
                t[idx] *= (0.5 if p >= 3 else 1.0) * (0.5 if q >= 3 else 1.0)
            elif mode != "elasticity":
                raise ValueError("Method `voigt_inv` did not receive valid input for keyword `mode`.")
        return t
    if matrix.shape == (6,):
        t = np.zeros((3, 3))
        for idx in np.ndindex(3, 3):
            p = _vidx(*idx)
            t[idx] = matrix[p]
            if mode is None or mode == "strain":
                if p >= 3:
                    t[idx] *= 0.5
            elif mode != "stress":
                raise ValueError("Method `voigt_inv` did not receive valid input for keyword `mode`.")
        return t
    raise ValueError("Method `voigt_inv` did not receive valid input for `matrix`.")
