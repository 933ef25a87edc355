"""``System``: a micromechanical system (nodes, cells, types, domain).

Same constructor, attributes and CHK I/O as the reference's ``System``
(micmec/system.py:38-316). HDF5 and XYZ output are left out: they need h5py /
molmod, which are not part of this build.
"""

import numpy as np

from micmec_gb300.chk import load_chk, dump_chk
from micmec_gb300.pes.ext import Domain

__all__ = ["System"]


class System(object):
    """Construct a micromechanical system (arguments as micmec/system.py:85-110)."""

    def __init__(self, pos, masses, rvecs, surrounding_cells, surrounding_nodes, boundary_nodes=None, grid=None,
                 types=None, params=None):
        self.masses = np.asarray(masses, dtype=np.float64)
        self.pos = np.array(pos, dtype=np.float64)
        self.domain = Domain(np.asarray(rvecs, dtype=np.float64).reshape(-1, 3))
        self.grid = None if grid is None else np.asarray(grid)
        self.types = None if types is None else np.asarray(types)
        self.params = params
        self.surrounding_cells = np.asarray(surrounding_cells)
        self.surrounding_nodes = np.asarray(surrounding_nodes)
        self.boundary_nodes = boundary_nodes
        self.nnodes = len(self.surrounding_cells)
        self.ncells = len(self.surrounding_nodes)

    def update_params(self, new_params, type_=1):
        for key, val in new_params.items():
            self.params.update({f"type{int(type_)}/{key}": val})

    @classmethod
    def from_file(cls, fn, **user_kwargs):
        """Construct a system from a CHK file (micmec/system.py:213-259)."""
        if not fn.endswith(".chk"):
            raise IOError('Cannot read from file "%s".' % fn)
        allowed = ["pos", "masses", "rvecs", "surrounding_cells", "surrounding_nodes", "boundary_nodes", "grid",
                   "types"]
        kwargs, params = {}, {}
        for key, value in load_chk(fn).items():
            if key in allowed:
                kwargs[key] = value
            if "type" in key and key != "types":
                params[key] = value
        kwargs["params"] = params
        kwargs.update(user_kwargs)
        return cls(**kwargs)

    @classmethod
    def from_dict(cls, data):
        """Construct a system from a ``build_system`` dictionary."""
        keys = ["pos", "masses", "rvecs", "surrounding_cells", "surrounding_nodes", "boundary_nodes", "grid", "types"]
        kw = {k: data[k] for k in keys if k in data}
        kw["params"] = {k: v for k, v in data.items() if "/" in k}
        return cls(**kw)

    def to_file(self, fn):
        """Write the system to a CHK file."""
        if not fn.endswith(".chk"):
            raise NotImplementedError("The extension of %s does not correspond to any known format." % fn)
        output = {
            "pos": self.pos,
            "masses": self.masses,
            "rvecs": self.domain.rvecs,
            "surrounding_cells": self.surrounding_cells,
            "surrounding_nodes": self.surrounding_nodes,
            "boundary_nodes": self.boundary_nodes,
            "grid": self.grid,
            "types": self.types,
        }
        output.update(self.params)
        dump_chk(fn, {k: v for k, v in output.items() if v is not None})
