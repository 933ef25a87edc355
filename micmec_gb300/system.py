"""``System``: a micromechanical system (nodes, cells, types, domain).

Same constructor, attributes and file I/O as the reference's ``System``
(micmec/system.py:38-370): CHK text files, HDF5 system groups (through any
``h5py.File``-like object; ``.h5`` file names use ``micmec_gb300.h5lite``, the h5py subset
this package needs, which writes and reads HDF5 files itself since h5py is not installed) and
XYZ snapshots.
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
        """Construct a system from a CHK or .h5 file (micmec/system.py:213-259)."""
        if fn.endswith(".h5"):
            from micmec_gb300 import h5lite

            with h5lite.File(fn, "r") as f:
                return cls.from_hdf5(f, **user_kwargs)
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

    @classmethod
    def from_hdf5(cls, f, **user_kwargs):
        """Construct a system from the ``system`` group of an h5py-like file (micmec/system.py:383-420)."""
        sgrp = f["system"]
        kwargs = {}
        for key in ("pos", "masses", "rvecs", "surrounding_cells", "surrounding_nodes", "boundary_nodes", "grid",
                    "types"):
            if key in sgrp:
                kwargs[key] = np.asarray(sgrp[key][:])
        params = {}
        if "params" in sgrp:
            for name, item in sgrp["params"].items():
                for key, ds in item.items():
                    params["%s/%s" % (name, key)] = np.asarray(ds[()]) if len(ds.shape) else ds[()]
        kwargs["params"] = params
        kwargs.update(user_kwargs)
        return cls(**kwargs)

    def to_hdf5(self, f):
        """Write the system to the ``system`` group of an h5py-like file (micmec/system.py:352-370);
        the topology, domain and parameters are written too, so that ``from_hdf5`` restores it."""
        if "system" in f:
            raise ValueError("The HDF5 file already contains a system description.")
        sgrp = f.create_group("system")
        sgrp.create_dataset("pos", data=self.pos)
        if self.masses is not None:
            sgrp.create_dataset("masses", data=self.masses)
        sgrp.create_dataset("rvecs", data=self.domain.rvecs)
        sgrp.create_dataset("surrounding_cells", data=self.surrounding_cells)
        sgrp.create_dataset("surrounding_nodes", data=self.surrounding_nodes)
        for key in ("boundary_nodes", "grid", "types"):
            value = getattr(self, key)
            if value is not None:
                sgrp.create_dataset(key, data=np.asarray(value))
        for key, value in (self.params or {}).items():
            sgrp.create_dataset("params/" + key, data=np.asarray(value))

    def to_file(self, fn):
        """Write the system to a CHK, .h5 or XYZ file (micmec/system.py:298-350)."""
        if fn.endswith(".h5"):
            from micmec_gb300 import h5lite

            with h5lite.File(fn, "w") as f:
                self.to_hdf5(f)
            return
        if fn.endswith(".xyz"):
            from micmec_gb300.sampling.trajectory import write_xyz_frame

            with open(fn, "w") as fh:
                write_xyz_frame(fh, str(self), self.pos)
            return
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
