"""Trajectory writers (interface of micmec/sampling/trajectory.py:31-128).

``HDF5Writer(f)`` appends every state item of the iterative to growing datasets under
``trajectory/`` of ``f`` and writes the system once under ``system/`` (trajectory.py:31-85);
``f`` is an ``h5py.File``-like object, e.g. ``micmec_gb300.h5lite.File``. ``XYZWriter``
writes node positions in angstrom as caesium atoms, one frame per call
(trajectory.py:88-128). Both only read the state: the device MD paths may run the next
steps while they write.
"""

import numpy as np

from micmec_gb300.sampling.iterative import Hook
from micmec_gb300.units import angstrom

__all__ = ["BaseHDF5Writer", "HDF5Writer", "XYZWriter"]


class BaseHDF5Writer(Hook):
    modifies_state = False

    def __init__(self, f, start=0, step=1):
        self.f = f
        Hook.__init__(self, start, step)

    def __call__(self, iterative):
        if "trajectory" not in self.f:
            self.init_trajectory(iterative)
        tgrp = self.f["trajectory"]
        row = min(tgrp[key].shape[0] for key in iterative.state if key in tgrp.keys())
        for key, item in iterative.state.items():
            if item.value is None:
                continue
            if len(item.shape) > 0 and min(item.shape) == 0:
                continue
            ds = tgrp[key]
            if ds.shape[0] <= row:
                ds.resize(row + 1, axis=0)
            ds[row] = item.value

    def dump_system(self, system, grp):
        system.to_hdf5(grp)

    def init_trajectory(self, iterative):
        tgrp = self.f.create_group("trajectory")
        for key, item in iterative.state.items():
            if item.value is None:
                continue
            if len(item.shape) > 0 and min(item.shape) == 0:
                continue
            tgrp.create_dataset(key, (0,) + item.shape, maxshape=(None,) + item.shape, dtype=item.dtype)
            for name, value in item.iter_attrs(iterative):
                tgrp.attrs[name] = value


class HDF5Writer(BaseHDF5Writer):
    def __call__(self, iterative):
        if "system" not in self.f:
            self.dump_system(iterative.mmf.system, self.f)
        BaseHDF5Writer.__call__(self, iterative)


def write_xyz_frame(fh, title, pos):
    """One XYZ frame: node count, title, then 'Cs x y z' rows in angstrom."""
    fh.write("%8i\n%s\n" % (len(pos), title))
    np.savetxt(fh, np.asarray(pos) / angstrom, fmt="Cs %15.10f %15.10f %15.10f")


class XYZWriter(Hook):
    modifies_state = False

    def __init__(self, fn_xyz, select=None, start=0, step=1):
        self.fn_xyz = fn_xyz
        self.select = select
        self._fh = None
        Hook.__init__(self, start, step)

    def __call__(self, iterative):
        if self._fh is None:
            self._fh = open(self.fn_xyz, "w")
        pos = iterative.mmf.system.pos if self.select is None else iterative.mmf.system.pos[self.select]
        write_xyz_frame(self._fh, "%7i E_pot = %.10f     " % (iterative.counter, iterative.epot), pos)
        self._fh.flush()

    def close(self):
        if self._fh is not None:
            self._fh.close()
            self._fh = None
