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
    """Records the iterative's state items, one row per call, in growing datasets of the
    ``trajectory`` group of ``f`` (created at the first call, with the items' attributes on
    the group). Items without a value or with an empty axis are not recorded."""

    modifies_state = False

    def __init__(self, f, start=0, step=1):
        self.f = f
        self._keys = None  # recorded state items, fixed when the group is found or made
        Hook.__init__(self, start, step)

    @staticmethod
    def _recordable(item):
        return item.value is not None and not (len(item.shape) > 0 and min(item.shape) == 0)

    def _group(self, iterative):
        if "trajectory" not in self.f:
            self.init_trajectory(iterative)
        grp = self.f["trajectory"]
        if self._keys is None:
            self._keys = [key for key in iterative.state if key in grp.keys()]
        return grp

    def __call__(self, iterative):
        grp = self._group(iterative)
        # the frame's row: the shortest dataset's length, so that a frame an earlier run left
        # half written (some datasets one row longer) is written again in place
        row = min(grp[key].shape[0] for key in self._keys)
        for key in self._keys:
            item = iterative.state[key]
            if not self._recordable(item):
                continue
            ds = grp[key]
            if ds.shape[0] == row:
                ds.resize(row + 1, axis=0)
            ds[row] = item.value

    def dump_system(self, system, grp):
        system.to_hdf5(grp)

    def init_trajectory(self, iterative):
        grp = self.f.create_group("trajectory")
        for key, item in iterative.state.items():
            if self._recordable(item):
                grp.create_dataset(key, (0,) + item.shape, maxshape=(None,) + item.shape, dtype=item.dtype)
                for name, value in item.iter_attrs(iterative):
                    grp.attrs[name] = value


class HDF5Writer(BaseHDF5Writer):
    """Also writes the system once, under ``system`` (System.to_hdf5)."""

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
