"""A small stand-in for the part of h5py that trajectories and systems use.

h5py is not installed with this package. ``File`` offers the interface that the
reference's ``HDF5Writer`` (micmec/sampling/trajectory.py:31-85) and
``System.to_hdf5`` / ``from_hdf5`` (micmec/system.py:262-370) use: nested groups,
``create_group``, ``create_dataset(name, shape, maxshape, dtype)`` or ``(name, data=...)``,
``in``, ``[...]`` lookups with "a/b" paths, datasets with ``shape``, ``dtype``,
``resize(n, axis=0)``, row assignment and slicing, and ``attrs`` dictionaries. The tree is
held in memory and written on ``flush`` / ``close`` as an HDF5 file
(:mod:`micmec_gb300.hdf5`: the classic format the HDF5 library writes by default, which h5py
reads); a file opened for reading or appending is read the same way. Datasets are stored
contiguous with their current shape, and read back resizable along their first axis.
"""

import os

import numpy as np

from micmec_gb300 import hdf5

__all__ = ["File", "Group", "Dataset"]


class Dataset(object):
    """An array whose first axis can grow (``maxshape[0] is None``)."""

    def __init__(self, data=None, shape=None, maxshape=None, dtype=None):
        if data is not None:
            self._buf = np.array(data, dtype=dtype)
            self._n = self._buf.shape[0] if self._buf.ndim else 0
        else:
            self._buf = np.zeros(shape, dtype=dtype or np.float64)
            self._n = shape[0] if len(shape) else 0
        self.maxshape = tuple(maxshape) if maxshape is not None else self._buf.shape
        self.attrs = {}

    @property
    def shape(self):
        if self._buf.ndim == 0:
            return ()
        return (self._n,) + self._buf.shape[1:]

    @property
    def dtype(self):
        return self._buf.dtype

    def __len__(self):
        return self._n

    def resize(self, size, axis=0):
        if axis != 0:
            raise ValueError("only the first axis can be resized")
        if self.maxshape[0] is not None and size > self.maxshape[0]:
            raise ValueError("size exceeds maxshape")
        if size > self._buf.shape[0]:  # geometric growth: amortised O(1) appends
            cap = max(size, 2 * self._buf.shape[0], 4)
            grown = np.zeros((cap,) + self._buf.shape[1:], dtype=self._buf.dtype)
            grown[: self._n] = self._buf[: self._n]
            self._buf = grown
        self._n = size

    def _view(self):
        return self._buf if self._buf.ndim == 0 else self._buf[: self._n]

    def __getitem__(self, idx):
        return self._view()[idx]

    def __setitem__(self, idx, value):
        self._view()[idx] = value

    def __array__(self, dtype=None, copy=None):
        v = self._view()
        return v if dtype is None else v.astype(dtype)


class Group(object):
    def __init__(self):
        self._items = {}
        self.attrs = {}

    def _walk(self, path, create=False):
        node = self
        parts = [p for p in path.split("/") if p]
        for p in parts[:-1]:
            if p not in node._items:
                if not create:
                    raise KeyError(path)
                node._items[p] = Group()
            node = node._items[p]
        return node, parts[-1]

    def __contains__(self, path):
        try:
            node, last = self._walk(path)
        except KeyError:
            return False
        return isinstance(node, Group) and last in node._items

    def __getitem__(self, path):
        node, last = self._walk(path)
        return node._items[last]

    def keys(self):
        return self._items.keys()

    def items(self):
        return self._items.items()

    def create_group(self, path):
        node, last = self._walk(path, create=True)
        if last in node._items:
            raise ValueError("%s already exists" % path)
        node._items[last] = Group()
        return node._items[last]

    def create_dataset(self, path, shape=None, maxshape=None, dtype=None, data=None):
        node, last = self._walk(path, create=True)
        if last in node._items:
            raise ValueError("%s already exists" % path)
        node._items[last] = Dataset(data=data, shape=shape, maxshape=maxshape, dtype=dtype)
        return node._items[last]


class File(Group):
    """``File(name, mode)``: "w" new, "a" read existing (or new) and write back, "r" read only."""

    def __init__(self, filename, mode="r"):
        Group.__init__(self)
        self.filename = filename
        self.mode = mode
        if mode in ("r", "a") and os.path.exists(filename) and hdf5.is_hdf5(filename):
            self._load(hdf5.read(filename), self)
        elif mode in ("r", "a") and os.path.exists(filename):
            # the NumPy-archive files of earlier versions of this module
            with np.load(filename, allow_pickle=False) as z:
                for key in z.files:
                    path, _, attr = key.partition("@")
                    if attr == ".maxshape":
                        self[path].maxshape = tuple(None if m < 0 else int(m) for m in z[key])
                    elif attr:
                        owner = self if path in ("", "/") else self[path.rstrip("/")]
                        owner.attrs[attr] = z[key][()] if z[key].ndim == 0 else z[key]
                    elif path.endswith("/"):
                        if path.rstrip("/") not in self:
                            self.create_group(path.rstrip("/"))
                    else:
                        self.create_dataset(path, data=z[key])
        elif mode == "r":
            raise IOError('Cannot read from file "%s".' % filename)

    @staticmethod
    def _load(hg, group):
        group.attrs.update(hg.attrs)
        for name, item in hg.members.items():
            if isinstance(item, hdf5.HGroup):
                File._load(item, group.create_group(name))
            else:
                data = np.asarray(item.data)
                maxshape = (None,) + data.shape[1:] if data.ndim else ()
                ds = group.create_dataset(name, data=data, maxshape=maxshape)
                ds.attrs.update(item.attrs)

    @staticmethod
    def _tree(group):
        out = hdf5.HGroup(attrs=group.attrs)
        for name, item in group.items():
            if isinstance(item, Group):
                out.members[name] = File._tree(item)
            else:
                out.members[name] = hdf5.HDataset(np.asarray(item), item.attrs)
        return out

    def flush(self):
        if self.mode == "r":
            return
        hdf5.write(self.filename, self._tree(self))

    def close(self):
        self.flush()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
