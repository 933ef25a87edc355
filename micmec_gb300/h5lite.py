"""A small stand-in for the part of h5py that trajectories and systems use.

h5py is not installed with this package. ``File`` offers the interface that the
reference's ``HDF5Writer`` (micmec/sampling/trajectory.py:31-85) and
``System.to_hdf5`` / ``from_hdf5`` (micmec/system.py:262-370) use: nested groups,
``create_group``, ``create_dataset(name, shape, maxshape, dtype)`` or ``(name, data=...)``,
``in``, ``[...]`` lookups with "a/b" paths, datasets with ``shape``, ``dtype``,
``resize(n, axis=0)``, row assignment and slicing, and ``attrs`` dictionaries. The file
on disk is a NumPy ``.npz`` archive (one array per dataset, keyed by its path; attributes
under ``path@name``, a dataset's maxshape under ``path@.maxshape``), written on ``flush`` /
``close``; it is not an HDF5 file.
"""

import os

import numpy as np

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

    def _flat(self, prefix=""):
        for name, item in self._items.items():
            path = prefix + name
            if isinstance(item, Group):
                yield path + "/", None, item.attrs
                yield from item._flat(path + "/")
            else:
                yield path, item, item.attrs


class File(Group):
    """``File(name, mode)``: "w" new, "a" read existing (or new) and write back, "r" read only."""

    def __init__(self, filename, mode="r"):
        Group.__init__(self)
        self.filename = filename
        self.mode = mode
        if mode in ("r", "a") and os.path.exists(filename):
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

    def flush(self):
        if self.mode == "r":
            return
        arrays = {}
        for name, value in self.attrs.items():
            arrays["/@" + name] = np.asarray(value)
        for path, ds, attrs in self._flat():
            if ds is not None:
                arrays[path] = np.asarray(ds)
                arrays[path + "@.maxshape"] = np.array([-1 if m is None else m for m in ds.maxshape], dtype=np.int64)
            else:
                arrays[path] = np.zeros(0)
            for name, value in attrs.items():
                arrays[path + "@" + name] = np.asarray(value)
        with open(self.filename, "wb") as f:
            np.savez(f, **arrays)

    def close(self):
        self.flush()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
