"""HDF5 files without h5py (micmec_gb300.hdf5, used by micmec_gb300.h5lite).

The reader is checked against a file written by the HDF5 library (the MATLAB 7.3 test file
that scipy ships, read as test data when it is installed); the writer's files are checked
field by field against the on-disk format (superblock, object headers, group B-tree, local
heap, symbol table nodes) and read back.
"""
import os
import struct

import numpy as np
import pytest


def _library_file():
    try:
        import scipy.io.matlab as m
    except ImportError:
        return None
    fn = os.path.join(os.path.dirname(m.__file__), "tests", "data", "testhdf5_7.4_GLNX86.mat")
    return fn if os.path.exists(fn) else None


def test_reader_takes_a_file_written_by_the_hdf5_library():
    from micmec_gb300 import hdf5

    fn = _library_file()
    if fn is None:
        pytest.skip("scipy's HDF5 test file is not installed")
    assert hdf5.is_hdf5(fn)  # superblock after a 512-byte user block
    g = hdf5.read(fn)
    assert list(g.members) == ["testdouble"]
    d = g.members["testdouble"]
    assert d.data.shape == (9, 1) and d.data.dtype == np.float64
    assert np.allclose(d.data.ravel(), np.arange(9) * np.pi / 4, rtol=0, atol=1e-15)
    assert d.attrs["MATLAB_class"] == b"double"


def _tree(nmembers=40):
    from micmec_gb300.hdf5 import HDataset, HGroup

    rng = np.random.default_rng(3)
    root = HGroup(attrs={"title": "micmec", "count": 3, "vec": np.arange(3.0), "names": np.array(["a", "bé"])})
    s = HGroup()
    root.members["system"] = s
    s.members["pos"] = HDataset(rng.normal(size=(27, 3)))
    s.members["types"] = HDataset(np.arange(8, dtype=np.int32), {"unit": "none"})
    s.members["masses"] = HDataset(rng.uniform(1, 2, 27).astype(np.float32))
    s.members["empty"] = HDataset(np.zeros((0, 3)))
    s.members["flags"] = HDataset(np.array([True, False, True]))
    s.members["big_endian"] = HDataset(np.arange(4, dtype=">f8"))
    s.members["scalar"] = HDataset(np.float64(2.5))
    s.members["label"] = HDataset(np.array([b"fcu", b"reo"]))
    s.members["u64"] = HDataset(np.array([0, 2**63 + 5], dtype=np.uint64))
    p = HGroup(attrs={"kind": "parameters"})
    s.members["params"] = p
    for i in range(nmembers):  # several symbol table nodes under one B-tree node
        p.members["key%03d" % i] = HDataset(np.full(i + 1, i, dtype=np.int64))
    root.members["a_first"] = HGroup()  # empty group
    return root


def test_written_file_follows_the_format(tmp_path):
    from micmec_gb300 import hdf5

    fn = str(tmp_path / "t.h5")
    hdf5.write(fn, _tree())
    b = open(fn, "rb").read()
    assert b[:8] == hdf5.SIGNATURE
    assert b[8:16] == bytes([0, 0, 0, 0, 0, 8, 8, 0])  # versions, 8-byte offsets and lengths
    assert struct.unpack_from("<HHI", b, 16) == (4, 16, 0)
    base, free, eof, drv = struct.unpack_from("<QQQQ", b, 24)
    assert base == 0 and free == hdf5.UNDEF and drv == hdf5.UNDEF and eof == len(b)
    _, root_oh, cache, _, btree, heap = struct.unpack_from("<QQIIQQ", b, 56)
    assert cache == 1
    ver, _, nmsg, refc, size = struct.unpack_from("<BBHII", b, root_oh)
    assert (ver, refc) == (1, 1) and size % 8 == 0
    mtype, msize = struct.unpack_from("<HH", b, root_oh + 16)
    assert mtype == 0x11 and struct.unpack_from("<QQ", b, root_oh + 24) == (btree, heap)
    assert b[heap:heap + 4] == b"HEAP"
    dsize, free_at, data = struct.unpack_from("<QQQ", b, heap + 8)
    assert struct.unpack_from("<QQ", b, data + free_at) == (1, dsize - free_at)  # one free block, list end 1
    assert b[btree:btree + 4] == b"TREE" and b[btree + 4] == 0 and b[btree + 5] == 0
    # the parameters group: 40 members in 5 symbol table nodes of 8, names in byte order
    g = hdf5.read(fn)
    names = list(g.members["system"].members["params"].members)
    assert names == sorted(names) and len(names) == 40
    assert all(off % 8 == 0 for off in (root_oh, btree, heap, data))


def test_roundtrip_keeps_values_types_and_attributes(tmp_path):
    from micmec_gb300 import hdf5

    src = _tree(nmembers=255)
    fn = str(tmp_path / "t.h5")
    hdf5.write(fn, src)
    got = hdf5.read(fn)
    assert got.attrs["title"] == "micmec" and got.attrs["count"] == 3
    assert np.array_equal(got.attrs["vec"], np.arange(3.0)) and list(got.attrs["names"]) == ["a", "bé"]
    s, r = src.members["system"], got.members["system"]
    for name in ("pos", "types", "masses", "empty", "big_endian", "label", "u64"):
        a, b = np.asarray(s.members[name].data), np.asarray(r.members[name].data)
        assert a.shape == b.shape and np.array_equal(a, b), name
        assert b.dtype.kind == a.dtype.kind and b.dtype.itemsize == a.dtype.itemsize, name
    assert r.members["types"].attrs["unit"] == "none"
    assert np.array_equal(r.members["flags"].data, [1, 0, 1])  # booleans come back as uint8
    assert r.members["scalar"].data == 2.5
    p = r.members["params"]
    assert p.attrs["kind"] == "parameters" and len(p.members) == 255
    for i in (0, 7, 8, 100, 254):
        assert np.array_equal(p.members["key%03d" % i].data, np.full(i + 1, i))
    assert got.members["a_first"].members == {}


def test_groups_beyond_one_btree_node_are_refused(tmp_path):
    from micmec_gb300 import hdf5

    with pytest.raises(ValueError):
        hdf5.write(str(tmp_path / "t.h5"), _tree(nmembers=257))


def test_h5lite_files_are_hdf5(tmp_path):
    from micmec_gb300 import h5lite, hdf5

    fn = str(tmp_path / "t.h5")
    with h5lite.File(fn, "w") as f:
        d = f.create_dataset("trajectory/epot", (0,), maxshape=(None,), dtype=np.float64)
        d.resize(3, axis=0)
        d[:] = [1.0, 2.0, 3.0]
        f["trajectory"].attrs["ndof"] = 78
    assert hdf5.is_hdf5(fn)
    g = hdf5.read(fn)
    assert np.array_equal(g.members["trajectory"].members["epot"].data, [1.0, 2.0, 3.0])
    assert g.members["trajectory"].attrs["ndof"] == 78
