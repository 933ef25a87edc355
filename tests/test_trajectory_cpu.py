"""Trajectory writers, the h5py stand-in and System file I/O, on the CPU (oracle forces)."""
import os

import numpy as np

from conftest import load_golden, make_system, system_dict
from test_hooks_cpu import _oracle_ff


def test_h5lite_groups_datasets_attrs_roundtrip(tmp_path):
    from micmec_gb300 import h5lite

    fn = str(tmp_path / "t.h5")
    with h5lite.File(fn, "w") as f:
        g = f.create_group("trajectory")
        d = g.create_dataset("pos", (0, 4, 3), maxshape=(None, 4, 3), dtype=np.float64)
        for i in range(7):
            d.resize(i + 1, axis=0)
            d[i] = i
        g.attrs["unit"] = "bohr"
        f.create_dataset("system/masses", data=np.arange(4.0))
    with h5lite.File(fn, "r") as f:
        assert f["trajectory/pos"].shape == (7, 4, 3)
        assert np.array_equal(f["trajectory/pos"][:, 2, 1], np.arange(7.0))
        assert str(f["trajectory"].attrs["unit"]) == "bohr"
        assert "system" in f and "system/masses" in f and "nothing" not in f
    with h5lite.File(fn, "a") as f:  # append mode keeps and extends
        d = f["trajectory/pos"]
        d.resize(8, axis=0)
        d[7] = 7
    with h5lite.File(fn, "r") as f:
        assert f["trajectory/pos"].shape[0] == 8


def test_system_h5_and_xyz_files(tmp_path):
    from micmec_gb300.system import System

    s = make_system(system_dict(load_golden("md_nve_nanocell"), "sys/"))
    s.to_file(str(tmp_path / "s.h5"))
    s.to_file(str(tmp_path / "s.xyz"))
    t = System.from_file(str(tmp_path / "s.h5"))
    assert np.array_equal(t.pos, s.pos) and np.array_equal(t.masses, s.masses)
    assert np.array_equal(t.surrounding_nodes, s.surrounding_nodes)
    assert np.array_equal(t.domain.rvecs, s.domain.rvecs)
    for key, value in s.params.items():
        assert np.array_equal(np.asarray(t.params[key]), np.asarray(value)), key
    lines = open(str(tmp_path / "s.xyz")).read().splitlines()
    assert int(lines[0]) == s.nnodes and len(lines) == s.nnodes + 2
    from micmec_gb300.units import angstrom

    xyz = np.array([[float(v) for v in ln.split()[1:]] for ln in lines[2:]])
    assert np.abs(xyz * angstrom - s.pos).max() < 1e-9 * angstrom


def test_writers_record_the_host_trajectory(tmp_path):
    from micmec_gb300 import h5lite
    from micmec_gb300.sampling.iterative import Hook
    from micmec_gb300.sampling.trajectory import HDF5Writer, XYZWriter
    from micmec_gb300.sampling.verlet import VerletIntegrator

    g = load_golden("md_nve_nanocell")
    s, ff = _oracle_ff(g)
    snaps = {}

    class Snap(Hook):
        def __call__(self, it):
            snaps[it.counter] = (it.pos.copy(), it.epot)

    fn = str(tmp_path / "traj.h5")
    f = h5lite.File(fn, "w")
    xyz = XYZWriter(str(tmp_path / "traj.xyz"), start=0, step=5)
    vi = VerletIntegrator(ff, float(g["timestep"]), hooks=[HDF5Writer(f, step=5), xyz, Snap(0, 5)],
                          vel0=g["vel0"].copy(), device=False)
    vi.run(20)
    f.close()
    xyz.close()
    with h5lite.File(fn, "r") as h:
        counters = h["trajectory/counter"][:]
        assert list(counters) == [0, 5, 10, 15, 20]
        for row, c in enumerate(counters):
            assert np.array_equal(h["trajectory/pos"][row], snaps[int(c)][0])
            assert h["trajectory/epot"][row] == snaps[int(c)][1]
        assert np.array_equal(h["system/masses"][:], s.masses)
    text = open(str(tmp_path / "traj.xyz")).read().splitlines()
    assert len(text) == 5 * (s.nnodes + 2)
    assert text[1].split()[0] == "0" and "E_pot" in text[1]
    assert os.path.getsize(fn) > 0
