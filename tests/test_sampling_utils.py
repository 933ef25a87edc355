"""Sampling utilities and the external-pressure part against the reference (CPU only).

Initial velocities (micmec/sampling/utils.py:28-65), barostat velocities (450-475),
momentum removal for periodic and isolated systems (142-174), degree-of-freedom
counts (322-343, 478-501) and domain symmetrisation (346-383) are compared with
outputs of the reference's own functions on the same seeded inputs
(tests/golden/make_golden.py, ``sampling_utils.npz``). The reference draws from the
global ``np.random`` stream, so each case re-seeds it exactly as the generator did.
ForcePartPressure has no reference counterpart; it is checked against its
definition (E = P V, virial P V I) and the homogeneous-deformation derivative.
"""
import numpy as np
import pytest

from conftest import load_golden

G = load_golden("sampling_utils")


def test_get_random_vel_matches_reference():
    from micmec_gb300.sampling.utils import get_random_vel

    cases = [(300.0, True, None), (300.0, False, None), (600.0, True, np.array([1, 5, 7, 30])), (0.0, True, None)]
    for i, (temp, scale, select) in enumerate(cases):
        np.random.seed(int(G["vel_seeds"][i]))
        v = get_random_vel(temp, scale, G["masses"], select=select)
        assert v.shape == G["vel%d" % i].shape
        assert np.allclose(v, G["vel%d" % i], rtol=1e-14, atol=0.0), i


def test_get_random_vel_press_matches_reference():
    from micmec_gb300.sampling.utils import get_random_vel_press

    np.random.seed(200)
    vp = get_random_vel_press(float(G["baro_mass"]), 300.0)
    assert np.allclose(vp, G["vel_press"], rtol=1e-14, atol=0.0)
    assert np.array_equal(vp, vp.T)


@pytest.mark.parametrize("tag,rvecs", [("pbc", np.eye(3) * 100.0), ("iso", np.zeros((0, 3)))])
def test_clean_momenta_matches_reference(tag, rvecs):
    from micmec_gb300.pes.ext import Domain
    from micmec_gb300.sampling.utils import clean_momenta

    p, v = G["clean_pos0"].copy(), G["clean_vel0"].copy()
    m = G["masses"]
    clean_momenta(p, v, m, Domain(rvecs))
    assert np.allclose(p, G["clean_%s_pos" % tag], rtol=0, atol=1e-12)
    ref = G["clean_%s_vel" % tag]
    assert np.abs(v - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.abs(m @ v).max() <= 1e-12 * np.abs(m[:, None] * v).sum(axis=0).max()


def test_dof_counts_match_reference():
    from micmec_gb300.sampling.utils import get_ndof_baro, get_ndof_internal_md

    assert [get_ndof_internal_md(57, n) for n in (0, 1, 2, 3)] == list(G["ndof_internal"])
    combos = ((True, False), (True, True), (False, False))
    assert [get_ndof_baro(3, a, c) for a, c in combos] == list(G["ndof_baro"])
    with pytest.raises(AssertionError):
        get_ndof_baro(3, False, True)


def test_domain_symmetrize_matches_reference():
    from micmec_gb300.pes.ext import Domain
    from micmec_gb300.sampling.utils import domain_symmetrize

    class FF(object):
        def __init__(self, pos, rvecs):
            self.system = type("S", (), {})()
            self.system.pos = np.array(pos)
            self.system.domain = Domain(np.array(rvecs))

        def update_rvecs(self, rvecs):
            self.system.domain.update_rvecs(rvecs)

        def update_pos(self, pos):
            self.system.pos[:] = pos

    vel = G["clean_vel0"]
    ff = FF(G["clean_pos0"], G["sym_rvecs0"])
    vecs, tens = domain_symmetrize(ff, vector_lst=[vel[:3].copy()], tensor_lst=[np.outer(vel[0], vel[1])])
    rv = np.asarray(ff.system.domain.rvecs)
    assert np.allclose(rv, G["sym_rvecs"], rtol=0, atol=1e-12 * np.abs(rv).max())
    assert np.allclose(rv, rv.T, rtol=0, atol=1e-12 * np.abs(rv).max())
    assert np.allclose(ff.system.pos, G["sym_pos"], rtol=0, atol=1e-11)
    assert np.allclose(vecs[0], G["sym_vec"], rtol=1e-12, atol=0)
    assert np.allclose(tens[0], G["sym_tens"], rtol=1e-12, atol=1e-30)


# ---------------------------------------------------------------- ForcePartPressure


def _pressure_system():
    from micmec_gb300.system import System

    rv = np.array([[40.0, 1.5, -0.7], [0.9, 41.0, 2.1], [-1.2, 0.3, 39.0]])
    sn = np.zeros((0, 8), dtype=np.int64)
    sc = np.zeros((2, 8), dtype=np.int64) - 1
    return System(pos=np.zeros((2, 3)), masses=np.ones(2), rvecs=rv, surrounding_cells=sc, surrounding_nodes=sn,
                  grid=None, types=np.zeros(0, dtype=np.int64), params={})


def test_force_part_pressure_energy_and_virial():
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartPressure, MicMecForceField

    s = _pressure_system()
    P = 250e6 * units.pascal
    part = ForcePartPressure(s, P)
    ff = MicMecForceField(s, [part])
    V = abs(np.linalg.det(s.domain.rvecs))
    gpos = np.full((s.nnodes, 3), 0.5)
    vtens = np.full((3, 3), 0.25)
    e = ff.compute(gpos, vtens)
    assert e == pytest.approx(P * V, rel=1e-14)
    assert np.array_equal(gpos, np.full((s.nnodes, 3), 0.5))  # no node gradient
    assert np.allclose(vtens - 0.25, P * V * np.eye(3), rtol=1e-14, atol=0)
    assert ff.part_press is part


def test_force_part_pressure_virial_is_the_homogeneous_strain_derivative():
    """vtens^T = dE/dD for rvecs -> rvecs (I + D), central differences."""
    from micmec_gb300 import units
    from micmec_gb300.pes.mmff import ForcePartPressure

    s = _pressure_system()
    part = ForcePartPressure(s, 1e9 * units.pascal)
    rv0 = np.array(s.domain.rvecs)
    vtens = np.zeros((3, 3))
    part.compute(None, vtens)
    h = 1e-6
    fd = np.zeros((3, 3))
    for i in range(3):
        for j in range(3):
            D = np.zeros((3, 3))
            D[i, j] = h
            s.domain.update_rvecs(rv0 @ (np.eye(3) + D))
            ep = part.compute()
            s.domain.update_rvecs(rv0 @ (np.eye(3) - D))
            em = part.compute()
            fd[i, j] = (ep - em) / (2 * h)
    s.domain.update_rvecs(rv0)
    assert np.allclose(fd, vtens.T, rtol=1e-7, atol=1e-9 * np.abs(vtens).max())
