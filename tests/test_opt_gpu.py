"""Optimisers on GPU forces: QN against the reference's QNOptimizer trajectory; CG and cell DOFs by invariants."""
import numpy as np
import pytest

from conftest import load_golden, make_system, system_dict

pytestmark = pytest.mark.gpu


def _ff(g, model="nanocell"):
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    s = make_system(system_dict(g, "sys/"))
    return s, MicMecForceField(s, [ForcePartMechanical(s, model=model)])


def test_qn_matches_reference():
    from micmec_gb300.sampling.dof import CartesianDOF
    from micmec_gb300.sampling.iterative import Hook
    from micmec_gb300.sampling.opt import QNOptimizer

    g = load_golden("opt_qn_nanocell")
    s, ff = _ff(g)
    energies = []

    class E(Hook):
        def __call__(self, it):
            energies.append(it.epot)

    opt = QNOptimizer(CartesianDOF(ff, gpos_rms=1e-6, dpos_rms=1e-4), hooks=[E()])
    opt.run(60)
    ref = g["energies"]
    assert len(energies) == len(ref)
    assert np.allclose(energies, ref, rtol=1e-9, atol=0)
    assert np.abs(s.pos - g["pos_end"]).max() < 1e-6


def test_cg_reaches_reference_minimum():
    from micmec_gb300.sampling.dof import CartesianDOF
    from micmec_gb300.sampling.opt import CGOptimizer

    g = load_golden("opt_qn_nanocell")
    s, ff = _ff(g)
    dof = CartesianDOF(ff, gpos_rms=1e-7, dpos_rms=1e-5)
    CGOptimizer(dof).run(2000)
    e = ff.compute()
    assert e <= g["energies"][-1] + 1e-9 * abs(g["energies"][-1])
    gpos = np.zeros((s.nnodes, 3))
    ff.compute(gpos)
    assert np.sqrt((gpos**2).sum(axis=1)).max() < 3e-6


def test_strain_cell_dof_gradient():
    from micmec_gb300.sampling.dof import StrainCellDOF, FullCellDOF

    g = load_golden("opt_qn_nanocell")
    s, ff = _ff(g)
    for cls in (StrainCellDOF, FullCellDOF):
        dof = cls(ff)
        assert dof.check_delta(eps=1e-6) < 1e-3


@pytest.mark.parametrize("kind", ["strain", "full", "host-strain"])
def test_cell_relaxation_reaches_reference_minimum(kind):
    """CGOptimizer with StrainCellDOF / FullCellDOF: on the device (batched cell-relaxation
    kernel) and on the host (GPU forces) it reaches the minimum of the reference's
    QNOptimizer run from the same start."""
    from micmec_gb300.sampling.dof import FullCellDOF, StrainCellDOF
    from micmec_gb300.sampling.opt import CGOptimizer

    tag = "full" if kind == "full" else "strain"
    g = load_golden("opt_cell_%s_nanocell" % tag)
    s, ff = _ff(g)
    cls = FullCellDOF if tag == "full" else StrainCellDOF
    dof = cls(ff, gpos_rms=1e-8, dpos_rms=1e-6, grvecs_rms=1e-8, drvecs_rms=1e-6)
    opt = CGOptimizer(dof, device=not kind.startswith("host"))
    if opt.device:
        assert opt._device_kind() == tag
    opt.run(3000)
    e = ff.compute()
    assert abs(e - float(g["epot_end"])) <= 1e-9 * abs(float(g["epot_end"]))
    rv, ref = np.asarray(s.domain.rvecs), g["rvecs_end"]
    assert np.abs(rv @ rv.T - ref @ ref.T).max() <= 1e-5 * np.abs(ref @ ref.T).max()


def test_device_cg_positions_reach_reference_minimum():
    from micmec_gb300.sampling.dof import CartesianDOF
    from micmec_gb300.sampling.opt import CGOptimizer

    g = load_golden("opt_qn_nanocell")
    s, ff = _ff(g)
    opt = CGOptimizer(CartesianDOF(ff, gpos_rms=1e-7, dpos_rms=1e-5), device=True)
    assert opt._device_kind() is None
    opt.run(2000)
    assert opt.dof.converged
    e = ff.compute()
    assert e <= g["energies"][-1] + 1e-9 * abs(g["energies"][-1])
    assert np.abs(s.pos - g["pos_end"]).max() < 1e-3


def test_strain_cell_relaxation_with_pressure_part_matches_batched_relaxer():
    """ForcePartPressure beside ForcePartMechanical under StrainCellDOF + CG (host optimiser,
    GPU forces): the relaxed enthalpy E + P V, domain and residual stress vtens / V + P I
    equal those of the batched device relaxer run at the same external pressure."""
    from micmec_gb300 import units
    from micmec_gb300.batch import BatchSystems
    from micmec_gb300.pes.mmff import ForcePartMechanical, ForcePartPressure, MicMecForceField
    from micmec_gb300.sampling.dof import StrainCellDOF
    from micmec_gb300.sampling.opt import CGOptimizer

    P = 500e6 * units.pascal
    g = load_golden("opt_cell_strain_nanocell")
    d = system_dict(g, "sys/")
    s = make_system(d)
    mech = ForcePartMechanical(s, model="nanocell")
    ff = MicMecForceField(s, [mech, ForcePartPressure(s, P)])
    dof = StrainCellDOF(ff, gpos_rms=1e-9, dpos_rms=1e-7, grvecs_rms=1e-9, drvecs_rms=1e-7)
    CGOptimizer(dof).run(4000)
    vtens = np.zeros((3, 3))
    h_host = ff.compute(None, vtens)
    V = s.domain.volume
    assert np.abs(vtens / V).max() < 1e-9  # mechanical virial / V balances -P I
    b = BatchSystems([make_system(d)], model="nanocell", precision="fp64")
    b.set_state([d["pos"]], None, [d["rvecs"]])
    gmax, iters = b.relax(max_iter=4000, gtol=1e-8, cell="strain", press=P, stress_tol=1e-11)
    assert gmax[0] < 1e-8, iters
    h_batch = b.energies()[0] + P * b.control()[0, 18]
    assert abs(h_host - h_batch) <= 1e-9 * abs(h_batch)
    rv, ref = np.asarray(s.domain.rvecs), b.get_state()[2][0]
    assert np.abs(rv @ rv.T - ref @ ref.T).max() <= 1e-5 * np.abs(ref @ ref.T).max()
