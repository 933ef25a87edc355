"""GPU force path (C ABI through ForcePartMechanical) against the reference's golden forces."""
import numpy as np
import pytest

from conftest import load_golden, make_system, system_dict

pytestmark = pytest.mark.gpu

G = load_golden("forces")
CASES = [str(c) for c in G["cases"]]


def _ff(case, model, precision):
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    s = make_system(system_dict(G, case + "/sys/"))
    fp = ForcePartMechanical(s, model=model, precision=precision)
    return s, fp, MicMecForceField(s, [fp])


@pytest.mark.parametrize("model", ["original", "nanocell"])
@pytest.mark.parametrize("case", CASES)
def test_fp64_matches_reference(case, model):
    s, fp, ff = _ff(case, model, "fp64")
    gpos = np.zeros((s.nnodes, 3))
    vtens = np.zeros((3, 3))
    e = ff.compute(gpos, vtens)
    key = f"{case}/{model}/"
    e_ref, g_ref, v_ref = float(G[key + "energy"]), G[key + "gpos"], G[key + "vtens"]
    # FP64 tolerance: 1e-10 relative to the largest component
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)
    assert np.abs(gpos - g_ref).max() <= 1e-10 * np.abs(g_ref).max()
    assert np.abs(vtens - v_ref).max() <= 1e-10 * np.abs(v_ref).max()
    assert np.allclose(fp.epot_cells, G[key + "epot_cells"], rtol=1e-10, atol=1e-14)
    assert np.abs(fp.gpos_cells - G[key + "gpos_cells"]).max() <= 1e-10 * np.abs(G[key + "gpos_cells"]).max()


@pytest.mark.parametrize("model", ["original", "nanocell"])
@pytest.mark.parametrize("case", CASES)
def test_fp32_within_tolerance(case, model):
    s, fp, ff = _ff(case, model, "fp32")
    gpos = np.zeros((s.nnodes, 3))
    vtens = np.zeros((3, 3))
    e = ff.compute(gpos, vtens)
    key = f"{case}/{model}/"
    e_ref, g_ref, v_ref = float(G[key + "energy"]), G[key + "gpos"], G[key + "vtens"]
    # FP32 per-cell arithmetic: force error <= 1e-5 of the largest force component
    assert np.abs(gpos - g_ref).max() <= 1e-5 * np.abs(g_ref).max()
    assert abs(e - e_ref) <= 1e-5 * abs(e_ref)
    assert np.abs(vtens - v_ref).max() <= 1e-5 * np.abs(v_ref).max()


def test_add_into_semantics_and_repeatability():
    case = "synth_4x4x4_2types_2states"
    s, fp, ff = _ff(case, "nanocell", "fp64")
    g1 = np.ones((s.nnodes, 3))
    v1 = np.ones((3, 3))
    ff.compute(g1, v1)
    g2 = np.zeros((s.nnodes, 3))
    v2 = np.zeros((3, 3))
    ff.compute(g2, v2)
    assert np.array_equal(g1 - 1.0, g2 + 0.0) or np.abs(g1 - 1.0 - g2).max() < 1e-15
    g3 = np.zeros((s.nnodes, 3))
    ff.compute(g3)
    assert np.array_equal(g2, g3)  # deterministic gather: bitwise repeatable


def test_nan_raises_value_error():
    case = "3x3x3_test_micmec"
    s, fp, ff = _ff(case, "nanocell", "fp64")
    s.pos[3, 1] = np.nan
    with pytest.raises(ValueError):
        ff.compute(np.zeros((s.nnodes, 3)), np.zeros((3, 3)))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("fp32", 1e-5)])
@pytest.mark.parametrize("case", CASES)
def test_eight_lane_cell_kernel_matches_reference(case, precision, tol, monkeypatch):
    """The nanocell model's eight-lanes-per-cell kernel (selected with MICMEC_CELL_KERNEL=8; the
    default is one thread per cell) against the reference's forces."""
    monkeypatch.setenv("MICMEC_CELL_KERNEL", "8")
    s, fp, ff = _ff(case, "nanocell", precision)
    gpos = np.zeros((s.nnodes, 3))
    vtens = np.zeros((3, 3))
    e = ff.compute(gpos, vtens)
    key = f"{case}/nanocell/"
    e_ref, g_ref, v_ref = float(G[key + "energy"]), G[key + "gpos"], G[key + "vtens"]
    assert abs(e - e_ref) <= tol * abs(e_ref)
    assert np.abs(gpos - g_ref).max() <= tol * np.abs(g_ref).max()
    assert np.abs(vtens - v_ref).max() <= tol * np.abs(v_ref).max()

