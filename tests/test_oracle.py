"""The CPU oracle against the golden fixtures produced by the reference implementation."""
import numpy as np
import pytest

from conftest import load_golden, system_dict
from oracle import mmff as om

G = load_golden("forces")
CASES = [str(c) for c in G["cases"]]


@pytest.mark.parametrize("model", ["original", "nanocell"])
@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case, model):
    sysd = system_dict(G, case + "/sys/")
    e, gpos, vtens = om.compute(sysd, model)
    key = f"{case}/{model}/"
    e_ref, g_ref, v_ref = float(G[key + "energy"]), G[key + "gpos"], G[key + "vtens"]
    assert abs(e - e_ref) <= 1e-12 * abs(e_ref)
    assert np.abs(gpos - g_ref).max() <= 1e-12 * np.abs(g_ref).max()
    assert np.abs(vtens - v_ref).max() <= 1e-12 * np.abs(v_ref).max()
    ecells, gcells, _ = om.deformation(sysd["pos"], sysd["rvecs"], sysd["grid"], sysd["surrounding_nodes"],
                                       sysd["types"], sysd["params"], model)
    assert np.allclose(ecells, G[key + "epot_cells"], rtol=1e-12, atol=0)
    assert np.abs(gcells - G[key + "gpos_cells"]).max() <= 1e-12 * np.abs(G[key + "gpos_cells"]).max()


def test_net_force_vanishes():
    sysd = system_dict(G, "synth_4x4x4_2types_2states/sys/")
    for model in ("original", "nanocell"):
        _, gpos, _ = om.compute(sysd, model)
        assert np.abs(gpos.sum(axis=0)).max() < 1e-14 * np.abs(gpos).max() * len(gpos)


def test_gradient_matches_finite_differences():
    """Central differences of the oracle energy (symmetric elasticity tensors)."""
    sysd = system_dict(G, "synth_4x4x4_2types_2states/sys/")
    rng = np.random.default_rng(3)
    for model in ("original", "nanocell"):
        e0, gpos, _ = om.compute(sysd, model)
        for _ in range(4):
            n, x = rng.integers(len(gpos)), rng.integers(3)
            h = 1e-4
            p = dict(sysd)
            pp = sysd["pos"].copy()
            pp[n, x] += h
            p["pos"] = pp
            ep = om.compute(p, model)[0]
            pp[n, x] -= 2 * h
            em = om.compute(p, model)[0]
            fd = (ep - em) / (2 * h)
            assert abs(fd - gpos[n, x]) <= 1e-6 * np.abs(gpos).max()


def test_virial_is_homogeneous_strain_derivative():
    """vtens[k, l] = dE/d(deformation) under pos -> pos (I + D), rvecs -> rvecs (I + D)."""
    sysd = system_dict(G, "synth_4x4x4_2types_2states/sys/")
    _, _, vtens = om.compute(sysd, "nanocell")
    h = 1e-6
    fd = np.zeros((3, 3))
    for k in range(3):
        for l in range(3):
            es = []
            for sgn in (1, -1):
                D = np.eye(3)
                D[k, l] += sgn * h
                p = dict(sysd)
                p["pos"] = sysd["pos"] @ D
                p["rvecs"] = sysd["rvecs"] @ D
                es.append(om.compute(p, "nanocell")[0])
            fd[k, l] = (es[0] - es[1]) / (2 * h)
    assert np.abs(fd - vtens).max() <= 1e-6 * np.abs(vtens).max()


def test_torch_oracle_matches_numpy_oracle():
    torch = pytest.importorskip("torch")
    from oracle import torch_mmff
    from micmec_gb300.pes.mmff import type_parameters

    sysd = system_dict(G, "synth_4x4x4_2types_2states/sys/")
    ids = sorted(set(int(t) for t in sysd["types"]))
    nstates, h0, C, df, temp = type_parameters(sysd["params"], ids)
    iu = np.triu_indices(6)
    pairs = [(0, 0), (1, 1), (2, 2), (1, 2), (0, 2), (0, 1)]
    c21 = np.zeros((len(ids), 4, 21))
    for t in range(len(ids)):
        for s in range(nstates[t]):
            Ct = C[4 * t + s].reshape(3, 3, 3, 3)
            c21[t, s] = np.array([[Ct[pairs[p] + pairs[q]] for q in range(6)] for p in range(6)])[iu]
    pos = torch.tensor(sysd["pos"], requires_grad=True)
    for model in ("nanocell", "original"):
        E = torch_mmff.energy(pos, sysd["rvecs"], sysd["grid"], sysd["surrounding_nodes"], sysd["types"], ids,
                              nstates, torch.tensor(c21), torch.tensor(h0.reshape(-1, 4, 3, 3)),
                              torch.tensor(df.reshape(-1, 4)), temp, model=model)
        g, = torch.autograd.grad(E, pos)
        e_ref, g_ref, _ = om.compute(sysd, model)
        assert abs(E.item() - e_ref) <= 1e-12 * abs(e_ref)
        assert np.abs(g.numpy() - g_ref).max() <= 1e-11 * np.abs(g_ref).max()
