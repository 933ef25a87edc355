"""The reference-side ctypes binding (micmec_gb300/binding/mmff_gb300.py), executed.

That file is what a maintainer adds to the reference tree as ``micmec/pes/mmff_gb300.py``;
it imports ``micmec.pes.mmff.ForcePart`` and ``micmec.utils.Grid``. Here it runs
unchanged on a ``micmec`` namespace whose two modules are this package's mirrors of
those reference modules, on every golden force case, so its argument types, table
packing, domain handling and status handling are exercised against the reference's
own numbers (FP64: 1e-10 of the largest component).
"""
import importlib.util
import os
import sys
import types

import numpy as np
import pytest

from conftest import ROOT, load_golden, make_system, system_dict

pytestmark = pytest.mark.gpu

G = load_golden("forces")
CASES = [str(c) for c in G["cases"]]


@pytest.fixture(scope="module")
def binding():
    import micmec_gb300.pes.mmff as mmff
    import micmec_gb300.utils as utils

    saved = {k: sys.modules.get(k) for k in ("micmec", "micmec.pes", "micmec.pes.mmff", "micmec.utils")}
    pkg = types.ModuleType("micmec")
    pes = types.ModuleType("micmec.pes")
    pkg.pes, pkg.utils, pes.mmff = pes, utils, mmff
    sys.modules.update({"micmec": pkg, "micmec.pes": pes, "micmec.pes.mmff": mmff, "micmec.utils": utils})
    try:
        path = os.path.join(ROOT, "micmec_gb300", "binding", "mmff_gb300.py")
        spec = importlib.util.spec_from_file_location("micmec_pes_mmff_gb300", path)
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        yield mod
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v


@pytest.mark.parametrize("model", ["original", "nanocell"])
@pytest.mark.parametrize("case", CASES)
def test_binding_matches_reference_forces(binding, case, model):
    from micmec_gb300.pes.mmff import MicMecForceField

    s = make_system(system_dict(G, case + "/sys/"))
    part = binding.ForcePartMechanicalGPU(s, model=model)
    ff = MicMecForceField(s, [part])
    g0 = np.full((s.nnodes, 3), 0.125)
    v0 = np.full((3, 3), -0.5)
    gpos, vtens = g0.copy(), v0.copy()
    e = ff.compute(gpos, vtens)
    key = "%s/%s/" % (case, model)
    e_ref, g_ref, v_ref = float(G[key + "energy"]), G[key + "gpos"], G[key + "vtens"]
    assert abs(e - e_ref) <= 1e-10 * abs(e_ref)
    assert np.abs(gpos - g0 - g_ref).max() <= 1e-10 * np.abs(g_ref).max()
    assert np.abs(vtens - v0 - v_ref).max() <= 1e-10 * np.abs(v_ref).max()


def test_binding_follows_domain_updates_and_reports_nan(binding):
    from micmec_gb300.pes.mmff import ForcePartMechanical, MicMecForceField

    case = "synth_4x4x4_2types_2states"
    s = make_system(system_dict(G, case + "/sys/"))
    s2 = make_system(system_dict(G, case + "/sys/"))
    ff = MicMecForceField(s, [binding.ForcePartMechanicalGPU(s)])
    ff2 = MicMecForceField(s2, [ForcePartMechanical(s2)])
    F = np.eye(3) + np.array([[0.01, 0.002, 0.0], [0.0, -0.005, 0.001], [0.003, 0.0, 0.004]])
    for f in (ff, ff2):
        f.update_rvecs(f.system.domain.rvecs @ F)
        f.update_pos(f.system.pos @ F)
    out = []
    for f in (ff, ff2):
        g, v = np.zeros((s.nnodes, 3)), np.zeros((3, 3))
        out.append((f.compute(g, v), g, v))
    (e1, g1, v1), (e2, g2, v2) = out
    assert abs(e1 - e2) <= 1e-12 * abs(e2)
    assert np.abs(g1 - g2).max() <= 1e-12 * np.abs(g2).max()
    assert np.abs(v1 - v2).max() <= 1e-12 * np.abs(v2).max()
    s.pos[2, 0] = np.nan
    ff.update_pos(s.pos)
    with pytest.raises(ValueError):
        ff.compute(np.zeros((s.nnodes, 3)))
