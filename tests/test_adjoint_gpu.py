"""Adjoint kernel behind torch.autograd: parameter and position gradients of energy, force and
trajectory losses, against an FP64 autograd reference and central finite differences."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(n=4, model="nanocell", seed=0):
    import torch

    from micmec_gb300 import lattices, units
    from micmec_gb300.autograd import MicMecParameters
    from micmec_gb300.pes.mmff import ForcePartMechanical
    from micmec_gb300.system import System

    rng = np.random.default_rng(seed)
    d = lattices.make_lattice(lattices.defect_grid(n, 0.25, rng), nstates=2)
    d["pos"] = lattices.displace(d["pos"], 0.1 * units.angstrom, rng)
    s = System.from_dict(d)
    part = ForcePartMechanical(s, model=model, precision="fp64")
    params = MicMecParameters(part)
    pos = torch.tensor(s.pos, dtype=torch.float64, device="cuda")
    return s, part, params, pos, rng


def _ref_energy(s, part, params, pos_t, c21, h0, df, model):
    from oracle import torch_mmff

    return torch_mmff.energy(pos_t, s.domain.rvecs, s.grid, s.surrounding_nodes, s.types, part.type_ids,
                             params.nstates, c21, h0, df, params.temp, model=model)


@pytest.mark.parametrize("model", ["nanocell", "original"])
def test_force_loss_gradients_match_fp64_autograd_reference(model):
    import torch

    from micmec_gb300.autograd import energy_and_gradient

    s, part, params, pos, rng = _setup(model=model)
    w = torch.tensor(rng.normal(size=(s.nnodes, 3)), dtype=torch.float64, device="cuda")
    pos.requires_grad_(True)
    E, g = energy_and_gradient(pos, params)
    loss = 1e3 * E + (w * g).sum() * 10.0
    gp, gc, gh, gd = torch.autograd.grad(loss, [pos, params.c21, params.h0, params.free_energy])
    # FP64 autograd reference on the CPU
    c21 = params.c21.detach().clone().requires_grad_(True)
    h0 = params.h0.detach().clone().requires_grad_(True)
    df = params.free_energy.detach().clone().requires_grad_(True)
    pt = torch.tensor(s.pos, dtype=torch.float64, requires_grad=True)
    Er = _ref_energy(s, part, params, pt, c21, h0, df, model)
    gr, = torch.autograd.grad(Er, pt, create_graph=True)
    lr = 1e3 * Er + (w.cpu() * gr).sum() * 10.0
    rp, rc, rh, rd = torch.autograd.grad(lr, [pt, c21, h0, df])
    assert abs(E.item() - Er.item()) <= 1e-10 * abs(Er.item())
    assert (g.detach().cpu() - gr.detach()).abs().max() <= 1e-10 * gr.abs().max()
    for a, b in ((gp.cpu(), rp), (gc.cpu(), rc), (gh.cpu(), rh), (gd.cpu(), rd)):
        assert (a - b).abs().max() <= 1e-8 * b.abs().max() + 1e-300, (a - b).abs().max()


def test_force_loss_gradient_matches_central_differences():
    import torch

    from micmec_gb300.autograd import energy_and_gradient

    s, part, params, pos, rng = _setup(n=3)
    w = torch.tensor(rng.normal(size=(s.nnodes, 3)), dtype=torch.float64, device="cuda")

    def loss():
        E, g = energy_and_gradient(pos, params)
        return (w * g).sum()

    l0 = loss()
    gc, gh, gd = torch.autograd.grad(l0, [params.c21, params.h0, params.free_energy])
    # the free-energy slot with the largest effect (in a lattice built on state 0's rest cell the
    # other states carry weights ~exp(-E/kT) far below rounding)
    fe = tuple(int(i) for i in np.unravel_index(int(gd.abs().argmax()), gd.shape))
    checks = [(params.c21, gc, (0, 1, 0)), (params.c21, gc, (1, 0, 3)), (params.h0, gh, (0, 0, 0, 0)),
              (params.h0, gh, (1, 1, 2, 1)), (params.free_energy, gd, fe)]
    for tensor, grad, idx in checks:
        base = tensor.detach()[idx].item()
        h = 1e-4 * max(abs(base), 1e-2 * tensor.detach().abs().max().item())
        vals = []
        for sgn in (1, -1):
            with torch.no_grad():
                tensor[idx] = base + sgn * h
            vals.append(loss().item())
        with torch.no_grad():
            tensor[idx] = base
        fd = (vals[0] - vals[1]) / (2 * h)
        floor = 1e-13 * abs(l0.item()) / h  # rounding of the central difference
        assert abs(fd - grad[idx].item()) <= 1e-6 * max(abs(fd), 1e-3 * grad.abs().max().item()) + floor, \
            (idx, fd, grad[idx])


def test_trajectory_gradient_with_checkpointing():
    import torch

    from micmec_gb300 import units
    from micmec_gb300.autograd import verlet_trajectory

    s, part, params, pos, rng = _setup(n=3, seed=2)
    masses = torch.tensor(s.masses, dtype=torch.float64, device="cuda")
    vel = torch.tensor(rng.normal(size=(s.nnodes, 3)) * np.sqrt(units.boltzmann * 300.0 / s.masses)[:, None],
                       dtype=torch.float64, device="cuda")
    target = torch.tensor(rng.normal(size=(s.nnodes, 3)) * 1e-3, dtype=torch.float64, device="cuda")
    dt = 1.0 * units.femtosecond

    def loss():
        grads, _, _ = verlet_trajectory(pos, vel, masses, params, dt, 12, checkpoint_every=5)
        mean_force = -torch.stack(grads).mean(dim=0)
        return ((mean_force - target) ** 2).mean()

    l0 = loss()
    gc, gh, gd = torch.autograd.grad(l0, [params.c21, params.h0, params.free_energy])
    fe = tuple(int(i) for i in np.unravel_index(int(gd.abs().argmax()), gd.shape))
    for tensor, grad, idx in ((params.c21, gc, (0, 0, 0)), (params.h0, gh, (0, 1, 1, 1)),
                              (params.free_energy, gd, fe)):
        base = tensor.detach()[idx].item()
        h = 1e-4 * max(abs(base), 1e-2 * tensor.detach().abs().max().item())
        vals = []
        for sgn in (1, -1):
            with torch.no_grad():
                tensor[idx] = base + sgn * h
            vals.append(loss().item())
        with torch.no_grad():
            tensor[idx] = base
        fd = (vals[0] - vals[1]) / (2 * h)
        floor = 1e-13 * abs(l0.item()) / h
        assert abs(fd - grad[idx].item()) <= 1e-6 * max(abs(fd), 1e-3 * grad.abs().max().item()) + floor, \
            (idx, fd, grad[idx])


def test_relaxed_stress_loss_gradient_matches_central_differences():
    """Loss on relaxed stresses over strain points (each point relaxed for the current
    parameters): the implicit-differentiation gradient against central differences that
    re-relax every point (h = 1e-4 relative)."""
    import torch
    from scipy.optimize import minimize

    from micmec_gb300.autograd import energy_and_gradient, relaxed_stress

    s, part, params, pos, rng = _setup(n=3, seed=4)
    base_rv = np.array(s.domain.rvecs)
    pos0 = np.array(s.pos)
    strains = [0.0, 0.01, 0.02]
    targets = [torch.tensor(rng.normal(size=(3, 3)) * 1e-5, dtype=torch.float64, device="cuda") for _ in strains]

    def relax(x0):
        def f(x):
            pt = torch.tensor(x.reshape(-1, 3), dtype=torch.float64, device="cuda")
            with torch.no_grad():
                E, g = energy_and_gradient(pt, params)
            return float(E), g.cpu().numpy().ravel()

        r = minimize(f, x0.ravel(), jac=True, method="L-BFGS-B",
                     options=dict(gtol=1e-14, ftol=1e-22, maxiter=20000, maxcor=40))
        return r.x.reshape(-1, 3)

    def set_strain(e):
        F = np.eye(3)
        F[0, 0] += e
        rv = base_rv @ F
        s.domain.update_rvecs(rv)
        part.update_rvecs(rv)
        return F

    def loss_value():
        total = 0.0
        for e, tgt in zip(strains, targets):
            F = set_strain(e)
            x = torch.tensor(relax(pos0 @ F), dtype=torch.float64, device="cuda")
            with torch.no_grad():
                sig = relaxed_stress(x, params)
            total += float(((sig - tgt) ** 2).sum())
        return total

    # analytic gradient
    grads = [torch.zeros_like(t) for t in params.tensors()]
    for e, tgt in zip(strains, targets):
        F = set_strain(e)
        x = torch.tensor(relax(pos0 @ F), dtype=torch.float64, device="cuda")
        sig = relaxed_stress(x, params)
        loss = ((sig - tgt) ** 2).sum()
        for acc, gr in zip(grads, torch.autograd.grad(loss, list(params.tensors()))):
            acc += gr
    # central differences on a few parameters: C11 (type 0, state 0), h0_xx (type 1,
    # state 1), the free energy of type 0 state 1
    picks = [(0, (0, 0, 0)), (1, (1, 1, 0, 0)), (2, (0, 1))]
    for which, idx in picks:
        t = params.tensors()[which]
        v0 = float(t.data[idx])
        h = 1e-4 * abs(v0) if v0 != 0.0 else 1e-4 * float(t.data.abs().max())
        with torch.no_grad():
            t.data[idx] = v0 + h
            lp = loss_value()
            t.data[idx] = v0 - h
            lm = loss_value()
            t.data[idx] = v0
        fd = (lp - lm) / (2 * h)
        an = float(grads[which][idx])
        assert abs(an - fd) <= 1e-4 * abs(fd) + 1e-8 * abs(lp) / h, (which, idx, an, fd)
