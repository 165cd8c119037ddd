"""Adjoint of CheFSI w.r.t. the local potential: hand-written backward vs central finite
differences (h = 1e-5, frozen spectrum bounds) and vs the density of the summed states."""
import numpy as np
import pytest
import torch

from dftfe_gb300 import problems

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def adj(cuda):
    from dftfe_gb300 import adjoint
    return adjoint


def _setup(adj, n_iter=2, degree=8, seed=4, nwfc=12, nsum=6):
    pr = problems.make_problem(n=2, L=4.0, p=3, n_wells=2, n_wfc=nwfc, seed=seed, projectors=True)
    v0 = torch.from_numpy(
        pr.info["vjxw"] / np.broadcast_to(pr.mesh.quadrature()[1], pr.info["vjxw"].shape)).cuda()
    s = adj.AdjointSetup.from_problem(pr, n_iter=n_iter, n_sum=nsum, degree=degree, checkpoint=3)
    return pr, s, v0.contiguous()


def test_cell_assembly_matches_fe_module(adj, cuda):
    from dftfe_gb300 import chefsi
    pr, s, v0 = _setup(adj)
    mats = chefsi.assemble_cell_hamiltonians(s.shape, s.stiffness, (v0 * s.jxw).contiguous())
    ref = torch.from_numpy(pr.cell_mats).cuda()
    assert (mats - ref).abs().max().item() < 1e-12 * ref.abs().max().item()


def test_adjoint_matches_central_differences(adj):
    pr, s, v0 = _setup(adj)
    v = v0.clone().requires_grad_(True)
    L = adj.ritz_sum(v, s)
    L.backward()
    g = v.grad.detach().cpu().numpy()
    _, _, _, tape = adj.run_forward(s, v0)
    s.bounds_per_iter = [t[2] for t in tape]
    rng = np.random.default_rng(0)
    h = 1e-5
    idx = [(int(rng.integers(v0.shape[0])), int(rng.integers(v0.shape[1]))) for _ in range(8)]
    for c, q in idx:
        vp, vm = v0.clone(), v0.clone()
        vp[c, q] += h
        vm[c, q] -= h
        fd = (adj.run_forward(s, vp)[0] - adj.run_forward(s, vm)[0]) / (2 * h)
        assert abs(fd - g[c, q]) <= 2e-6 * max(1.0, abs(fd)) + 1e-8, (c, q, fd, g[c, q])


def test_adjoint_tends_to_density_at_convergence(adj):
    pr, s, v0 = _setup(adj, n_iter=12, degree=12)
    v = v0.clone().requires_grad_(True)
    adj.ritz_sum(v, s).backward()
    _, ev, X, _ = adj.run_forward(s, v0)
    rho = adj.density_term(s, X)
    g = v.grad.detach()
    rel = ((g - rho).abs().max() / rho.abs().max()).item()
    assert rel < 1e-4, rel
    # and the density integrates to the number of summed states
    assert abs(rho.sum().item() - s.n_sum) < 2e-2 * s.n_sum
