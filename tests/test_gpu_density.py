"""Electron density of the Ritz vectors at the quadrature points (`chefsi_density`, DFT-FE's
densityCalculator) against the oracle's direct interpolate-square-sum: FP64 to 1e-12, the
tensor-core path to 2e-5 of the largest value."""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import small_problem

pytestmark = pytest.mark.gpu


def quadrature(pr):
    """Shape values [n_q][n_e] at the (p+3)^3 Gauss points and JxW [n_cells][n_q]."""
    from dftfe_gb300 import fe
    mesh = pr.mesh
    nq1 = mesh.p + 3
    xq, _ = fe.gauss_nodes_weights(nq1)
    phi, _ = mesh.shape_1d(xq)
    q = np.arange(nq1 ** 3)
    qx, qy, qz = q % nq1, (q // nq1) % nq1, q // (nq1 * nq1)
    i = np.arange(mesh.nodes_per_cell)
    p1 = mesh.p + 1
    N = phi[qx][:, i % p1] * phi[qy][:, (i // p1) % p1] * phi[qz][:, i // (p1 * p1)]
    _, w3 = mesh.quadrature(nq1)
    return N, np.broadcast_to(w3, (mesh.n_cells, len(w3))).copy()


@pytest.mark.parametrize("p,n,N", [(2, 3, 8), (4, 2, 37), (6, 2, 16)])
def test_density_matches_oracle(cuda, p, n, N):
    from dftfe_gb300 import chefsi as C
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=2)
    op = C.KohnShamOperator.from_problem(pr)
    rng = np.random.default_rng(p + n)
    X = rng.standard_normal((pr.n_dofs, N))
    occ = rng.uniform(0.0, 2.0, N)
    shape, jxw = quadrature(pr)
    ref = orc.density(pr.cell_map, pr.inv_sqrt_mass, shape, X, occ, jxw)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    rho = C.density(op, t(X), t(occ), t(shape), t(jxw)).cpu().numpy()
    assert np.abs(rho - ref).max() <= 1e-12 * np.abs(ref).max()
    # accumulate: a second set of states (another k-point / spin) adds
    X2 = rng.standard_normal((pr.n_dofs, N))
    ref2 = ref + orc.density(pr.cell_map, pr.inv_sqrt_mass, shape, X2, occ, jxw)
    rho2 = C.density(op, t(X2), t(occ), t(shape), t(jxw), rho=t(rho), accumulate=True)
    assert np.abs(rho2.cpu().numpy() - ref2).max() <= 1e-12 * np.abs(ref2).max()


@pytest.mark.parametrize("p,n,N", [(2, 3, 8), (4, 2, 136), (6, 2, 256)])
def test_density_tensor_cores_match_oracle(cuda, p, n, N):
    """The tensor-core density (FP16 split of M^{-1/2} x and of the shape functions, FP32
    accumulation; quadrature points in one, two or three row parts): within 2e-5 of the
    largest density value of the FP64 oracle."""
    from dftfe_gb300 import chefsi as C
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=2)
    op = C.KohnShamOperator.from_problem(pr)
    rng = np.random.default_rng(3 * p + n)
    X = rng.standard_normal((pr.n_dofs, N))
    occ = rng.uniform(0.0, 2.0, N)
    shape, jxw = quadrature(pr)
    ref = orc.density(pr.cell_map, pr.inv_sqrt_mass, shape, X, occ, jxw)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    rho = C.density(op, t(X), t(occ), t(shape), t(jxw), precision="mixed").cpu().numpy()
    assert np.abs(rho - ref).max() <= 2e-5 * np.abs(ref).max()
    rho2 = C.density(op, t(X), t(occ), t(shape), t(jxw), rho=t(rho), accumulate=True,
                     precision="mixed").cpu().numpy()
    assert np.abs(rho2 - 2 * ref).max() <= 4e-5 * np.abs(ref).max()


def test_density_integrates_to_the_electron_count(cuda):
    """For the lowest eigenvectors of the operator (M^{1/2}-scaled, orthonormal: CheFSI's
    basis) sum_q rho JxW = sum_i f_i up to the difference between the GLL-lumped mass and the
    Gauss quadrature of smooth states (0.05% at p = 4)."""
    from dftfe_gb300 import chefsi as C
    from tests.helpers import oracle_op
    pr = small_problem(n=2, L=4.0, p=4, wells=2)
    op = C.KohnShamOperator.from_problem(pr)
    _, V = np.linalg.eigh(oracle_op(pr).dense())
    X = V[:, :6]
    occ = np.full(6, 2.0)
    shape, jxw = quadrature(pr)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    rho = C.density(op, t(X), t(occ), t(shape), t(jxw)).cpu().numpy()
    assert abs(rho.sum() - occ.sum()) < 2e-3 * occ.sum()
