"""Tensor-core (FP16 hi/lo split) dense products of the mixed Rayleigh-Ritz step against FP64.

The Gram product A^T B (long K) and the rotation X W (long M) run through the C ABI
(`chefsi_gemm` with CHEFSI_PREC_MIXED, `chefsi_overlap`, `chefsi_cholesky_gs`).

Tolerances, per element against b = |A|^T |B| (or |X| |W|):
  max |C - C_ref| / b <= 2^-15   (22-bit operand split, FP32 accumulation of 16-term MMA steps
                                  over <= 2048-term chunks, FP64 across chunks: worst case)
  rms(C - C_ref) / rms(b) <= 2^-19   (the typical error)
Columns are scaled over six decades so the per-column power-of-two scaling is exercised.
"""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def scaled(rng, M, N, decades=3.0):
    X = rng.standard_normal((M, N))
    return X * (10.0 ** rng.uniform(-decades, decades, N))[None, :]


def check_close(got, ref, bound):
    err = np.abs(got - ref)
    tiny = np.finfo(np.float64).tiny
    assert float((err / np.maximum(bound, tiny)).max()) <= 2.0 ** -15
    assert float(np.sqrt((err ** 2).mean()) / np.sqrt((bound ** 2).mean())) <= 2.0 ** -19


@pytest.mark.parametrize("M,N1,N2", [(1, 1, 1), (777, 70, 33), (64, 256, 256),
                                     (100003, 300, 130), (300007, 129, 129)])
def test_gram_tc_matches_fp64(C, M, N1, N2):
    rng = np.random.default_rng(M + 7 * N1 + N2)
    A = scaled(rng, M, N1)
    B = scaled(rng, M, N2)
    At, Bt = torch.from_numpy(A).cuda(), torch.from_numpy(B).cuda()
    got = C.gemm(At, Bt, ta="T", precision="mixed").cpu().numpy()
    check_close(got, A.T @ B, np.abs(A).T @ np.abs(B))


@pytest.mark.parametrize("M,N", [(5000, 70), (200001, 257)])
def test_gram_tc_same_operand(C, M, N):
    """A^T A with one operand: the diagonal tiles load A once."""
    rng = np.random.default_rng(M)
    A = scaled(rng, M, N)
    At = torch.from_numpy(A).cuda()
    got = C.gemm(At, At, ta="T", precision="mixed").cpu().numpy()
    check_close(got, A.T @ A, np.abs(A).T @ np.abs(A))


@pytest.mark.parametrize("M,K,N", [(1, 1, 1), (1000, 70, 70), (5000, 130, 257),
                                   (70001, 300, 300)])
def test_rotation_tc_matches_fp64(C, M, K, N):
    rng = np.random.default_rng(M + K + N)
    X = scaled(rng, M, K)
    W = rng.standard_normal((K, N)) * (10.0 ** rng.uniform(-3, 3, (K, 1)))
    got = C.gemm(torch.from_numpy(X).cuda(), torch.from_numpy(W).cuda(),
                 precision="mixed").cpu().numpy()
    check_close(got, X @ W, np.abs(X) @ np.abs(W))


def test_overlap_tc_lower_tiles(C):
    """chefsi_overlap (lower 128x128 tiles, mirrored) on a 64,000-dof operator."""
    from dftfe_gb300 import problems
    pr = problems.make_problem(n=10, L=15.0, p=4, n_wells=2, n_wfc=8, seed=3)
    op = C.KohnShamOperator.from_problem(pr)
    rng = np.random.default_rng(5)
    X = scaled(rng, pr.n_dofs, 300)
    S = op.overlap(torch.from_numpy(X).cuda(), "mixed").cpu().numpy()
    check_close(S, X.T @ X, np.abs(X).T @ np.abs(X))


def test_cholesky_gs_mixed_in_place(C):
    """The in-place tensor-core rotation inside Cholesky-GS leaves an orthonormal block."""
    from dftfe_gb300 import problems
    pr = problems.make_problem(n=10, L=15.0, p=4, n_wells=2, n_wfc=8, seed=3)
    op = C.KohnShamOperator.from_problem(pr)
    X = np.random.default_rng(9).standard_normal((pr.n_dofs, 200))
    Xt = torch.from_numpy(X).cuda()
    C.pseudoGramSchmidtOrthogonalization(op, Xt, precision="mixed")
    Y = Xt.cpu().numpy()
    assert np.abs(Y.T @ Y - np.eye(200)).max() < 1e-5
    # same span: the projection of X onto span(Y) is X (formed as Y (Y^T X))
    assert np.abs(Y @ (Y.T @ X) - X).max() < 1e-4 * np.abs(X).max()
