"""The memory-bounded (column-blocked, row-slabbed) Rayleigh-Ritz step against the full-size
one on the same filtered block, FP64 and mixed.

Tolerances: FP64 Ritz values 1e-10 relative to the spectrum's scale and residual norms 1e-9;
mixed (tensor-core Gram per row slab with its own exponents, three-term tensor-core H X per
column block) Ritz values 2e-6 relative against the full-size mixed step and against FP64.
"""
import numpy as np
import pytest
import torch

from tests.helpers import small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def iterate(C, op, X0, mixed, bounds=(-3.0, 3.0, 12.0), degree=10, **kw):
    s = C.ChebyshevOrthogonalizedSubspaceIterationSolver(C.SolverParams(
        chebyshevOrder=degree, rr_precision="fp32tc" if mixed else "fp64", **kw))
    s.reinitSpectrumBounds(*bounds)
    X = torch.from_numpy(X0.copy()).cuda()
    ev, res = s.solve(op, X, useMixedPrec=mixed)
    return ev, res, X.cpu().numpy()


@pytest.mark.parametrize("block,slab", [(8, 64), (7, 100), (24, 0)])
def test_blocked_rr_fp64_matches_full(C, block, slab):
    from dftfe_gb300 import problems
    pr = problems.make_problem(n=3, L=6.0, p=2, n_wells=3, n_wfc=12, seed=7, projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    X0 = np.random.default_rng(3).uniform(-1, 1, (pr.n_dofs, 24))
    ev_f, res_f, X_f = iterate(C, op, X0, False, rr_block=-1)
    ev_b, res_b, X_b = iterate(C, op, X0, False, rr_block=block, rr_slab_rows=slab)
    scale = max(1.0, np.abs(ev_f).max())
    assert np.abs(ev_b - ev_f).max() < 1e-10 * scale
    assert np.abs(res_b - res_f).max() < 1e-9
    assert np.abs(X_b.T @ X_b - np.eye(24)).max() < 1e-10
    # the lowest 12 Ritz vectors span the same space
    P_f, P_b = X_f[:, :12] @ X_f[:, :12].T, X_b[:, :12] @ X_b[:, :12].T
    assert np.abs(P_f - P_b).max() < 1e-8


def test_blocked_rr_mixed_matches_full(C):
    """64 vectors in two column blocks of 32 and four row slabs; a degree-4 filter keeps the
    block well conditioned, so the two mixed forms differ only by rounding."""
    pr = small_problem(n=4, L=8.0, p=3, wells=3, projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    lo, up = C.lanczosLowerUpperBoundEigenSpectrum(op, 20)
    bounds = (lo, lo + 0.3 * (up - lo), up)
    X0 = np.random.default_rng(5).uniform(-1, 1, (pr.n_dofs, 64))
    kw = dict(bounds=bounds, degree=4)
    ev_f, res_f, _ = iterate(C, op, X0, True, rr_block=-1, **kw)
    ev_b, res_b, X_b = iterate(C, op, X0, True, rr_block=32, rr_slab_rows=512, **kw)
    ev_d, _, _ = iterate(C, op, X0, False, rr_block=-1, **kw)
    scale = max(1.0, np.abs(ev_d).max())
    assert np.abs(ev_b - ev_f).max() < 2e-6 * scale
    assert np.abs(ev_b[:16] - ev_d[:16]).max() < 1e-5 * scale
    assert np.abs(res_b - res_f).max() < 1e-4 * max(1.0, res_f.max())
    assert np.abs(X_b.T @ X_b - np.eye(64)).max() < 1e-4
