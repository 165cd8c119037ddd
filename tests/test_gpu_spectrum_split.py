"""Spectrum-split Rayleigh-Ritz (rayleighRitzGEPSpectrumSplitDirect) through the C ABI against
the FP64 oracle.

Tolerances: FP64 eigenvalues 1e-10 relative to the spectrum's scale, orthonormalised X and
XFrac projectors 1e-9; mixed (tensor-core Gram/rotation, three-term tensor-core H X, FP64 or
reduced fractional block) eigenvalues 2e-6 relative, XFrac projector 1e-5.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import dense_operator, oracle_op, small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def chefsi(cuda):
    from dftfe_gb300 import chefsi as C
    return C


def proj_diff(A, B):
    """max |A A^T - B B^T| (compares column spans, blind to signs and rotations)."""
    return float(np.abs(A @ A.T - B @ B.T).max())


def run_ss(C, op, X, n_occ, precision="fp64", frac_reduced=False):
    Xt = torch.from_numpy(X.copy()).cuda()
    XF = torch.empty((X.shape[0], X.shape[1] - n_occ), dtype=torch.float64, device="cuda")
    ev, HXF = C.rayleighRitzGEPSpectrumSplitDirect(op, Xt, XF, n_occ, precision=precision,
                                                   want_hx=True, frac_reduced=frac_reduced)
    return ev, Xt.cpu().numpy(), XF.cpu().numpy(), HXF.cpu().numpy()


@pytest.mark.parametrize("N,n_occ", [(24, 18), (16, 0), (16, 15), (40, 33)])
def test_spectrum_split_fp64_matches_oracle(chefsi, N, n_occ):
    pr = small_problem(projectors=True)
    op, ora = chefsi.KohnShamOperator.from_problem(pr), oracle_op(pr)
    X = np.random.default_rng(N + n_occ).standard_normal((pr.n_dofs, N))
    ev_o, Xo, XFo, HXFo = orc.rayleigh_ritz_spectrum_split(ora, X, n_occ)
    ev, Xg, XFg, HXFg = run_ss(chefsi, op, X, n_occ)
    scale = max(1.0, np.abs(ev_o).max())
    assert ev.shape == (N - n_occ,)
    assert np.abs(ev - ev_o).max() < 1e-10 * scale
    # Cholesky-GS is unique: the orthonormalised X itself matches
    assert np.abs(Xg - Xo).max() < 1e-9 * np.abs(Xo).max()
    assert np.abs(Xg.T @ Xg - np.eye(N)).max() < 1e-11
    assert proj_diff(XFg, XFo) < 1e-9
    assert np.abs(XFg.T @ XFg - np.eye(N - n_occ)).max() < 1e-10
    # H XFrac is the operator applied to XFrac, and XFrac holds Ritz pairs of span(X)
    A = dense_operator(pr)
    assert np.abs(HXFg - A @ XFg).max() < 1e-10 * scale
    assert np.abs(XFg.T @ HXFg - np.diag(ev)).max() < 1e-10 * scale


def test_spectrum_split_equals_top_of_full_rayleigh_ritz(chefsi):
    pr = small_problem(projectors=True)
    op = chefsi.KohnShamOperator.from_problem(pr)
    X = np.random.default_rng(5).standard_normal((pr.n_dofs, 30))
    ev_full, HXr = chefsi.rayleighRitzGEP(op, torch.from_numpy(X.copy()).cuda(), want_hx=True)
    ev, _, XFg, _ = run_ss(chefsi, op, X, 22)
    assert np.abs(ev - ev_full[22:]).max() < 1e-10 * max(1.0, np.abs(ev_full).max())


@pytest.mark.parametrize("frac_reduced", [False, True])
def test_spectrum_split_mixed_close_to_fp64(chefsi, frac_reduced):
    # N = 200 puts the Gram, rotation and H X products on the tensor-core paths; n_occ = 170
    # is not a multiple of the 400-vector block, so the FP64 block starts at vector 0
    pr = small_problem(n=4, L=8.0, p=3, wells=3, projectors=True)
    op, ora = chefsi.KohnShamOperator.from_problem(pr), oracle_op(pr)
    X = np.random.default_rng(11).standard_normal((pr.n_dofs, 200))
    ev_o, Xo, XFo, _ = orc.rayleigh_ritz_spectrum_split(ora, X, 170)
    ev, Xg, XFg, HXFg = run_ss(chefsi, op, X, 170, precision="mixed", frac_reduced=frac_reduced)
    scale = max(1.0, np.abs(ev_o).max())
    assert np.abs(ev - ev_o).max() < 2e-6 * scale, np.abs(ev - ev_o).max()
    assert np.abs(Xg.T @ Xg - np.eye(200)).max() < 1e-5
    assert proj_diff(XFg, XFo) < 1e-5


def test_spectrum_split_rejects_bad_arguments(chefsi):
    from dftfe_gb300._lib import ChefsiError
    pr = small_problem(projectors=True)
    op = chefsi.KohnShamOperator.from_problem(pr)
    Xt = torch.zeros((pr.n_dofs, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        chefsi.rayleighRitzGEPSpectrumSplitDirect(
            op, Xt, torch.zeros((pr.n_dofs, 3), dtype=torch.float64, device="cuda"), 4)
    with pytest.raises(ChefsiError):
        chefsi.rayleighRitzGEPSpectrumSplitDirect(
            op, Xt, torch.zeros((pr.n_dofs, 0), dtype=torch.float64, device="cuda"), 8)


def make_solvers(C, mixed, n=2):
    params = C.SolverParams(chebyshevOrder=10, rr_precision="fp32tc" if mixed else "fp64")
    out = [C.ChebyshevOrthogonalizedSubspaceIterationSolver(params) for _ in range(n)]
    for s in out:
        s.reinitSpectrumBounds(-3.0, 3.0, 12.0)
    return out


def test_solve_spectrum_split_matches_solve_fp64(chefsi):
    """One FP64 CheFSI iteration with the spectrum split gives the top Ritz values and the
    residual norms of the full iteration from the same input (the filter is identical)."""
    from dftfe_gb300 import problems
    pr = problems.make_problem(n=3, L=6.0, p=2, n_wells=3, n_wfc=12, seed=7, projectors=True)
    op = chefsi.KohnShamOperator.from_problem(pr)
    X0 = np.random.default_rng(3).uniform(-1, 1, (pr.n_dofs, 24))
    s_full, s_ss = make_solvers(chefsi, False)
    X1 = torch.from_numpy(X0.copy()).cuda()
    X2 = torch.from_numpy(X0.copy()).cuda()
    ev_f, res_f = s_full.solve(op, X1)
    ev_s, res_s, XF = s_ss.solveSpectrumSplit(op, X2, 18)
    assert np.abs(ev_s - ev_f[18:]).max() < 1e-10 * max(1.0, np.abs(ev_f).max())
    assert np.abs(res_s - res_f[18:]).max() < 1e-9
    Y = X2.cpu().numpy()
    assert np.abs(Y.T @ Y - np.eye(24)).max() < 1e-11
    # XFrac spans the top Ritz vectors of the full iteration
    assert proj_diff(XF.cpu().numpy(), X1.cpu().numpy()[:, 18:]) < 1e-8
    t = s_ss.timings(False)
    assert t["total"] > 0 and t["eig"] > 0


def test_solve_spectrum_split_mixed_no_worse_than_full(chefsi):
    """Mixed iteration (tensor-core filter, Gram, rotation and H X): its fractional Ritz values
    and residuals against the FP64 spectrum-split iteration stay within the error the mixed
    full iteration has against the FP64 full iteration (filtered blocks are ill-conditioned,
    and both reduced-precision Rayleigh-Ritz forms carry errors of O(2^-22 cond(L)))."""
    from dftfe_gb300 import problems
    pr = problems.make_problem(n=3, L=6.0, p=2, n_wells=3, n_wfc=12, seed=7, projectors=True)
    op = chefsi.KohnShamOperator.from_problem(pr)
    X0 = np.random.default_rng(3).uniform(-1, 1, (pr.n_dofs, 24))
    run = {}
    for mixed in (False, True):
        s_full, s_ss = make_solvers(chefsi, mixed)
        X1 = torch.from_numpy(X0.copy()).cuda()
        X2 = torch.from_numpy(X0.copy()).cuda()
        ev_f, _ = s_full.solve(op, X1, useMixedPrec=mixed)
        ev_s, res_s, XF = s_ss.solveSpectrumSplit(op, X2, 18, useMixedPrec=mixed)
        run[mixed] = (ev_f, ev_s, res_s, X2.cpu().numpy())
    scale = max(1.0, np.abs(run[False][0]).max())
    err_full = np.abs(run[True][0][18:] - run[False][0][18:]).max()
    err_ss = np.abs(run[True][1] - run[False][1]).max()
    assert err_ss < max(2e-6 * scale, 2.0 * err_full), (err_ss, err_full)
    assert np.abs(run[True][2] - run[False][2]).max() < 1e-4
    Y = run[True][3]
    assert np.abs(Y.T @ Y - np.eye(24)).max() < 1e-3
