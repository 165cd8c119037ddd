"""GPU parity tests: every CheFSI stage through the C ABI against the FP64 oracle.

Tolerances (written per test): FP64 stages <= 1e-12 relative (HX) / 1e-10 (filter, Ritz);
FP32 SIMT HX <= 2e-6 relative; the mixed (FP16-split tensor-core) HX and the three-term split
(fp32tc) HX <= 2e-6 relative;
mixed CheFSI Ritz values <= 1e-6 Ha.
"""
import os

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import cheb_scalar, dense_operator, oracle_op, small_problem, unfolded_setup

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


@pytest.fixture(scope="module")
def chefsi(cuda):
    from dftfe_gb300 import chefsi as C
    return C


def gpu_op(C, pr, **kw):
    return C.KohnShamOperator.from_problem(pr, **kw)


@pytest.mark.parametrize("p,n,proj,B", [(2, 3, True, 8), (4, 2, True, 37), (3, 2, False, 1),
                                        (6, 2, True, 64)])
def test_hx_fp64_matches_oracle(chefsi, p, n, proj, B):
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=2, projectors=proj)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(p).standard_normal((pr.n_dofs, B))
    Y = op.apply(torch.from_numpy(X).cuda()).cpu().numpy()
    assert rel(Y, ora.HX(X)) < 1e-12


def test_hx_scaleflag_semantics(chefsi):
    pr = small_problem(projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(1).standard_normal((pr.n_dofs, 6))
    D = np.random.default_rng(2).standard_normal((pr.n_dofs, 6))
    d = torch.from_numpy(D).cuda()
    op.HX(torch.from_numpy(X).cuda(), d, scalar=0.37, scaleFlag=True)
    ref = ora.HX(X, scalar=0.37, dst=D.copy(), accumulate=True)
    assert rel(d.cpu().numpy(), ref) < 1e-12


@pytest.mark.parametrize("prec,p,n,B", [("fp32", 4, 2, 96), ("mixed", 4, 2, 96),
                                         ("mixed", 6, 2, 136), ("mixed", 2, 3, 8),
                                         ("mixed", 5, 2, 256), ("fp32tc", 4, 2, 96),
                                         ("fp32tc", 6, 2, 136), ("fp32tc", 2, 3, 8),
                                         ("fp32tc", 5, 2, 256)])
def test_hx_reduced_precision(chefsi, prec, p, n, B):
    """FP32 SIMT and tensor-core (FP16-split) HX: cell sizes with one K-block (p = 2), one
    row half (p = 4, 5) and two row halves (p = 6); partial and several 128-vector chunks."""
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=2, projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(5).uniform(-1, 1, (pr.n_dofs, B))
    Xt = torch.from_numpy(X).float().cuda()
    Y = torch.zeros_like(Xt)
    try:
        op.HX(Xt, Y, precision=prec)
    except Exception as e:  # tensor path must exist on sm_103a
        pytest.fail(f"{prec} HX failed: {e}")
    ref = ora.HX(Xt.double().cpu().numpy())
    assert rel(Y.double().cpu().numpy(), ref) < 2e-6


@pytest.mark.parametrize("p,n,B", [(6, 2, 128), (4, 3, 64)])
def test_hx_tc_three_term_split_is_fp32_class(chefsi, p, n, B):
    """The three-term split apply (FP32 operands exactly, six products, FP32 accumulation) is
    as accurate as the FP32 SIMT apply: both against the FP64 oracle on the FP32-rounded
    input, with inputs spanning three decades per vector."""
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=2, projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    rng = np.random.default_rng(11)
    X = rng.uniform(-1, 1, (pr.n_dofs, B)) * 10.0 ** rng.uniform(-3, 0, B)[None, :]
    Xt = torch.from_numpy(X).float().cuda()
    ref = ora.HX(Xt.double().cpu().numpy())
    errs = {}
    for prec in ("fp32", "fp32tc", "mixed"):
        Y = torch.zeros_like(Xt)
        op.HX(Xt, Y, precision=prec)
        d = Y.double().cpu().numpy() - ref
        errs[prec] = float(np.sqrt((d ** 2).mean()) / np.sqrt((ref ** 2).mean()))
    assert errs["fp32tc"] <= 2.0 * errs["fp32"] + 1e-8, errs
    assert errs["fp32tc"] < errs["mixed"], errs


@pytest.mark.parametrize("p,n,B", [(4, 3, 40), (6, 2, 128), (3, 1, 16)])
def test_hx_tc_accumulates_into_owned_and_shared_rows(chefsi, p, n, B):
    """dst += scalar * A X on the tensor path: rows owned by one cell (plain load + store)
    and rows shared by several cells (reductions) both keep dst's previous value. n = 1 is a
    single periodic cell whose own nodes fold onto the same dofs (no owned face rows)."""
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=2, projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    rng = np.random.default_rng(p + n)
    X = rng.uniform(-1, 1, (pr.n_dofs, B))
    D = rng.uniform(-1, 1, (pr.n_dofs, B))
    Xt = torch.from_numpy(X).float().cuda()
    Dt = torch.from_numpy(D).float().cuda()
    op.HX(Xt, Dt, scalar=-0.61, scaleFlag=True, precision="mixed")
    ref = ora.HX(Xt.double().cpu().numpy(), scalar=-0.61,
                 dst=D.astype(np.float32).astype(np.float64), accumulate=True)
    assert rel(Dt.double().cpu().numpy(), ref) < 2e-6


def test_hx_complex_matches_oracle(chefsi):
    pr = small_problem(n=2, L=4.0, p=3, wells=2, kpoint=[0.2, -0.1, 0.3])
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    rng = np.random.default_rng(9)
    X = rng.standard_normal((pr.n_dofs, 5)) + 1j * rng.standard_normal((pr.n_dofs, 5))
    Y = op.apply(torch.from_numpy(X).cuda()).cpu().numpy()
    assert rel(Y, ora.HX(X)) < 1e-12


def test_hx_constraint_rows_match_oracle(chefsi):
    pr = small_problem(n=2, L=4.0, p=2, wells=2)
    emap, n_ext, cons, mass_ext = unfolded_setup(pr)
    op = chefsi.KohnShamOperator(emap, pr.cell_mats, np.sqrt(mass_ext), 1 / np.sqrt(mass_ext),
                                 n_ext, constraints=cons)
    ora = orc.OracleOperator(emap, pr.cell_mats, 1 / np.sqrt(mass_ext), n_ext, constraints=cons)
    X = np.random.default_rng(3).standard_normal((n_ext, 4))
    Y = op.apply(torch.from_numpy(X).cuda()).cpu().numpy()
    assert rel(Y, ora.HX(X)) < 1e-12


def test_filter_fp64_matches_oracle_and_polynomial(chefsi):
    pr = small_problem(projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    A = dense_operator(pr)
    lam, Q = np.linalg.eigh(A)
    X = np.random.default_rng(4).standard_normal((pr.n_dofs, 9))
    a, b, a0, m = lam[20], lam[-1] + 0.5, lam[0] - 0.5, 9
    Xt = torch.from_numpy(X).cuda()
    chefsi.chebyshevFilter(op, Xt, m, a, b, a0)
    ref = ora.chebyshev_filter(X, m, a, b, a0)
    poly = Q @ (cheb_scalar(lam, m, a, b, a0)[:, None] * (Q.T @ X))
    assert rel(Xt.cpu().numpy(), ref) < 1e-10
    assert rel(ref, poly) < 1e-10


# The default mixed filter carries the Chebyshev shift c on the tensor-core tiles' diagonals.
# Its per-cell partial sums are then ~ c |x| in size instead of ~ |A x| (small for the smooth,
# wanted components), and the tensor core's FP32 accumulation, which behaves like
# round-toward-zero after each K = 16 step (a CPU model with that rounding reproduces the
# measured errors of both the shifted and the unshifted filter), leaves a bias of ~2^-23 per
# step relative to those sums: about 1e-5 of max |p(A) X| after 10 to 30 degrees, against 5e-7
# with the shift applied in FP32 by a recurrence pass. The Ritz values do not see it (they are
# set by the Rayleigh-Ritz step: the 20-iteration 64,000-dof test holds 1e-6 Ha either way).
MIXED_SHIFTED_TOL = 4e-5


def test_filter_mixed_close_to_fp64(chefsi):
    pr = small_problem(n=2, L=4.0, p=4, wells=2, projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(7).uniform(-1, 1, (pr.n_dofs, 32))
    lo, up = orc.lanczos_bounds(ora, np.ones(pr.n_dofs), 20)
    Xt = torch.from_numpy(X).cuda()
    chefsi.chebyshevFilter(op, Xt, 10, lo + 0.3 * (up - lo), up, lo, precision="mixed")
    ref = ora.chebyshev_filter(X, 10, lo + 0.3 * (up - lo), up, lo)
    assert rel(Xt.cpu().numpy(), ref) < MIXED_SHIFTED_TOL


def test_filter_mixed_after_cell_matrix_update(chefsi):
    """An SCF step replaces the cell matrices: the filter plan keeps its map and projector
    tables and rebuilds its tiles on the device (new scale, new diagonals, the projector
    columns re-scattered). The mixed filter and the mixed HX after the update match the oracle
    of the new matrices, and a second update back to the first matrices reproduces the first
    filter."""
    pr = small_problem(n=2, L=4.0, p=4, wells=2, projectors=True)
    op = gpu_op(chefsi, pr)
    X = np.random.default_rng(9).uniform(-1, 1, (pr.n_dofs, 32))
    mats2 = 1.7 * pr.cell_mats + 0.3 * np.swapaxes(pr.cell_mats, 1, 2)
    out = []
    for mats in (pr.cell_mats, mats2, pr.cell_mats):
        op.update_cell_matrices(torch.from_numpy(np.ascontiguousarray(mats)).cuda())
        ora = orc.OracleOperator(pr.cell_map, mats, pr.inv_sqrt_mass, pr.n_dofs,
                                 projectors=pr.nonlocal_)
        lo, up = orc.lanczos_bounds(ora, np.ones(pr.n_dofs), 20)
        a = lo + 0.3 * (up - lo)
        Xt = torch.from_numpy(X.copy()).cuda()
        chefsi.chebyshevFilter(op, Xt, 10, a, up, lo, precision="mixed")
        out.append(Xt.cpu().numpy())
        assert rel(out[-1], ora.chebyshev_filter(X, 10, a, up, lo)) < MIXED_SHIFTED_TOL
        Y = torch.zeros((pr.n_dofs, 32), dtype=torch.float32, device="cuda")
        op.HX(torch.from_numpy(X.astype(np.float32)).cuda(), Y, precision="mixed")
        assert rel(Y.cpu().numpy(), ora.HX(X.astype(np.float32).astype(np.float64))) < 2e-6
    assert rel(out[2], out[0]) < 1e-5   # reduction order differs between runs


def test_filter_mixed_shift_beyond_tiles_falls_back(chefsi):
    """A damped interval reaching far past the spectrum puts the Chebyshev shift c beyond what
    the FP16 tiles' diagonals can hold (here c / max|A| ~ 19): the default filter then runs
    the recurrence pass with the shift in FP32 and meets that variant's 5e-6 bound; a normal
    filter afterwards on the same operator takes the shifted path again."""
    pr = small_problem(n=2, L=4.0, p=4, wells=2, projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(8).uniform(-1, 1, (pr.n_dofs, 32))
    lo, up = orc.lanczos_bounds(ora, np.ones(pr.n_dofs), 20)
    a, b = lo + 0.3 * (up - lo), 8.0 * up
    Xt = torch.from_numpy(X.copy()).cuda()
    chefsi.chebyshevFilter(op, Xt, 10, a, b, lo, precision="mixed")
    assert rel(Xt.cpu().numpy(), ora.chebyshev_filter(X, 10, a, b, lo)) < 5e-6
    Xt = torch.from_numpy(X.copy()).cuda()
    chefsi.chebyshevFilter(op, Xt, 10, a, up, lo, precision="mixed")
    assert rel(Xt.cpu().numpy(), ora.chebyshev_filter(X, 10, a, up, lo)) < MIXED_SHIFTED_TOL


@pytest.mark.parametrize("N,degenerate", [(1, False), (7, False), (50, False), (130, True),
                                          (257, True)])
def test_syevd_matches_numpy(chefsi, N, degenerate):
    rng = np.random.default_rng(N)
    Q, _ = np.linalg.qr(rng.standard_normal((N, N)))
    w = np.sort(rng.standard_normal(N))
    if degenerate and N > 10:
        w[3:9] = w[3]
        w[20:23] = w[20] + np.array([0, 1e-13, 2e-13])
    A = (Q * w) @ Q.T
    A = 0.5 * (A + A.T)
    wg, Z = chefsi.syevd(torch.from_numpy(A).cuda())
    wg, Z = wg.cpu().numpy(), Z.cpu().numpy()
    assert np.abs(wg - np.linalg.eigvalsh(A)).max() < 1e-12 * max(1, np.abs(w).max()) * N
    assert np.abs(Z.T @ Z - np.eye(N)).max() < 1e-10
    assert np.abs(A @ Z - Z * wg).max() < 1e-10 * max(1, np.abs(w).max())


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-13), ("mixed", 2e-6)])
def test_overlap_and_xthx(chefsi, prec, tol):
    pr = small_problem(n=3, L=6.0, p=3, wells=2, projectors=True)
    op = gpu_op(chefsi, pr)
    A = dense_operator(pr)
    X = np.random.default_rng(8).standard_normal((pr.n_dofs, 70))
    Xt = torch.from_numpy(X).cuda()
    S = op.overlap(Xt, prec).cpu().numpy()
    Hp = op.XtHX(Xt, prec).cpu().numpy()
    assert rel(S, X.T @ X) < tol
    assert rel(Hp, X.T @ A @ X) < tol


def test_cholesky_gs_orthonormalises(chefsi):
    pr = small_problem(projectors=True)
    op = gpu_op(chefsi, pr)
    X = np.random.default_rng(2).standard_normal((pr.n_dofs, 20))
    Xt = torch.from_numpy(X).cuda()
    chefsi.pseudoGramSchmidtOrthogonalization(op, Xt)
    Y = Xt.cpu().numpy()
    assert np.abs(Y.T @ Y - np.eye(20)).max() < 1e-12
    # same span
    P = Y @ Y.T
    assert np.abs(P @ X - X).max() < 1e-10 * np.abs(X).max()


def test_rayleigh_ritz_matches_oracle(chefsi):
    pr = small_problem(projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(6).standard_normal((pr.n_dofs, 16))
    ev_o, Xo, HXo = orc.rayleigh_ritz_gep(ora, X)
    ev_g = chefsi.rayleighRitzGEP(op, torch.from_numpy(X.copy()).cuda())
    assert np.abs(ev_g - ev_o).max() < 1e-10 * max(1.0, np.abs(ev_o).max())


def test_residual_norms(chefsi):
    pr = small_problem(projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(1).standard_normal((pr.n_dofs, 10))
    lam = np.linspace(-1, 1, 10)
    r_g = chefsi.computeEigenResidualNorm(op, torch.from_numpy(X).cuda(), lam)
    assert rel(r_g, ora.residual_norms(X, lam)) < 1e-12


def test_lanczos_bounds_match_oracle(chefsi):
    pr = small_problem(projectors=True)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    v0 = np.random.default_rng(0).uniform(0, 1, pr.n_dofs)
    assert chefsi.lanczosLowerUpperBoundEigenSpectrum(op, 20, False, v0) == \
        orc.lanczos_bounds(ora, v0, 20)


def test_solve_reproduces_golden_fixture(chefsi):
    from dftfe_gb300 import problems
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "small_p2.npz"))
    pr = problems.make_problem(n=3, L=6.0, p=2, n_wells=3, n_wfc=12, seed=7, projectors=True)
    op = gpu_op(chefsi, pr)
    for mixed, tol in ((False, 1e-10), (True, 1e-6)):
        s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(
            chefsi.SolverParams(chebyshevOrder=10))
        s.reinitSpectrumBounds(-3.0, 3.0, 12.0)
        X = torch.from_numpy(g["X"].copy()).cuda()
        for _ in range(5):
            ev, res = s.solve(op, X, useMixedPrec=mixed)
            s.reinitSpectrumBounds(ev[0], ev[-1], 12.0)
        occ = 6
        assert np.abs(ev[:occ] - g["ritz"][:occ]).max() < tol, (mixed, ev - g["ritz"])
        if not mixed:
            assert np.abs(ev - g["ritz"]).max() < tol
            assert np.abs(res - g["res"]).max() < 1e-8


def test_hx_golden_fixture(chefsi):
    from dftfe_gb300 import problems
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "small_p2.npz"))
    pr = problems.make_problem(n=3, L=6.0, p=2, n_wells=3, n_wfc=12, seed=7, projectors=True)
    op = gpu_op(chefsi, pr)
    Y = op.apply(torch.from_numpy(g["X"]).cuda()).cpu().numpy()
    assert rel(Y, g["hx"]) < 1e-12


@pytest.mark.parametrize("p,n,B,proj", [(2, 3, 8, True), (4, 2, 136, True), (6, 2, 136, True),
                                        (5, 2, 256, True), (4, 3, 64, False)])
def test_filter_variants_match_oracle(chefsi, p, n, B, proj):
    """The four mixed tensor-core filters against the oracle's FP64 filter (relative to
    max |p(A) X|: 5e-6, the shifted default MIXED_SHIFTED_TOL) and against each other:
    * folded: one HX launch per degree with the shift c on the tiles' diagonals and the
      nonlocal apply as extra tensor-core K columns of the cell matrices (the projector
      coefficients 2^t C^T x as extra split rows), reducing into the older vector's buffer;
    * axpby: recurrence pass + the same HX launch without the shift;
    * fused: the recurrence finished in the HX launch's epilogue (vectors kept as FP16 hi + lo);
    * separate: recurrence pass, HX launch and the SIMT nonlocal kernels.
    Cell sizes with one K-block of nodes (p = 2, several atoms per cell), one row half (p = 4,
    5) and two (p = 6); partial and several 128-vector chunks; a second filter call on the same
    solver."""
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=3, projectors=proj)
    op, ora = gpu_op(chefsi, pr), oracle_op(pr)
    X = np.random.default_rng(p + B).uniform(-1, 1, (pr.n_dofs, B))
    lo, up = orc.lanczos_bounds(ora, np.ones(pr.n_dofs), 20)
    a, b, a0, m = lo + 0.3 * (up - lo), up, lo, 10
    ref = ora.chebyshev_filter(X, m, a, b, a0)
    out = {}
    for variant in ("separate", "folded", "axpby", "fused"):
        s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(chefsi.SolverParams(
            chebyshevOrder=m, chebyWfcBlockSize=B, wfcBlockSize=B, filter_variant=variant))
        s.reinitSpectrumBounds(a0, a, b)
        for _ in range(2):
            Xt = torch.from_numpy(X.copy()).cuda()
            s.solveNoRR(op, Xt, 1, useMixedPrec=True)
        out[variant] = Xt.cpu().numpy()
        tol = MIXED_SHIFTED_TOL if variant == "folded" else 5e-6
        assert rel(out[variant], ref) < tol, variant
        assert rel(out[variant], out.get("separate", ref)) < tol + 5e-6, variant


def _unfolded_operators(chefsi, pr, projectors):
    """The problem's operator on the unfolded lattice with periodicity as constraint rows
    (slave = master, weight 1), on the GPU and in the oracle; projectors (optional) moved to
    the masters' extended numbering."""
    from dftfe_gb300 import fe
    emap, n_ext, cons, mass_ext = unfolded_setup(pr)
    nl = None
    if projectors and pr.nonlocal_ is not None:
        npt, m = pr.mesh.npts, pr.mesh.npts + 1
        f = pr.nonlocal_.dofs.astype(np.int64)
        ext = (f % npt) + m * ((f // npt) % npt + m * (f // (npt * npt)))
        nl = fe.NonlocalProjectors(pr.nonlocal_.n_atoms, pr.nonlocal_.n_proj, pr.nonlocal_.ptr,
                                   ext.astype(np.int32), pr.nonlocal_.values,
                                   pr.nonlocal_.couplings)
    op = chefsi.KohnShamOperator(emap, pr.cell_mats, np.sqrt(mass_ext), 1 / np.sqrt(mass_ext),
                                 n_ext, projectors=nl, constraints=cons)
    ora = orc.OracleOperator(emap, pr.cell_mats, 1 / np.sqrt(mass_ext), n_ext, projectors=nl,
                             constraints=cons)
    return op, ora, n_ext, cons[0]


@pytest.mark.parametrize("p,n,B,proj", [(4, 2, 96, False), (2, 3, 8, True), (6, 2, 136, False),
                                        (4, 2, 64, True)])
def test_hx_tensor_cores_with_constraint_rows(chefsi, p, n, B, proj):
    """The mixed (tensor-core) HX of an operator with constraint rows (the periodic cube
    unfolded, periodicity as slave rows): distribute on the FP16 split rows, the plan's tiles
    with M^{-1/2} folded in, the adjoint after the launch; against the oracle's constrained HX,
    2e-6 relative (the tolerance of the unconstrained tensor-core HX)."""
    pr = small_problem(n=n, L=2.0 * n, p=p, wells=3, projectors=proj)
    op, ora, n_ext, _ = _unfolded_operators(chefsi, pr, proj)
    X = np.random.default_rng(p + B).uniform(-1, 1, (n_ext, B))
    Xt = torch.from_numpy(X).float().cuda()
    Y = torch.zeros_like(Xt)
    op.HX(Xt, Y, precision="mixed")
    ref = ora.HX(Xt.double().cpu().numpy())
    assert rel(Y.double().cpu().numpy(), ref) < 2e-6


def test_mixed_solve_with_constraint_rows_matches_oracle(chefsi):
    """Ten mixed CheFSI iterations (tensor-core filter with the constraint rows, mixed
    Rayleigh-Ritz) on the unfolded periodic operator with projectors, from X0 with zero slave
    rows (as DFT-FE keeps them), with the oracle's bounds before every iteration: the occupied
    Ritz values within 1e-6 Ha of the oracle's FP64 CheFSI."""
    pr = small_problem(n=3, L=6.0, p=4, wells=3, nwfc=16, seed=5, projectors=True)
    op, ora, n_ext, slaves = _unfolded_operators(chefsi, pr, True)
    X0 = np.random.default_rng(9).uniform(-1, 1, (n_ext, 16))
    X0[slaves] = 0.0
    lo, up = orc.lanczos_bounds(ora, np.ones(n_ext), 20)
    st = orc.SolverState(lo, lo + 0.3 * (up - lo), up)
    s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(chefsi.SolverParams(
        chebyshevOrder=16, chebyWfcBlockSize=16, wfcBlockSize=16, rr_precision="fp32tc"))
    Xo, Xg = X0.copy(), torch.from_numpy(X0.copy()).cuda()
    for _ in range(10):
        s.reinitSpectrumBounds(st.a0, st.b_low, st.b_up)
        ev, _ = s.solve(op, Xg, useMixedPrec=True)
        ev_o, res_o, Xo = orc.solve(ora, Xo, st, m=16)
    assert np.abs(ev[:8] - ev_o[:8]).max() < 1e-6, ev[:8] - ev_o[:8]
