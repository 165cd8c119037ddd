"""Complex (Bloch) Rayleigh-Ritz path through the C ABI against FP64 references.

Tolerances: Hermitian eigensolver eigenvalues <= 1e-12 |A|, residual and orthogonality
<= 1e-10; FP64 complex Rayleigh-Ritz and CheFSI <= 1e-10 Ha against the oracle; the mixed
step (real-view tensor-core Gram products and rotation) <= 1e-6 Ha.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import oracle_op, small_problem

pytestmark = pytest.mark.gpu

K = [0.2, -0.1, 0.3]


@pytest.fixture(scope="module")
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


@pytest.mark.parametrize("N,degenerate", [(1, False), (2, False), (37, False), (130, True)])
def test_heevd_matches_numpy(C, N, degenerate):
    rng = np.random.default_rng(N)
    if degenerate:
        Q, _ = np.linalg.qr(rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N)))
        w = np.sort(rng.standard_normal(N))
        w[10:14] = w[10]
        w[50:53] = w[50]
        A = (Q * w) @ Q.conj().T
    else:
        B = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
        A = B + B.conj().T
    A = 0.5 * (A + A.conj().T)
    wg, Z = C.syevd(torch.from_numpy(A).cuda())
    wg, Z = wg.cpu().numpy(), Z.cpu().numpy()
    scale = max(1.0, np.abs(np.linalg.eigvalsh(A)).max())
    assert np.abs(wg - np.linalg.eigvalsh(A)).max() < 1e-12 * scale * max(N, 1)
    assert np.abs(Z.conj().T @ Z - np.eye(N)).max() < 1e-10
    assert np.abs(A @ Z - Z * wg).max() < 1e-10 * scale


def test_cholesky_gs_complex(C):
    pr = small_problem(n=2, L=4.0, p=3, wells=2, kpoint=K)
    op = C.KohnShamOperator.from_problem(pr)
    rng = np.random.default_rng(4)
    X = rng.standard_normal((pr.n_dofs, 20)) + 1j * rng.standard_normal((pr.n_dofs, 20))
    Xt = torch.from_numpy(X.copy()).cuda()
    C.pseudoGramSchmidtOrthogonalization(op, Xt)
    Y = Xt.cpu().numpy()
    assert np.abs(Y.conj().T @ Y - np.eye(20)).max() < 1e-12
    assert np.abs(Y @ (Y.conj().T @ X) - X).max() < 1e-10 * np.abs(X).max()


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-10), ("mixed", 1e-6)])
def test_rayleigh_ritz_complex_matches_oracle(C, prec, tol):
    pr = small_problem(n=3, L=6.0, p=3, wells=2, kpoint=K)
    op, ora = C.KohnShamOperator.from_problem(pr), oracle_op(pr)
    rng = np.random.default_rng(6)
    X = rng.standard_normal((pr.n_dofs, 24)) + 1j * rng.standard_normal((pr.n_dofs, 24))
    ev_o, Xo, HXo = orc.rayleigh_ritz_gep(ora, X)
    Xt = torch.from_numpy(X.copy()).cuda()
    ev_g, HXg = C.rayleighRitzGEP(op, Xt, precision=prec, want_hx=True)
    assert np.abs(ev_g - ev_o).max() < tol * max(1.0, np.abs(ev_o).max())
    # Ritz vectors: residual A x - lambda x matches the oracle's residual norms
    Xg, HXg = Xt.cpu().numpy(), HXg.cpu().numpy()
    r_g = np.linalg.norm(HXg - Xg * ev_g, axis=0)
    r_o = np.linalg.norm(HXo - Xo * ev_o, axis=0)
    assert np.abs(r_g - r_o).max() < (1e-8 if prec == "fp64" else 1e-4) * max(1.0, r_o.max())


@pytest.mark.parametrize("mixed,tol,rr", [(False, 1e-10, "fp64"), (True, 1e-6, "fp64"),
                                          (True, 1e-6, "fp32"), (True, 1e-6, "fp32tc")])
def test_solve_complex_matches_oracle(C, mixed, tol, rr):
    pr = small_problem(n=3, L=6.0, p=2, wells=3, nwfc=12, seed=7, kpoint=K)
    op, ora = C.KohnShamOperator.from_problem(pr), oracle_op(pr)
    rng = np.random.default_rng(8)
    X0 = rng.uniform(-1, 1, (pr.n_dofs, 12)) + 1j * rng.uniform(-1, 1, (pr.n_dofs, 12))
    st = orc.SolverState(a0=-3.0, b_low=3.0, b_up=12.0)
    Xo = X0.copy()
    for _ in range(5):
        ev_o, res_o, Xo = orc.solve(ora, Xo, st, m=10)
    s = C.ChebyshevOrthogonalizedSubspaceIterationSolver(
        C.SolverParams(chebyshevOrder=10, rr_precision=rr))
    s.reinitSpectrumBounds(-3.0, 3.0, 12.0)
    X = torch.from_numpy(X0.copy()).cuda()
    for _ in range(5):
        ev, res = s.solve(op, X, useMixedPrec=mixed)
        s.reinitSpectrumBounds(ev[0], ev[-1], 12.0)
    occ = 6
    assert np.abs(ev[:occ] - ev_o[:occ]).max() < tol
    if not mixed:
        assert np.abs(ev - ev_o).max() < tol
        assert np.abs(res - res_o).max() < 1e-8


@pytest.mark.parametrize("mixed", [False, True])
def test_solve_batched_matches_sequential(C, mixed):
    """Independent problems (three Bloch k-points and one real operator) solved concurrently
    on four streams give the same iterations as one-by-one solves."""
    probs = [small_problem(n=3, L=6.0, p=2, wells=3, nwfc=12, seed=7, kpoint=k)
             for k in ([0.2, -0.1, 0.3], [0.0, 0.4, -0.2], [-0.3, 0.1, 0.1])]
    probs.append(small_problem(n=3, L=6.0, p=2, wells=3, nwfc=12, seed=7))
    ops = [C.KohnShamOperator.from_problem(p) for p in probs]
    rng = np.random.default_rng(3)
    X0 = []
    for p in probs:
        x = rng.uniform(-1, 1, (p.n_dofs, 12))
        if p.is_complex:
            x = x + 1j * rng.uniform(-1, 1, (p.n_dofs, 12))
        X0.append(x)

    def make():
        out = []
        for _ in probs:
            s = C.ChebyshevOrthogonalizedSubspaceIterationSolver(C.SolverParams(chebyshevOrder=10))
            s.reinitSpectrumBounds(-3.0, 3.0, 12.0)
            out.append(s)
        return out

    seq, bat = make(), make()
    Xs = [torch.from_numpy(x.copy()).cuda() for x in X0]
    Xb = [torch.from_numpy(x.copy()).cuda() for x in X0]
    for _ in range(3):
        ev_s = []
        for s, op, X in zip(seq, ops, Xs):
            ev, _ = s.solve(op, X, useMixedPrec=mixed)
            s.reinitSpectrumBounds(ev[0], ev[-1], 12.0)
            ev_s.append(ev)
        ev_b, _ = C.solve_batched(bat, ops, Xb, useMixedPrec=mixed, n_streams=4)
        for s, ev in zip(bat, ev_b):
            s.reinitSpectrumBounds(ev[0], ev[-1], 12.0)
        # the tensor-core HX scatters with FP32 atomics, so mixed runs differ by rounding
        tol = 1e-5 if mixed else 1e-10
        for a, b in zip(ev_s, ev_b):
            assert np.abs(a - b).max() < tol


def test_solve_batched_grouped_uneven_bloch(C):
    """Bloch Hamiltonians of uneven mesh (2^3 and 3^3 cells) and block size (8 and 16
    wavefunctions), different bounds and degrees: the batched solve filters them together
    (grouped recurrence and tensor-core launches in one CUDA graph) and gives the same Ritz
    values as one-by-one solves of the same iterations (mixed tolerance: FP32 atomics)."""
    from dftfe_gb300 import problems
    probs = problems.bloch_set(6, seed=11, small=True)
    ops = [C.KohnShamOperator.from_problem(p) for p in probs]
    X0 = [p.initial_vectors() for p in probs]

    bounds = []
    for op, p in zip(ops, probs):
        lo, blow, up = C.initial_bounds(op, p.n_wfc)
        bounds.append((lo, min(blow, lo + 0.5 * (up - lo)), up))

    def make():
        out = []
        for i, b in enumerate(bounds):
            s = C.ChebyshevOrthogonalizedSubspaceIterationSolver(
                C.SolverParams(chebyshevOrder=8 + 2 * (i % 3), mixed_precision="mixed",
                               rr_precision="fp32"))
            s.reinitSpectrumBounds(*b)
            out.append(s)
        return out

    seq, bat = make(), make()
    Xs = [torch.from_numpy(x.copy()).cuda() for x in X0]
    Xb = [torch.from_numpy(x.copy()).cuda() for x in X0]
    for _ in range(2):
        ev_s = []
        for s, op, X in zip(seq, ops, Xs):
            ev, _ = s.solve(op, X, useMixedPrec=True)
            ev_s.append(ev)
        ev_b, _ = C.solve_batched(bat, ops, Xb, useMixedPrec=True, n_streams=3)
        for a, b in zip(ev_s, ev_b):
            assert np.abs(a - b).max() < 1e-5 * max(1.0, np.abs(a).max())
        for s1, s2, a, b, bd in zip(seq, bat, ev_s, ev_b, bounds):
            s1.reinitSpectrumBounds(a[0], a[-1], bd[2])
            s2.reinitSpectrumBounds(b[0], b[-1], bd[2])


def test_lanczos_bounds_complex_match_oracle(C):
    pr = small_problem(n=2, L=4.0, p=3, wells=2, kpoint=K)
    op, ora = C.KohnShamOperator.from_problem(pr), oracle_op(pr)
    v0 = np.random.default_rng(0).uniform(0, 1, pr.n_dofs)
    lo, up = C.lanczosLowerUpperBoundEigenSpectrum(op, 20, False, v0)
    assert (lo, up) == orc.lanczos_bounds(ora, v0, 20)
