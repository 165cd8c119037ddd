"""Failure detection on the GPU path, made on the host (no GPU fault): injected allocation
failure, a non-SPD overlap handed to the Cholesky, non-finite operator input. Each must come
back as a status code with the context still usable."""
import numpy as np
import pytest
import torch

from tests.helpers import small_problem

pytestmark = pytest.mark.gpu


@pytest.fixture()
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def test_not_spd_overlap_is_reported(C, monkeypatch):
    from dftfe_gb300 import _lib
    pr = small_problem(projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    X = torch.from_numpy(pr.initial_vectors()).cuda()
    monkeypatch.setenv("CHEFSI_FAULT_INJECT", "not_spd")
    with pytest.raises(_lib.ChefsiError) as ei:
        C.pseudoGramSchmidtOrthogonalization(op, X)
    assert ei.value.code == _lib.CHEFSI_ERR_NOT_SPD
    monkeypatch.delenv("CHEFSI_FAULT_INJECT")
    C.pseudoGramSchmidtOrthogonalization(op, X)       # context still usable
    Y = X.cpu().numpy()
    assert np.abs(Y.T @ Y - np.eye(Y.shape[1])).max() < 1e-12


def test_mixed_overlap_beyond_its_precision_is_taken_again_in_fp64(C, monkeypatch):
    """A tensor-core overlap whose Cholesky fails (made on the host: CHEFSI_FAULT_INJECT=
    not_spd_mixed spoils the tensor-core S only) is recomputed with the FP64 Gram: the mixed
    iteration then succeeds and its lowest Ritz values meet the mixed bar against the oracle
    (the setup of smoke(): 1e-5 Ha after one degree-12 iteration). With every S spoiled
    (not_spd) the mixed iteration still reports CHEFSI_ERR_NOT_SPD."""
    from dftfe_gb300 import _lib, problems
    from oracle import oracle as orc
    pr = problems.make_problem(n=2, L=4.0, p=4, n_wells=2, n_wfc=16, seed=3, projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    ora = orc.OracleOperator(pr.cell_map, pr.cell_mats, pr.inv_sqrt_mass, pr.n_dofs,
                             projectors=pr.nonlocal_)
    X0 = pr.initial_vectors()
    lo, up = orc.lanczos_bounds(ora, np.ones(pr.n_dofs), 20)
    bl = lo + 0.2 * (up - lo)
    ev_o, _, _ = orc.solve(ora, X0.copy(), orc.SolverState(lo, bl, up), m=12)

    def mixed_solve():
        s = C.ChebyshevOrthogonalizedSubspaceIterationSolver(C.SolverParams(chebyshevOrder=12))
        s.reinitSpectrumBounds(lo, bl, up)
        return s.solve(op, torch.from_numpy(X0.copy()).cuda(), useMixedPrec=True)[0]

    monkeypatch.setenv("CHEFSI_FAULT_INJECT", "not_spd_mixed")
    ev = mixed_solve()
    assert np.abs(ev[:8] - ev_o[:8]).max() < 1e-5
    monkeypatch.setenv("CHEFSI_FAULT_INJECT", "not_spd")
    with pytest.raises(_lib.ChefsiError) as ei:
        mixed_solve()
    assert ei.value.code == _lib.CHEFSI_ERR_NOT_SPD
    monkeypatch.delenv("CHEFSI_FAULT_INJECT")
    ev = mixed_solve()
    assert np.abs(ev[:8] - ev_o[:8]).max() < 1e-5


def test_rank_deficient_overlap_is_not_spd(C):
    from dftfe_gb300 import _lib
    pr = small_problem(projectors=True)
    op = C.KohnShamOperator.from_problem(pr)
    X = torch.zeros((pr.n_dofs, 6), dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.ChefsiError) as ei:
        C.pseudoGramSchmidtOrthogonalization(op, X)
    assert ei.value.code == _lib.CHEFSI_ERR_NOT_SPD


def test_nan_input_is_rejected(C):
    from dftfe_gb300 import _lib
    pr = small_problem()
    pr.cell_mats[0, 0, 0] = np.nan
    with pytest.raises(_lib.ChefsiError) as ei:
        C.KohnShamOperator.from_problem(pr)
    assert ei.value.code == _lib.CHEFSI_ERR_NAN


def test_alloc_failure_is_reported(C, monkeypatch):
    from dftfe_gb300 import _lib
    pr = small_problem()
    monkeypatch.setenv("CHEFSI_FAULT_INJECT", "alloc")
    with pytest.raises(_lib.ChefsiError) as ei:
        C.KohnShamOperator.from_problem(pr)
    assert ei.value.code == _lib.CHEFSI_ERR_ALLOC
    monkeypatch.delenv("CHEFSI_FAULT_INJECT")
    op = C.KohnShamOperator.from_problem(pr)           # recovers
    assert op.n_dofs == pr.n_dofs


def test_bad_map_is_rejected(C):
    from dftfe_gb300 import _lib
    pr = small_problem()
    pr.cell_map[0, 0] = pr.n_dofs + 5
    with pytest.raises(_lib.ChefsiError) as ei:
        C.KohnShamOperator.from_problem(pr)
    assert ei.value.code == _lib.CHEFSI_ERR_INVALID


def test_bounded_device_waits_expire_and_context_stays_usable(C):
    """Every device-side wait is bounded. With the bounds lowered to zero (a wait expires at
    its first poll) the tensor-core filter HX, the tensor-core Gram of the mixed overlap and
    the cooperative tridiagonalisation of the eigensolver each return CHEFSI_ERR_TIMEOUT; with
    the bounds restored the same calls on the same context succeed and agree with the oracle."""
    from dftfe_gb300 import _lib
    from oracle import oracle as orc
    from tests.helpers import oracle_op
    lib = _lib.load()
    pr = small_problem(n=2, L=4.0, p=4, wells=2, projectors=True)
    op, ora = C.KohnShamOperator.from_problem(pr), oracle_op(pr)
    X = np.random.default_rng(3).uniform(-1, 1, (pr.n_dofs, 32))
    lo, up = orc.lanczos_bounds(ora, np.ones(pr.n_dofs), 20)
    a, b, a0 = lo + 0.3 * (up - lo), up, lo
    rng = np.random.default_rng(4)
    Q, _ = np.linalg.qr(rng.standard_normal((300, 300)))
    A = (Q * np.sort(rng.standard_normal(300))) @ Q.T
    A = 0.5 * (A + A.T)
    try:
        _lib.check(lib.chefsi_set_wait_limits(0, _lib.DEFAULT_BARRIER_SPINS))
        with pytest.raises(_lib.ChefsiError) as ei:
            C.chebyshevFilter(op, torch.from_numpy(X.copy()).cuda(), 10, a, b, a0, precision="mixed")
        assert ei.value.code == _lib.CHEFSI_ERR_TIMEOUT
        with pytest.raises(_lib.ChefsiError) as ei:
            C.pseudoGramSchmidtOrthogonalization(op, torch.from_numpy(X.copy()).cuda(),
                                                 precision="mixed")
        assert ei.value.code == _lib.CHEFSI_ERR_TIMEOUT
        _lib.check(lib.chefsi_set_wait_limits(_lib.DEFAULT_WAIT_TRIES, 0))
        with pytest.raises(_lib.ChefsiError) as ei:
            C.syevd(torch.from_numpy(A.copy()).cuda())
        assert ei.value.code == _lib.CHEFSI_ERR_TIMEOUT
    finally:
        _lib.check(lib.chefsi_set_wait_limits(_lib.DEFAULT_WAIT_TRIES, _lib.DEFAULT_BARRIER_SPINS))
    Xt = torch.from_numpy(X.copy()).cuda()
    C.chebyshevFilter(op, Xt, 10, a, b, a0, precision="mixed")
    ref = ora.chebyshev_filter(X, 10, a, b, a0)
    # the default (shifted) mixed filter's bound (tests/test_gpu_parity.py)
    assert np.abs(Xt.cpu().numpy() - ref).max() < 4e-5 * np.abs(ref).max()
    w, _ = C.syevd(torch.from_numpy(A.copy()).cuda())
    assert np.abs(w.cpu().numpy() - np.linalg.eigvalsh(A)).max() < 1e-11
