"""CheFSI at the 64,000-dof workload against the oracle's CheFSI, 20 iterations.

Workload: periodic cube L = 15 bohr, 10^3 cells, FE degree 4 (64,000 dofs), 8 seeded Gaussian
wells, 96 wavefunctions (48 occupied) from X0 ~ U(-1, 1), Chebyshev degree 24, 20 CheFSI
iterations (chebyshevOrthogonalizedSubspaceIterationSolver::solve,
src/solvers/eigenSolvers/chebyshevOrthogonalizedSubspaceIterationSolver.cc:116-607, with the
bounds update of kohnShamEigenSpaceCompute, src/dft/kohnShamEigenSolve.cc:296-501).

The oracle runs its 20 iterations once (FP64, CPU) and records the bounds (a0, bLow, b) it
used before each one; the GPU solver runs through the C ABI with exactly those bounds before
each of its iterations, so the two runs differ only in arithmetic. Tolerances, written in the
tests:

* FP64: every Ritz value within 1e-8 Ha, every residual norm within 1e-8, the largest
  principal angle between the occupied (48-state) subspaces below 1e-8 rad;
* mixed (FP16-split tensor-core filter, mixed Rayleigh-Ritz): the occupied Ritz values within
  1e-6 Ha, the occupied residual norms below 1e-4, the occupied subspace angle below 1e-3 rad.

Collected after the other GPU parity files (the oracle's 20 iterations take about a minute).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

N_ITER = 20
DEGREE = 24


@pytest.fixture(scope="module")
def ref():
    from dftfe_gb300 import problems
    pr = problems.workload("small", seed=0)
    ora = orc.OracleOperator(pr.cell_map, pr.cell_mats, pr.inv_sqrt_mass, pr.n_dofs,
                             projectors=pr.nonlocal_)
    v0 = np.random.default_rng(0).uniform(0.0, 1.0, pr.n_dofs)
    st = orc.initial_bounds(ora, pr.n_wfc, v0)
    X = pr.initial_vectors()
    bounds = []
    for _ in range(N_ITER):
        bounds.append((st.a0, st.b_low, st.b_up))
        ev, res, X = orc.solve(ora, X, st, m=DEGREE)
    return pr, bounds, ev, res, X


def gpu_run(pr, bounds, mixed):
    from dftfe_gb300 import chefsi
    op = chefsi.KohnShamOperator.from_problem(pr)
    s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(
        chefsi.SolverParams(chebyshevOrder=DEGREE, chebyWfcBlockSize=pr.n_wfc,
                            wfcBlockSize=pr.n_wfc, rr_precision="fp32tc"))
    X = torch.from_numpy(pr.initial_vectors()).cuda()
    for b in bounds:
        s.reinitSpectrumBounds(*b)
        ev, res = s.solve(op, X, useMixedPrec=mixed)
    return ev, res, X.cpu().numpy()


def occupied_angle(Xa, Xb, nocc):
    """Largest principal angle between the spans of the first nocc columns (orthonormal
    bases): arcsin of the spectral norm of Qb - Qa (Qa^T Qb), which stays accurate for small
    angles (the arccos of the smallest singular value of Qa^T Qb bottoms out near 5e-8)."""
    Qa, Qb = Xa[:, :nocc], Xb[:, :nocc]
    r = Qb - Qa @ (Qa.T @ Qb)
    return float(np.arcsin(min(1.0, np.linalg.norm(r, 2))))


def test_config0_fp64_matches_oracle(cuda, ref):
    pr, bounds, ev_o, res_o, X_o = ref
    ev, res, X = gpu_run(pr, bounds, mixed=False)
    nocc = pr.n_occupied
    d_ev = np.abs(ev - ev_o).max()
    d_res = np.abs(res - res_o).max()
    ang = occupied_angle(X_o, X, nocc)
    print(f"config0 fp64: max|dRitz| {d_ev:.3e} Ha, max|dres| {d_res:.3e}, angle {ang:.3e} rad, "
          f"res_occ_max {res[:nocc].max():.3e} (oracle {res_o[:nocc].max():.3e})")
    assert d_ev < 1e-8, ev - ev_o
    assert d_res < 1e-8
    assert ang < 1e-8


def test_config0_mixed_matches_oracle(cuda, ref):
    pr, bounds, ev_o, res_o, X_o = ref
    ev, res, X = gpu_run(pr, bounds, mixed=True)
    nocc = pr.n_occupied
    d_occ = np.abs(ev[:nocc] - ev_o[:nocc]).max()
    d_all = np.abs(ev - ev_o).max()
    ang = occupied_angle(X_o, X, nocc)
    print(f"config0 mixed: max|dRitz| occupied {d_occ:.3e} Ha, all {d_all:.3e} Ha, angle "
          f"{ang:.3e} rad, res_occ_max {res[:nocc].max():.3e} (oracle {res_o[:nocc].max():.3e})")
    assert d_occ < 1e-6, ev[:nocc] - ev_o[:nocc]
    assert res[:nocc].max() < 1e-4
    assert ang < 1e-3
