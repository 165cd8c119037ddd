"""CheFSI on the 1.7M-dof operator of the benchmark against the oracle's CheFSI.

Workload: periodic cube L = 30 bohr, 20^3 cells, FE degree 6 (1,728,000 dofs), 64 seeded
Gaussian wells with 8 projectors each: the operator the benchmark times. The oracle's CPU
iterations at 1024 vectors would take minutes each, so the block is 16 vectors from
X0 ~ U(-1, 1), Chebyshev degree 30, 4 iterations (chebyshevOrthogonalizedSubspaceIterationSolver
::solve, src/solvers/eigenSolvers/chebyshevOrthogonalizedSubspaceIterationSolver.cc:116-607,
with the bounds update of kohnShamEigenSpaceCompute, src/dft/kohnShamEigenSolve.cc:296-501).
The oracle records the bounds (a0, bLow, b) it used before each iteration and the GPU solver
runs with exactly those, so the runs differ only in arithmetic.

Tolerance, written in the test: FP64, every Ritz value within 1e-8 Ha and every residual norm
within 1e-8 (measured: 4e-15 Ha, 7e-15). The mixed path is not compared here: from random
vectors, the first-call bounds for 16 vectors (a short Lanczos run puts a0 above the spectrum's
bottom and bLow just above it) make the filtered block more ill-conditioned than its FP32
storage resolves, so its overlap is not positive definite even when taken again in FP64 and
the mixed iteration reports CHEFSI_ERR_NOT_SPD (the reference's FP32 filter vectors have the
same limit); the mixed path is compared with the oracle over 20 iterations at the 64,000-dof
workload and with the FP64 path at this operator with 1024 vectors (the benchmark's FP64 leg).

Collected after the other GPU files (building the workload and the oracle's iterations take
about a minute on the host).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc

pytestmark = pytest.mark.gpu

N_VEC, N_ITER, DEGREE = 16, 4, 30


@pytest.fixture(scope="module")
def ref():
    from dftfe_gb300 import problems
    pr = problems.workload("mixed", seed=0)
    ora = orc.OracleOperator(pr.cell_map, pr.cell_mats, pr.inv_sqrt_mass, pr.n_dofs,
                             projectors=pr.nonlocal_)
    v0 = np.random.default_rng(0).uniform(0.0, 1.0, pr.n_dofs)
    st = orc.initial_bounds(ora, N_VEC, v0)
    X = pr.initial_vectors(N_VEC)
    bounds = []
    for _ in range(N_ITER):
        bounds.append((st.a0, st.b_low, st.b_up))
        ev, res, X = orc.solve(ora, X, st, m=DEGREE)
    return pr, bounds, ev, res


def gpu_run(pr, bounds, mixed):
    from dftfe_gb300 import chefsi
    op = chefsi.KohnShamOperator.from_problem(pr)
    s = chefsi.ChebyshevOrthogonalizedSubspaceIterationSolver(
        chefsi.SolverParams(chebyshevOrder=DEGREE, chebyWfcBlockSize=N_VEC, wfcBlockSize=N_VEC,
                            rr_precision="fp32tc"))
    X = torch.from_numpy(pr.initial_vectors(N_VEC)).cuda()
    for b in bounds:
        s.reinitSpectrumBounds(*b)
        ev, res = s.solve(op, X, useMixedPrec=mixed)
    return ev, res


def test_config1_operator_fp64_matches_oracle(cuda, ref):
    pr, bounds, ev_o, res_o = ref
    ev, res = gpu_run(pr, bounds, mixed=False)
    print(f"1.7M dofs fp64: max|dRitz| {np.abs(ev - ev_o).max():.3e} Ha, "
          f"max|dres| {np.abs(res - res_o).max():.3e}, res max {res.max():.3e}")
    assert np.abs(ev - ev_o).max() < 1e-8, ev - ev_o
    assert np.abs(res - res_o).max() < 1e-8
