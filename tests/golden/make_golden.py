"""Generate tests/golden/small_p2.npz: oracle outputs on a small seeded problem.

The reference has no CheFSI-level golden vectors and cannot be built here, so this fixture
pins the oracle against its own committed outputs (regression) and gives the GPU tests a
fixed target: HX of a fixed block, one Chebyshev filter, and the Ritz values / residuals of
five CheFSI iterations with explicit bounds. Run: python -m tests.golden.make_golden
"""
import os

import numpy as np

from dftfe_gb300 import problems
from oracle import oracle as orc


def build_case():
    pr = problems.make_problem(n=3, L=6.0, p=2, n_wells=3, n_wfc=12, seed=7, projectors=True)
    op = orc.OracleOperator(pr.cell_map, pr.cell_mats, pr.inv_sqrt_mass, pr.n_dofs,
                            projectors=pr.nonlocal_)
    X = pr.initial_vectors()
    hx = op.HX(X)
    filt = op.chebyshev_filter(X, 8, 3.0, 12.0, -3.0)
    st = orc.SolverState(a0=-3.0, b_low=3.0, b_up=12.0)
    Xi = X.copy()
    for _ in range(5):
        ev, res, Xi = orc.solve(op, Xi, st, m=10)
    return dict(X=X, hx=hx, filt=filt, ritz=ev, res=res)


if __name__ == "__main__":
    out = build_case()
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "small_p2.npz")
    np.savez_compressed(path, **out)
    print(path, {k: v.shape for k, v in out.items()})
