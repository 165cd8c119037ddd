"""Spectrum-split Rayleigh-Ritz and first-order density-matrix response for complex (Bloch)
operators through the C ABI against the FP64 oracle.

Tolerances: FP64 eigenvalues 1e-10 relative to the spectrum's scale, XFrac projector and
X P' 1e-9 / 1e-10; densityMatDerFermiEnergy 1e-12; the mixed step (reduced H X of the real
form, FP64 complex dense products) 2e-6 in the eigenvalues.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from tests.helpers import dense_operator, oracle_op, small_problem

pytestmark = pytest.mark.gpu

K = [0.2, -0.1, 0.3]


@pytest.fixture(scope="module")
def C(cuda):
    from dftfe_gb300 import chefsi
    return chefsi


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("prec,frac_reduced,tol", [("fp64", False, 1e-10), ("mixed", False, 2e-6),
                                                   ("mixed", True, 2e-6)])
def test_spectrum_split_complex_matches_oracle(C, prec, frac_reduced, tol):
    pr = small_problem(n=3, L=6.0, p=3, wells=2, kpoint=K)
    op, ora = C.KohnShamOperator.from_problem(pr), oracle_op(pr)
    rng = np.random.default_rng(12)
    X = rng.standard_normal((pr.n_dofs, 24)) + 1j * rng.standard_normal((pr.n_dofs, 24))
    ev_o, Xo, XFo, HXFo = orc.rayleigh_ritz_spectrum_split(ora, X, 17)
    Xt = torch.from_numpy(X.copy()).cuda()
    XF = torch.empty((pr.n_dofs, 7), dtype=torch.complex128, device="cuda")
    ev, HXF = C.rayleighRitzGEPSpectrumSplitDirect(op, Xt, XF, 17, precision=prec, want_hx=True,
                                                   frac_reduced=frac_reduced)
    scale = max(1.0, np.abs(ev_o).max())
    assert np.abs(ev - ev_o).max() < tol * scale
    Xg, XFg, HXFg = Xt.cpu().numpy(), XF.cpu().numpy(), HXF.cpu().numpy()
    assert np.abs(Xg.conj().T @ Xg - np.eye(24)).max() < 1e-11
    assert np.abs(XFg @ XFg.conj().T - XFo @ XFo.conj().T).max() < (1e-9 if prec == "fp64" else 1e-4)
    if prec == "fp64":
        assert np.abs(Xg - Xo).max() < 1e-9 * np.abs(Xo).max()
        assert np.abs(HXFg - dense_operator(pr) @ XFg).max() < 1e-10 * scale


def test_solve_spectrum_split_complex_matches_solve(C):
    pr = small_problem(n=3, L=6.0, p=2, wells=3, nwfc=12, seed=7, kpoint=K)
    op = C.KohnShamOperator.from_problem(pr)
    rng = np.random.default_rng(8)
    X0 = rng.uniform(-1, 1, (pr.n_dofs, 20)) + 1j * rng.uniform(-1, 1, (pr.n_dofs, 20))
    sol = []
    for _ in range(2):
        s = C.ChebyshevOrthogonalizedSubspaceIterationSolver(C.SolverParams(chebyshevOrder=10))
        s.reinitSpectrumBounds(-3.0, 3.0, 12.0)
        sol.append(s)
    X1 = torch.from_numpy(X0.copy()).cuda()
    X2 = torch.from_numpy(X0.copy()).cuda()
    ev_f, res_f = sol[0].solve(C.KohnShamOperator.from_problem(pr), X1)
    ev_s, res_s, XF = sol[1].solveSpectrumSplit(op, X2, 14)
    assert np.abs(ev_s - ev_f[14:]).max() < 1e-10 * max(1.0, np.abs(ev_f).max())
    assert np.abs(res_s - res_f[14:]).max() < 1e-9


@pytest.mark.parametrize("T", [500.0, 20000.0])
def test_dm_response_complex_matches_oracle(C, T):
    pr = small_problem(n=3, L=6.0, p=2, kpoint=K)
    pr2 = small_problem(n=3, L=6.0, p=2, kpoint=K, seed=5, wells=3)
    pert = pr2.cell_mats - pr.cell_mats
    op_prime = C.KohnShamOperator(pr.cell_map, pert, pr.sqrt_mass, pr.inv_sqrt_mass, pr.n_dofs)
    ora_prime = orc.OracleOperator(pr.cell_map, pert, pr.inv_sqrt_mass, pr.n_dofs)
    w, Q = np.linalg.eigh(dense_operator(pr))
    X, eig = Q[:, :24].copy(), w[:24].copy()
    mu = 0.5 * (eig[10] + eig[11])
    XP_o, dmu_o = orc.density_matrix_first_order_response(ora_prime, X, eig, mu, T)
    Xt = torch.from_numpy(X.copy()).cuda()
    dmu = C.densityMatrixEigenBasisFirstOrderResponse(op_prime, Xt, eig, mu, T)
    assert rel(Xt.cpu().numpy(), XP_o) < 1e-10
    assert rel(dmu, dmu_o) < 1e-12


@pytest.mark.parametrize("p", [2, 4])
def test_bloch_cell_assembly_matches_oracle(C, p):
    """On-device Bloch cell matrices for three k-points against the oracle's q-loop and
    against the workload's own (sum-factorised) matrices; p = 4 has 125 nodes per cell, so
    the 32 x 32 output tiles have a ragged edge."""
    from tests.helpers import shape_tables
    pr = small_problem(n=2, L=4.0, p=p, wells=2, kpoint=K)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    jxw = np.broadcast_to(w3, (mesh.n_cells, len(w3))).copy()
    vjxw = pr.info["vjxw"]
    kp = np.array([K, [0.0, 0.0, 0.0], [0.5, 0.25, -0.4]])
    ref = orc.cell_hamiltonians_bloch_direct(mesh.stiffness_cell(), N, dN, vjxw, jxw, kp)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    out = C.assemble_cell_hamiltonians_bloch(t(N), t(dN), t(mesh.stiffness_cell()), t(vjxw),
                                             t(jxw), kp).cpu().numpy()
    assert rel(out, ref) < 1e-12
    assert rel(out[0], pr.cell_mats) < 1e-12

