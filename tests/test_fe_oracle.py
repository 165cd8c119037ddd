"""CPU tests: finite-element inputs and the FP64 oracle against analytic known answers.

The reference ships no golden vectors at the CheFSI boundary (its regression tests pin total
energies only), so the oracle is pinned here by known answers: free-particle spectra
1/2|G+k|^2, dense eigendecompositions of small assembled operators, and the scalar
Chebyshev polynomial of the sigma-form recurrence.
"""
import numpy as np
import pytest

from dftfe_gb300 import fe
from oracle import oracle as orc
from tests.helpers import cheb_scalar, dense_operator, oracle_op, small_problem


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6, 7])
def test_gll_rule_exactness(p):
    x, w = fe.gll_nodes_weights(p)
    assert abs(w.sum() - 1.0) < 1e-14
    for k in range(2 * p):  # GLL with p+1 points is exact to degree 2p-1
        assert abs((w * x ** k).sum() - 1.0 / (k + 1)) < 1e-13


def test_lagrange_basis_interpolates():
    x, _ = fe.gll_nodes_weights(4)
    phi, dphi = fe.lagrange_1d(x, x)
    assert np.allclose(phi, np.eye(5), atol=1e-13)
    assert np.allclose(dphi.sum(1), 0.0, atol=1e-11)   # derivative of the constant 1


def test_mass_and_map():
    m = fe.PeriodicCubeMesh(3, 6.0, 3)
    assert abs(m.lumped_mass().sum() - 6.0 ** 3) < 1e-10
    cm = m.cell_dof_map()
    assert cm.min() == 0 and cm.max() == m.n_dofs - 1
    assert len(np.unique(cm)) == m.n_dofs


def test_cell_matrix_sum_factorisation_matches_direct_formula():
    pr = small_problem(n=2, L=4.0, p=3, wells=3)
    mesh = pr.mesh
    nq1 = mesh.p + 3
    xq, _ = fe.gauss_nodes_weights(nq1)
    phi, _ = mesh.shape_1d(xq)
    q = np.arange(nq1 ** 3)
    qx, qy, qz = q % nq1, (q // nq1) % nq1, q // (nq1 * nq1)
    i = np.arange(mesh.nodes_per_cell)
    p1 = mesh.p + 1
    N = phi[qx][:, i % p1] * phi[qy][:, (i // p1) % p1] * phi[qz][:, i // (p1 * p1)]
    Hdir = orc.cell_hamiltonians_direct(mesh.stiffness_cell(), N, pr.info["vjxw"])
    assert np.abs(Hdir - pr.cell_mats).max() < 1e-12 * np.abs(Hdir).max()


@pytest.mark.parametrize("n,L,p", [(2, 6.0, 4), (3, 6.0, 3)])
def test_free_particle_spectrum_matches_plane_waves(n, L, p):
    """K1: V = 0 gives 1/2|G|^2 to FE accuracy (degenerate multiplets intact)."""
    mesh = fe.PeriodicCubeMesh(n, L, p)
    K = mesh.stiffness_cell()
    mats = np.broadcast_to(0.5 * K, (mesh.n_cells,) + K.shape).copy()
    op = orc.OracleOperator(mesh.cell_dof_map(), mats, 1 / np.sqrt(mesh.lumped_mass()), mesh.n_dofs)
    ev = np.linalg.eigvalsh(op.dense())
    g = 2 * np.pi / L
    assert abs(ev[0]) < 1e-10
    assert np.allclose(ev[1:7], 0.5 * g * g, rtol=2e-2)
    assert np.ptp(ev[1:4]) < 1e-9     # cubic symmetry: exact 3-fold (x, y, z) degeneracy


def test_bloch_free_particle():
    """Complex Bloch cell matrices: Hermitian assembly, eigenvalues 1/2|G+k|^2."""
    mesh = fe.PeriodicCubeMesh(2, 6.0, 4)
    k = np.array([0.1, -0.2, 0.15])
    v = np.zeros((mesh.n_cells, (mesh.p + 3) ** 3))
    Hc = fe.cell_hamiltonians(mesh, v, kpoint=k)
    op = orc.OracleOperator(mesh.cell_dof_map(), Hc, 1 / np.sqrt(mesh.lumped_mass()), mesh.n_dofs)
    A = op.dense()
    assert np.abs(A - A.conj().T).max() < 1e-12
    ev = np.linalg.eigvalsh(A)
    g = 2 * np.pi / 6.0
    pw = sorted(0.5 * np.sum((g * np.array([i, j, l]) + k) ** 2)
                for i in range(-2, 3) for j in range(-2, 3) for l in range(-2, 3))
    assert np.allclose(ev[:6], pw[:6], rtol=1e-3)


def test_oracle_hx_matches_dense_assembly_with_projectors():
    pr = small_problem(projectors=True, wells=2)
    op = oracle_op(pr)
    A = dense_operator(pr)
    X = np.random.default_rng(3).standard_normal((pr.n_dofs, 5))
    Y = op.HX(X)
    assert np.abs(Y - A @ X).max() < 1e-12 * np.abs(A @ X).max()
    # scaleFlag semantics: dst + scalar * A src
    Z = np.ones_like(X)
    op.HX(X, scalar=0.5, dst=Z, accumulate=True)
    assert np.allclose(Z, 1.0 + 0.5 * (A @ X), atol=1e-12)


def test_oracle_constraint_path_matches_folded_map():
    """Periodicity as constraint rows on the unfolded lattice == folded map (masters)."""
    pr = small_problem(n=2, L=4.0, p=2, wells=2)
    folded = oracle_op(pr)
    emap, n_ext, cons, mass_ext = __import__("tests.helpers", fromlist=["x"]).unfolded_setup(pr)
    unf = orc.OracleOperator(emap, pr.cell_mats, 1 / np.sqrt(mass_ext), n_ext, constraints=cons)
    X = np.random.default_rng(4).standard_normal((pr.n_dofs, 3))
    e2f = pr.mesh.extended_to_folded()
    Xe = X[e2f]
    Ye = unf.HX(Xe)
    Yf = folded.HX(X)
    is_master = np.ones(n_ext, bool)
    is_master[cons[0]] = False
    assert np.abs(Ye[cons[0]]).max() == 0.0
    assert np.allclose(Ye[is_master], Yf[e2f[is_master]], atol=1e-12)


def test_oracle_filter_is_the_chebyshev_polynomial():
    pr = small_problem(wells=2)
    op = oracle_op(pr)
    A = dense_operator(pr)
    lam, Q = np.linalg.eigh(A)
    X = Q[:, :4] + 0.1 * Q[:, 10:14]
    a, b, a0, m = lam[8], lam[-1] + 0.1, lam[0] - 0.5, 7
    Y = op.chebyshev_filter(X, m, a, b, a0)
    ref = Q @ (cheb_scalar(lam, m, a, b, a0)[:, None] * (Q.T @ X))
    assert np.abs(Y - ref).max() < 1e-10 * np.abs(ref).max()


def test_oracle_chefsi_converges_to_dense_eigenvalues():
    """K2: CheFSI Ritz values equal the dense eigenvalues (tiny mesh)."""
    pr = small_problem(projectors=True, nwfc=10)
    op = oracle_op(pr)
    exact = np.linalg.eigvalsh(dense_operator(pr))
    X = pr.initial_vectors()
    st = orc.SolverState(a0=np.floor(exact[0]), b_low=exact[14], b_up=np.ceil(exact[-1] + 0.5))
    for _ in range(25):
        ev, res, X = orc.solve(op, X, st, m=12)
    assert np.abs(ev[:8] - exact[:8]).max() < 1e-10
    assert res[:8].max() < 1e-8


def test_chebyshev_order_table():
    assert orc.chebyshev_order(400) == 24
    assert orc.chebyshev_order(600) == 30
    assert orc.chebyshev_order(1e9) == 1250


def test_lanczos_bounds_enclose_spectrum():
    pr = small_problem(wells=2)
    op = oracle_op(pr)
    ev = np.linalg.eigvalsh(dense_operator(pr))
    lo, up = orc.lanczos_bounds(op, np.random.default_rng(0).uniform(0, 1, pr.n_dofs), k=20)
    assert lo <= ev[0] and up >= ev[-1] - 1e-8


def test_golden_fixture_reproduces():
    """The committed golden fixture (tests/golden/make_golden.py) still matches the oracle."""
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "small_p2.npz")
    if not os.path.exists(path):
        pytest.skip("golden fixture not generated")
    from tests.golden.make_golden import build_case
    g = np.load(path)
    out = build_case()
    for k in g.files:
        assert np.allclose(out[k], g[k], rtol=1e-11, atol=1e-12), k


def test_oracle_density_of_a_constant_state():
    """psi = M^{-1/2} x = 1 at every node (x = M^{1/2} 1) interpolates to 1 at every Gauss
    point, so rho = sum_i f_i there and its integral is sum_i f_i times the volume."""
    pr = small_problem(n=2, L=4.0, p=3, wells=2)
    mesh = pr.mesh
    nq1 = mesh.p + 3
    xq, _ = fe.gauss_nodes_weights(nq1)
    phi, _ = mesh.shape_1d(xq)
    q = np.arange(nq1 ** 3)
    qx, qy, qz = q % nq1, (q // nq1) % nq1, q // (nq1 * nq1)
    i = np.arange(mesh.nodes_per_cell)
    p1 = mesh.p + 1
    N = phi[qx][:, i % p1] * phi[qy][:, (i // p1) % p1] * phi[qz][:, i // (p1 * p1)]
    _, w3 = mesh.quadrature(nq1)
    jxw = np.broadcast_to(w3, (mesh.n_cells, len(w3))).copy()
    X = np.repeat((1.0 / pr.inv_sqrt_mass)[:, None], 2, axis=1)
    occ = np.array([2.0, 0.5])
    rho = orc.density(pr.cell_map, pr.inv_sqrt_mass, N, X, occ)
    assert np.abs(rho - occ.sum()).max() < 1e-12
    rho_w = orc.density(pr.cell_map, pr.inv_sqrt_mass, N, X, occ, jxw)
    assert abs(rho_w.sum() - occ.sum() * 4.0 ** 3) < 1e-9


def test_oracle_spectrum_split_is_the_top_of_the_full_rayleigh_ritz():
    """The spectrum-split RR returns the top N - Noc Ritz pairs of the generalised RR on the
    same X: equal eigenvalues, XFrac spanning the top rotated vectors, X left orthonormal."""
    pr = small_problem(projectors=True)
    ora = oracle_op(pr)
    X = np.random.default_rng(9).standard_normal((pr.n_dofs, 20))
    ev, Xr, HXr = orc.rayleigh_ritz_gep(ora, X)
    ev_s, Xo, XF, HXF = orc.rayleigh_ritz_spectrum_split(ora, X, 14)
    assert np.abs(ev_s - ev[14:]).max() < 1e-11 * np.abs(ev).max()
    assert np.abs(Xo.T @ Xo - np.eye(20)).max() < 1e-12
    assert np.abs(XF @ XF.T - Xr[:, 14:] @ Xr[:, 14:].T).max() < 1e-10
    assert np.abs(HXF - dense_operator(pr) @ XF).max() < 1e-10 * np.abs(ev).max()


def test_oracle_density_matrix_response_is_the_divided_difference():
    """The first-order recursion gives the derivative of the matrix function g(H) that the
    zeroth-order recursion applies: in the eigenbasis, P'_ij = g[e_i, e_j] H'_ij (divided
    difference; g'(e_i) on the diagonal), and g is close to the Fermi-Dirac occupation f.
    densityMatDerFermiEnergy is beta g (1 - g), the Fermi-Dirac identity -f' = beta f (1 - f)
    evaluated with g, so it matches -g' to the accuracy of g ~ f."""
    pr = small_problem(projectors=False)
    ora = oracle_op(pr)
    A = dense_operator(pr)
    w, Q = np.linalg.eigh(A)
    N = 24
    X = Q[:, :N]
    eig = w[:N]
    mu, T = 0.5 * (eig[10] + eig[11]), 5000.0
    XP, dmu = orc.density_matrix_first_order_response(ora, X, eig, mu, T)
    P = X.T @ XP
    Hp = X.T @ A @ X
    g = lambda x: orc.fermi_recursion_scalar(x, mu, T)
    h = 1e-6
    D = np.empty((N, N))
    for i in range(N):
        for j in range(N):
            if abs(eig[i] - eig[j]) > 1e-4:
                D[i, j] = (g(eig[i]) - g(eig[j])) / (eig[i] - eig[j])
            else:
                D[i, j] = (g(eig[i] + h) - g(eig[i] - h)) / (2 * h)
    assert np.abs(P - D * Hp).max() < 1e-6 * np.abs(D * Hp).max()
    assert np.abs(-np.diag(D) - dmu).max() < 1e-4 * np.abs(dmu).max()
    beta = 1.0 / orc.K_B_HARTREE_PER_KELVIN / T
    fd = 1.0 / (1.0 + np.exp(beta * (eig - mu)))
    assert np.abs(g(eig) - fd).max() < 1e-3


def test_oracle_bloch_cell_matrices_match_fe_module():
    """The direct q-loop of the k-point cell-matrix formula equals the sum-factorised
    construction the workloads use (both restate hamMatrixKernelLDA's k-point form)."""
    from tests.helpers import shape_tables
    k = [0.2, -0.1, 0.3]
    pr = small_problem(n=2, L=4.0, p=2, wells=2, kpoint=k)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    jxw = np.broadcast_to(w3, (mesh.n_cells, len(w3))).copy()
    vjxw = pr.info["vjxw"]
    H = orc.cell_hamiltonians_bloch_direct(mesh.stiffness_cell(), N, dN, vjxw, jxw,
                                           np.array([k, [0.0, 0.0, 0.0]]))
    assert np.abs(H[0] - pr.cell_mats).max() < 1e-12 * np.abs(pr.cell_mats).max()
    real = fe.cell_hamiltonians(mesh, vjxw)
    assert np.abs(H[1] - real).max() < 1e-12 * np.abs(real).max()


def test_oracle_gga_cell_matrices():
    """The GGA q-loop against a matrix form of the same sums, its symmetry, and its LDA limit."""
    from tests.helpers import shape_tables
    pr = small_problem(n=2, L=4.0, p=2, wells=2)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    vjxw = pr.info["vjxw"]
    g = np.random.default_rng(3).standard_normal((mesh.n_cells, len(w3), 3)) * w3[None, :, None]
    K = mesh.stiffness_cell()
    H = orc.cell_hamiltonians_gga_direct(K, N, dN, vjxw, g)
    G = np.einsum('cqd,dqi,qj->cij', g, dN, N)
    ref = 0.5 * K[None] + np.einsum('cq,qi,qj->cij', vjxw, N, N) + 2.0 * (G + G.transpose(0, 2, 1))
    assert np.abs(H - ref).max() < 1e-12 * np.abs(ref).max()
    assert np.abs(H - H.transpose(0, 2, 1)).max() < 1e-13 * np.abs(H).max()
    lda = orc.cell_hamiltonians_gga_direct(K, N, dN, vjxw, np.zeros_like(g))
    assert np.abs(lda - fe.cell_hamiltonians(mesh, vjxw)).max() < 1e-12 * np.abs(lda).max()


def test_oracle_bloch_gga_is_bloch_lda_plus_the_real_gga_terms():
    from tests.helpers import shape_tables
    k = [0.2, -0.1, 0.3]
    pr = small_problem(n=2, L=4.0, p=2, wells=2, kpoint=k)
    mesh = pr.mesh
    N, dN, w3 = shape_tables(mesh)
    jxw = np.broadcast_to(w3, (mesh.n_cells, len(w3))).copy()
    vjxw = pr.info["vjxw"]
    g = np.random.default_rng(4).standard_normal((mesh.n_cells, len(w3), 3)) * w3[None, :, None]
    K = mesh.stiffness_cell()
    kp = np.array([k])
    lda = orc.cell_hamiltonians_bloch_direct(K, N, dN, vjxw, jxw, kp)[0]
    gga = orc.cell_hamiltonians_bloch_direct(K, N, dN, vjxw, jxw, kp, g)[0]
    real_term = orc.cell_hamiltonians_gga_direct(K, N, dN, vjxw, g) - \
        orc.cell_hamiltonians_gga_direct(K, N, dN, vjxw, np.zeros_like(g))
    assert np.abs(gga - lda - real_term).max() < 1e-12 * np.abs(gga).max()


def _box_geometry(mesh, scales):
    """Reference-cell gradients and Jacobian factors of the periodic mesh stretched by
    diag(scales): every cell is h diag(scales) times the reference cube."""
    from tests.helpers import shape_tables
    N, dN, w3 = shape_tables(mesh)
    h = mesh.h
    dNref = dN * h                                   # d/dxi on [0, 1]^3
    inv = np.diag(1.0 / (h * np.asarray(scales, float)))
    det = h ** 3 * np.prod(scales)
    F = np.einsum('ik,jk->ij', inv, inv)[None, None] * (w3 / h ** 3 * det)[None, :, None, None]
    F = np.broadcast_to(F, (mesh.n_cells,) + F.shape[1:]).copy()
    return N, dNref, F, det / h ** 3


def test_oracle_geometry_cell_matrices_uniform_and_stretched():
    """The per-cell stiffness from reference gradients and Jacobian factors: on the uniform mesh
    it equals 0.5 K + N^T diag(v) N. The free-particle operator (lumped mass scaled by the
    volume factor) is separable: stretched by 2 in every direction its spectrum is the uniform
    one over 4; stretched by diag(1, 1, 2) its two lowest nonzero eigenvalues are the two
    distinct wave-1 eigenvalues of the uniform mesh over 4 (the z modes), exact to rounding."""
    from tests.helpers import shape_tables
    pr = small_problem(n=2, L=4.0, p=3, wells=2)
    mesh = pr.mesh
    N, dNref, F, _ = _box_geometry(mesh, (1.0, 1.0, 1.0))
    vjxw = pr.info["vjxw"]
    H = orc.cell_hamiltonians_geometry_direct(N, dNref, F, vjxw)
    ref = fe.cell_hamiltonians(mesh, vjxw)
    assert np.abs(H - ref).max() < 1e-12 * np.abs(ref).max()
    mass = mesh.lumped_mass()
    zero = np.zeros_like(vjxw)
    ev = {}
    for sc in ((1.0, 1.0, 1.0), (2.0, 2.0, 2.0), (1.0, 1.0, 2.0)):
        N, dNref, F, vol = _box_geometry(mesh, sc)
        mats = orc.cell_hamiltonians_geometry_direct(N, dNref, F, zero)
        op = orc.OracleOperator(mesh.cell_dof_map(), mats, 1 / np.sqrt(mass * vol), mesh.n_dofs)
        ev[sc] = np.linalg.eigvalsh(op.dense())
    u, iso, z2 = ev[(1.0, 1.0, 1.0)], ev[(2.0, 2.0, 2.0)], ev[(1.0, 1.0, 2.0)]
    assert np.abs(iso - u / 4.0).max() < 1e-10 * u.max()
    waves = np.unique(np.round(u[1:7], 9))       # the two distinct wave-1 eigenvalues
    assert len(waves) == 2
    assert abs(z2[0]) < 1e-10
    assert np.allclose(z2[1:3], waves / 4.0, rtol=1e-9)
