"""Shared helpers for the CheFSI tests (small seeded problems, dense references)."""
from __future__ import annotations

import numpy as np

from dftfe_gb300 import fe, problems
from oracle import oracle as orc


def small_problem(n=3, L=6.0, p=2, wells=2, nwfc=8, seed=1, projectors=False, kpoint=None):
    return problems.make_problem(n=n, L=L, p=p, n_wells=wells, n_wfc=nwfc, seed=seed,
                                 projectors=projectors, kpoint=kpoint)


def oracle_op(pr, constraints=None, unfolded=False):
    if unfolded:
        emap, n_ext, cmap_args, mass_ext = unfolded_setup(pr)
        return orc.OracleOperator(emap, pr.cell_mats, 1.0 / np.sqrt(mass_ext), n_ext,
                                  projectors=None, constraints=cmap_args)
    return orc.OracleOperator(pr.cell_map, pr.cell_mats, pr.inv_sqrt_mass, pr.n_dofs,
                              projectors=pr.nonlocal_, constraints=constraints)


def unfolded_setup(pr):
    """The periodic operator on the unfolded (np+1)^3 lattice with periodicity expressed as
    constraint rows (slave = master, weight 1); masters carry the folded mass."""
    mesh = pr.mesh
    emap, n_ext, slaves, masters = mesh.unfolded_dof_map()
    e2f = mesh.extended_to_folded()
    mass_ext = pr.mass[e2f].copy()
    ptr = np.arange(len(slaves) + 1, dtype=np.int32)
    w = np.ones(len(slaves))
    return emap, n_ext, (slaves, ptr, masters, w), mass_ext


def shape_tables(mesh, nq1=None):
    """Shape values N [n_q][n_e], real-space gradients dN [3][n_q][n_e] and JxW [n_q] at the
    QGauss(nq1)^3 points of a uniform cell (q = qx + nq1 (qy + nq1 qz), I = a + p1 (b + p1 c))."""
    nq1 = mesh.p + 3 if nq1 is None else nq1
    xq, _ = fe.gauss_nodes_weights(nq1)
    phi, dphi = mesh.shape_1d(xq)
    q = np.arange(nq1 ** 3)
    qx, qy, qz = q % nq1, (q // nq1) % nq1, q // (nq1 * nq1)
    i = np.arange(mesh.nodes_per_cell)
    p1 = mesh.p + 1
    ia, ib, ic = i % p1, (i // p1) % p1, i // (p1 * p1)
    fx, fy, fz = phi[qx][:, ia], phi[qy][:, ib], phi[qz][:, ic]
    gx, gy, gz = dphi[qx][:, ia] / mesh.h, dphi[qy][:, ib] / mesh.h, dphi[qz][:, ic] / mesh.h
    N = fx * fy * fz
    dN = np.stack([gx * fy * fz, fx * gy * fz, fx * fy * gz])
    _, w3 = mesh.quadrature(nq1)
    return N, dN, w3


def dense_operator(pr) -> np.ndarray:
    cm = pr.cell_map
    H = np.zeros((pr.n_dofs, pr.n_dofs), dtype=pr.cell_mats.dtype)
    for c in range(pr.mesh.n_cells):
        H[np.ix_(cm[c], cm[c])] += pr.cell_mats[c]
    if pr.nonlocal_ is not None:
        C = pr.nonlocal_.dense(pr.n_dofs)
        H += C @ np.diag(pr.nonlocal_.couplings.reshape(-1)) @ C.T
    d = pr.inv_sqrt_mass
    return d[:, None] * H * d[None, :]


def cheb_scalar(lam, m, a, b, a0):
    """The scalar polynomial the sigma-form filter applies (same recurrence on numbers)."""
    lam = np.asarray(lam, dtype=np.float64)
    e, c = (b - a) / 2, (b + a) / 2
    sigma = e / (a0 - c)
    sigma1, gamma = sigma, 2 / sigma
    x = np.ones_like(lam)
    y = (sigma1 / e) * (lam - c) * x
    for _ in range(2, m + 1):
        sigma2 = 1 / (gamma - sigma)
        x, y = y, 2 * sigma2 / e * (lam - c) * y - sigma * sigma2 * x
        sigma = sigma2
    return y
