"""Finite-element discretisation of a periodic cube for the Kohn-Sham eigenproblem.

This module builds the inputs that DFT-FE's CheFSI path consumes, i.e. the caller side of
the boundary (in DFT-FE these come from deal.II's ``FE_Q`` / ``MatrixFree`` and from
``kohnShamDFTOperatorDeviceClass::reinit``):

* the degree-p Lagrange basis on Gauss-Lobatto-Legendre (GLL) nodes
  (``FE_Q<3>(QGaussLobatto<1>(p+1))``, src/dft/dft.cc:86-92);
* the quadrature rules DFT-FE registers (src/dft/initBoundaryConditions.cc:214-232,295-296):
  QGauss(p+1) for the stiffness matrix, QGauss(p+3) for V_eff and the k-point terms;
* the lumped GLL mass vector M_ii = sum_q N_i(q)^2 JxW with QGaussLobatto(p+1)
  (src/dftOperator/kohnShamDFTOperatorDevice.cc:940-1033);
* the periodic cell -> dof map with the periodic constraints folded in (each boundary node
  on a "+" face is the same dof as its image on the "-" face), and, for testing the
  constraint path, the unfolded map plus the equivalent constraint rows;
* cell Hamiltonian matrices H_e = 1/2 K_e + sum_q V(q) JxW(q) N_I(q) N_J(q)
  (+ 1/2|k|^2 M_e - i k . G_e for Bloch k-points), the formula of ``hamMatrixKernelLDA``
  (src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:61-115 real,
  :119-280 complex), evaluated here by sum factorisation over the tensor-product
  quadrature (same value, fewer flops);
* Gaussian local wells and Gaussian x real-solid-harmonic nonlocal projectors.

Conventions: Hartree atomic units; local node I = a + (p+1)*(b + (p+1)*c) (x fastest);
global node g = ix + np*(iy + np*iz) on the periodic lattice np = n*p; cells numbered in
Morton order of (cx, cy, cz) (``PeriodicCubeMesh.cell_xyz``).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


# ----------------------------------------------------------------------------- 1-D rules

def gll_nodes_weights(p: int):
    """GLL nodes and weights of degree p on [0, 1] (p+1 points).

    Nodes: the end points and the roots of P_p'(x); weights 2/(p(p+1) P_p(x_i)^2) on [-1, 1].
    """
    if p < 1:
        raise ValueError("degree must be >= 1")
    leg = np.polynomial.legendre.Legendre.basis(p)
    interior = np.sort(np.real(leg.deriv().roots())) if p > 1 else np.zeros(0)
    x = np.concatenate([[-1.0], interior, [1.0]])
    # one Newton polish of the interior roots in extended care
    for _ in range(3):
        if p > 1:
            d1 = leg.deriv()(x[1:-1])
            d2 = leg.deriv(2)(x[1:-1])
            x[1:-1] -= d1 / d2
    w = 2.0 / (p * (p + 1) * leg(x) ** 2)
    return 0.5 * (x + 1.0), 0.5 * w


def gauss_nodes_weights(n: int):
    """n-point Gauss-Legendre rule on [0, 1]."""
    x, w = np.polynomial.legendre.leggauss(n)
    return 0.5 * (x + 1.0), 0.5 * w


def lagrange_1d(nodes: np.ndarray, x: np.ndarray):
    """Values and first derivatives of the Lagrange polynomials on ``nodes`` at ``x``.

    Returns (phi, dphi), each of shape [len(x), len(nodes)].
    """
    nodes = np.asarray(nodes, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    k = len(nodes)
    phi = np.ones((len(x), k))
    dphi = np.zeros((len(x), k))
    for j in range(k):
        others = [m for m in range(k) if m != j]
        denom = np.prod([nodes[j] - nodes[m] for m in others])
        for m in others:
            phi[:, j] *= (x - nodes[m])
        # derivative: sum over dropped factor
        for m in others:
            term = np.ones(len(x))
            for l in others:
                if l != m:
                    term *= (x - nodes[l])
            dphi[:, j] += term
        phi[:, j] /= denom
        dphi[:, j] /= denom
    return phi, dphi


# ----------------------------------------------------------------------------- mesh

@dataclass
class PeriodicCubeMesh:
    """Uniform n^3 hex mesh of the periodic cube [0, L)^3 with a degree-p GLL basis."""

    n: int
    L: float
    p: int
    h: float = field(init=False)
    npts: int = field(init=False)          # lattice points per side = n*p
    n_cells: int = field(init=False)
    n_dofs: int = field(init=False)
    nodes_per_cell: int = field(init=False)

    def __post_init__(self):
        if self.n < 1 or self.p < 1:
            raise ValueError("need n >= 1 and p >= 1")
        self.h = self.L / self.n
        self.npts = self.n * self.p
        self.n_cells = self.n ** 3
        self.n_dofs = self.npts ** 3
        self.nodes_per_cell = (self.p + 1) ** 3
        self.gll_x, self.gll_w = gll_nodes_weights(self.p)
        # cells are numbered in Morton (Z) order of their integer coordinates, the order
        # p4est hands DFT-FE its cells in; neighbouring cells stay close in the numbering
        lex = np.arange(self.n_cells)
        lx, ly, lz = lex % self.n, (lex // self.n) % self.n, lex // (self.n * self.n)
        code = np.zeros(self.n_cells, dtype=np.int64)
        for bit in range(max(1, int(self.n - 1).bit_length())):
            code |= ((lx >> bit) & 1) << (3 * bit)
            code |= ((ly >> bit) & 1) << (3 * bit + 1)
            code |= ((lz >> bit) & 1) << (3 * bit + 2)
        order = np.argsort(code, kind="stable")
        self.cell_xyz = np.stack([lx[order], ly[order], lz[order]], axis=1)

    # -- maps ---------------------------------------------------------------------------
    def cell_origin(self):
        """[n_cells, 3] lower corners of the cells."""
        return self.cell_xyz.astype(np.float64) * self.h

    def cell_dof_map(self) -> np.ndarray:
        """[n_cells, n_e] int32 global dof of each cell node, periodic images folded."""
        n, p, npts = self.n, self.p, self.npts
        cx, cy, cz = self.cell_xyz[:, 0], self.cell_xyz[:, 1], self.cell_xyz[:, 2]
        a = np.arange(p + 1)
        ix = (cx[:, None] * p + a[None, :]) % npts          # [nc, p+1]
        iy = (cy[:, None] * p + a[None, :]) % npts
        iz = (cz[:, None] * p + a[None, :]) % npts
        g = (ix[:, None, None, :] + npts * (iy[:, None, :, None] + npts * iz[:, :, None, None]))
        return g.reshape(self.n_cells, -1).astype(np.int32)

    def unfolded_dof_map(self):
        """Map onto the (np+1)^3 lattice without folding, plus the periodic constraints.

        Returns (map [n_cells, n_e] int32, n_ext, slave_ids int32, master_ids int32) where
        every lattice point with some coordinate == np is a slave of its folded image with
        weight 1 (deal.II ``make_periodicity_constraints``; applied on the device by
        ``constraintMatrixInfoDevice::distribute``, utils/constraintMatrixInfoDevice.cc:546).
        """
        n, p, npts = self.n, self.p, self.npts
        m = npts + 1
        cx, cy, cz = self.cell_xyz[:, 0], self.cell_xyz[:, 1], self.cell_xyz[:, 2]
        a = np.arange(p + 1)
        ix = cx[:, None] * p + a[None, :]
        iy = cy[:, None] * p + a[None, :]
        iz = cz[:, None] * p + a[None, :]
        g = (ix[:, None, None, :] + m * (iy[:, None, :, None] + m * iz[:, :, None, None]))
        emap = g.reshape(self.n_cells, -1).astype(np.int32)
        # extended lattice -> folded lattice; folded dof ids are embedded in the extended
        # numbering at the same (ix, iy, iz) with all coords < np.
        lat = np.arange(m ** 3)
        lx, ly, lz = lat % m, (lat // m) % m, lat // (m * m)
        is_slave = (lx == npts) | (ly == npts) | (lz == npts)
        fx, fy, fz = lx % npts, ly % npts, lz % npts
        master = fx + m * (fy + m * fz)
        return emap, m ** 3, lat[is_slave].astype(np.int32), master[is_slave].astype(np.int32)

    def extended_to_folded(self):
        """For the unfolded lattice: index of each extended point in the folded numbering."""
        m = self.npts + 1
        lat = np.arange(m ** 3)
        lx, ly, lz = lat % m, (lat // m) % m, lat // (m * m)
        return ((lx % self.npts) + self.npts * ((ly % self.npts) + self.npts * (lz % self.npts))).astype(np.int64)

    # -- basis data -------------------------------------------------------------------
    def shape_1d(self, xq):
        return lagrange_1d(self.gll_x, xq)

    def lumped_mass(self) -> np.ndarray:
        """Lumped GLL mass vector M_g (QGaussLobatto(p+1) quadrature, nodes == points)."""
        w = self.gll_w
        we = (w[None, None, :] * w[None, :, None] * w[:, None, None]).reshape(-1) * self.h ** 3
        cmap = self.cell_dof_map()
        return np.bincount(cmap.reshape(-1), weights=np.tile(we, self.n_cells), minlength=self.n_dofs)

    def stiffness_cell(self) -> np.ndarray:
        """K_e[I, J] = int grad N_I . grad N_J over one (uniform) cell, QGauss(p+1)."""
        xq, wq = gauss_nodes_weights(self.p + 1)
        phi, dphi = self.shape_1d(xq)
        M1 = (phi * wq[:, None]).T @ phi
        K1 = (dphi * wq[:, None]).T @ dphi
        k = np.kron
        return self.h * (k(M1, k(M1, K1)) + k(M1, k(K1, M1)) + k(K1, k(M1, M1)))

    def quadrature(self, nq1: int | None = None):
        """QGauss(nq1) points of every cell: returns (points [n_cells, nq, 3], JxW [nq])."""
        nq1 = self.p + 3 if nq1 is None else nq1
        xq, wq = gauss_nodes_weights(nq1)
        qx = np.tile(xq, nq1 * nq1)
        qy = np.tile(np.repeat(xq, nq1), nq1)
        qz = np.repeat(xq, nq1 * nq1)
        ref = np.stack([qx, qy, qz], axis=1) * self.h
        w3 = (wq[None, None, :] * wq[None, :, None] * wq[:, None, None]).reshape(-1) * self.h ** 3
        return self.cell_origin()[:, None, :] + ref[None, :, :], w3


# ----------------------------------------------------------------------------- physics

def min_image(d: np.ndarray, L: float) -> np.ndarray:
    return d - L * np.round(d / L)


def gaussian_wells_potential(points: np.ndarray, centres: np.ndarray, depths: np.ndarray,
                             width: float, L: float, cutoff_sigmas: float = 8.0) -> np.ndarray:
    """V(r) = -sum_w d_w exp(-|r - R_w|^2 / (2 s^2)) under the minimum-image convention.

    ``points`` is [n_cells, nq, 3]; each well is evaluated on the cells whose bounding box
    lies within ``cutoff_sigmas`` widths of its centre (exp(-32) ~ 1e-14 beyond 8 widths).
    """
    pts = np.asarray(points)
    nc = pts.shape[0]
    out = np.zeros(pts.shape[:-1])
    lo_c = pts.min(axis=1)
    hi_c = pts.max(axis=1)
    rc = cutoff_sigmas * width
    for R, dep in zip(centres, depths):
        lo = min_image(lo_c - R[None, :], L)
        span = hi_c - lo_c
        gap = np.where((lo <= 0.0) & (lo + span >= 0.0), 0.0,
                       np.minimum(np.abs(lo), np.abs(lo + span)))
        sel = np.nonzero((gap * gap).sum(1) < rc * rc)[0] if nc > 1 else np.arange(nc)
        if len(sel) == 0:
            continue
        d = min_image(pts[sel] - R[None, None, :], L)
        out[sel] -= dep * np.exp(-(d * d).sum(-1) / (2.0 * width * width))
    return out


def cell_mass_like_matrices(mesh: PeriodicCubeMesh, weights: np.ndarray, nq1: int,
                            cells: np.ndarray | None = None, chunk: int = 256) -> np.ndarray:
    """sum_q weights[c, q] N_I(q) N_J(q) for each cell, by sum factorisation.

    ``weights`` is [n_sel, nq1^3] with q = qx + nq1*(qy + nq1*qz). Returns [n_sel, n_e, n_e].
    """
    p1 = mesh.p + 1
    xq, _ = gauss_nodes_weights(nq1)
    phi, _ = mesh.shape_1d(xq)                           # [nq1, p1]
    P = phi[:, :, None] * phi[:, None, :]                # [nq1, a, A]
    nsel = weights.shape[0]
    out = np.empty((nsel, p1 ** 3, p1 ** 3))
    for s in range(0, nsel, chunk):
        v = weights[s:s + chunk].reshape(-1, nq1, nq1, nq1)           # [c, z, y, x]
        t1 = np.einsum('czyx,xaA->czyaA', v, P, optimize=True)
        t2 = np.einsum('czyaA,ybB->czbBaA', t1, P, optimize=True)
        t3 = np.einsum('czbBaA,zkK->ckKbBaA', t2, P, optimize=True)
        # t3[c, k, K, b, B, a, A] -> [c, (k b a), (K B A)]
        out[s:s + chunk] = t3.transpose(0, 1, 3, 5, 2, 4, 6).reshape(-1, p1 ** 3, p1 ** 3)
    return out


def cell_gradient_mass_matrices(mesh: PeriodicCubeMesh, nq1: int) -> np.ndarray:
    """G_e[d, I, J] = int dN_I/dx_d N_J over one (uniform) cell, QGauss(nq1). [3, n_e, n_e]."""
    xq, wq = gauss_nodes_weights(nq1)
    phi, dphi = mesh.shape_1d(xq)
    M1 = (phi * wq[:, None]).T @ phi            # int phi_a phi_A
    D1 = (dphi * wq[:, None]).T @ phi           # int phi_a' phi_A
    k = np.kron
    h2 = mesh.h ** 2                            # h^3 volume / h derivative
    return np.stack([h2 * k(M1, k(M1, D1)), h2 * k(M1, k(D1, M1)), h2 * k(D1, k(M1, M1))])


def cell_hamiltonians(mesh: PeriodicCubeMesh, v_jxw: np.ndarray, kpoint=None,
                      nq1: int | None = None) -> np.ndarray:
    """Cell Hamiltonians H_e = 1/2 K_e + V_e (+ 1/2|k|^2 M_e - i k.G_e).

    The formula of hamMatrixKernelLDA
    (src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:61-115, :119-280):
    the real part is 1/2 cellShapeFunctionGradientIntegral + sum_q vEffJxW N_I N_J
    (+ kSquareTimesHalf * sum_q JxW N_I N_J), the imaginary part is
    -k . sum_q JxW gradN_I N_J.
    """
    nq1 = mesh.p + 3 if nq1 is None else nq1
    K = mesh.stiffness_cell()
    H = cell_mass_like_matrices(mesh, v_jxw, nq1)
    H += 0.5 * K[None]
    if kpoint is None:
        return H
    k = np.asarray(kpoint, dtype=np.float64)
    _, w3 = mesh.quadrature(nq1)
    Me = cell_mass_like_matrices(mesh, w3[None, :], nq1)[0]
    G = cell_gradient_mass_matrices(mesh, nq1)
    # The stored matrix is the one applied to the cell vector: A_e[I, J] = H_ref[J, I]
    # with H_ref the reference's flattened layout (its complex HX multiplies with OP_T,
    # src/dftOperator/matrixVectorProductImplementationsDevice.cc:48-66), so the imaginary
    # part is -k . int N_I grad N_J.
    Gt = G.transpose(0, 2, 1)
    Hc = H.astype(np.complex128)
    Hc += (0.5 * float(k @ k)) * Me[None]
    Hc += 1j * (-(k[0] * Gt[0] + k[1] * Gt[1] + k[2] * Gt[2]))[None]
    return Hc


def solid_harmonics(d: np.ndarray, sigma: float) -> np.ndarray:
    """The 8 real solid harmonics (s, p_x, p_y, p_z, d_xy, d_yz, d_zx, d_x2-y2), each
    normalised so that int (Y g)^2 = 1 for g = exp(-r^2/(2 sigma^2)). d: [..., 3]."""
    x, y, z = d[..., 0], d[..., 1], d[..., 2]
    n0 = (math.pi * sigma * sigma) ** 1.5
    s2, s4 = sigma ** 2, sigma ** 4
    cols = [np.ones_like(x) / math.sqrt(n0),
            x / math.sqrt(n0 * s2 / 2), y / math.sqrt(n0 * s2 / 2), z / math.sqrt(n0 * s2 / 2),
            x * y / math.sqrt(n0 * s4 / 4), y * z / math.sqrt(n0 * s4 / 4),
            z * x / math.sqrt(n0 * s4 / 4), (x * x - y * y) / math.sqrt(n0 * s4)]
    return np.stack(cols, axis=-1)


@dataclass
class NonlocalProjectors:
    """H_nl = sum_a C_a diag(V_a) C_a^T with C_a[d, j] = int N_d beta_{a,j} (assembled).

    Storage per atom a: dof list ``dofs[ptr[a]:ptr[a+1]]`` and dense block
    ``values[vptr[a]: vptr[a] + n_dofs_a * P]`` row-major [n_dofs_a][P]; couplings V_a [P].
    """
    n_atoms: int
    n_proj: int
    ptr: np.ndarray
    dofs: np.ndarray
    values: np.ndarray
    couplings: np.ndarray

    def dense(self, n_dofs: int) -> np.ndarray:
        C = np.zeros((n_dofs, self.n_atoms * self.n_proj))
        for a in range(self.n_atoms):
            d = self.dofs[self.ptr[a]:self.ptr[a + 1]]
            C[d, a * self.n_proj:(a + 1) * self.n_proj] = self.values[self.ptr[a]:self.ptr[a + 1]]
        return C


def gaussian_projectors(mesh: PeriodicCubeMesh, centres: np.ndarray, couplings: np.ndarray,
                        sigma: float = 1.0, rcut: float = 3.0, nq1: int | None = None
                        ) -> NonlocalProjectors:
    """Assemble C_a[d, j] = int N_d(r) Y_j(r - R_a) g(r - R_a) [|r - R_a| < rcut] dr.

    The cell-level integrals mirror DFT-FE's projector matrices C_{cell} (cell x projector,
    src/dftOperator/computeNonLocalHamiltonianTimesXMemoryOptBatchGEMMDevice.cc:27-283
    consumes them); cells are selected by their bounding-box distance to the centre.
    """
    nq1 = mesh.p + 3 if nq1 is None else nq1
    P = 8
    pts, w3 = mesh.quadrature(nq1)
    xq, _ = gauss_nodes_weights(nq1)
    phi, _ = mesh.shape_1d(xq)
    origin = mesh.cell_origin()
    cmap = mesh.cell_dof_map()
    ptr = [0]
    dofs_all, vals_all = [], []
    for R in centres:
        # bounding-box distance (minimum image) from R to each cell
        lo = min_image(origin - R[None, :], mesh.L)
        gap = np.where((lo <= 0.0) & (lo + mesh.h >= 0.0), 0.0,
                       np.minimum(np.abs(lo), np.abs(lo + mesh.h)))
        sel = np.nonzero((gap * gap).sum(1) < rcut * rcut)[0]
        d = min_image(pts[sel] - R[None, None, :], mesh.L)          # [ns, nq, 3]
        r2 = (d * d).sum(-1)
        beta = solid_harmonics(d, sigma) * (np.exp(-r2 / (2 * sigma * sigma)) * (r2 < rcut * rcut))[..., None]
        wb = beta * w3[None, :, None]                                # [ns, nq, P]
        wb = wb.reshape(len(sel), nq1, nq1, nq1, P)                  # [c, z, y, x, j]
        t = np.einsum('czyxj,xa->czyaj', wb, phi, optimize=True)
        t = np.einsum('czyaj,yb->czbaj', t, phi, optimize=True)
        t = np.einsum('czbaj,zk->ckbaj', t, phi, optimize=True)
        cellC = t.reshape(len(sel), -1, P)                           # [ns, n_e, P]
        gd = cmap[sel].reshape(-1)
        uniq, inv = np.unique(gd, return_inverse=True)
        acc = np.zeros((len(uniq), P))
        np.add.at(acc, inv, cellC.reshape(-1, P))
        keep = np.abs(acc).max(1) > 0
        dofs_all.append(uniq[keep].astype(np.int32))
        vals_all.append(acc[keep])
        ptr.append(ptr[-1] + int(keep.sum()))
    return NonlocalProjectors(
        n_atoms=len(centres), n_proj=P, ptr=np.asarray(ptr, dtype=np.int32),
        dofs=np.concatenate(dofs_all) if dofs_all else np.zeros(0, np.int32),
        values=np.concatenate(vals_all) if vals_all else np.zeros((0, P)),
        couplings=np.asarray(couplings, dtype=np.float64).reshape(len(centres), P))
