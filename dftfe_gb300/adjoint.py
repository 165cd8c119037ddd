"""Hand-written adjoint of Chebyshev-filtered subspace iteration w.r.t. the local potential.

Loss: L(V) = sum of the lowest ``n_sum`` Ritz values after ``n_iter`` CheFSI iterations
(filter of degree m, generalised Rayleigh-Ritz) started from a fixed block X0, with V the
local potential at the quadrature points of every cell. The spectrum bounds of each
iteration are recorded in the forward pass and held fixed in the backward pass.

Forward (FP64, on the GPU through the C ABI): assemble H_c = 1/2 K + N^T diag(V JxW) N on the
device, then per iteration: filter, Rayleigh-Ritz (which rotates X by W = L^{-T} Q).

Backward (reverse mode, on the GPU through the C ABI):
* explicit term dL/dA = sum_i x_i x_i^T over the summed Ritz vectors (Hellmann-Feynman;
  on its own it is the electron density of those states at the quadrature points);
* Rayleigh-Ritz: dL/dX_f = 2 (A X~ - X~ Lambda) W^T (restricted to the summed states);
* each filter is linear in its input block, p(A) X_in, so the adjoint runs the three-term
  recurrence backwards -- vbar_{k-1} += alpha1_k (A - c) vbar_k, vbar_{k-2} += alpha2_k vbar_k
  -- and accumulates dL/dA += alpha1_k vbar_k v_{k-1}^T at the cell level
  (chefsi_cell_outer_accumulate). The forward vectors v_k are recomputed segment by segment
  from checkpoints stored every ``checkpoint`` degrees;
* between iterations the gradient goes back through the fixed rotation: dL/dX_f = dL/dX_in W^T
  (the Ritz-value sum depends only on the span, so the W-dependence term vanishes);
* dL/dV(q) = JxW(q) sum_IJ N_I(q) G_c[I][J] N_J(q) (chefsi_cell_quadrature_contract).

DFT-FE computes this gradient only at convergence, through the density
(src/dft/densityCalculator.cc:39, densityCalculatorDeviceKernels.cc:34-86); here the
backward differentiates the finite algorithm and reduces to that density as the iteration
converges, which the tests check together with central finite differences.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import chefsi, fe


def filter_coefficients(m: int, a: float, b: float, a0: float):
    """(alpha1_k, alpha2_k) for k = 1..m of the sigma-form recurrence and the shift c
    (linearAlgebraOperationsOpt.cc:276-352)."""
    e, c = (b - a) / 2.0, (b + a) / 2.0
    sigma = e / (a0 - c)
    sigma1, gamma = sigma, 2.0 / sigma
    coef = [(sigma1 / e, 0.0)]
    for _ in range(2, m + 1):
        sigma2 = 1.0 / (gamma - sigma)
        coef.append((2.0 * sigma2 / e, -(sigma * sigma2)))
        sigma = sigma2
    return coef, c


@dataclass
class AdjointSetup:
    """Everything the forward pass needs besides V: operator, FE data, start block."""
    op: chefsi.KohnShamOperator
    shape: torch.Tensor        # [n_q][n_e] shape values at the V quadrature points
    stiffness: torch.Tensor    # [n_e][n_e] cell stiffness (uniform mesh)
    jxw: torch.Tensor          # [n_cells][n_q]
    X0: torch.Tensor           # [M][N]
    n_iter: int
    n_sum: int
    degree: int
    bounds: tuple              # (a0, bLow, bUp) of the first iteration
    checkpoint: int = 6
    bounds_per_iter: list | None = None   # fixed (bLow, bUp, a0) per iteration, if given

    @classmethod
    def from_problem(cls, pr, n_iter=5, n_sum=None, degree=None, checkpoint=6, bounds=None,
                     device="cuda"):
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
        op = chefsi.KohnShamOperator.from_problem(pr)
        if bounds is None:
            lo, blow, up = chefsi.initial_bounds(op, pr.n_wfc)
            # the first-call formula assumes n_dofs >> n_wfc; keep bLow inside (a0, b)
            bounds = (lo, min(blow, lo + 0.5 * (up - lo)), up)
        X0 = torch.from_numpy(pr.initial_vectors()).to(device)
        t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float64)).to(device)
        return cls(op=op, shape=t(N), stiffness=t(mesh.stiffness_cell()), jxw=t(jxw), X0=X0,
                   n_iter=n_iter, n_sum=n_sum or pr.n_occupied, degree=degree or pr.cheb_degree,
                   bounds=tuple(bounds), checkpoint=checkpoint)


def _set_potential(s: AdjointSetup, v: torch.Tensor):
    mats = chefsi.assemble_cell_hamiltonians(s.shape, s.stiffness, (v * s.jxw).contiguous())
    s.op.update_cell_matrices(mats)


def run_forward(s: AdjointSetup, v: torch.Tensor):
    """n_iter CheFSI iterations (FP64). Returns (loss, eigenvalues, Ritz vectors, tape)."""
    _set_potential(s, v)
    a0, blow, bup = s.bounds
    X = s.X0.clone()
    tape = []
    ev = None
    for it in range(s.n_iter):
        if s.bounds_per_iter is not None:
            blow, bup, a0 = s.bounds_per_iter[it]
        Xin = X.clone()
        chefsi.chebyshevFilter(s.op, X, s.degree, blow, bup, a0)
        ev, W = chefsi.rayleighRitzGEP(s.op, X, want_w=True)
        tape.append((Xin, W, (blow, bup, a0)))
        a0, blow = float(ev[0]), float(ev[-1])
    loss = float(np.sum(ev[: s.n_sum]))
    return loss, ev, X, tape


def _filter_backward(s: AdjointSetup, Xin: torch.Tensor, gbar: torch.Tensor, a, b, a0,
                     G: torch.Tensor) -> torch.Tensor:
    """Adjoint of X_f = p_m(A) Xin: returns dL/dXin, accumulates dL/dH_c into G."""
    op, m, ck = s.op, s.degree, s.checkpoint
    coef, c = filter_coefficients(m, a, b, a0)

    def step(k, v_km1, v_km2):
        """v_k = alpha1_k (A - c) v_{k-1} + alpha2_k v_{k-2}."""
        a1, a2 = coef[k - 1]
        out = torch.zeros_like(v_km1)
        if k >= 2 and a2 != 0.0:
            chefsi.axpby(a2, v_km2, 0.0, out)
        chefsi.axpby(-c * a1, v_km1, 1.0, out)
        op.HX(v_km1, out, scalar=a1, scaleFlag=True)
        return out

    # forward sweep storing checkpoint pairs (v_{j-1}, v_j) at j = 0, ck, 2ck, ...
    checkpoints = {0: (None, Xin)}
    prev, cur = None, Xin
    for k in range(1, m + 1):
        nxt = step(k, cur, prev)
        prev, cur = cur, nxt
        if k % ck == 0 and k < m:
            checkpoints[k] = (prev, cur)

    def segment(start):
        """v_start .. v_{start+ck-1} recomputed from the checkpoint at start."""
        p, c0 = checkpoints[start]
        vs = {start: c0}
        if p is not None:
            vs[start - 1] = p
        for k in range(start + 1, min(start + ck, m + 1)):
            vs[k] = step(k, vs[k - 1], vs.get(k - 2))
        return vs

    vbar = {m: gbar}
    seg_start, seg = None, None
    for k in range(m, 0, -1):
        need = k - 1
        st = (need // ck) * ck
        if st != seg_start:
            seg_start, seg = st, segment(st)
        v_km1 = seg[need]
        a1, a2 = coef[k - 1]
        vb = vbar.pop(k)
        op.cell_outer_accumulate(vb, v_km1, a1, G)
        tgt = vbar.get(k - 1)
        if tgt is None:
            tgt = torch.zeros_like(vb)
            vbar[k - 1] = tgt
        chefsi.axpby(-c * a1, vb, 1.0, tgt)
        op.HX(vb, tgt, scalar=a1, scaleFlag=True)
        if k >= 2 and a2 != 0.0:
            t2 = vbar.get(k - 2)
            if t2 is None:
                t2 = torch.zeros_like(vb)
                vbar[k - 2] = t2
            chefsi.axpby(a2, vb, 1.0, t2)
    return vbar[0]


def run_backward(s: AdjointSetup, gL: float, ev, X, tape):
    """dL/dV at every quadrature point, [n_cells][n_q]."""
    op = s.op
    n = s.n_sum
    nc, ne = op.n_cells, op.nodes_per_cell
    G = torch.zeros((nc, ne, ne), dtype=torch.float64, device=X.device)
    Xocc = X[:, :n].contiguous()
    lam = torch.from_numpy(np.asarray(ev[:n])).to(X.device)
    # explicit (Hellmann-Feynman) term
    op.cell_outer_accumulate(Xocc, Xocc, gL, G)
    # Rayleigh-Ritz: dL/dX_f = 2 (A X~ - X~ Lambda) W_occ^T
    R = op.apply(Xocc)
    chefsi.gemm(Xocc, torch.diag(lam), alpha=-1.0, beta=1.0, C=R)
    _project_out(X, R)
    _, W_last, _ = tape[-1]
    gbar = chefsi.gemm(R, W_last[:, :n].contiguous(), tb="T", alpha=2.0 * gL)
    for it in range(len(tape) - 1, -1, -1):
        Xin, W, (blow, bup, a0) = tape[it]
        gin = _filter_backward(s, Xin, gbar, blow, bup, a0, G)
        if it > 0:
            # the loss depends on span(Xin) only, so its exact gradient is orthogonal to that
            # span; removing the within-span part drops roundoff that the next rotation W^T
            # would amplify by up to 1/p(lambda_top) per iteration
            _project_out(Xin, gin)
            _, Wprev, _ = tape[it - 1]
            gbar = chefsi.gemm(gin, Wprev, tb="T")
    return chefsi.cell_quadrature_contract(s.shape, G, s.jxw)


def _project_out(Q: torch.Tensor, G: torch.Tensor):
    """G <- G - Q (Q^T G) for a block Q with orthonormal columns (in place)."""
    C = chefsi.gemm(Q, G, ta="T")
    chefsi.gemm(Q, C, alpha=-1.0, beta=1.0, C=G)


def density_term(s: AdjointSetup, X: torch.Tensor) -> torch.Tensor:
    """JxW(q) sum_i |psi_i(q)|^2 over the summed Ritz vectors (psi = M^{-1/2} x interpolated)."""
    nc, ne = s.op.n_cells, s.op.nodes_per_cell
    G = torch.zeros((nc, ne, ne), dtype=torch.float64, device=X.device)
    Xocc = X[:, : s.n_sum].contiguous()
    s.op.cell_outer_accumulate(Xocc, Xocc, 1.0, G)
    return chefsi.cell_quadrature_contract(s.shape, G, s.jxw)


class FilteredRitzSum(torch.autograd.Function):
    """L(V) = sum of the lowest n_sum Ritz values after n_iter CheFSI iterations."""

    @staticmethod
    def forward(ctx, v: torch.Tensor, setup: AdjointSetup):
        loss, ev, X, tape = run_forward(setup, v)
        ctx.setup = setup
        ctx.saved = (ev, X, tape)
        return torch.tensor(loss, dtype=torch.float64, device=v.device)

    @staticmethod
    def backward(ctx, grad_out):
        ev, X, tape = ctx.saved
        g = run_backward(ctx.setup, float(grad_out), ev, X, tape)
        return g, None


def ritz_sum(v: torch.Tensor, setup: AdjointSetup) -> torch.Tensor:
    return FilteredRitzSum.apply(v, setup)
