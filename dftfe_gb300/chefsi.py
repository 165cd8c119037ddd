"""Host-side mirror of DFT-FE's CheFSI interface over the GB300 C ABI.

Names and argument meaning follow the reference:

* ``KohnShamOperator`` -- ``operatorDFTDeviceClass`` (include/operatorDevice.h:43-420):
  ``HX`` (:176-185, with ``scaleFlag`` / ``scalar``), ``XtHX`` (:230-241),
  ``getSqrtMassVec`` / ``getInvSqrtMassVec`` (:68-72);
* ``ChebyshevOrthogonalizedSubspaceIterationSolver`` --
  ``chebyshevOrthogonalizedSubspaceIterationSolverDevice``
  (include/chebyshevOrthogonalizedSubspaceIterationSolverDevice.h:37-166): ``solve`` (with
  the spectrum-split branch), ``solveNoRR``, ``densityMatrixEigenBasisFirstOrderResponse``,
  ``reinitSpectrumBounds``;
* ``lanczosLowerUpperBoundEigenSpectrum``, ``chebyshevFilter``, ``fillOverlapMatrix``,
  ``rayleighRitzGEP``, ``rayleighRitzGEPSpectrumSplitDirect``,
  ``densityMatrixEigenBasisFirstOrderResponse``, ``pseudoGramSchmidtOrthogonalization``,
  ``computeEigenResidualNorm`` -- the linearAlgebraOperationsDevice functions of the same
  names; ``copyValueType1ArrToValueType2Arr`` (deviceKernelsGeneric);
* ``density`` (densityCalculator), the cell-matrix assembly functions
  (hamiltonianMatrixCalculatorFlattenedDevice), ``solve_batched`` (the k-point loop).

Vectors are torch CUDA tensors in DFT-FE's flattened layout [n_dofs, n_vectors]
(vector index fastest). Every call goes through libchefsi_gb300.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib
from ._lib import PRECISIONS, check


def _ptr(t: torch.Tensor | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if t is None else t.data_ptr())


def _np_ptr(a: np.ndarray | None) -> ctypes.c_void_p:
    return ctypes.c_void_p(0 if a is None else a.ctypes.data)


def _stream(stream=None) -> ctypes.c_void_p:
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _prec(p) -> int:
    return PRECISIONS[p] if isinstance(p, str) else int(p)


class KohnShamOperator:
    """A = M^{-1/2}(H_loc + H_nl)M^{-1/2} on one GPU (operatorDFTDeviceClass)."""

    def __init__(self, cell_map, cell_mats, sqrt_mass, inv_sqrt_mass, n_dofs: int | None = None,
                 projectors=None, constraints=None):
        lib = _lib.load()
        cm = np.ascontiguousarray(cell_map, dtype=np.int32)
        self.is_complex = bool(np.iscomplexobj(cell_mats))
        mats = np.ascontiguousarray(cell_mats, dtype=np.complex128 if self.is_complex else np.float64)
        sm = np.ascontiguousarray(sqrt_mass, dtype=np.float64)
        ism = np.ascontiguousarray(inv_sqrt_mass, dtype=np.float64)
        self.n_dofs = int(n_dofs if n_dofs is not None else len(sm))
        self.n_cells, self.nodes_per_cell = cm.shape
        d = _lib.OperatorDesc()
        d.n_dofs, d.n_cells, d.nodes_per_cell = self.n_dofs, self.n_cells, self.nodes_per_cell
        d.is_complex = int(self.is_complex)
        d.cell_dof_map, d.cell_matrices = _np_ptr(cm), _np_ptr(mats)
        d.sqrt_mass, d.inv_sqrt_mass = _np_ptr(sm), _np_ptr(ism)
        keep = [cm, mats, sm, ism]
        if constraints is not None:
            ids, ptr, mas, w = (np.ascontiguousarray(a, dt) for a, dt in
                                zip(constraints, (np.int32, np.int32, np.int32, np.float64)))
            keep += [ids, ptr, mas, w]
            d.n_constrained = len(ids)
            d.constrained_ids, d.constraint_ptr = _np_ptr(ids), _np_ptr(ptr)
            d.master_ids, d.master_weights = _np_ptr(mas), _np_ptr(w)
        if projectors is not None and projectors.n_atoms > 0:
            ap = np.ascontiguousarray(projectors.ptr, np.int32)
            ad = np.ascontiguousarray(projectors.dofs, np.int32)
            av = np.ascontiguousarray(projectors.values, np.float64)
            cp = np.ascontiguousarray(projectors.couplings, np.float64)
            keep += [ap, ad, av, cp]
            d.n_atoms, d.n_proj = projectors.n_atoms, projectors.n_proj
            d.atom_dof_ptr, d.atom_dofs = _np_ptr(ap), _np_ptr(ad)
            d.atom_proj, d.couplings = _np_ptr(av), _np_ptr(cp)
        h = ctypes.c_void_p()
        check(lib.chefsi_operator_create(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        self._sqrt = torch.from_numpy(sm).cuda()
        self._isqrt = torch.from_numpy(ism).cuda()
        self.dtype = torch.complex128 if self.is_complex else torch.float64

    @classmethod
    def from_problem(cls, pr, constraints=None):
        return cls(pr.cell_map, pr.cell_mats, pr.sqrt_mass, pr.inv_sqrt_mass, pr.n_dofs,
                   projectors=pr.nonlocal_, constraints=constraints)

    @property
    def handle(self):
        return self._h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._lib is not None:
            _lib._lib.chefsi_operator_destroy(h)
            self._h = None

    def getSqrtMassVec(self) -> torch.Tensor:
        return self._sqrt

    def getInvSqrtMassVec(self) -> torch.Tensor:
        return self._isqrt

    def HX(self, src: torch.Tensor, dst: torch.Tensor, scalar: float = 1.0,
           scaleFlag: bool = False, precision="fp64", stream=None) -> torch.Tensor:
        """dst = (scaleFlag ? dst : 0) + scalar * A src (operatorDFTDeviceClass::HX)."""
        n_vec = 1 if src.dim() == 1 else src.shape[1]
        ld_s = 1 if src.dim() == 1 else src.stride(0)
        ld_d = 1 if dst.dim() == 1 else dst.stride(0)
        check(_lib.load().chefsi_hx(self._h, _ptr(src), ld_s, _ptr(dst), ld_d, n_vec,
                                    float(scalar), int(bool(scaleFlag)), _prec(precision),
                                    _stream(stream)))
        return dst

    def apply(self, X: torch.Tensor, precision="fp64") -> torch.Tensor:
        Y = torch.empty_like(X)
        return self.HX(X, Y, 1.0, False, precision)

    def XtHX(self, X: torch.Tensor, precision="fp64") -> torch.Tensor:
        N = X.shape[1]
        Hp = torch.zeros((N, N), dtype=X.dtype, device=X.device)
        check(_lib.load().chefsi_xthx(self._h, _ptr(X), X.stride(0), N, _ptr(Hp), _prec(precision),
                                      _stream()))
        return Hp

    def update_cell_matrices(self, mats: torch.Tensor):
        """Replace the cell Hamiltonians (device FP64 [n_cells][n_e][n_e], unscaled)."""
        check(_lib.load().chefsi_operator_update_cell_matrices(self._h, _ptr(mats), _stream()))

    def cell_outer_accumulate(self, U: torch.Tensor, V: torch.Tensor, alpha: float,
                              G: torch.Tensor):
        """G_c += alpha * (D U)_c (D V)_c^T over the vectors (adjoint building block)."""
        check(_lib.load().chefsi_cell_outer_accumulate(self._h, _ptr(U), _ptr(V), U.stride(0),
                                                       U.shape[1], float(alpha), _ptr(G),
                                                       _stream()))
        return G

    def overlap(self, X: torch.Tensor, precision="fp64") -> torch.Tensor:
        N = X.shape[1]
        S = torch.zeros((N, N), dtype=X.dtype, device=X.device)
        check(_lib.load().chefsi_overlap(self._h, _ptr(X), X.stride(0), N, _ptr(S), _prec(precision),
                                         _stream()))
        return S


fillOverlapMatrix = KohnShamOperator.overlap


def density(op: "KohnShamOperator", X: torch.Tensor, occupation: torch.Tensor,
            shape: torch.Tensor, jxw: torch.Tensor | None = None,
            rho: torch.Tensor | None = None, accumulate: bool = False,
            precision: str = "fp64") -> torch.Tensor:
    """rho[c][q] (+)= jxw[c][q] sum_i f_i |psi_i(x_q)|^2 (densityCalculator: the density of the
    Ritz vectors at the quadrature points; psi = M^{-1/2} x interpolated by shape [n_q][n_e])."""
    nq = shape.shape[0]
    if rho is None:
        rho = torch.zeros((op.n_cells, nq), dtype=torch.float64, device=X.device)
    occ = occupation.to(device=X.device, dtype=torch.float64).contiguous()
    check(_lib.load().chefsi_density(op.handle, _ptr(X), X.stride(0), X.shape[1], _ptr(occ), nq,
                                     _ptr(shape), _ptr(jxw), _ptr(rho), int(accumulate),
                                     _prec(precision), _stream()))
    return rho


def cell_quadrature_contract(shape: torch.Tensor, G: torch.Tensor, jxw: torch.Tensor | None):
    nc, ne, _ = G.shape
    nq = shape.shape[0]
    out = torch.empty((nc, nq), dtype=torch.float64, device=G.device)
    check(_lib.load().chefsi_cell_quadrature_contract(nc, ne, nq, _ptr(shape), _ptr(G), _ptr(jxw),
                                                      _ptr(out), _stream()))
    return out


def lanczosLowerUpperBoundEigenSpectrum(op: KohnShamOperator, k: int = 20,
                                        reproducible: bool = False, v0: np.ndarray | None = None,
                                        seed: int = 0):
    lo, up = ctypes.c_double(), ctypes.c_double()
    v = None if v0 is None else np.ascontiguousarray(v0, np.float64)
    check(_lib.load().chefsi_lanczos_bounds(op.handle, k, int(reproducible), _np_ptr(v), seed,
                                            ctypes.byref(lo), ctypes.byref(up), _stream()))
    return lo.value, up.value


def chebyshevFilter(op: KohnShamOperator, X: torch.Tensor, m: int, a: float, b: float, a0: float,
                    precision="fp64") -> torch.Tensor:
    check(_lib.load().chefsi_chebyshev_filter(op.handle, _ptr(X), X.stride(0), X.shape[1], m,
                                              float(a), float(b), float(a0), _prec(precision),
                                              _stream()))
    return X


def pseudoGramSchmidtOrthogonalization(op: KohnShamOperator, X: torch.Tensor, precision="fp64"):
    check(_lib.load().chefsi_cholesky_gs(op.handle, _ptr(X), X.stride(0), X.shape[1],
                                         _prec(precision), _stream()))
    return X


def rayleighRitzGEP(op: KohnShamOperator, X: torch.Tensor, precision="fp64", want_hx=False,
                    want_w=False):
    """Generalised Rayleigh-Ritz in place on X; returns eigenvalues (and HX_rot, W if asked)."""
    N = X.shape[1]
    ev = np.zeros(N)
    HX = torch.empty_like(X) if want_hx else None
    W = torch.empty((N, N), dtype=X.dtype, device=X.device) if want_w else None
    check(_lib.load().chefsi_rayleigh_ritz(op.handle, _ptr(X), X.stride(0), N, _np_ptr(ev),
                                           _ptr(HX), _ptr(W), _prec(precision), _stream()))
    out = [ev]
    if want_hx:
        out.append(HX)
    if want_w:
        out.append(W)
    return out[0] if len(out) == 1 else tuple(out)


def rayleighRitzGEPSpectrumSplitDirect(op: KohnShamOperator, X: torch.Tensor, XFrac: torch.Tensor,
                                       Noc: int, precision="fp64", want_hx=False,
                                       frac_reduced=False):
    """Spectrum-split Rayleigh-Ritz (linearAlgebraOperationsDevice.h:279-298): X [n_dofs, N]
    is orthonormalised in place, XFrac [n_dofs, N - Noc] receives X Q_fr; returns the N - Noc
    eigenvalues (ascending), and H XFrac when want_hx."""
    N = X.shape[1]
    nfr = N - Noc
    if XFrac.shape != (X.shape[0], nfr) or XFrac.dtype != X.dtype:
        raise ValueError("XFrac must be [n_dofs, N - Noc] of X's dtype")
    ev = np.zeros(nfr)
    HXF = torch.empty_like(XFrac) if want_hx else None
    check(_lib.load().chefsi_rayleigh_ritz_spectrum_split(
        op.handle, _ptr(X), X.stride(0), N, int(Noc), _ptr(XFrac), XFrac.stride(0), _np_ptr(ev),
        _ptr(HXF), _prec(precision), int(bool(frac_reduced)), _stream()))
    return (ev, HXF) if want_hx else ev


def densityMatrixEigenBasisFirstOrderResponse(opPrime: KohnShamOperator, X: torch.Tensor,
                                              eigenValues, fermiEnergy: float, TVal: float,
                                              precision="fp64") -> np.ndarray:
    """First-order density-matrix response (linearAlgebraOperationsDevice.h:302-322): X
    [n_dofs, N] (orthonormal eigenvectors) becomes X P' in place, P' the first-order response
    of the recursive Fermi-operator expansion to the perturbation opPrime applies; returns
    densityMatDerFermiEnergy (N values)."""
    N = X.shape[1]
    ev = np.ascontiguousarray(eigenValues, dtype=np.float64)
    if ev.shape != (N,):
        raise ValueError("eigenValues must have N entries")
    dmu = np.zeros(N)
    check(_lib.load().chefsi_density_matrix_first_order_response(
        opPrime.handle, _ptr(X), X.stride(0), N, _np_ptr(ev), float(fermiEnergy), float(TVal),
        _np_ptr(dmu), _prec(precision), _stream()))
    return dmu


def gemm(A: torch.Tensor, B: torch.Tensor, ta: str = "N", tb: str = "N", alpha: float = 1.0,
         beta: float = 0.0, C: torch.Tensor | None = None, precision="fp64") -> torch.Tensor:
    """C = alpha op(A) op(B) + beta C on the GPU (row-major FP64)."""
    M = A.shape[1] if ta == "T" else A.shape[0]
    K = A.shape[0] if ta == "T" else A.shape[1]
    N = B.shape[0] if tb == "T" else B.shape[1]
    if C is None:
        C = torch.zeros((M, N), dtype=torch.float64, device=A.device)
    check(_lib.load().chefsi_gemm(ta.encode(), tb.encode(), M, N, K, float(alpha), _ptr(A),
                                  A.stride(0), _ptr(B), B.stride(0), float(beta), _ptr(C),
                                  C.stride(0), _prec(precision), _stream()))
    return C


def axpby(a: float, x: torch.Tensor, b: float, y: torch.Tensor) -> torch.Tensor:
    """y = a x + b y (FP64 device blocks) through the library."""
    n = 1 if y.dim() == 1 else y.shape[1]
    ldx = 1 if x.dim() == 1 else x.stride(0)
    ldy = 1 if y.dim() == 1 else y.stride(0)
    check(_lib.load().chefsi_axpby(y.shape[0], n, float(a), _ptr(x), ldx, float(b), _ptr(y), ldy,
                                   _stream()))
    return y


def copyValueType1ArrToValueType2Arr(src: torch.Tensor, dst: torch.Tensor,
                                     scale: float = 1.0) -> torch.Tensor:
    """dst = scale * src with precision conversion (FP32 / FP64 device blocks, 1-D or 2-D with
    unit column stride) through the library: a power-of-two scale is exact, one rounding."""
    bits = {torch.float32: 32, torch.float64: 64}
    rows = src.shape[0]
    n = 1 if src.dim() == 1 else src.shape[1]
    lds = n if src.dim() == 1 else src.stride(0)
    ldd = n if dst.dim() == 1 else dst.stride(0)
    if src.dim() == 1:
        rows, n, lds, ldd = 1, src.shape[0], src.shape[0], dst.shape[0]
    check(_lib.load().chefsi_convert_block(bits[src.dtype], _ptr(src), lds, bits[dst.dtype],
                                           _ptr(dst), ldd, rows, n, float(scale), _stream()))
    return dst


def assemble_cell_hamiltonians(shape: torch.Tensor, stiffness: torch.Tensor,
                               v_jxw: torch.Tensor) -> torch.Tensor:
    """H_c = 1/2 K + N^T diag(v_jxw_c) N for every cell, on the GPU."""
    nc, nq = v_jxw.shape
    ne = stiffness.shape[0]
    out = torch.empty((nc, ne, ne), dtype=torch.float64, device=v_jxw.device)
    check(_lib.load().chefsi_assemble_cell_hamiltonians(nc, ne, nq, _ptr(shape), _ptr(stiffness),
                                                        _ptr(v_jxw), _ptr(out), _stream()))
    return out


def assemble_cell_hamiltonians_geometry(shape: torch.Tensor, shape_grad_ref: torch.Tensor,
                                        jacobian_factor: torch.Tensor,
                                        v_jxw: torch.Tensor) -> torch.Tensor:
    """Cell Hamiltonians [n_cells, n_e, n_e] of cells of any shape on the GPU: the per-cell
    stiffness of FEBasisOperations::computeCellStiffnessMatrix from the reference-cell gradients
    shape_grad_ref [3, n_q, n_e] and the Jacobian factors jacobian_factor [n_cells, n_q, 3, 3]
    (J^-1 J^-T JxW), plus the LDA potential term v_jxw [n_cells, n_q]."""
    nc, nq = v_jxw.shape
    ne = shape.shape[1]
    if tuple(jacobian_factor.shape) != (nc, nq, 3, 3) or tuple(shape_grad_ref.shape) != (3, nq, ne):
        raise ValueError("jacobian_factor must be [n_cells, n_q, 3, 3], shape_grad_ref [3, n_q, n_e]")
    F = jacobian_factor.contiguous()
    out = torch.empty((nc, ne, ne), dtype=torch.float64, device=v_jxw.device)
    check(_lib.load().chefsi_assemble_cell_hamiltonians_geometry(
        nc, ne, nq, _ptr(shape), _ptr(shape_grad_ref), _ptr(F), _ptr(v_jxw), _ptr(out),
        _stream()))
    return out


def assemble_cell_hamiltonians_gga(shape: torch.Tensor, shape_grad: torch.Tensor,
                                   stiffness: torch.Tensor, v_jxw: torch.Tensor,
                                   gga_jxw: torch.Tensor) -> torch.Tensor:
    """GGA cell Hamiltonians [n_cells, n_e, n_e] on the GPU (hamMatrixKernelGGAMemOpt, real):
    gga_jxw is derExcWithSigmaTimesGradRhoJxW [n_cells, n_q, 3]."""
    nc, nq = v_jxw.shape
    ne = stiffness.shape[0]
    if tuple(gga_jxw.shape) != (nc, nq, 3):
        raise ValueError("gga_jxw must be [n_cells, n_q, 3]")
    g = gga_jxw.contiguous()
    out = torch.empty((nc, ne, ne), dtype=torch.float64, device=v_jxw.device)
    check(_lib.load().chefsi_assemble_cell_hamiltonians_gga(
        nc, ne, nq, _ptr(shape), _ptr(shape_grad), _ptr(stiffness), _ptr(v_jxw), _ptr(g),
        _ptr(out), _stream()))
    return out


def assemble_cell_hamiltonians_bloch(shape: torch.Tensor, shape_grad: torch.Tensor,
                                     stiffness: torch.Tensor, v_jxw: torch.Tensor,
                                     jxw: torch.Tensor, kpoints,
                                     gga_jxw: torch.Tensor | None = None) -> torch.Tensor:
    """Bloch cell Hamiltonians [n_k, n_cells, n_e, n_e] (complex128) for every k-point, on the
    GPU (the k-point form of hamMatrixKernelLDA, or of hamMatrixKernelGGAMemOpt with gga_jxw
    [n_cells, n_q, 3]; the matrix applied to the cell vector)."""
    nc, nq = v_jxw.shape
    ne = stiffness.shape[0]
    k = np.ascontiguousarray(np.asarray(kpoints, dtype=np.float64).reshape(-1, 3))
    out = torch.empty((k.shape[0], nc, ne, ne), dtype=torch.complex128, device=v_jxw.device)
    if gga_jxw is None:
        check(_lib.load().chefsi_assemble_cell_hamiltonians_bloch(
            nc, ne, nq, _ptr(shape), _ptr(shape_grad), _ptr(stiffness), _ptr(v_jxw), _ptr(jxw),
            k.shape[0], _np_ptr(k), _ptr(out), _stream()))
        return out
    if tuple(gga_jxw.shape) != (nc, nq, 3):
        raise ValueError("gga_jxw must be [n_cells, n_q, 3]")
    g = gga_jxw.contiguous()
    check(_lib.load().chefsi_assemble_cell_hamiltonians_bloch_gga(
        nc, ne, nq, _ptr(shape), _ptr(shape_grad), _ptr(stiffness), _ptr(v_jxw), _ptr(g),
        _ptr(jxw), k.shape[0], _np_ptr(k), _ptr(out), _stream()))
    return out


def computeEigenResidualNorm(op: KohnShamOperator, X: torch.Tensor, eig) -> np.ndarray:
    N = X.shape[1]
    e = np.ascontiguousarray(eig, np.float64)
    r = np.zeros(N)
    check(_lib.load().chefsi_residual_norms(op.handle, _ptr(X), X.stride(0), N, _np_ptr(e),
                                            _np_ptr(r), _stream()))
    return r


def syevd(A: torch.Tensor):
    """Symmetric (real) or Hermitian (complex) eigensolve on the GPU in FP64: returns
    (w ascending, Z with the eigenvectors in its columns)."""
    N = A.shape[0]
    Ac = A.clone().contiguous()
    w = torch.empty(N, dtype=torch.float64, device=A.device)
    Z = torch.empty((N, N), dtype=A.dtype, device=A.device)
    fn = _lib.load().chefsi_heevd if A.is_complex() else _lib.load().chefsi_syevd
    check(fn(N, _ptr(Ac), _ptr(w), _ptr(Z), _stream()))
    return w, Z


def chebyshev_order(upper_bound: float) -> int:
    return int(_lib.load().chefsi_chebyshev_order(float(upper_bound)))


@dataclass
class SolverParams:
    """The dftParameters fields the CheFSI path reads (utils/dftParameters.cc:1224-1287)."""
    chebyshevOrder: int = 0
    chebyWfcBlockSize: int = 400
    wfcBlockSize: int = 400
    mixed_precision: str = "mixed"     # precision used when solve(useMixedPrec=True)
    lanczos_steps: int = 20
    reproducible_output: bool = False
    chebyshevFilterPolyDegreeFirstScfScalingFactor: float = 1.34
    keep_hx: bool = True
    rr_precision: str = "fp64"         # HX precision feeding X^T H X in mixed mode
    # spectrum split in mixed mode: the block of X^T H X coupling the fractional states from
    # an FP64 H X (False, useMixedPrecXTHXSpectrumSplit's map) or from the rr_precision H X
    spectrum_split_frac_reduced: bool = False
    # memory-bounded Rayleigh-Ritz: column block (0 automatic, > 0 forced, < 0 never) and
    # dofs per row slab (0 automatic)
    rr_block: int = 0
    rr_slab_rows: int = 0
    # mixed tensor-core filter: "folded" (one HX launch per degree with the Chebyshev shift on
    # the tiles' diagonals and the nonlocal apply as extra tensor-core K columns, no recurrence
    # pass), "axpby" (recurrence pass + that HX launch without the shift), "fused" (the
    # recurrence finished inside the HX launch) or "separate" (recurrence pass, HX launch,
    # separate nonlocal kernels)
    filter_variant: str = "folded"


class ChebyshevOrthogonalizedSubspaceIterationSolver:
    """chebyshevOrthogonalizedSubspaceIterationSolverDevice on the GB300 C ABI."""

    def __init__(self, params: SolverParams | None = None):
        self.params = params or SolverParams()
        self._h = {}
        self._lib = _lib.load()

    def _handle(self, mixed: bool):
        key = bool(mixed)
        if key not in self._h:
            p = _lib.Params()
            p.chebyshev_degree = self.params.chebyshevOrder
            p.cheby_wfc_block = self.params.chebyWfcBlockSize
            p.wfc_block = self.params.wfcBlockSize
            p.precision = _prec(self.params.mixed_precision) if mixed else _lib.PREC_FP64
            p.lanczos_steps = self.params.lanczos_steps
            p.reproducible = int(self.params.reproducible_output)
            p.first_scf_degree_scale = self.params.chebyshevFilterPolyDegreeFirstScfScalingFactor
            p.keep_hx = int(self.params.keep_hx)
            p.rr_precision = _prec(self.params.rr_precision)
            p.ss_frac_reduced = int(self.params.spectrum_split_frac_reduced)
            p.rr_block = int(self.params.rr_block)
            p.rr_slab_rows = int(self.params.rr_slab_rows)
            p.filter_variant = {"folded": 0, "fused": 1, "separate": -1, "axpby": 2}[self.params.filter_variant]
            h = ctypes.c_void_p()
            check(self._lib.chefsi_solver_create(ctypes.byref(p), ctypes.byref(h)))
            self._h[key] = h
            if hasattr(self, "_bounds"):
                check(self._lib.chefsi_solver_reinit_spectrum_bounds(h, *self._bounds))
        return self._h[key]

    def __del__(self):
        for h in getattr(self, "_h", {}).values():
            if _lib._lib is not None:
                _lib._lib.chefsi_solver_destroy(h)

    def reinitSpectrumBounds(self, lowerBoundWantedSpectrum: float,
                             lowerBoundUnWantedSpectrum: float,
                             upperBoundUnWantedSpectrum: float):
        self._bounds = (float(lowerBoundWantedSpectrum), float(lowerBoundUnWantedSpectrum),
                        float(upperBoundUnWantedSpectrum))
        for h in self._h.values():
            check(self._lib.chefsi_solver_reinit_spectrum_bounds(h, *self._bounds))

    def solve(self, operatorMatrix: KohnShamOperator, X: torch.Tensor, eigenValues=None,
              residualNorms=None, computeResidual: bool = True, useMixedPrec: bool = False,
              isFirstScf: bool = False, eigenVectorsRotFracDensity: torch.Tensor | None = None):
        """One CheFSI iteration on X [n_dofs, N] in place; returns (eigenValues, residualNorms).

        As the reference's solve, an eigenValues array shorter than N asks for the
        spectrum-split Rayleigh-Ritz step: its N - len(eigenValues) lowest states are the core
        states, eigenVectorsRotFracDensity [n_dofs, len(eigenValues)] receives the fractional
        Ritz vectors, and eigenValues / residualNorms are filled for those."""
        N = X.shape[1]
        if eigenValues is not None and len(eigenValues) < N:
            nfr = len(eigenValues)
            if eigenVectorsRotFracDensity is None:
                raise ValueError("a spectrum-split solve needs eigenVectorsRotFracDensity")
            ev, rn, _ = self.solveSpectrumSplit(operatorMatrix, X, N - nfr,
                                                eigenVectorsRotFracDensity, computeResidual,
                                                useMixedPrec, isFirstScf)
            eigenValues[:] = ev
            if residualNorms is None:
                return eigenValues, rn
            residualNorms[:nfr] = rn
            return eigenValues, residualNorms
        ev = np.zeros(N) if eigenValues is None else eigenValues
        rn = np.zeros(N) if residualNorms is None else residualNorms
        h = self._handle(useMixedPrec)
        check(self._lib.chefsi_solve(h, operatorMatrix.handle, _ptr(X), N, _np_ptr(ev),
                                     _np_ptr(rn), int(computeResidual), int(isFirstScf), _stream()))
        return ev, rn

    def solveSpectrumSplit(self, operatorMatrix: KohnShamOperator, X: torch.Tensor, Noc: int,
                           XFrac: torch.Tensor | None = None, computeResidual: bool = True,
                           useMixedPrec: bool = False, isFirstScf: bool = False):
        """solve() with N - Noc wanted eigenvalues: filter, spectrum-split Rayleigh-Ritz.
        X is left orthonormalised; returns (eigenValues, residualNorms, XFrac)."""
        N = X.shape[1]
        nfr = N - Noc
        if XFrac is None:
            XFrac = torch.empty((X.shape[0], nfr), dtype=X.dtype, device=X.device)
        ev, rn = np.zeros(nfr), np.zeros(nfr)
        h = self._handle(useMixedPrec)
        check(self._lib.chefsi_solve_spectrum_split(
            h, operatorMatrix.handle, _ptr(X), N, int(Noc), _ptr(XFrac), _np_ptr(ev), _np_ptr(rn),
            int(computeResidual), int(isFirstScf), _stream()))
        return ev, rn, XFrac

    def densityMatrixEigenBasisFirstOrderResponse(self, operatorMatrix: KohnShamOperator,
                                                  eigenVectors: torch.Tensor, eigenValues,
                                                  fermiEnergy: float, TVal: float,
                                                  useMixedPrec: bool = False) -> np.ndarray:
        """The solver member of the reference
        (chebyshevOrthogonalizedSubspaceIterationSolverDevice.cc:1083-1189): eigenVectors in the
        FE basis are scaled by M^{1/2} into the Loewdin basis, the response is applied there
        (operatorMatrix is the first-order operator H'), and the result is scaled back by
        M^{-1/2}. Returns densityMatDerFermiEnergy."""
        sq = operatorMatrix.getSqrtMassVec().reshape(-1, 1)
        eigenVectors.mul_(sq)
        try:
            dmu = densityMatrixEigenBasisFirstOrderResponse(
                operatorMatrix, eigenVectors, eigenValues, fermiEnergy, TVal,
                precision=self.params.mixed_precision if useMixedPrec else "fp64")
        finally:
            eigenVectors.mul_(operatorMatrix.getInvSqrtMassVec().reshape(-1, 1))
        return dmu

    def solveNoRR(self, operatorMatrix: KohnShamOperator, X: torch.Tensor, numberPasses: int = 1,
                  useMixedPrec: bool = False, isFirstScf: bool = False):
        h = self._handle(useMixedPrec)
        check(self._lib.chefsi_solve_no_rr(h, operatorMatrix.handle, _ptr(X), X.shape[1],
                                           numberPasses, int(isFirstScf), _stream()))
        return X

    def timings(self, mixed: bool = False) -> dict:
        t = (ctypes.c_double * 7)()
        check(self._lib.chefsi_solver_timings(self._handle(mixed), t))
        keys = ["filter", "overlap_cholesky", "xthx", "eig", "rotation", "residual", "total"]
        return dict(zip(keys, list(t)))

    def set_profiling(self, enable: bool = True, mixed: bool = True):
        check(self._lib.chefsi_solver_set_profiling(self._handle(mixed), int(enable)))

    def hx_stats(self, mixed: bool = True):
        n, t = ctypes.c_int32(), ctypes.c_double()
        check(self._lib.chefsi_solver_hx_stats(self._handle(mixed), ctypes.byref(n), ctypes.byref(t)))
        return n.value, t.value

    def last_degree(self, mixed: bool = False) -> int:
        d = ctypes.c_int32()
        check(self._lib.chefsi_solver_get_bounds(self._handle(mixed), None, None, None,
                                                 ctypes.byref(d)))
        return d.value


def initial_bounds(op: KohnShamOperator, n_wfc: int, k: int = 20, reproducible: bool = False,
                   v0=None, seed: int = 0):
    """First-call bounds of kohnShamEigenSpaceCompute (src/dft/kohnShamEigenSolve.cc:335-365)."""
    lo, up = lanczosLowerUpperBoundEigenSpectrum(op, k, reproducible, v0, seed)
    blow = lo + (up - lo) / op.n_dofs * n_wfc * (10.0 if reproducible else 200.0)
    return lo, blow, up


def solve_batched(solvers, operators, Xs, useMixedPrec: bool = False,
                  computeResidual: bool = True, isFirstScf: bool = False, n_streams: int = 0,
                  group: bool = True):
    """One CheFSI iteration on each independent problem (k-points, spins, Bloch Hamiltonians)
    through chefsi_solve_batched; returns (list of eigenvalues, list of residual norms).
    group: filter the eligible problems together (grouped launches in a CUDA graph)."""
    count = len(Xs)
    if not (len(solvers) == len(operators) == count):
        raise ValueError("solvers, operators and Xs must have the same length")
    lib = _lib.load()
    vp = ctypes.c_void_p
    hs = (vp * count)(*[s._handle(useMixedPrec).value for s in solvers])
    ops = (vp * count)(*[o.handle.value for o in operators])
    xs = (vp * count)(*[X.data_ptr() for X in Xs])
    ns = (ctypes.c_int32 * count)(*[X.shape[1] for X in Xs])
    evs = [np.zeros(X.shape[1]) for X in Xs]
    rns = [np.zeros(X.shape[1]) for X in Xs]
    ev_p = (vp * count)(*[e.ctypes.data for e in evs])
    rn_p = (vp * count)(*[r.ctypes.data for r in rns])
    torch.cuda.synchronize()  # the worker streams do not order after the caller's stream
    check(lib.chefsi_solve_batched(count, hs, ops, xs, ns, ev_p, rn_p, int(computeResidual),
                                   int(isFirstScf), int(n_streams), int(group)))
    return evs, rns
