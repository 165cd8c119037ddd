/*
 * chefsi.h -- C ABI of the GB300-native Chebyshev-filtered subspace iteration (CheFSI).
 *
 * A drop-in for DFT-FE's CheFSI hot path on one GPU. The entry points replace these
 * reference interfaces (paths inside the DFT-FE source tree):
 *
 *   chefsi_operator_create / _destroy
 *       kohnShamDFTOperatorDeviceClass::init + reinit + computeHamiltonianMatricesAllkpt
 *       (src/dftOperator/kohnShamDFTOperatorDevice.cc:494-933,
 *        src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:1075-1375);
 *       the cell Hamiltonians, cell->dof map, mass vector, constraints and nonlocal
 *       projectors are passed in instead of being built from deal.II objects.
 *   chefsi_hx        operatorDFTDeviceClass::HX / HXCheby (include/operatorDevice.h:176-197;
 *                    src/dftOperator/kohnShamDFTOperatorDevice.cc:3767-3860, :3876-3997)
 *   chefsi_xthx      operatorDFTDeviceClass::XtHX (include/operatorDevice.h:230-241;
 *                    src/dftOperator/kohnShamDFTOperatorDevice.cc:4003-4157)
 *   chefsi_overlap   linearAlgebraOperationsDevice::fillParallelOverlapMatScalapack[MixedPrec]
 *                    (src/linAlg/linearAlgebraOperationsDevice.cc:3079-3240, :3544-3798)
 *   chefsi_chebyshev_filter
 *                    linearAlgebraOperationsDevice::chebyshevFilter
 *                    (src/linAlg/linearAlgebraOperationsDevice.cc:531-727)
 *   chefsi_lanczos_bounds
 *                    linearAlgebraOperationsDevice::lanczosLowerUpperBoundEigenSpectrum
 *                    (src/linAlg/linearAlgebraOperationsDevice.cc:341-527)
 *   chefsi_cholesky_gs
 *                    pseudoGramSchmidtOrthogonalization (src/linAlg/pseudoGSDevice.cc:82-463)
 *   chefsi_rayleigh_ritz
 *                    rayleighRitzGEP (src/linAlg/rayleighRitzDevice.cc:356-819)
 *   chefsi_density_matrix_first_order_response
 *                    densityMatrixEigenBasisFirstOrderResponse
 *                    (include/linearAlgebraOperationsDevice.h:302-322,
 *                    src/linAlg/rayleighRitzDevice.cc:1455-1721)
 *   chefsi_rayleigh_ritz_spectrum_split / chefsi_solve_spectrum_split
 *                    rayleighRitzGEPSpectrumSplitDirect
 *                    (include/linearAlgebraOperationsDevice.h:279-298,
 *                    src/linAlg/rayleighRitzDevice.cc:822-1455) and the solve() branch that
 *                    calls it (chebyshevOrthogonalizedSubspaceIterationSolverDevice.cc:584-690)
 *   chefsi_residual_norms
 *                    computeEigenResidualNorm (src/linAlg/linearAlgebraOperationsDevice.cc:4611-)
 *   chefsi_solver_create / _reinit_spectrum_bounds / chefsi_solve / chefsi_solve_no_rr
 *                    chebyshevOrthogonalizedSubspaceIterationSolverDevice constructor,
 *                    reinitSpectrumBounds, solve, solveNoRR
 *                    (include/chebyshevOrthogonalizedSubspaceIterationSolverDevice.h:37-166)
 *   chefsi_syevd     the projected eigensolve done by ELPA/ScaLAPACK in the reference
 *                    (src/linAlg/rayleighRitzDevice.cc:720-749), here FP64 on the GPU
 *
 * Conventions
 *   - Block vectors are dof-major, wavefunction-fastest: X[i * ld + j] for dof i, vector j
 *     (DFT-FE's flattened layout, include/MultiVector.h:126). All vector and matrix
 *     pointers passed to compute calls are DEVICE pointers unless the name says host.
 *   - Small N x N matrices (overlap, projected Hamiltonian, rotations) are row-major on the
 *     device.
 *   - The operator is A = M^{-1/2} (H_loc + H_nl) M^{-1/2} in Hartree; CheFSI works on
 *     vectors already scaled by M^{1/2} (src/dft/kohnShamEigenSolve.cc:322-329).
 *   - Every call returns an int status (CHEFSI_OK == 0); no C++ exception crosses the ABI.
 *     chefsi_last_error() returns the message of the last failure on the calling thread.
 *   - Compute calls take a cudaStream_t (passed as void*) and enqueue work on it. Calls that
 *     return host results (eigenvalues, residuals, bounds) synchronise that stream.
 *   - Stream capture: the FP64 and FP32 SIMT chefsi_hx only enqueue work once their
 *     workspaces exist (capture them after a first call). The tensor-core paths read their
 *     bounded-wait status back and the mixed filter reads its block's largest entry back (to
 *     scale the block by a power of two), so those calls synchronise their stream and cannot
 *     be captured; chefsi_solve_batched captures its own grouped filter.
 *   - Handles are not thread-safe: one host thread per handle.
 *   - Precision: CHEFSI_PREC_FP64 computes everything in FP64. CHEFSI_PREC_MIXED runs the
 *     filter HX on the tensor cores with FP16-split operands (hi+lo, three products,
 *     FP32 accumulation) on FP32 block vectors, and the overlap / projected-Hamiltonian Gram
 *     products and the rotations on the tensor cores with the same split of column-scaled
 *     operands (FP32 accumulation over 128-dof chunks, compensated sums across chunks); the
 *     HX feeding the projected Hamiltonian follows rr_precision; the Cholesky, the projected
 *     eigensolve and the residual norms stay in FP64. CHEFSI_PREC_FP32 is the SIMT FP32
 *     apply (no tensor cores), kept for comparison. CHEFSI_PREC_FP32_TC (chefsi_hx and
 *     rr_precision) is the FP32-accurate tensor-core apply: three-term FP16 split (FP32
 *     operands exactly, cell matrices to 2^-33), six products, FP32 accumulation.
 */
#ifndef CHEFSI_GB300_H
#define CHEFSI_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CHEFSI_OK 0
#define CHEFSI_ERR_INVALID 1     /* bad argument (null pointer, size out of range) */
#define CHEFSI_ERR_CUDA 2        /* a CUDA runtime call failed */
#define CHEFSI_ERR_NOT_SPD 3     /* Cholesky met a non-positive pivot */
#define CHEFSI_ERR_NO_CONVERGENCE 4
#define CHEFSI_ERR_ALLOC 5       /* device allocation failed */
#define CHEFSI_ERR_TIMEOUT 6     /* a bounded device wait ran out */
#define CHEFSI_ERR_NAN 7         /* non-finite input detected */
#define CHEFSI_ERR_UNSUPPORTED 8 /* valid request this build does not implement */

/* precision modes */
#define CHEFSI_PREC_FP64 0
#define CHEFSI_PREC_MIXED 1
#define CHEFSI_PREC_FP32 2
#define CHEFSI_PREC_FP32_TC 3

typedef struct chefsi_operator_s* chefsi_operator;
typedef struct chefsi_solver_s* chefsi_solver;

/* Description of one Kohn-Sham operator (one k-point / spin). Host pointers. */
typedef struct {
  int64_t n_dofs;               /* M: locally owned dofs (length of a vector) */
  int32_t n_cells;              /* number of cells */
  int32_t nodes_per_cell;       /* n_e = (p+1)^3 */
  int32_t is_complex;           /* 0: real (Gamma point), 1: complex Bloch */
  const int32_t* cell_dof_map;  /* [n_cells][n_e] dof of each cell node */
  const void* cell_matrices;    /* [n_cells][n_e][n_e] FP64 (or interleaved complex FP64),
                                   row I column J, the matrix applied to the cell vector */
  const double* sqrt_mass;      /* [n_dofs] M^{1/2} (lumped) */
  const double* inv_sqrt_mass;  /* [n_dofs] M^{-1/2} */
  /* constraints: slave rows in CSR form over master dofs (0 rows = none). When present the
     operator runs DFT-FE's sequence (scale, distribute, cell products, adjoint distribute,
     scale); otherwise the mass scaling is folded into the cell matrices. The inhomogeneities
     g_s of the reference's distribute (utils/constraintMatrixInfoDevice.cc:62-63) are taken
     as zero: x_s = sum_m w_sm x_m, which is the reference's case for wavefunctions (their
     constraints are homogeneous; only the electrostatics carries nonzero g_s). */
  int32_t n_constrained;
  const int32_t* constrained_ids; /* [n_constrained] */
  const int32_t* constraint_ptr;  /* [n_constrained+1] */
  const int32_t* master_ids;      /* [nnz] */
  const double* master_weights;   /* [nnz] */
  /* nonlocal projectors: H_nl = sum_a C_a diag(V_a) C_a^T, C_a dense over its dof list */
  int32_t n_atoms;
  int32_t n_proj;               /* projectors per atom (uniform) */
  const int32_t* atom_dof_ptr;  /* [n_atoms+1] */
  const int32_t* atom_dofs;     /* [nnz_dofs] */
  const double* atom_proj;      /* [nnz_dofs][n_proj] */
  const double* couplings;      /* [n_atoms][n_proj] */
} chefsi_operator_desc;

/* Solver parameters (subset of dftParameters that the path reads). */
typedef struct {
  int32_t chebyshev_degree;     /* 0: from the upper bound via DFT-FE's lookup table */
  int32_t cheby_wfc_block;      /* chebyWfcBlockSize */
  int32_t wfc_block;            /* wfcBlockSize (residual / XtHX blocks) */
  int32_t precision;            /* CHEFSI_PREC_* */
  int32_t lanczos_steps;        /* 20 (40 with reproducible output) */
  int32_t reproducible;         /* REPRODUCIBLE OUTPUT */
  double first_scf_degree_scale;/* chebyshevFilterPolyDegreeFirstScfScalingFactor */
  int32_t keep_hx;              /* 1: keep H X from the RR step for the residuals */
  int32_t rr_precision;         /* precision of the H X feeding X^T H X in mixed mode:
                                   CHEFSI_PREC_FP64 (default), CHEFSI_PREC_FP32 (FP32 SIMT
                                   apply), CHEFSI_PREC_FP32_TC (tensor-core apply with the
                                   three-term FP16 split: FP32 operands exactly, FP32
                                   accumulation) or CHEFSI_PREC_MIXED (the filter's two-term
                                   split) */
  int32_t ss_frac_reduced;      /* spectrum-split Rayleigh-Ritz in mixed mode: 0 (default)
                                   recomputes the block of X^T H X that couples the
                                   fractionally occupied states from an FP64 H X (the
                                   precision map of useMixedPrecXTHXSpectrumSplit); 1 keeps
                                   the rr_precision H X there too */
  int32_t rr_block;             /* real Rayleigh-Ritz step in column blocks (X^T H X one block
                                   of H X at a time, Gram and rotation by row slabs, no
                                   full-size H X): 0 (default) when the full-size workspaces
                                   would not fit the free device memory, > 0 always with
                                   blocks of that many vectors, < 0 never */
  int32_t rr_slab_rows;         /* dofs per row slab of the blocked step (0: about 2^30 / N) */
  int32_t filter_variant;       /* mixed tensor-core filter: 0 (default) one HX launch per
                                   degree with the Chebyshev shift on the tiles' diagonals and
                                   the nonlocal apply as extra tensor-core K columns, reducing
                                   into the older vector's buffer (kept up to a scalar factor:
                                   no recurrence pass; the launch splits its FP32 input); 2 a
                                   recurrence pass per degree and that HX launch without the
                                   shift; 1 the fused step (the recurrence finished in the HX
                                   launch, vectors kept as FP16 hi + lo rows); -1 the recurrence
                                   pass, the HX launch and separate nonlocal kernels */
} chefsi_params;

/* Bounds of the device-side waits (no counterpart in the reference: a test hook for failure
   detection). mbarrier_tries: tries of every mbarrier wait in the tensor-core kernels (each a
   hardware suspend of up to 20 us; default CHEFSI_DEFAULT_WAIT_TRIES, about 1.3 s);
   barrier_spins: polls of a grid-barrier wait in the cooperative tridiagonalisation (default
   CHEFSI_DEFAULT_BARRIER_SPINS). A wait that runs out records CHEFSI_ERR_TIMEOUT, the kernel
   returns after its own copies and tensor-core operations have finished, and the call that
   launched it returns CHEFSI_ERR_TIMEOUT with the context still usable; 0 makes every such
   wait expire at once. Applies to kernels launched after the call, on the current device. */
#define CHEFSI_DEFAULT_WAIT_TRIES 65536u
#define CHEFSI_DEFAULT_BARRIER_SPINS 67108864u
int chefsi_set_wait_limits(uint32_t mbarrier_tries, uint32_t barrier_spins);

const char* chefsi_last_error(void);
const char* chefsi_version(void);
/* number of kernels this library has launched in the process (all streams) */
uint64_t chefsi_launch_count(void);

int chefsi_operator_create(const chefsi_operator_desc* desc, chefsi_operator* out);
int chefsi_operator_destroy(chefsi_operator op);
int chefsi_operator_info(chefsi_operator op, int64_t* n_dofs, int32_t* n_cells,
                         int32_t* nodes_per_cell, int32_t* is_complex);

/* dst = (accumulate ? dst : 0) + scalar * A src over n_vec vectors (DFT-FE's HX with
   scaleFlag == accumulate). Real: src/dst FP64 (precision FP64) or FP32 (FP32 / FP32_TC /
   MIXED).
   Complex: interleaved complex FP64 only. ld_* are leading dimensions in elements. */
int chefsi_hx(chefsi_operator op, const void* src, int64_t ld_src, void* dst, int64_t ld_dst,
              int32_t n_vec, double scalar, int32_t accumulate, int32_t precision, void* stream);

/* S = X^H X (lower triangle mirrored, N x N row-major FP64, device). */
int chefsi_overlap(chefsi_operator op, const void* X, int64_t ld, int32_t N, double* S,
                   int32_t precision, void* stream);

/* Hp = X^H A X (N x N row-major FP64, device). The HX is FP64 in every mode. */
int chefsi_xthx(chefsi_operator op, const void* X, int64_t ld, int32_t N, double* Hp,
                int32_t precision, void* stream);

/* In-place Chebyshev filter of the n_vec columns starting at X (ld): degree m on the
   unwanted interval [a, b] with lower wanted bound a0 (sigma-scaled recurrence). */
int chefsi_chebyshev_filter(chefsi_operator op, void* X, int64_t ld, int32_t n_vec,
                            int32_t m, double a, double b, double a0, int32_t precision,
                            void* stream);

/* k-step Lanczos from the host start vector v0 (length n_dofs; null: seeded uniform(0,1)).
   Returns floor(lambda_min(T)) and ceil(lambda_max(T) + |f| (reproducible) or |f|/10). */
int chefsi_lanczos_bounds(chefsi_operator op, int32_t k, int32_t reproducible,
                          const double* v0_host, uint64_t seed, double* lower, double* upper,
                          void* stream);

/* Symmetric (Hermitian for complex) eigensolve of an N x N row-major device matrix:
   eigenvalues ascending into w (device, N), eigenvectors into the columns of Z (device).
   A is overwritten. */
int chefsi_syevd(int32_t N, double* A, double* w, double* Z, void* stream);

/* Hermitian eigensolve of an N x N row-major interleaved-complex device matrix A (ELPA /
   zheevd in rayleighRitzGEP, src/linAlg/rayleighRitzDevice.cc:720-749): eigenvalues
   ascending into w (device, N doubles), eigenvectors into the columns of Z (device, N x N
   interleaved complex). A is overwritten. */
int chefsi_heevd(int32_t N, double* A, double* w, double* Z, void* stream);

/* Allocation-free variant of chefsi_syevd (no counterpart in the reference).
   For callers that cannot allocate device memory during a solve -- an application whose
   pool allocator owns the GPU's memory, or one that cannot take the device-wide
   synchronisation of cudaFree. The workspace is a file-scope device array sized for
   N <= 256 (about 3.3 MB per device); larger N returns CHEFSI_ERR_INVALID. The CUDA runtime
   loads the library's device code lazily, so the array is placed in device memory when the
   first call on a device looks up its address (cudaGetSymbolAddress): make one warm-up call
   (any N <= 256) on each device before the caller's pool reserves the device memory, and
   before any stream capture. From then on the array stays allocated on that device until the
   process exits, and later calls allocate nothing. Every call synchronises its stream (it
   reads the cluster tolerance back to the host). All calls share the array, so calls that
   overlap on the GPU race; serialise them. Same arguments and results as chefsi_syevd. */
int chefsi_syevd_noalloc(int32_t N, double* A, double* w, double* Z, void* stream);

/* Cholesky-Gram-Schmidt: S = X^H X, S = L L^H, X <- X L^{-H}. */
int chefsi_cholesky_gs(chefsi_operator op, void* X, int64_t ld, int32_t N, int32_t precision,
                       void* stream);

/* Rayleigh-Ritz in the generalised form; eigenvalues to host eig_host (N), X rotated in
   place to the Ritz vectors. If HX_out is non-null it receives A X_rot (FP64, [M][N]); if
   W_out is non-null it receives the N x N coefficient matrix W = L^{-T} Q (X_rot = X W).
   precision MIXED takes the Gram and rotation products to the tensor cores and keeps the H X
   that feeds X^T H X in FP64 (the solver's rr_precision default); a solver created with
   rr_precision = CHEFSI_PREC_FP32_TC uses the three-term tensor-core H X instead. */
int chefsi_rayleigh_ritz(chefsi_operator op, void* X, int64_t ld, int32_t N, double* eig_host,
                         double* HX_out, double* W_out, int32_t precision, void* stream);

/* Spectrum-split Rayleigh-Ritz. X ([n_dofs][N], ld) is orthonormalised in place by
   Cholesky-GS (X <- X L^{-H}, X^H X = L L^H) and stays in that basis; the projected
   Hamiltonian X^H H X of the orthonormal X is diagonalised for its top n_fr = N - n_occ
   eigenpairs only, and XFrac ([n_dofs][n_fr], ld_frac) = X Q_fr. eig_host receives the n_fr
   eigenvalues in ascending order; HXFrac_out, if non-null, H XFrac ([n_dofs][n_fr] FP64).
   precision MIXED: the reduced-precision H X (three-term tensor-core split) for the occupied
   column blocks and, unless frac_reduced, an FP64 H X and Gram product for the block that
   couples the fractional states; real operators also take the Gram and rotation products
   to the tensor cores (complex operators keep them in FP64). */
int chefsi_rayleigh_ritz_spectrum_split(chefsi_operator op, void* X, int64_t ld, int32_t N,
                                        int32_t n_occ, void* XFrac, int64_t ld_frac,
                                        double* eig_host, void* HXFrac_out, int32_t precision,
                                        int32_t frac_reduced, void* stream);

/* First-order response of the density matrix in the eigenbasis. op_prime
   applies the perturbation H' only (DFT-FE's onlyHPrimePart apply: build it from the cell
   matrices of the first-order potential). X ([n_dofs][N], ld) holds the N orthonormal
   eigenvectors (Loewdin basis, as the solve works on) with eigenvalues eig_host[N]:
   Hp' = X^H H' X; P' from 10 steps of the first-order recursive Fermi-operator expansion at
   beta = 1 / (k_B temperature) (Kelvin; k_B = 3.166811429e-6 Ha/K) around fermi_energy;
   X <- X P' in place; dmu_host[N] receives densityMatDerFermiEnergy = beta X0 (1 - X0).
   precision MIXED: tensor-core H X, Gram and rotation for real operators (the reference's
   singlePrecLRD), the reduced H X of the real form with FP64 complex products for complex
   ones. */
int chefsi_density_matrix_first_order_response(chefsi_operator op_prime, void* X, int64_t ld,
                                               int32_t N, const double* eig_host,
                                               double fermi_energy, double temperature,
                                               double* dmu_host, int32_t precision,
                                               void* stream);

/* y = a x + b y on [rows][n_vec] FP64 device blocks (leading dimensions ldx, ldy). */
int chefsi_axpby(int64_t rows, int32_t n_vec, double a, const double* x, int64_t ldx, double b,
                 double* y, int64_t ldy, void* stream);

/* dst = scale * src with precision conversion on [rows][n_vec] device blocks (leading
   dimensions ld_src, ld_dst); src_bits / dst_bits = 32 (FP32) or 64 (FP64). A power-of-two
   scale is applied exactly and the result rounded once to the destination type; any other
   scale multiplies in the destination's precision.
   Replaces dftfe::utils::deviceKernelsGeneric::copyValueType1ArrToValueType2Arr
   (include/deviceKernelsGeneric.h:53) and the scaled block copies of the mixed-precision
   filter. */
int chefsi_convert_block(int32_t src_bits, const void* src, int64_t ld_src, int32_t dst_bits,
                         void* dst, int64_t ld_dst, int64_t rows, int32_t n_vec, double scale,
                         void* stream);

/* C = alpha op(A) op(B) + beta C, row-major device matrices, op = 'N' or 'T'. FP64, or FP32
   products with FP64 accumulation across K chunks (CHEFSI_PREC_MIXED / FP32). */
int chefsi_gemm(char ta, char tb, int64_t M, int32_t N, int32_t K, double alpha, const double* A,
                int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                int32_t precision, void* stream);

/* Cell Hamiltonians on the device (the real-case formula of hamMatrixKernelLDA,
   src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:61-115):
   out[c][I][J] = 0.5 stiffness[I][J] + sum_q shape[q][I] v_jxw[c][q] shape[q][J].
   shape [n_q][n_e], stiffness [n_e][n_e], v_jxw [n_cells][n_q], out [n_cells][n_e][n_e]. */
int chefsi_assemble_cell_hamiltonians(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                      const double* shape, const double* stiffness,
                                      const double* v_jxw, double* out, void* stream);

/* Cell Hamiltonians of cells of any shape (the per-cell stiffness of
   FEBasisOperations::computeCellStiffnessMatrix, utils/FEBasisOperations.cc:1133-1300, with the
   potential term of hamMatrixKernelLDA):
   out[c][I][J] = sum_q ( 0.5 sum_ij shape_grad_ref[i][q][I] jacobian_factor[c][q][i][j]
                          shape_grad_ref[j][q][J] + v_jxw[c][q] shape[q][I] shape[q][J] )
   shape [n_q][n_e], shape_grad_ref [3][n_q][n_e] the gradients on the reference cell,
   jacobian_factor [n_cells][n_q][3][3] = sum_k invJ[i][k] invJ[j][k] JxW (invJ[i][k] =
   d xi_i / d x_k, the reference's jacobianFactor), v_jxw [n_cells][n_q], out
   [n_cells][n_e][n_e]; device pointers. */
int chefsi_assemble_cell_hamiltonians_geometry(int32_t n_cells, int32_t nodes_per_cell,
                                               int32_t n_q, const double* shape,
                                               const double* shape_grad_ref,
                                               const double* jacobian_factor,
                                               const double* v_jxw, double* out, void* stream);

/* GGA cell Hamiltonians, real (hamMatrixKernelGGAMemOpt,
   src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:283-456):
   out[c][I][J] = 0.5 stiffness[I][J] + sum_q ( v_jxw[c][q] N_qI N_qJ
                  + 2 sum_d gga_jxw[c][q][d] (shape_grad[d][q][I] N_qJ + N_qI shape_grad[d][q][J]) )
   with gga_jxw = derExcWithSigmaTimesGradRhoJxW [n_cells][n_q][3] and shape_grad
   [3][n_q][n_e] the real-space shape-function gradients; device pointers. */
int chefsi_assemble_cell_hamiltonians_gga(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                          const double* shape, const double* shape_grad,
                                          const double* stiffness, const double* v_jxw,
                                          const double* gga_jxw, double* out, void* stream);

/* Bloch cell Hamiltonians for n_k k-points (the k-point form of hamMatrixKernelLDA,
   src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:119-280), stored as the matrix
   applied to the cell vector (interleaved complex, the layout chefsi_operator_create takes):
   Re out[k][c][I][J] = 0.5 stiffness[I][J] + sum_q (v_jxw[c][q] + |k|^2/2 jxw[c][q]) N_qI N_qJ
   Im out[k][c][I][J] = -sum_d k_d sum_q jxw[c][q] N_qI shape_grad[d][q][J].
   shape [n_q][n_e], shape_grad [3][n_q][n_e] (real-space gradients), stiffness [n_e][n_e],
   v_jxw and jxw [n_cells][n_q] on the device; kpoints_host [n_k][3] (Cartesian, 1/bohr) on
   the host; out [n_k][n_cells][n_e][n_e] complex on the device. */
int chefsi_assemble_cell_hamiltonians_bloch(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                            const double* shape, const double* shape_grad,
                                            const double* stiffness, const double* v_jxw,
                                            const double* jxw, int32_t n_k,
                                            const double* kpoints_host, void* out, void* stream);

/* The GGA form of chefsi_assemble_cell_hamiltonians_bloch (hamMatrixKernelGGAMemOpt, complex,
   src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:458-655): the real part also
   carries 2 sum_q sum_d gga_jxw[c][q][d] (shape_grad[d][q][I] N_qJ + N_qI shape_grad[d][q][J]),
   gga_jxw [n_cells][n_q][3] on the device. */
int chefsi_assemble_cell_hamiltonians_bloch_gga(int32_t n_cells, int32_t nodes_per_cell,
                                                int32_t n_q, const double* shape,
                                                const double* shape_grad, const double* stiffness,
                                                const double* v_jxw, const double* gga_jxw,
                                                const double* jxw, int32_t n_k,
                                                const double* kpoints_host, void* out,
                                                void* stream);

/* Replace the operator's cell matrices with new unscaled ones (device pointer), as
   computeHamiltonianMatricesAllkpt does each SCF step; derived copies are refreshed. */
int chefsi_operator_update_cell_matrices(chefsi_operator op, const double* cell_matrices,
                                         void* stream);

/* Adjoint building block: G[c][I][J] += alpha * sum_b (D U)[map I][b] (D V)[map J][b], D = M^{-1/2},
   U, V device [n_dofs][ld] FP64, G device [n_cells][n_e][n_e] (dL/dH_c for L = U^T A V terms). */
int chefsi_cell_outer_accumulate(chefsi_operator op, const double* U, const double* V, int64_t ld,
                                 int32_t n_vec, double alpha, double* G, void* stream);

/* out[c][q] = jxw[c][q] * sum_IJ shape[q][I] G[c][I][J] shape[q][J]  (jxw may be null):
   dL/dV at the quadrature points from dL/dH_c. */
int chefsi_cell_quadrature_contract(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                    const double* shape, const double* G, const double* jxw,
                                    double* out, void* stream);

/* Electron density of the Ritz vectors at the quadrature points:
   rho[c][q] (+)= jxw[c][q] * sum_i occupation[i] |psi_i(x_q)|^2, with psi_i = M^{-1/2} x_i
   interpolated by the cell's shape functions shape[q][I] ([n_q][nodes_per_cell], device) and
   occupation (device, N entries) carrying the occupation, spin and k-point weights; jxw may be
   null (weight 1); accumulate != 0 adds to rho (the sum over k-points and spins). Real
   operators. precision CHEFSI_PREC_FP64: the occupation-weighted cell outer products
   sum_i f_i psi_c,i psi_c,i^T and one contraction with the shape functions, FP64.
   CHEFSI_PREC_MIXED: tensor cores interpolate psi at the quadrature points (FP16 split of
   M^{-1/2} x and of the shape functions, FP32 accumulation) and add f_i psi^2 in FP32.
   Replaces the per-(k, spin) density accumulation of densityCalculator
   (src/dft/densityCalculator.cc:39; densityCalculatorDeviceKernels.cc:34-86). */
int chefsi_density(chefsi_operator op, const double* X, int64_t ld, int32_t N,
                   const double* occupation, int32_t n_q, const double* shape, const double* jxw,
                   double* rho, int32_t accumulate, int32_t precision, void* stream);

/* residual norms r_i = || A x_i - lambda_i x_i || (host arrays eig, res). */
int chefsi_residual_norms(chefsi_operator op, const void* X, int64_t ld, int32_t N,
                          const double* eig_host, double* res_host, void* stream);

int chefsi_solver_create(const chefsi_params* params, chefsi_solver* out);
int chefsi_solver_destroy(chefsi_solver s);
int chefsi_solver_reinit_spectrum_bounds(chefsi_solver s, double lower_wanted,
                                         double lower_unwanted, double upper_unwanted);
int chefsi_solver_get_bounds(chefsi_solver s, double* lower_wanted, double* lower_unwanted,
                             double* upper_unwanted, int32_t* last_degree);
/* Per-phase device times of the last solve in milliseconds:
   [filter, overlap+cholesky, xthx(hx+gemm), eig, rotation, residual, total]. */
int chefsi_solver_timings(chefsi_solver s, double* ms7);
/* Filter HX launches of the last solve: their count and summed device time (CUDA events
   recorded on the solve's stream around every filter HX when profiling is enabled). */
int chefsi_solver_set_profiling(chefsi_solver s, int32_t enable);
int chefsi_solver_hx_stats(chefsi_solver s, int32_t* launches, double* total_ms);

/* One CheFSI iteration on X (device, [n_dofs][N], ld = N; FP64 or complex FP64):
   filter all vectors, Rayleigh-Ritz (GEP), residual norms. Eigenvalues and residual norms
   are written to host arrays. The bounds are NOT updated (the caller owns a0 / bLow, as
   kohnShamEigenSpaceCompute does); see chefsi_solver_reinit_spectrum_bounds. */
int chefsi_solve(chefsi_solver s, chefsi_operator op, void* X, int32_t N, double* eig_host,
                 double* res_host, int32_t compute_residual, int32_t is_first_scf,
                 void* stream);

/* One CheFSI iteration whose Rayleigh-Ritz step is the spectrum-split one (the solve()
   branch taken when N - n_occ < N eigenvalues are wanted): filter all N vectors of X, then
   X <- orthonormalised X, XFrac ([n_dofs][N - n_occ], ld N - n_occ, device) = X Q_fr.
   eig_host / res_host receive the N - n_occ eigenvalues and the residual norms of the
   XFrac columns (H XFrac - lambda XFrac, with H XFrac = (H X) Q_fr). */
int chefsi_solve_spectrum_split(chefsi_solver s, chefsi_operator op, void* X, int32_t N,
                                int32_t n_occ, void* XFrac, double* eig_host, double* res_host,
                                int32_t compute_residual, int32_t is_first_scf, void* stream);

/* One CheFSI iteration on each of count independent problems (the k-point / spin loop of
   dftClass::kohnShamEigenSpaceCompute, src/dft/kohnShamEigenSolve.cc:507-655, which calls
   solve() once per (k, spin)): problem i is (solvers[i], ops[i], X[i], N[i]) with its
   eigenvalues (and residual norms) written to eig_host[i] (res_host[i]); res_host may be
   null. Every entry needs its own solver (bounds and workspaces) and its own operator (the
   entries run concurrently, and a mixed filter writes its shift into the operator's
   tensor-core tiles; as in DFT-FE, every (k, spin) has its own Hamiltonian). The same holds
   for operators used by several host threads or streams at once.
   With group_filter != 0, the entries whose mixed filter runs on the tensor cores in one
   block (chebyWfcBlockSize >= N) are filtered together: per Chebyshev degree one grouped
   recurrence launch and one persistent tensor-core HX launch cover all problems of a cell
   type, with their own coefficients, and the lockstep recurrence is captured and replayed as
   a CUDA graph; the HX pipeline shape is chosen by a built-in autotuner (timed once per cell
   type and work size). The Rayleigh-Ritz steps (and every other entry) then run
   concurrently on n_streams CUDA streams (n_streams <= 0: min(count, 8)), each driven by a
   host worker thread, largest problems first. Returns the first failing entry's status. */
int chefsi_solve_batched(int32_t count, chefsi_solver* solvers, chefsi_operator* ops, void** X,
                         const int32_t* N, double** eig_host, double** res_host,
                         int32_t compute_residual, int32_t is_first_scf, int32_t n_streams,
                         int32_t group_filter);

/* Filter only (no Rayleigh-Ritz), solveNoRR. */
int chefsi_solve_no_rr(chefsi_solver s, chefsi_operator op, void* X, int32_t N,
                       int32_t n_passes, int32_t is_first_scf, void* stream);

/* Chebyshev degree from DFT-FE's lookup table (solver .cc:24-56). */
int32_t chefsi_chebyshev_order(double upper_bound_unwanted);

#ifdef __cplusplus
}
#endif
#endif /* CHEFSI_GB300_H */
