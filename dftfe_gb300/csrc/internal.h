// Internal types shared by the CheFSI translation units (not part of the C ABI).
#pragma once

#include "common.cuh"

#include <functional>
#include <memory>
#include <string>
#include <vector>

namespace chefsi {

struct cplx {
  double x, y;
};
__device__ __forceinline__ cplx cadd(cplx a, cplx b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cplx csub(cplx a, cplx b) { return {a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cplx cmul(cplx a, cplx b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ cplx cconj(cplx a) { return {a.x, -a.y}; }
__device__ __forceinline__ cplx cscale(cplx a, double s) { return {a.x * s, a.y * s}; }

// Tensor-core copy of the cell matrices: FP16 hi/lo split of 2^s * A_e (s a power-of-two
// exponent putting max |A_e| in [2^14, 2^15)), rows and columns zero-padded to npad (a
// multiple of 32), stored [n_cells][npad][npad] so that one TMA box of [rows][32 halves] is
// one 64-byte-swizzled operand tile.
struct TensorCellMats {
  DeviceBuffer<__half> hi, lo;
  DeviceBuffer<__half> lo3;  // third term of the three-term split (built on first use)
  int npad = 0;
  int kpad = 0;
  float scale = 1.f;   // power of two applied before the split
  bool ready = false;
  bool lo3_ready = false;
};

// Tables of the fused filter step (tc.cu, fused.cu), built once per operator on first use:
// * rows: every cell entry (cell, node) is "single" when its dof has no other cell entry (its
//   row is finished by the one unit that reduces into it) or "shared" (arrival counters per
//   128-vector chunk decide which unit finishes it);
// * the nonlocal term as extra K columns of the cell matrices: each (atom, dof) pair of the
//   projectors is given to one cell entry of its dof (greedily, so that few cells take more
//   than one atom), a cell's atoms occupy n_proj K columns each after its n_e nodes, holding
//   2^-t C V for the entry's dof; the K side gathers those columns from rows n_dofs + a P + j
//   of the split buffer, where 2^t W = 2^t C^T x sits. Cells with fewer atoms get zero columns.
struct FusedPlan {
  bool ready = false;
  int nkb = 0;            // K-blocks of 32 (nodes and projector columns)
  int kstride = 0;        // = 32 nkb
  int max_slots = 0;      // most atoms any cell takes
  int64_t n_shared = 0;
  int64_t rows = 0;       // split-buffer rows: n_dofs + n_atoms n_proj
  float scale = 1.f;      // 2^s of the tiles
  float wscale = 1.f;     // 2^t of the W rows
  DeviceBuffer<int> mapk;         // [n_cells][kstride]
  DeviceBuffer<int> rowinfo;      // [n_cells][n_e] x {dof, shared index or -1}
  DeviceBuffer<unsigned char> ncontrib;  // [n_shared]
  DeviceBuffer<__half> hi, lo;    // extended cell-matrix tiles [n_cells][halves][nkb][n_half x 32]
  // the tiles' diagonal entries (operators with M^{-1/2} folded in): the shifted filter keeps
  // 2^s (A_II - c / n_I) there (n_I = cell entries of the row's dof, so the shift adds up to
  // c once per dof); shift = the c the tiles hold now
  double diag_max = 0.0;          // max |A_II| over the cells
  double shift = 0.0;
  // the tiles depend on the cell matrices, the tables above on the map and the projectors:
  // a cell-matrix update rebuilds the tiles only (on the device)
  bool tiles_ready = false;
  DeviceBuffer<int64_t> ext_idx;  // tile elements of the projector columns
  DeviceBuffer<double> ext_val;   // their values C V / 2^t (the tile scale applied on scatter)
  double ext_max = 0.0;           // max |ext_val|
  double dmax2 = 1.0;             // constraint rows: max(M^{-1/2})^2 (the tiles fold it in)
  // operators with constraint rows (M^{-1/2} folded in by the plan, not the operator):
  DeviceBuffer<float> nl_c32;     // M^{-1/2} C in FP32 for the projection
  DeviceBuffer<double> con_wp;    // constraint weights in the folded basis, w d_m / d_s
};

}  // namespace chefsi

struct chefsi_operator_s {
  int64_t n_dofs = 0;
  int n_cells = 0;
  int n_e = 0;
  int is_complex = 0;
  bool folded = true;  // M^{-1/2} folded into the cell matrices / projectors

  chefsi::DeviceBuffer<int> map;          // [n_cells][n_e]
  chefsi::DeviceBuffer<double> mats64;    // [n_cells][n_e][n_e] (x2 for complex)
  chefsi::DeviceBuffer<float> mats32;     // FP32 copy (real only)
  chefsi::TensorCellMats tc;              // FP16 split copy for the tensor-core filter HX
  chefsi::FusedPlan fz;                   // tables of the fused filter step
  chefsi::DeviceBuffer<double> sqrt_mass, inv_sqrt_mass;

  // constraints
  int n_con = 0;
  chefsi::DeviceBuffer<int> con_ids, con_ptr, con_master;
  chefsi::DeviceBuffer<double> con_w;

  // nonlocal projectors
  int n_atoms = 0, n_proj = 0;
  int64_t nl_nnz = 0;
  chefsi::DeviceBuffer<int> nl_ptr, nl_dofs;
  chefsi::DeviceBuffer<double> nl_vals64, couplings;
  chefsi::DeviceBuffer<float> nl_vals32;
  int nl_n_chunks = 0;
  chefsi::DeviceBuffer<int> nl_chunk_atom, nl_chunk_row0;


  chefsi::DeviceBuffer<int> tc_err;       // timeout flag of the tensor-core kernel
  chefsi::DeviceBuffer<__half> xs_hi, xs_lo, xs_lo3;  // FP16 split of the HX input (chefsi_hx path)

  // real form of a complex operator (2 n_dofs real unknowns, 2 n_e x 2 n_e real cell
  // matrices) for the FP32 / tensor-core filter; built on first use
  std::unique_ptr<chefsi_operator_s> rv;

  // workspaces (grow-only)
  chefsi::DeviceBuffer<double> ws64a, ws64b, nlW64;
  chefsi::DeviceBuffer<float> nlW32, ws32x;
};

namespace chefsi {

// ---- operator apply (operator.cu) -------------------------------------------------------
// dst = (accumulate ? dst : 0) + scalar * A src
void hx_f64(chefsi_operator_s* op, const double* src, int64_t lds, double* dst, int64_t ldd,
            int B, double scalar, bool accumulate, cudaStream_t st);
void hx_f32(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd,
            int B, double scalar, bool accumulate, cudaStream_t st);
void hx_c64(chefsi_operator_s* op, const cplx* src, int64_t lds, cplx* dst, int64_t ldd, int B,
            double scalar, bool accumulate, cudaStream_t st);
// tensor-core (FP16 split) apply on FP32 vectors; returns false if unavailable for this op
bool hx_tc(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd, int B,
           double scalar, bool accumulate, cudaStream_t st);
// One member of a grouped tensor-core apply: dst += scalar * A src (local part only), the
// input given by its FP16 split rows [n_dofs][B] (xlo3 for the three-term split).
struct TcGroupItem {
  chefsi_operator_s* op;
  const __half* xhi;
  const __half* xlo;
  const __half* xlo3;
  float* dst;
  int64_t ldd;
  int B;
  double scalar;
};
// pipeline shape of the tensor-core apply (X-ring depth, K-blocks of copies in flight)
struct TcPipeline {
  int xstages;
  int lookahead;
  int cell_tile;   // > 1: (cell, chunk) pairs dealt as tiles of that many cells, chunk-major
};
// one block of a grouped recurrence step: y = a x + b y (b == 0: y not read), (hi, lo) = split(x)
struct AxpbyGroupItem {
  const float* x;
  float* y;
  __half* hi;
  __half* lo;
  int64_t n;  // entries (a multiple of 4)
  double a, b;
};
void axpby_split_group(const AxpbyGroupItem* items, int n, cudaStream_t st);
// one persistent launch over up to 32 applies of operators with the same cell type
void hx_tc_group_launch(const TcGroupItem* items, int n, int ns, const TcPipeline* pipe,
                        cudaStream_t st);
int device_sms();
// the density on tensor cores (FP16 split of M^{-1/2} x and of the shape functions, FP32 sums):
// rho[c][q] (+)= jxw * sum_v occ_v psi_v(x_q)^2; false if the tensor path does not apply
bool density_tc(chefsi_operator_s* op, const double* X, int64_t ld, int B, const double* occ,
                int n_q, const double* shape, const double* jxw, double* rho, bool accumulate,
                cudaStream_t st);
// the same with the three-term split (33 bits: src exactly, the cell matrices to 2^-33; six
// products, FP32 accumulation): the accuracy class of the FP32 apply. src must be scaled so
// that max |src| < 2^15.
bool hx_tc3(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd, int B,
            double scalar, bool accumulate, cudaStream_t st);
bool tc_usable(chefsi_operator_s* op);
// the tensor-core apply reads the input as FP16 hi + lo rows [n_dofs][B] (B % 8 == 0);
// src (FP32) feeds the nonlocal term
bool tc_split_usable(chefsi_operator_s* op, int B);
bool hx_tc_split(chefsi_operator_s* op, const __half* xhi, const __half* xlo, const float* src,
                 int64_t lds, float* dst, int64_t ldd, int B, double scalar, bool accumulate,
                 cudaStream_t st);
void split_rows_f32(const float* x, int64_t ldx, int64_t M, int B, __half* hi, __half* lo,
                    cudaStream_t st);
// y = a x + b y on contiguous [M][B] blocks (b == 0: y is not read) and (hi, lo) = split(x)
void axpby_split_f32(const float* x, float* y, int64_t M, int B, double a, double b, __half* hi,
                     __half* lo, cudaStream_t st);
// W[a][j][b] = sum_r C[r][j] x[dof_r][b] for FP32 vectors (W zeroed here)
void nl_project_f32(chefsi_operator_s* op, const float* x, int64_t ldx, float* W, int B,
                    cudaStream_t st);
void prepare_tensor_mats(chefsi_operator_s* op, cudaStream_t st);
// one fused filter step (tc.cu): x_j from the split rows of x_{j-1} (xhi/xlo, rows n_dofs +
// n_atoms n_proj: the last ones hold 2^t W) and x_{j-2} (ohi/olo on entry, single rows);
// x_j = a A x_{j-1} + c x_{j-1} + b x_{j-2} into ohi/olo; shared rows through acc / counter,
// whose accumulators are left pre-set to cn x_j + bn x_{j-1} when has_next
struct TcFusedLaunch {
  chefsi_operator_s* op;
  const __half* xhi;
  const __half* xlo;
  __half* ohi;
  __half* olo;
  float* acc;
  unsigned* counter;
  int B;
  double a, c, b, cn, bn;
  int has_next;
};
void hx_tc_fused_launch(const TcFusedLaunch& f, cudaStream_t st);
// dst += scalar (A + C V C^T) x on the tensor cores with the nonlocal apply as the plan's extra
// K columns: x given by split rows [plan rows][B], the projector rows holding 2^t C^T x
// (shift != 0: dst += scalar (A - shift I + C V C^T) x, the shift held on the tiles' diagonals;
// set_tile_shift must have accepted it)
void hx_tc_folded_launch(chefsi_operator_s* op, const __half* xhi, const __half* xlo, float* dst,
                         int64_t ldd, int B, double scalar, cudaStream_t st, double shift = 0.0);
// the same launch with x given as FP32 rows x32 [plan rows][B] (the projector rows holding
// C^T x unscaled), split by the kernel's producer warps after scaling by xf
void hx_tc_folded_f32_launch(chefsi_operator_s* op, const float* x32, float* dst, int64_t ldd,
                             int B, double scalar, double xf, cudaStream_t st, double shift);
// the projector rows of a split buffer: (hi, lo)[n_dofs + a P + j] = split(2^t (C^T f x)[a][j])
// from FP32 vectors x [n_dofs][B] (W: n_atoms n_proj B floats of workspace)
void nl_project_to_split(chefsi_operator_s* op, const float* x, int B, float* W, __half* hi,
                         __half* lo, cudaStream_t st, double f = 1.0);
// the plan's tiles with 2^s (A_II - shift / n_I) on their diagonals; false (tiles unchanged) if
// the shifted entries would leave FP16's range or the operator has constraint rows
bool set_tile_shift(chefsi_operator_s* op, double shift, cudaStream_t st);
// (hi, lo) = split(f x) over a contiguous block of n FP32 entries (n a multiple of 4); with
// rewrite also x = f x
void split_scaled_f32(float* x, int64_t n, double f, bool rewrite, __half* hi, __half* lo,
                      cudaStream_t st);
// row halves of the tensor-core tiles for n_e nodes (n_half rows each)
void tc_row_split(int n_e, int* n_half, int* n_halves);
// (cell, half, K-block) tiles of 2^s A_e over nkb K-blocks (columns past n_e zero)
void split_mats_ext(chefsi_operator_s* op, int nkb, double scale, __half* hi, __half* lo,
                    cudaStream_t st);
// workspaces of the fused filter (grow-only): two split buffers (x_{j-1}; x_j), the rows' FP32
// accumulators [n_dofs][B], the shared rows' arrival counters, the projector coefficients W
struct FusedWork {
  DeviceBuffer<__half> hi[2], lo[2];
  DeviceBuffer<float> acc, W;
  DeviceBuffer<unsigned> counter;
};
// the Chebyshev filter of one FP32 block X [M][B] (max |x| ~ 2^8) with the fused steps; mark()
// is called before and after every degree (profiling events)
void cheb_filter_fused(chefsi_operator_s* op, FusedWork& w, float* X, int64_t M, int B, int m,
                       double a, double b, double a0, const std::function<void()>& mark,
                       cudaStream_t st);
// the tables of the fused step (fused.cu); false if the operator does not take the fused path
bool fused_plan_usable(chefsi_operator_s* op);
// an operator with constraint rows on the tensor cores (the plan's tiles fold M^{-1/2} in)
bool constrained_tc_usable(chefsi_operator_s* op, int B);
// dst (+)= scalar A x for an operator with constraint rows, x given by its FP16 split rows
// (hi, lo) [plan rows][B]: the slave rows of the split are overwritten by the distributed
// values (sum w' x_m), the projector rows by 2^t C^T x; dst's slave rows keep their values
// (the launch's contributions to them are moved to their masters). W: n_atoms n_proj B floats,
// save: n_constrained B floats of workspace.
void hx_tc_constrained_split(chefsi_operator_s* op, __half* hi, __half* lo, float* dst,
                             int64_t ldd, int B, double scalar, float* W, float* save,
                             cudaStream_t st);
// the same from FP32 vectors src [n_dofs][lds] (split into the operator's workspace); dst is
// zeroed first unless accumulate
void hx_tc_constrained(chefsi_operator_s* op, const float* src, int64_t lds, float* dst,
                       int64_t ldd, int B, double scalar, bool accumulate, cudaStream_t st);
void prepare_fused_plan(chefsi_operator_s* op, cudaStream_t st);
// device error flag of the tensor-core kernel (CHEFSI_OK or CHEFSI_ERR_TIMEOUT); clears it
int tc_check_error(chefsi_operator_s* op, cudaStream_t st);
// nonlocal term y += scalar * C V C^T x for FP32 vectors (used by the tensor-core path)
void apply_nonlocal_f32(chefsi_operator_s* op, const float* src, int64_t lds, float* dst,
                        int64_t ldd, int B, double scalar, cudaStream_t st);

// ---- elementwise helpers (operator.cu) ----------------------------------------------------
template <typename T>
void scale_block(T* x, int64_t ld, int64_t rows, int B, double s, cudaStream_t st);
// y = a*x + b*y on [rows][B] blocks
template <typename T>
void axpby_block(const T* x, int64_t ldx, T* y, int64_t ldy, int64_t rows, int B, double a,
                 double b, cudaStream_t st);
// column block copy / precision conversion: dst[i][j] = s * src[i][j]
template <typename Ts, typename Td>
void copy_block(const Ts* src, int64_t lds, Td* dst, int64_t ldd, int64_t rows, int B, double s,
                cudaStream_t st);
// max |x| over a block (device scalar out, as float bits via atomicMax)
void absmax_block_f64(const double* x, int64_t ld, int64_t rows, int B, double* out_dev,
                      cudaStream_t st);
void absmax_block_f32(const float* x, int64_t ld, int64_t rows, int B, double* out_dev,
                      cudaStream_t st);

// ---- tensor-core dense products (dense_tc.cu) ---------------------------------------------
// FP16 hi/lo split of a block of vectors, each column scaled by 2^e[j] (max |entry| in
// [2^14, 2^15)). The transposed split (ld = rows padded to 64) is stored as tiles of 128
// columns x 32 rows, each the swizzled shared-memory image of a K-major Gram operand
// ([padded / 128][ld / 32][4096 halves]); the row split [rows][ld = padded columns] feeds the
// rotation.
struct TcOperand {
  DeviceBuffer<__half> hi, lo;
  DeviceBuffer<int> e;                     // column exponents
  DeviceBuffer<double> sc;                 // 2^e per column
  DeviceBuffer<unsigned long long> bits;   // column maxima (bit patterns)
  int64_t rows = 0;  // logical rows (dofs)
  int cols = 0;      // logical columns (vectors)
  int64_t ld = 0;    // leading dimension of the FP16 layout
  int padded = 0;    // padded column count
  bool transposed = false;
};
struct TcDenseWork {
  DeviceBuffer<double> part;      // Gram k-slice partials
  DeviceBuffer<__half> whi, wlo;  // rotation matrix operand
  DeviceBuffer<int> et;           // rotation output column exponents
  DeviceBuffer<int> err;          // bounded-wait expiry flag
};
bool dense_tc_available();
template <typename T>
void tc_exponents(const T* X, int64_t ld, int64_t M, int N, TcOperand& op, cudaStream_t st);
template <typename T>
void tc_split_transposed(const T* X, int64_t ld, int64_t M, int N, TcOperand& op, cudaStream_t st);
template <typename T>
void tc_split_rows(const T* X, int64_t ld, int64_t M, int N, TcOperand& op, cudaStream_t st);
// C += A^T B (B == nullptr: A^T A); lower: only 128x128 tiles on or below the diagonal
void tc_gram(const TcOperand& A, const TcOperand* B, double* C, int64_t ldc, bool lower,
             TcDenseWork& w, cudaStream_t st);
// Y[M][n_out] = X W, W [X.cols][n_out] (X given by its row split; Y may be X itself)
void tc_rotate(const TcOperand& Xr, const double* W, int64_t ldw, int n_out, double* Y,
               int64_t ldy, TcDenseWork& w, cudaStream_t st);
int tc_dense_check_error(TcDenseWork& w, cudaStream_t st);
void gram_tc_f64(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t K, int N1,
                 int N2, double* C, int ldc, bool lower_only, cudaStream_t st);
void rotate_tc_f64(const double* X, int64_t ld, int64_t M, int K, const double* W, int64_t ldw,
                   int n_out, double* Y, int64_t ldy, cudaStream_t st);

// ---- dense linear algebra (dense.cu) ------------------------------------------------------
// C (N x N, row-major, ldc) += A^H B for A [K][N1] (lda), B [K][N2] (ldb), K split across CTAs.
// prec FP64: FP64 throughout; MIXED/FP32: FP32 products inside K chunks, FP64 across chunks.
// lower_only: only tiles with row-tile >= col-tile (for A == B)
void gram_f64(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t K, int N1,
              int N2, double* C, int ldc, int prec, bool lower_only, cudaStream_t st);
void gram_c64(const cplx* A, int64_t lda, const cplx* B, int64_t ldb, int64_t K, int N1, int N2,
              cplx* C, int ldc, bool lower_only, cudaStream_t st);
// C[M][N] = alpha * op(A) op(B) + beta * C  (row-major; op: 'N' or 'T' (conj for complex))
void gemm_f64(char ta, char tb, int64_t M, int N, int K, double alpha, const double* A,
              int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
              int prec, cudaStream_t st);
void gemm_c64(char ta, char tb, int64_t M, int N, int K, cplx alpha, const cplx* A, int64_t lda,
              const cplx* B, int64_t ldb, cplx beta, cplx* C, int64_t ldc, cudaStream_t st);
void symmetrize_lower(double* A, int N, cudaStream_t st);
void symmetrize_lower_c(cplx* A, int N, cudaStream_t st);
// in-place lower Cholesky of N x N row-major A (upper part zeroed). Returns CHEFSI_OK or
// CHEFSI_ERR_NOT_SPD (synchronises the stream to read the flag).
int cholesky_lower(double* A, int N, cudaStream_t st);
// lower-triangular inverse in place
void trtri_lower(double* L, int N, cudaStream_t st);
// symmetric eigensolve (Householder tridiagonalisation, bisection, inverse iteration,
// back-transformation); A overwritten; eigenvalues ascending in w; vectors in columns of Z.
int syevd(double* A, int N, double* w, double* Z, cudaStream_t st);
// polls of a grid-barrier wait in the cooperative tridiagonalisation before it expires
void dense_set_barrier_spins(uint32_t spins);
namespace tcx {
// tries of the bounded mbarrier waits of the tensor-core kernels (tc.cu, dense_tc.cu)
void tc_set_wait_tries(uint32_t tries);
void dense_tc_set_wait_tries(uint32_t tries);
}  // namespace tcx
int syevd_range(double* A, int N, int il, int count, double* w, double* Z, cudaStream_t st);
// complex Hermitian counterparts (dense_c.cu)
int cholesky_lower_c(cplx* A, int N, cudaStream_t st);
void trtri_lower_c(cplx* L, int N, cudaStream_t st);
int heevd(cplx* A, int N, double* w, cplx* Z, cudaStream_t st);
int heevd_range(cplx* A, int N, int il, int count, double* w, cplx* Z, cudaStream_t st);
// residual norms of columns: out[j] = || HX[:,j] - lam[j] X[:,j] ||
void residual_norms_f64(const double* X, int64_t ldx, const double* HX, int64_t ldh, int64_t M,
                        int N, const double* lam_dev, double* out_dev, cudaStream_t st);
void residual_norms_c64(const cplx* X, int64_t ldx, const cplx* HX, int64_t ldh, int64_t M, int N,
                        const double* lam_dev, double* out_dev, cudaStream_t st);
// dot / norm helpers for Lanczos (device scalar results)
void dot_f64(const double* x, const double* y, int64_t n, double* out_dev, cudaStream_t st);

// adjoint / assembly building blocks (adjoint.cu)
void assemble_cells(int n_cells, int n_e, int n_q, const double* N, const double* K,
                    const double* v, double* out, cudaStream_t st);
// cells of any shape: 0.5 sum_q dN^T F_cq dN (F = J^-1 J^-T JxW per point) + N^T diag(v_c) N
void assemble_cells_geometry(int n_cells, int n_e, int n_q, const double* N, const double* dN,
                             const double* F, const double* v, double* out, cudaStream_t st);
void assemble_cells_gga(int n_cells, int n_e, int n_q, const double* N, const double* dN,
                        const double* K, const double* v, const double* g, double* out,
                        cudaStream_t st);
// g (nullable): derExcWithSigmaTimesGradRhoJxW [n_cells][n_q][3] for the GGA terms
void assemble_cells_bloch(int n_cells, int n_e, int n_q, const double* N, const double* dN,
                          const double* K, const double* v, const double* w, int n_k,
                          const double* kpts, double* out, cudaStream_t st,
                          const double* g = nullptr);
// G_c += alpha * sum_b weights[b] (D u_b)_c (D w_b)_c^T (weights null: 1), D = M^{-1/2}
void cell_outer(chefsi_operator_s* op, const double* u, const double* w, int64_t ld, int B,
                double alpha, double* G, cudaStream_t st, const double* weights = nullptr);
// out[c][q] (+)= jxw[c][q] * sum_IJ N[q][I] G[c][I][J] N[q][J]
void quad_contract(int n_cells, int n_e, int n_q, const double* N, const double* G,
                   const double* jxw, double* out, cudaStream_t st, bool accumulate = false);
// replace the operator's cell matrices (device, unscaled) and refresh the derived copies
void update_cell_matrices(chefsi_operator_s* op, const double* mats_dev, cudaStream_t st);
// the real form of a folded complex operator (cached in op->rv)
chefsi_operator_s* realified(chefsi_operator_s* op, cudaStream_t st);
// complex [M][B] block (ld) <-> FP32 real rows [2M][B] (row 2g = Re, 2g+1 = Im), scaled by s
void complex_to_real_rows(const cplx* X, int64_t ld, int64_t M, int B, double s, float* out,
                          cudaStream_t st);
void real_rows_to_complex(const float* in, int64_t M, int B, double s, cplx* X, int64_t ld,
                          cudaStream_t st);

// eigensolver kernels (dense.cu), launched by the eigensolver drivers
__global__ void k_hh_vector(double* A, int N, int k, double* V, double* tau, double* d, double* e);
__global__ void k_hh_symv(const double* A, int N, int k, const double* V, const double* tau,
                          double* p);
__global__ void k_hh_w(int N, int k, const double* V, const double* tau, double* p);
__global__ void k_hh_rank2(double* A, int N, int k, const double* V, const double* w);
__global__ void k_tail(const double* A, int N, double* d, double* e);
__global__ void k_bisect_warp(const double* d, const double* e, int n, int idx0, int count,
                              double* w);
__global__ void k_inverse_iteration(const double* d, const double* e, int n, const double* w,
                                    int count, int idx0, double* Z, int ldz, double* work,
                                    unsigned char* swaps, double ortol);
__global__ void k_bt_dot(const double* V, int N, int k, const double* Z, double* r);
__global__ void k_bt_update(const double* V, int N, int k, const double* tau, double* Z,
                            const double* r);

}  // namespace chefsi
