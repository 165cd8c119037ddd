// C ABI of the CheFSI library and the solver driver.
//
// chefsi_solve follows chebyshevOrthogonalizedSubspaceIterationSolverDevice::solve
// (src/solvers/eigenSolvers/chebyshevOrthogonalizedSubspaceIterationSolverDevice.cc:155-736)
// with the CGS / Rayleigh-Ritz-GEP branch: block-wise Chebyshev filtering of all N vectors
// (chebyWfcBlockSize columns at a time), then the generalised Rayleigh-Ritz step
// (rayleighRitzGEP, src/linAlg/rayleighRitzDevice.cc:356-819) and the residual norms
// (computeEigenResidualNorm). Every dense step runs on the device; only eigenvalues,
// residual norms and bounds come back to the host.
#include "internal.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <random>
#include <thread>
#include <vector>

namespace chefsi {
const char* last_error_cstr();
unsigned long long launch_count();
chefsi_operator_s* create_operator(const chefsi_operator_desc* d);
}  // namespace chefsi

using namespace chefsi;

struct chefsi_solver_s {
  chefsi_params p{};
  double a0 = 0.0, b_low = 0.0, b_up = 0.0;
  int last_degree = 0;
  DeviceBuffer<double> Xb64, Yb64, S, Hp, T1, Z, W, evals, HX, rot, resid, scal;
  DeviceBuffer<double> HXf, HXF;  // spectrum split: FP64 H X of the fractional columns, H XFrac
  DeviceBuffer<double> G2, W2;  // 2N x 2N real views for the complex tensor-core products
  DeviceBuffer<float> Xb32, Yb32;
  TcOperand tx, th;      // FP16 splits of X and HX for the tensor-core RR products
  DeviceBuffer<__half> xs_hi, xs_lo;  // FP16 split of the filter's HX input
  FusedWork fzw;                      // the fused filter's split buffers and accumulators
  TcDenseWork tcw;
  double times[7] = {0, 0, 0, 0, 0, 0, 0};
  cudaEvent_t ev[8] = {};
  bool profile = false;
  std::vector<cudaEvent_t> hx_ev;   // pairs around filter HX launches
  int hx_used = 0;
  int hx_launches = 0;
  double hx_ms = 0.0;
  void hx_mark(cudaStream_t st) {
    if (!profile) return;
    if (hx_used >= (int)hx_ev.size()) {
      cudaEvent_t e;
      CHEFSI_CUDA(cudaEventCreate(&e));
      hx_ev.push_back(e);
    }
    CHEFSI_CUDA(cudaEventRecord(hx_ev[hx_used++], st));
  }
  void hx_collect() {
    hx_launches = 0;
    hx_ms = 0.0;
    for (int i = 0; i + 1 < hx_used; i += 2) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, hx_ev[i], hx_ev[i + 1]) == cudaSuccess) {
        hx_ms += ms;
        ++hx_launches;
      } else {
        cudaGetLastError();
      }
    }
    hx_used = 0;
  }
  chefsi_solver_s() {
    for (auto& e : ev) cudaEventCreate(&e);
  }
  ~chefsi_solver_s() {
    for (auto& e : ev)
      if (e) cudaEventDestroy(e);
    for (auto& e : hx_ev) cudaEventDestroy(e);
  }
};

#define CHEFSI_API_BEGIN try {
#define CHEFSI_API_END                                        \
  return CHEFSI_OK;                                           \
  }                                                           \
  catch (const chefsi::Error& e) {                            \
    chefsi::set_last_error(e.what());                         \
    return e.code;                                            \
  }                                                           \
  catch (const std::exception& e) {                           \
    chefsi::set_last_error(e.what());                         \
    return CHEFSI_ERR_INVALID;                                \
  }                                                           \
  catch (...) {                                               \
    chefsi::set_last_error("unknown error");                  \
    return CHEFSI_ERR_INVALID;                                \
  }

namespace {

const int kOrderLookup[][2] = {{500, 24},    {750, 30},     {1000, 39},    {1500, 50},
                               {2000, 53},   {3000, 57},    {4000, 62},    {5000, 69},
                               {9000, 77},   {14000, 104},  {20000, 119},  {30000, 162},
                               {50000, 300}, {80000, 450},  {100000, 550}, {200000, 700},
                               {500000, 1000}};

bool is_mixed(int prec) { return prec == CHEFSI_PREC_MIXED || prec == CHEFSI_PREC_FP32; }

// HX of the FP32 filter vectors: tensor cores (FP16 split) for MIXED, SIMT FP32 otherwise
void hx_filter32(chefsi_operator_s* op, int prec, const float* src, float* dst, int B,
                 double scalar, bool acc, cudaStream_t st) {
  if (prec == CHEFSI_PREC_MIXED && hx_tc(op, src, B, dst, B, B, scalar, acc, st)) return;
  hx_f32(op, src, B, dst, B, B, scalar, acc, st);
}

// Chebyshev filter (sigma form) of a contiguous block [M][B]; result returned in X.
// linearAlgebraOperationsDevice::chebyshevFilter, src/linAlg/linearAlgebraOperationsDevice.cc:531-727:
//   Y = (sigma1/e)(A X - c X);  for degree 2..m: X = alpha2 X - c alpha1 Y;  X += alpha1 A Y; swap.
// The reference's combinedDeviceKernel step is the axpby; HX accumulates into its output.
template <typename T, typename HXF>
void cheb_filter(T* X, T* Y, int64_t M, int B, int m, double a, double b, double a0, HXF hx,
                 cudaStream_t st) {
  const double e = (b - a) / 2.0, c = (b + a) / 2.0;
  double sigma = e / (a0 - c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  double alpha1 = sigma1 / e, alpha2 = -c;
  copy_block<T, T>(X, B, Y, B, M, B, alpha1 * alpha2, st);
  hx(X, Y, alpha1, true);
  T* x = X;
  T* y = Y;
  for (int degree = 2; degree < m + 1; ++degree) {
    const double sigma2 = 1.0 / (gamma - sigma);
    alpha1 = 2.0 * sigma2 / e;
    alpha2 = -(sigma * sigma2);
    axpby_block<T>(y, B, x, B, M, B, -c * alpha1, alpha2, st);
    hx(y, x, alpha1, true);
    std::swap(x, y);
    sigma = sigma2;
  }
  if (y != X) copy_block<T, T>(y, B, X, B, M, B, 1.0, st);
}

// rows of the filter's FP32 work blocks: the vectors, then (shifted filter) the projector rows
int64_t filter_rows(chefsi_operator_s* op) {
  return op->n_dofs + (op->is_complex ? 0 : (int64_t)op->n_atoms * op->n_proj);
}

// where a mixed filter left its result: the block out (X or Y) times factor
struct FilterOut {
  const float* out;
  double factor;
};

// Mixed Chebyshev filter with the shift on the tensor-core tiles. In the sigma form every degree
// is x_j = alpha1_j (A - c) x_{j-1} + alpha2_j x_{j-2} with the same c, so the plan's tiles carry
// 2^s (A_II - c / n_I) on their diagonals for the whole call and each degree is one HX launch
// reducing into the buffer of x_{j-2}. Each buffer holds its vector up to a factor kept here
// (vector = factor * buffer): the update alpha2 x_{j-2} only changes the factor, so no
// recurrence pass runs (the reference's combinedDeviceKernel,
// linearAlgebraOperationsDevice.cc:37-104, reads and writes both vectors every degree), and
// no split pass either: the launch gathers x_{j-1} as FP32 rows and its producer warps write
// the FP16 split of f x_{j-1} (f the power of two nearest its factor, which keeps the split at
// the vector's own magnitude). Besides the launch, a degree only runs the projection C^T x_{j-1}
// into the buffer's rows past n_dofs. X and Y hold filter_rows(op) rows; the result is left in
// one of them up to a factor (*res). Returns false (nothing done) when the shifted diagonals
// would leave FP16's range.
bool cheb_filter_shifted(chefsi_solver_s* s, chefsi_operator_s* op, float* X, float* Y, int64_t M,
                         int B, int m, double a, double b, double a0, cudaStream_t st,
                         FilterOut* res) {
  prepare_fused_plan(op, st);
  const double e = (b - a) / 2.0, c = (b + a) / 2.0;
  if (!set_tile_shift(op, c, st)) return false;
  const int64_t n = M * (int64_t)B;
  // out += scalar (A - c) v for the vector v = s_in in: the launch's producer warps split f in
  // (f the power of two nearest s_in: the split sees the vector's own magnitude), so its scalar
  // is scalar s_in / f; the projection writes C^T in into the buffer's rows past n_dofs. A
  // factor beyond 2^+-64 is first moved into the buffer (one scaling pass; rare).
  auto apply = [&](float* in, double& s_in, float* out, double scalar) {
    double f = std::ldexp(1.0, (int)std::lround(std::log2(std::fabs(s_in))));
    if (std::fabs(std::log2(f)) > 64.0) {
      scale_block<float>(in, B, M, B, f, st);
      s_in /= f;
      f = 1.0;
    }
    s->hx_mark(st);
    nl_project_f32(op, in, B, in + n, B, st);
    hx_tc_folded_f32_launch(op, in, out, B, B, scalar * s_in / f, f, st, c);
    s->hx_mark(st);
  };
  double sigma = e / (a0 - c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  double sx = 1.0, sy = 1.0;   // x_0 = X, x_1 = sy Y
  CHEFSI_CUDA(cudaMemsetAsync(Y, 0, sizeof(float) * (size_t)n, st));
  apply(X, sx, Y, sigma1 / e);
  float* x = X;   // x_{j-2}
  float* y = Y;   // x_{j-1}
  for (int degree = 2; degree < m + 1; ++degree) {
    const double sigma2 = 1.0 / (gamma - sigma);
    const double alpha1 = 2.0 * sigma2 / e, alpha2 = -(sigma * sigma2);
    // x_j = alpha2 sx [x + alpha1 / (alpha2 sx) (A - c) x_{j-1}] in the buffer of x_{j-2}
    apply(y, sy, x, alpha1 / (alpha2 * sx));
    sx *= alpha2;
    std::swap(x, y);
    std::swap(sx, sy);
    sigma = sigma2;
  }
  *res = FilterOut{y, sy};   // applied by the caller's conversion back to FP64
  return true;
}

// Mixed Chebyshev filter on the tensor cores (same recurrence as cheb_filter): the shifted
// filter by default; otherwise (variant 2, operators with constraint rows, shifts beyond the
// tiles' range) a recurrence step per degree y_{k-1} <- -c alpha1 y_k + alpha2 y_{k-1} that also
// writes the FP16 hi + lo split of y_k, the next HX's input. Returns the block holding the
// result and its factor.
FilterOut cheb_filter_tc(chefsi_solver_s* s, chefsi_operator_s* op, float* X, float* Y,
                         int64_t M, int B, int m, double a, double b, double a0, cudaStream_t st) {
  if (s->p.filter_variant == 1 && fused_plan_usable(op)) {
    // one launch per degree finishes the recurrence and applies the nonlocal term
    cheb_filter_fused(op, s->fzw, X, M, B, m, a, b, a0, [&] { s->hx_mark(st); }, st);
    return FilterOut{X, 1.0};
  }
  // the nonlocal apply folded into the tensor-core launch (extra K columns of the cell
  // matrices fed by split rows of 2^t C^T x after the dof rows), unless the separate nonlocal
  // kernels are asked for
  // operators with constraint rows: distribute on the split rows, the plan's tiles (M^{-1/2}
  // folded in by the plan), the adjoint after the launch
  const bool constrained = !op->folded;
  FilterOut res{X, 1.0};
  if (s->p.filter_variant == 0 && !constrained && fused_plan_usable(op) &&
      cheb_filter_shifted(s, op, X, Y, M, B, m, a, b, a0, st, &res))
    return res;
  // variant 2 (and variant 0 when the shift does not fit the tiles): a recurrence pass per
  // degree and the HX launch with the nonlocal apply folded in
  const bool fold = constrained || ((s->p.filter_variant == 0 || s->p.filter_variant == 2) &&
                                    op->n_atoms > 0 && fused_plan_usable(op));
  if (fold) prepare_fused_plan(op, st);
  const size_t rows = fold ? (size_t)op->fz.rows : (size_t)M;
  __half* hi = s->xs_hi.ensure(rows * B);
  __half* lo = s->xs_lo.ensure(rows * B);
  float* W = fold && op->n_atoms ? s->fzw.W.ensure((size_t)op->n_atoms * op->n_proj * B) : nullptr;
  float* save = constrained ? s->fzw.acc.ensure((size_t)op->n_con * B) : nullptr;
  const double e = (b - a) / 2.0, c = (b + a) / 2.0;
  double sigma = e / (a0 - c);
  const double sigma1 = sigma, gamma = 2.0 / sigma1;
  double alpha1 = sigma1 / e, alpha2 = -c;
  auto hx = [&](const float* src, float* dst, double sc) {
    s->hx_mark(st);
    if (constrained) {
      hx_tc_constrained_split(op, hi, lo, dst, B, B, sc, W, save, st);
    } else if (fold) {
      nl_project_to_split(op, src, B, W, hi, lo, st);
      hx_tc_folded_launch(op, hi, lo, dst, B, B, sc, st);
    } else if (!hx_tc_split(op, hi, lo, src, B, dst, B, B, sc, true, st)) {
      throw Error(CHEFSI_ERR_INVALID, "tensor-core filter HX not applicable to this block");
    }
    s->hx_mark(st);
  };
  axpby_split_f32(X, Y, M, B, alpha1 * alpha2, 0.0, hi, lo, st);   // Y = a X, split(X)
  hx(X, Y, alpha1);
  float* x = X;
  float* y = Y;
  for (int degree = 2; degree < m + 1; ++degree) {
    const double sigma2 = 1.0 / (gamma - sigma);
    alpha1 = 2.0 * sigma2 / e;
    alpha2 = -(sigma * sigma2);
    axpby_split_f32(y, x, M, B, -c * alpha1, alpha2, hi, lo, st);
    hx(y, x, alpha1);
    std::swap(x, y);
    sigma = sigma2;
  }
  return FilterOut{y, 1.0};
}

// filter columns [j0, j0+B) of X (ld) in place
void filter_columns(chefsi_solver_s* s, chefsi_operator_s* op, double* X, int64_t ld, int j0,
                    int B, int m, double a, double b, double a0, int prec, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  if (!is_mixed(prec)) {
    double* Xb = s->Xb64.ensure((size_t)M * B);
    double* Yb = s->Yb64.ensure((size_t)M * B);
    copy_block<double, double>(X + j0, ld, Xb, B, M, B, 1.0, st);
    cheb_filter<double>(Xb, Yb, M, B, m, a, b, a0,
                        [&](const double* src, double* dst, double sc, bool acc) {
                          s->hx_mark(st);
                          hx_f64(op, src, B, dst, B, B, sc, acc, st);
                          s->hx_mark(st);
                        },
                        st);
    copy_block<double, double>(Xb, B, X + j0, ld, M, B, 1.0, st);
    return;
  }
  // FP32 block vectors scaled by a power of two so that the largest entry is ~2^8 (keeps the
  // FP16 split of the tensor-core HX in its normal range; the recurrence is linear)
  double* sc = s->scal.ensure(1);
  absmax_block_f64(X + j0, ld, M, B, sc, st);
  double amax = 0.0;
  CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  double scale = 1.0;
  if (amax > 0.0 && std::isfinite(amax)) scale = std::ldexp(1.0, 8 - (int)std::ceil(std::log2(amax)));
  // (rows past n_dofs: the shifted filter's projector rows)
  float* Xb = s->Xb32.ensure((size_t)filter_rows(op) * B);
  float* Yb = s->Yb32.ensure((size_t)filter_rows(op) * B);
  copy_block<double, float>(X + j0, ld, Xb, B, M, B, scale, st);
  FilterOut fo{Xb, 1.0};
  if (prec == CHEFSI_PREC_MIXED && (tc_split_usable(op, B) || constrained_tc_usable(op, B))) {
    fo = cheb_filter_tc(s, op, Xb, Yb, M, B, m, a, b, a0, st);
  } else {
    cheb_filter<float>(Xb, Yb, M, B, m, a, b, a0,
                       [&](const float* src, float* dst, double scv, bool acc) {
                         s->hx_mark(st);
                         hx_filter32(op, prec, src, dst, B, scv, acc, st);
                         s->hx_mark(st);
                       },
                       st);
  }
  if (prec == CHEFSI_PREC_MIXED) {
    const int tc = tc_check_error(op, st);
    if (tc != CHEFSI_OK) throw Error(tc, "tensor-core HX: a bounded device wait expired");
  }
  // the filter's own factor rides in the conversion back to FP64
  copy_block<float, double>(fo.out, B, X + j0, ld, M, B, fo.factor / scale, st);
}

void filter_all(chefsi_solver_s* s, chefsi_operator_s* op, void* X, int N, int m, int prec,
                cudaStream_t st) {
  const int Bmax = std::max(1, std::min(s->p.cheby_wfc_block > 0 ? s->p.cheby_wfc_block : N, N));
  for (int j0 = 0; j0 < N; j0 += Bmax) {
    const int B = std::min(Bmax, N - j0);
    if (op->is_complex && is_mixed(prec) && op->folded) {
      // mixed Bloch filter: the real form of the operator (2 n_dofs unknowns) on FP32 rows,
      // so the tensor-core (FP16 split) or FP32 HX applies
      chefsi_operator_s* rv = realified(op, st);
      cplx* Xc = reinterpret_cast<cplx*>(X);
      const int64_t M = op->n_dofs;
      double* sc = s->scal.ensure(1);
      absmax_block_f64(reinterpret_cast<double*>(Xc + j0), 2 * (int64_t)N, M, 2 * B, sc, st);
      double amax = 0.0;
      CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
      CHEFSI_CUDA(cudaStreamSynchronize(st));
      double scale = 1.0;
      if (amax > 0.0 && std::isfinite(amax))
        scale = std::ldexp(1.0, 8 - (int)std::ceil(std::log2(amax)));
      float* xr = s->Xb32.ensure((size_t)filter_rows(rv) * B);
      float* yr = s->Yb32.ensure((size_t)filter_rows(rv) * B);
      complex_to_real_rows(Xc + j0, N, M, B, scale, xr, st);
      FilterOut fo{xr, 1.0};
      if (prec == CHEFSI_PREC_MIXED && tc_split_usable(rv, B)) {
        fo = cheb_filter_tc(s, rv, xr, yr, 2 * M, B, m, s->b_low, s->b_up, s->a0, st);
      } else {
        cheb_filter<float>(xr, yr, 2 * M, B, m, s->b_low, s->b_up, s->a0,
                           [&](const float* src, float* dst, double scv, bool acc) {
                             s->hx_mark(st);
                             hx_filter32(rv, prec, src, dst, B, scv, acc, st);
                             s->hx_mark(st);
                           },
                           st);
      }
      if (prec == CHEFSI_PREC_MIXED) {
        const int tc = tc_check_error(rv, st);
        if (tc != CHEFSI_OK) throw Error(tc, "tensor-core HX: a bounded device wait expired");
      }
      real_rows_to_complex(fo.out, M, B, fo.factor / scale, Xc + j0, N, st);
    } else if (op->is_complex) {
      cplx* Xc = reinterpret_cast<cplx*>(X);
      cplx* Xb = reinterpret_cast<cplx*>(s->Xb64.ensure((size_t)op->n_dofs * B * 2));
      cplx* Yb = reinterpret_cast<cplx*>(s->Yb64.ensure((size_t)op->n_dofs * B * 2));
      copy_block<cplx, cplx>(Xc + j0, N, Xb, B, op->n_dofs, B, 1.0, st);
      cheb_filter<cplx>(Xb, Yb, op->n_dofs, B, m, s->b_low, s->b_up, s->a0,
                        [&](const cplx* src, cplx* dst, double sc, bool acc) {
                          hx_c64(op, src, B, dst, B, B, sc, acc, st);
                        },
                        st);
      copy_block<cplx, cplx>(Xb, B, Xc + j0, N, op->n_dofs, B, 1.0, st);
    } else {
      filter_columns(s, op, reinterpret_cast<double*>(X), N, j0, B, m, s->b_low, s->b_up, s->a0,
                     prec, st);
    }
  }
}

// FP64 HX of all N columns of X into HX (blocks of wfc_block columns)
void hx_all_f64(chefsi_operator_s* op, const double* X, int64_t ld, int N, double* HX, int wfc_block,
                cudaStream_t st) {
  const int Bmax = std::max(1, std::min(wfc_block > 0 ? wfc_block : N, N));
  for (int j0 = 0; j0 < N; j0 += Bmax) {
    const int B = std::min(Bmax, N - j0);
    hx_f64(op, X + j0, ld, HX + j0, N, B, 1.0, false, st);
  }
}

// X[M][N] <- X W (row blocks through a temporary)
void rotate_rows(chefsi_solver_s* s, double* X, int64_t ld, int64_t M, int N, const double* W,
                 int prec, cudaStream_t st) {
  if (prec == CHEFSI_PREC_MIXED && dense_tc_available()) {
    tc_exponents<double>(X, ld, M, N, s->tx, st);
    tc_split_rows<double>(X, ld, M, N, s->tx, st);
    tc_rotate(s->tx, W, N, N, X, ld, s->tcw, st);
    const int rc = tc_dense_check_error(s->tcw, st);
    if (rc != CHEFSI_OK) throw Error(rc, "tensor-core rotation: a bounded device wait expired");
    return;
  }
  const int64_t rows = std::min<int64_t>(M, std::max<int64_t>(4096, (int64_t)(256ll << 20) / (8ll * N)));
  double* tmp = s->rot.ensure((size_t)rows * N);
  for (int64_t r0 = 0; r0 < M; r0 += rows) {
    const int64_t nr = std::min(rows, M - r0);
    gemm_f64('N', 'N', nr, N, N, 1.0, X + r0 * ld, ld, W, N, 0.0, tmp, N, prec, st);
    copy_block<double, double>(tmp, N, X + r0 * ld, ld, nr, N, 1.0, st);
  }
}

__global__ void k_negate_diag0(double* S) { S[0] = -fabs(S[0]) - 1.0; }

__global__ void k_conj_transpose(const cplx* __restrict__ A, cplx* __restrict__ B, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    B[t] = cconj(A[(t % N) * N + t / N]);
}

__global__ void k_transpose(const double* __restrict__ A, double* __restrict__ B, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    B[t] = A[(t % N) * N + t / N];
}

// The overlap's Cholesky factor (lower, in place of S). A tensor-core S resolves 22 bits: for a
// block whose overlap is conditioned beyond that (a filtered block far from convergence), its
// Cholesky fails although the FP64 one would not, so S is taken again with the FP64 Gram
// before CHEFSI_ERR_NOT_SPD is reported. CHEFSI_FAULT_INJECT=not_spd spoils every S,
// =not_spd_mixed only the tensor-core one (to exercise the second attempt).
int cholesky_overlap(double* S, const double* X, int64_t ld, int64_t M, int N, bool tc_gram_used,
                     cudaStream_t st) {
  if (fault_injected("not_spd") || (tc_gram_used && fault_injected("not_spd_mixed"))) {
    k_negate_diag0<<<1, 1, 0, st>>>(S);
    CHEFSI_CHECK_LAUNCH();
  }
  int rc = cholesky_lower(S, N, st);
  if (rc != CHEFSI_OK && tc_gram_used) {
    CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
    gram_f64(X, ld, X, ld, M, N, N, S, N, CHEFSI_PREC_FP64, true, st);
    symmetrize_lower(S, N, st);
    if (fault_injected("not_spd")) {
      k_negate_diag0<<<1, 1, 0, st>>>(S);
      CHEFSI_CHECK_LAUNCH();
    }
    rc = cholesky_lower(S, N, st);
  }
  if (rc != CHEFSI_OK) set_last_error("overlap matrix is not positive definite (Cholesky pivot <= 0)");
  return rc;
}

// Rayleigh-Ritz, generalised form (rayleighRitzGEP): returns eigenvalues (device) and
// rotates X (and HX if requested) to the Ritz basis.
int rayleigh_ritz_real(chefsi_solver_s* s, chefsi_operator_s* op, double* X, int64_t ld, int N,
                       int prec, bool want_hx, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  // mixed mode on tensor cores: FP16-split Gram products and rotations (dense_tc.cu)
  const bool tcd = prec == CHEFSI_PREC_MIXED && dense_tc_available();
  double* S = s->S.ensure((size_t)N * N);
  double* Hp = s->Hp.ensure((size_t)N * N);
  double* T1 = s->T1.ensure((size_t)N * N);
  double* Z = s->Z.ensure((size_t)N * N);
  double* W = s->W.ensure((size_t)N * N);
  double* w = s->evals.ensure(N);
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  // S = X^T X (lower), then mirrored
  CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
  if (tcd) {
    tc_exponents<double>(X, ld, M, N, s->tx, st);
    tc_split_transposed<double>(X, ld, M, N, s->tx, st);
    tc_gram(s->tx, nullptr, S, N, true, s->tcw, st);
  } else {
    gram_f64(X, ld, X, ld, M, N, N, S, N, prec, true, st);
  }
  symmetrize_lower(S, N, st);
  int rc = cholesky_overlap(S, X, ld, M, N, tcd, st);
  if (rc != CHEFSI_OK) return rc;
  trtri_lower(S, N, st);  // S now holds L^{-1}
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  // Hp = X^T (A X). The HX is FP64 unless the mixed mode asks for the FP32 SIMT apply; then
  // X is rounded to FP32 once and the same rounded basis enters S (the mixed Gram converts on
  // load), HX and Hp, so the generalised problem stays consistent.
  double* HX = s->HX.ensure((size_t)M * N);
  // rr_precision FP32_TC: X rounded to FP32 and applied with the three-term tensor-core split
  // (exact FP32 operands, six products, FP32 accumulation; the FP32 SIMT apply where the tensor
  // path does not apply). FP32: the FP32 SIMT apply. MIXED: the filter's two-term split (22
  // bits). The tensor paths scale X by a power of two into the split's range.
  const int rrp = s->p.rr_precision;
  const bool tc3 = is_mixed(prec) && rrp == CHEFSI_PREC_FP32_TC && tc_split_usable(op, N);
  const bool tc2 = is_mixed(prec) && rrp == CHEFSI_PREC_MIXED && tc_split_usable(op, N);
  const bool hx32 = is_mixed(prec) && (rrp == CHEFSI_PREC_FP32 || rrp == CHEFSI_PREC_FP32_TC || tc2);
  float* y32 = nullptr;
  if (hx32) {
    float* x32 = s->Xb32.ensure((size_t)M * N);
    y32 = s->Yb32.ensure((size_t)M * N);
    double scale = 1.0;
    if (tc2 || tc3) {
      double amax = 0.0;
      if (tcd) {
        // the largest of the column maxima the tensor-core Gram just took (no pass over X)
        std::vector<unsigned long long> bits(N);
        CHEFSI_CUDA(cudaMemcpyAsync(bits.data(), s->tx.bits.ptr, sizeof(unsigned long long) * N,
                                    cudaMemcpyDeviceToHost, st));
        CHEFSI_CUDA(cudaStreamSynchronize(st));
        const unsigned long long mb = *std::max_element(bits.begin(), bits.end());
        std::memcpy(&amax, &mb, sizeof(double));
      } else {
        double* sc = s->scal.ensure(1);
        absmax_block_f64(X, ld, M, N, sc, st);
        CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
        CHEFSI_CUDA(cudaStreamSynchronize(st));
      }
      if (amax > 0.0 && std::isfinite(amax))
        scale = std::ldexp(1.0, (tc3 ? 14 : 8) - (int)std::ceil(std::log2(amax)));
    }
    copy_block<double, float>(X, ld, x32, N, M, N, scale, st);
    bool done = false;
    if (tc3)
      done = hx_tc3(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    else if (tc2)
      done = hx_tc(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    if (!done) hx_f32(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    // the tensor-core path reads the FP32 HX directly; its rotation writes the FP64 HX
    if (!tcd) copy_block<float, double>(y32, N, HX, N, M, N, 1.0, st);
  } else {
    hx_all_f64(op, X, ld, N, HX, s->p.wfc_block, st);
  }
  CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(double) * N * N, st));
  if (tcd) {
    if (hx32) {
      tc_exponents<float>(y32, N, M, N, s->th, st);
      tc_split_transposed<float>(y32, N, M, N, s->th, st);
    } else {
      tc_exponents<double>(HX, N, M, N, s->th, st);
      tc_split_transposed<double>(HX, N, M, N, s->th, st);
    }
    tc_gram(s->tx, &s->th, Hp, N, true, s->tcw, st);
  } else {
    gram_f64(X, ld, HX, N, M, N, N, Hp, N, prec, true, st);
  }
  symmetrize_lower(Hp, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  // C = L^{-1} Hp L^{-T}
  gemm_f64('N', 'N', N, N, N, 1.0, S, N, Hp, N, 0.0, T1, N, CHEFSI_PREC_FP64, st);
  gemm_f64('N', 'T', N, N, N, 1.0, T1, N, S, N, 0.0, Hp, N, CHEFSI_PREC_FP64, st);
  symmetrize_lower(Hp, N, st);
  rc = syevd(Hp, N, w, Z, st);
  if (rc != CHEFSI_OK) return rc;
  // W = L^{-T} Q
  gemm_f64('T', 'N', N, N, N, 1.0, S, N, Z, N, 0.0, W, N, CHEFSI_PREC_FP64, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  if (tcd) {
    // X <- X W in place from its FP16 row split (the column exponents of X are reused)
    tc_split_rows<double>(X, ld, M, N, s->tx, st);
    tc_rotate(s->tx, W, N, N, X, ld, s->tcw, st);
    if (want_hx) {
      if (hx32)
        tc_split_rows<float>(y32, N, M, N, s->th, st);
      else
        tc_split_rows<double>(HX, N, M, N, s->th, st);
      tc_rotate(s->th, W, N, N, HX, N, s->tcw, st);
    }
    rc = tc_dense_check_error(s->tcw, st);
    if (rc != CHEFSI_OK) {
      set_last_error("tensor-core Rayleigh-Ritz products: a bounded device wait expired");
      return rc;
    }
  } else {
    rotate_rows(s, X, ld, M, N, W, prec, st);
    if (want_hx) rotate_rows(s, HX, N, M, N, W, prec, st);
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[5], st));
  return CHEFSI_OK;
}

// Rayleigh-Ritz of rayleigh_ritz_real with its workspaces bounded by a column block of rr_block
// vectors and a row slab of dofs, for blocks whose full-size workspaces do not fit the GPU (4096
// vectors over 4.1M dofs: 134 GB for X alone). The reference forms X^T H X the same way, one
// wfcBlockSize column block at a time (XtHX, kohnShamDFTOperatorDevice.cc:4003-4157):
//   S = X^T X: the tensor-core Gram accumulated over row slabs (each slab split with its own
//     column exponents) or the FP64 / FP32 Gram directly;
//   Hp[j0:, j0:j0+b] = X[:, j0:]^T H X[:, j0:j0+b] per column block, H X of one block at a time;
//   X <- X W by row slabs (in place; the rotation reads the slab's split);
//   residual norms from a fresh H X of each rotated block (no full-size H X is kept).
int rayleigh_ritz_real_blocked(chefsi_solver_s* s, chefsi_operator_s* op, double* X, int64_t ld,
                               int N, int prec, double* res, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  const bool tcd = prec == CHEFSI_PREC_MIXED && dense_tc_available();
  const int blk = std::max(1, std::min(s->p.rr_block > 0 ? s->p.rr_block : 256, N));
  int64_t ms = s->p.rr_slab_rows > 0 ? s->p.rr_slab_rows
                                     : std::max<int64_t>(64, (int64_t)(1ll << 30) / std::max(1, N));
  ms = std::min<int64_t>(M, std::max<int64_t>(64, (ms + 63) / 64 * 64));
  double* S = s->S.ensure((size_t)N * N);
  double* Hp = s->Hp.ensure((size_t)N * N);
  double* T1 = s->T1.ensure((size_t)N * N);
  double* Z = s->Z.ensure((size_t)N * N);
  double* W = s->W.ensure((size_t)N * N);
  double* w = s->evals.ensure(N);
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
  if (tcd) {
    for (int64_t r0 = 0; r0 < M; r0 += ms) {
      const int64_t mr = std::min(ms, M - r0);
      tc_exponents<double>(X + r0 * ld, ld, mr, N, s->tx, st);
      tc_split_transposed<double>(X + r0 * ld, ld, mr, N, s->tx, st);
      tc_gram(s->tx, nullptr, S, N, true, s->tcw, st);
    }
  } else {
    gram_f64(X, ld, X, ld, M, N, N, S, N, prec, true, st);
  }
  symmetrize_lower(S, N, st);
  int rc = cholesky_overlap(S, X, ld, M, N, tcd, st);
  if (rc != CHEFSI_OK) return rc;
  trtri_lower(S, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  const int rrp = s->p.rr_precision;
  const bool tc3 = is_mixed(prec) && rrp == CHEFSI_PREC_FP32_TC && tc_split_usable(op, blk);
  const bool tc2 = is_mixed(prec) && rrp == CHEFSI_PREC_MIXED && tc_split_usable(op, blk);
  const bool hx32 = is_mixed(prec) && (rrp == CHEFSI_PREC_FP32 || rrp == CHEFSI_PREC_FP32_TC || tc2);
  float* x32 = hx32 ? s->Xb32.ensure((size_t)M * blk) : nullptr;
  float* y32 = hx32 ? s->Yb32.ensure((size_t)M * blk) : nullptr;
  double* HXb = s->HX.ensure((size_t)M * blk);
  // H X of columns [j0, j0 + b) into y32 (reduced precision) or HXb (FP64), leading dim b;
  // with to_f64 the reduced result is also widened into HXb
  auto hx_block = [&](int j0, int b, bool to_f64) {
    if (hx32) {
      double scale = 1.0;
      if (tc2 || tc3) {
        double* sc = s->scal.ensure(1);
        absmax_block_f64(X + j0, ld, M, b, sc, st);
        double amax = 0.0;
        CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
        CHEFSI_CUDA(cudaStreamSynchronize(st));
        if (amax > 0.0 && std::isfinite(amax))
          scale = std::ldexp(1.0, (tc3 ? 14 : 8) - (int)std::ceil(std::log2(amax)));
      }
      copy_block<double, float>(X + j0, ld, x32, b, M, b, scale, st);
      bool done = false;
      if (tc3)
        done = hx_tc3(op, x32, b, y32, b, b, 1.0 / scale, false, st);
      else if (tc2)
        done = hx_tc(op, x32, b, y32, b, b, 1.0 / scale, false, st);
      if (!done) hx_f32(op, x32, b, y32, b, b, 1.0 / scale, false, st);
      if (to_f64) copy_block<float, double>(y32, b, HXb, b, M, b, 1.0, st);
    } else {
      hx_f64(op, X + j0, ld, HXb, b, b, 1.0, false, st);
    }
  };
  CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(double) * N * N, st));
  for (int j0 = 0; j0 < N; j0 += blk) {
    const int b = std::min(blk, N - j0);
    const int nr = N - j0;
    hx_block(j0, b, !tcd);
    double* C = Hp + (int64_t)j0 * N + j0;
    if (tcd) {
      for (int64_t r0 = 0; r0 < M; r0 += ms) {
        const int64_t mr = std::min(ms, M - r0);
        tc_exponents<double>(X + r0 * ld + j0, ld, mr, nr, s->tx, st);
        tc_split_transposed<double>(X + r0 * ld + j0, ld, mr, nr, s->tx, st);
        if (hx32) {
          tc_exponents<float>(y32 + r0 * b, b, mr, b, s->th, st);
          tc_split_transposed<float>(y32 + r0 * b, b, mr, b, s->th, st);
        } else {
          tc_exponents<double>(HXb + r0 * b, b, mr, b, s->th, st);
          tc_split_transposed<double>(HXb + r0 * b, b, mr, b, s->th, st);
        }
        tc_gram(s->tx, &s->th, C, N, false, s->tcw, st);
      }
    } else {
      gram_f64(X + j0, ld, HXb, b, M, nr, b, C, N, prec, false, st);
    }
  }
  symmetrize_lower(Hp, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  gemm_f64('N', 'N', N, N, N, 1.0, S, N, Hp, N, 0.0, T1, N, CHEFSI_PREC_FP64, st);
  gemm_f64('N', 'T', N, N, N, 1.0, T1, N, S, N, 0.0, Hp, N, CHEFSI_PREC_FP64, st);
  symmetrize_lower(Hp, N, st);
  rc = syevd(Hp, N, w, Z, st);
  if (rc != CHEFSI_OK) return rc;
  gemm_f64('T', 'N', N, N, N, 1.0, S, N, Z, N, 0.0, W, N, CHEFSI_PREC_FP64, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  if (tcd) {
    for (int64_t r0 = 0; r0 < M; r0 += ms) {
      const int64_t mr = std::min(ms, M - r0);
      tc_exponents<double>(X + r0 * ld, ld, mr, N, s->tx, st);
      tc_split_rows<double>(X + r0 * ld, ld, mr, N, s->tx, st);
      tc_rotate(s->tx, W, N, N, X + r0 * ld, ld, s->tcw, st);
    }
  } else {
    rotate_rows(s, X, ld, M, N, W, prec, st);
  }
  rc = tc_dense_check_error(s->tcw, st);
  if (rc != CHEFSI_OK) {
    set_last_error("tensor-core Rayleigh-Ritz products: a bounded device wait expired");
    return rc;
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[5], st));
  if (res) {
    for (int j0 = 0; j0 < N; j0 += blk) {
      const int b = std::min(blk, N - j0);
      hx_block(j0, b, true);
      residual_norms_f64(X + j0, ld, HXb, b, M, b, w + j0, res + j0, st);
    }
  }
  if (hx32) {
    const int tc = tc_check_error(op, st);
    if (tc != CHEFSI_OK) {
      set_last_error("tensor-core HX: a bounded device wait expired");
      return tc;
    }
  }
  return CHEFSI_OK;
}

// Whether a real Rayleigh-Ritz step of N vectors takes the blocked form: forced by rr_block > 0,
// never with rr_block < 0, otherwise when the full-size workspaces it still has to allocate
// (about 30 bytes per dof and vector in the mixed mode, 8 in FP64) exceed 90% of the free
// device memory.
bool rr_blocked(chefsi_solver_s* s, chefsi_operator_s* op, int N, int prec) {
  if (s->p.rr_block > 0) return true;
  if (s->p.rr_block < 0) return false;
  size_t fr = 0, tot = 0;
  if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  const double mn = (double)op->n_dofs * N;
  const double need = (is_mixed(prec) ? 30.0 : 8.0) * mn;
  const double held = 8.0 * s->HX.n + 4.0 * (double)(s->Xb32.n + s->Yb32.n) +
                      2.0 * (double)(s->tx.hi.n + s->tx.lo.n + s->th.hi.n + s->th.lo.n);
  return need > held + 0.9 * (double)fr;
}

// Spectrum-split Rayleigh-Ritz (rayleighRitzGEPSpectrumSplitDirect,
// src/linAlg/rayleighRitzDevice.cc:822-1455) for a real operator:
//   S = X^T X = L L^T;  X <- X L^{-T} (Cholesky-GS, X stays in this orthonormal basis);
//   Hp = X^T H X;  the top n_fr = N - n_occ eigenpairs (Q_fr, eigenvalues ascending) only;
//   XFrac = X Q_fr ([M][n_fr], ldf);  with want_hxf, H XFrac = (H X) Q_fr into s->HXF.
// Precision map of X^T H X in the mixed mode (XtHXMixedPrecOverlapComputeCommun,
// src/dftOperator/kohnShamDFTOperatorDevice.cc:4553): the column blocks of wfc_block vectors
// that lie inside the first n_occ vectors use the reduced-precision H X (rr_precision), and
// the trailing square from the block that holds vector n_occ on, i.e. the block that couples
// the fractionally occupied states, is recomputed from an FP64 H X and an FP64 Gram product
// (unless ss_frac_reduced). rr_precision FP64 keeps every H X in FP64.
int rayleigh_ritz_ss_real(chefsi_solver_s* s, chefsi_operator_s* op, double* X, int64_t ld, int N,
                          int n_occ, double* XF, int64_t ldf, int prec, bool want_hxf,
                          cudaStream_t st) {
  const int64_t M = op->n_dofs;
  const int nfr = N - n_occ;
  const bool tcd = prec == CHEFSI_PREC_MIXED && dense_tc_available();
  double* S = s->S.ensure((size_t)N * N);
  double* Hp = s->Hp.ensure((size_t)N * N);
  double* T1 = s->T1.ensure((size_t)N * N);
  double* Z = s->Z.ensure((size_t)N * nfr);
  double* W = s->W.ensure((size_t)N * N);
  double* w = s->evals.ensure(N);
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  // S = X^T X, Cholesky, L^{-1}; X <- X L^{-T}
  CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
  if (tcd) {
    tc_exponents<double>(X, ld, M, N, s->tx, st);
    tc_split_transposed<double>(X, ld, M, N, s->tx, st);
    tc_gram(s->tx, nullptr, S, N, true, s->tcw, st);
  } else {
    gram_f64(X, ld, X, ld, M, N, N, S, N, prec, true, st);
  }
  symmetrize_lower(S, N, st);
  int rc = cholesky_overlap(S, X, ld, M, N, tcd, st);
  if (rc != CHEFSI_OK) return rc;
  trtri_lower(S, N, st);
  k_transpose<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(S, W, N);
  CHEFSI_CHECK_LAUNCH();
  rotate_rows(s, X, ld, M, N, W, prec, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  // H X of the orthonormal X (same precision choices as the full Rayleigh-Ritz step)
  double* HX = s->HX.ensure((size_t)M * N);
  const int rrp = s->p.rr_precision;
  const bool tc3 = is_mixed(prec) && rrp == CHEFSI_PREC_FP32_TC && tc_split_usable(op, N);
  const bool tc2 = is_mixed(prec) && rrp == CHEFSI_PREC_MIXED && tc_split_usable(op, N);
  const bool hx32 = is_mixed(prec) && (rrp == CHEFSI_PREC_FP32 || rrp == CHEFSI_PREC_FP32_TC || tc2);
  float* y32 = nullptr;
  if (hx32) {
    float* x32 = s->Xb32.ensure((size_t)M * N);
    y32 = s->Yb32.ensure((size_t)M * N);
    double scale = 1.0;
    if (tc2 || tc3) {
      double* sc = s->scal.ensure(1);
      absmax_block_f64(X, ld, M, N, sc, st);
      double amax = 0.0;
      CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
      CHEFSI_CUDA(cudaStreamSynchronize(st));
      if (amax > 0.0 && std::isfinite(amax))
        scale = std::ldexp(1.0, (tc3 ? 14 : 8) - (int)std::ceil(std::log2(amax)));
    }
    copy_block<double, float>(X, ld, x32, N, M, N, scale, st);
    bool done = false;
    if (tc3)
      done = hx_tc3(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    else if (tc2)
      done = hx_tc(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    if (!done) hx_f32(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    if (!tcd) copy_block<float, double>(y32, N, HX, N, M, N, 1.0, st);
  } else {
    hx_all_f64(op, X, ld, N, HX, s->p.wfc_block, st);
  }
  // Hp = X^T (H X), lower triangle
  CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(double) * N * N, st));
  if (tcd) {
    tc_exponents<double>(X, ld, M, N, s->tx, st);
    tc_split_transposed<double>(X, ld, M, N, s->tx, st);
    if (hx32) {
      tc_exponents<float>(y32, N, M, N, s->th, st);
      tc_split_transposed<float>(y32, N, M, N, s->th, st);
    } else {
      tc_exponents<double>(HX, N, M, N, s->th, st);
      tc_split_transposed<double>(HX, N, M, N, s->th, st);
    }
    tc_gram(s->tx, &s->th, Hp, N, true, s->tcw, st);
  } else {
    gram_f64(X, ld, HX, N, M, N, N, Hp, N, prec, true, st);
  }
  if (hx32 && !s->p.ss_frac_reduced) {
    // the trailing square from the wfc block holding vector n_occ on, in FP64
    const int blk = std::max(1, std::min(s->p.wfc_block > 0 ? s->p.wfc_block : N, N));
    const int n_lo = (n_occ / blk) * blk;
    const int nf = N - n_lo;
    double* HXf = s->HXf.ensure((size_t)M * nf);
    hx_all_f64(op, X + n_lo, ld, nf, HXf, s->p.wfc_block, st);
    CHEFSI_CUDA(cudaMemsetAsync(T1, 0, sizeof(double) * nf * nf, st));
    gram_f64(X + n_lo, ld, HXf, nf, M, nf, nf, T1, nf, CHEFSI_PREC_FP64, true, st);
    copy_block<double, double>(T1, nf, Hp + (int64_t)n_lo * N + n_lo, N, nf, nf, 1.0, st);
  }
  symmetrize_lower(Hp, N, st);
  // Mixed mode: the reduced-precision rotation leaves X^T X = I + O(2^-22 cond(L)), and a
  // filtered block has a large cond(L); the projected problem is then solved in the
  // generalised form with this well-conditioned Gram (S2 = L2 L2^T, C = L2^{-1} Hp L2^{-T},
  // Ritz coefficients L2^{-T} Q) instead of taking the basis as exactly orthonormal. One more
  // Gram product of the split already made for Hp; FP64 mode keeps the standard form.
  const bool reproject = is_mixed(prec);
  if (reproject) {
    CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
    if (tcd)
      tc_gram(s->tx, nullptr, S, N, true, s->tcw, st);
    else
      gram_f64(X, ld, X, ld, M, N, N, S, N, prec, true, st);
    symmetrize_lower(S, N, st);
    rc = cholesky_lower(S, N, st);
    if (rc != CHEFSI_OK) {
      set_last_error("Gram matrix of the orthonormalised basis is not positive definite");
      return rc;
    }
    trtri_lower(S, N, st);
    gemm_f64('N', 'N', N, N, N, 1.0, S, N, Hp, N, 0.0, T1, N, CHEFSI_PREC_FP64, st);
    gemm_f64('N', 'T', N, N, N, 1.0, T1, N, S, N, 0.0, Hp, N, CHEFSI_PREC_FP64, st);
    symmetrize_lower(Hp, N, st);
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  // the top n_fr eigenpairs of the standard problem (eigenpairs_hermitian_by_index (Noc, N-1))
  rc = syevd_range(Hp, N, n_occ, nfr, w, Z, st);
  if (rc != CHEFSI_OK) return rc;
  const double* R = Z;   // Ritz coefficients [N][n_fr]
  if (reproject) {
    gemm_f64('T', 'N', N, nfr, N, 1.0, S, N, Z, nfr, 0.0, W, nfr, CHEFSI_PREC_FP64, st);
    R = W;
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  // XFrac = X Q_fr (subspaceRotationSpectrumSplitScalapack); H XFrac = (H X) Q_fr
  double* HXF = want_hxf ? s->HXF.ensure((size_t)M * nfr) : nullptr;
  if (tcd) {
    tc_split_rows<double>(X, ld, M, N, s->tx, st);
    tc_rotate(s->tx, R, nfr, nfr, XF, ldf, s->tcw, st);
    if (want_hxf) {
      if (hx32)
        tc_split_rows<float>(y32, N, M, N, s->th, st);
      else
        tc_split_rows<double>(HX, N, M, N, s->th, st);
      tc_rotate(s->th, R, nfr, nfr, HXF, nfr, s->tcw, st);
    }
    rc = tc_dense_check_error(s->tcw, st);
    if (rc != CHEFSI_OK) {
      set_last_error("tensor-core spectrum-split rotation: a bounded device wait expired");
      return rc;
    }
  } else {
    gemm_f64('N', 'N', M, nfr, N, 1.0, X, ld, R, nfr, 0.0, XF, ldf, prec, st);
    if (want_hxf) gemm_f64('N', 'N', M, nfr, N, 1.0, HX, N, R, nfr, 0.0, HXF, nfr, prec, st);
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[5], st));
  return CHEFSI_OK;
}

// ---------------------------------------------------------------- density-matrix response
// First-order response of the density matrix in the eigenbasis
// (densityMatrixEigenBasisFirstOrderResponse, src/linAlg/rayleighRitzDevice.cc:1455-1721).
// The recursive Fermi-operator expansion X_{k+1} = Y_k X_k^2, Y_k = (2 X_k (X_k - 1) + 1)^{-1},
// from X_0 = 1/2 - c (H - mu), c = 2^{-2-m} beta, is diagonal in the eigenbasis; its first-order
// part P (from P_0 = -c H') obeys, entry by entry, with i the row and j the column,
//   T = P X0_i + P X0_j;  P <- (Y0_i T - 2 (T X0'_j) Y0_i) + 2 (P X0'_j) Y0_i
// (X0' the updated diagonal): the reference's sequence of row / column scalings of dense
// matrices, which here is one pass over the entries of the lower triangle (row >= column)
// with the diagonal sequences precomputed; the upper triangle is its mirror.
constexpr int kDmforSteps = 10;

// X0[k][i] (k = 0..m), Y0[k][i] (k = 0..m-1); dmu[i] = beta X0_m (1 - X0_m). Every operation
// is an explicitly rounded one (no FMA contraction), in the reference's order: near the
// occupied end 1 - X0 is a difference of nearly equal numbers and carries the rounding of
// every step into densityMatDerFermiEnergy.
__global__ void k_dmfor_diag(const double* __restrict__ eig, int N, double mu, double beta,
                             double c, double* __restrict__ X0, double* __restrict__ Y0,
                             double* __restrict__ dmu) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  double x = __dsub_rn(0.5, __dmul_rn(c, __dsub_rn(eig[i], mu)));
  X0[i] = x;
  for (int k = 0; k < kDmforSteps; ++k) {
    const double y =
        __ddiv_rn(1.0, __dadd_rn(__dmul_rn(__dmul_rn(2.0, x), __dsub_rn(x, 1.0)), 1.0));
    x = __dmul_rn(__dmul_rn(y, x), x);
    Y0[(int64_t)k * N + i] = y;
    X0[(int64_t)(k + 1) * N + i] = x;
  }
  dmu[i] = __dmul_rn(__dmul_rn(beta, x), __dsub_rn(1.0, x));
}

// The recursion of entry (row i, column j) on one real component (the factors are real, so a
// complex entry runs it on its real and imaginary parts separately)
__device__ __forceinline__ double dmfor_entry(double h, int i, int j, int N, double c,
                                              const double* __restrict__ X0,
                                              const double* __restrict__ Y0) {
  double p = __dmul_rn(-c, h);
  for (int k = 0; k < kDmforSteps; ++k) {
    const double xi = X0[(int64_t)k * N + i], xj = X0[(int64_t)k * N + j];
    const double y = Y0[(int64_t)k * N + i];
    const double xn = X0[(int64_t)(k + 1) * N + j];
    const double T = __dadd_rn(__dmul_rn(p, xi), __dmul_rn(p, xj));
    const double a = __dsub_rn(__dmul_rn(T, y), __dmul_rn(2.0, __dmul_rn(__dmul_rn(T, xn), y)));
    p = __dadd_rn(a, __dmul_rn(2.0, __dmul_rn(__dmul_rn(p, xn), y)));
  }
  return p;
}

// P[i][j] <- first-order density-matrix response from Hp[i][j] (full symmetric input;
// the entry of row max(i, j), column min(i, j) is computed and written to both places)
__global__ void k_dmfor_apply(double* __restrict__ P, int N, double c,
                              const double* __restrict__ X0, const double* __restrict__ Y0) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / N), j = (int)(t % N);
    if (j > i) continue;  // row i >= column j
    const double p = dmfor_entry(P[t], i, j, N, c, X0, Y0);
    P[t] = p;
    P[(int64_t)j * N + i] = p;
  }
}

// complex Hermitian P: the lower entry from the recursion, the upper one its conjugate
__global__ void k_dmfor_apply_c(cplx* __restrict__ P, int N, double c,
                                const double* __restrict__ X0, const double* __restrict__ Y0) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / N), j = (int)(t % N);
    if (j > i) continue;
    const cplx h = P[t];
    const double re = dmfor_entry(h.x, i, j, N, c, X0, Y0);
    const double im = i == j ? 0.0 : dmfor_entry(h.y, i, j, N, c, X0, Y0);
    P[t] = {re, im};
    P[(int64_t)j * N + i] = {re, -im};
  }
}

// Hp' = X^T H' X (lower triangle mirrored), P' by the recursion, X <- X P'. dmu (device, N)
// receives densityMatDerFermiEnergy. Mixed: the three-term tensor-core H X, tensor-core Gram
// and rotation (the reference's singlePrecLRD path runs every block of X^T H' X in FP32).
int dm_first_order_response_real(chefsi_solver_s* s, chefsi_operator_s* op, double* X, int64_t ld,
                                 int N, const double* eig, double mu, double beta, double* dmu,
                                 int prec, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  const bool tcd = prec == CHEFSI_PREC_MIXED && dense_tc_available();
  double* Hp = s->Hp.ensure((size_t)N * N);
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  const bool tc3 = is_mixed(prec) && tc_split_usable(op, N);
  float* y32 = nullptr;
  double* HX = nullptr;
  if (is_mixed(prec)) {
    float* x32 = s->Xb32.ensure((size_t)M * N);
    y32 = s->Yb32.ensure((size_t)M * N);
    double scale = 1.0;
    if (tc3) {
      double* sc = s->scal.ensure(1);
      absmax_block_f64(X, ld, M, N, sc, st);
      double amax = 0.0;
      CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
      CHEFSI_CUDA(cudaStreamSynchronize(st));
      if (amax > 0.0 && std::isfinite(amax))
        scale = std::ldexp(1.0, 14 - (int)std::ceil(std::log2(amax)));
    }
    copy_block<double, float>(X, ld, x32, N, M, N, scale, st);
    if (!(tc3 && hx_tc3(op, x32, N, y32, N, N, 1.0 / scale, false, st)))
      hx_f32(op, x32, N, y32, N, N, 1.0 / scale, false, st);
    const int tc = tc_check_error(op, st);
    if (tc != CHEFSI_OK) throw Error(tc, "tensor-core HX: a bounded device wait expired");
    if (!tcd) {
      HX = s->HX.ensure((size_t)M * N);
      copy_block<float, double>(y32, N, HX, N, M, N, 1.0, st);
    }
  } else {
    HX = s->HX.ensure((size_t)M * N);
    hx_all_f64(op, X, ld, N, HX, s->p.wfc_block, st);
  }
  CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(double) * N * N, st));
  if (tcd) {
    tc_exponents<double>(X, ld, M, N, s->tx, st);
    tc_split_transposed<double>(X, ld, M, N, s->tx, st);
    tc_exponents<float>(y32, N, M, N, s->th, st);
    tc_split_transposed<float>(y32, N, M, N, s->th, st);
    tc_gram(s->tx, &s->th, Hp, N, true, s->tcw, st);
    const int rc = tc_dense_check_error(s->tcw, st);
    if (rc != CHEFSI_OK) {
      set_last_error("tensor-core Gram product: a bounded device wait expired");
      return rc;
    }
  } else {
    gram_f64(X, ld, HX, N, M, N, N, Hp, N, prec, true, st);
  }
  symmetrize_lower(Hp, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  const double c = std::ldexp(1.0, -2 - kDmforSteps) * beta;
  double* X0 = s->T1.ensure((size_t)(2 * kDmforSteps + 1) * N);
  double* Y0 = X0 + (size_t)(kDmforSteps + 1) * N;
  k_dmfor_diag<<<(N + 127) / 128, 128, 0, st>>>(eig, N, mu, beta, c, X0, Y0, dmu);
  CHEFSI_CHECK_LAUNCH();
  k_dmfor_apply<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(Hp, N, c, X0, Y0);
  CHEFSI_CHECK_LAUNCH();
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  // Y = X P' (P' symmetric: the reference rotates by its conjugate transpose)
  rotate_rows(s, X, ld, M, N, Hp, prec, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  return CHEFSI_OK;
}

// X[M][N] <- X W for complex blocks (row blocks through a temporary)
void rotate_rows_c(chefsi_solver_s* s, cplx* X, int64_t ld, int64_t M, int N, const cplx* W,
                   cudaStream_t st) {
  const int64_t rows = std::min<int64_t>(M, std::max<int64_t>(2048, (int64_t)(256ll << 20) / (16ll * N)));
  cplx* tmp = reinterpret_cast<cplx*>(s->rot.ensure((size_t)rows * N * 2));
  const cplx one = {1.0, 0.0}, zero = {0.0, 0.0};
  for (int64_t r0 = 0; r0 < M; r0 += rows) {
    const int64_t nr = std::min(rows, M - r0);
    gemm_c64('N', 'N', nr, N, N, one, X + r0 * ld, ld, W, N, zero, tmp, N, st);
    copy_block<cplx, cplx>(tmp, N, X + r0 * ld, ld, nr, N, 1.0, st);
  }
}

// The complex products of the mixed step run on the real tensor-core kernels through the
// real view of an interleaved complex block, Y = [Re x_0, Im x_0, Re x_1, ...] ([M][2N]):
// G = Y_a^T Y_b gives C = A^H B as C_ij = (G[2i][2j] + G[2i+1][2j+1]) + i (G[2i][2j+1] -
// G[2i+1][2j]), and X W is Y W_r with the 2N x 2N real matrix
// W_r = [[Re W, Im W], [-Im W, Re W]] interleaved the same way.
__global__ void k_gram_to_complex(const double* G, int N, cplx* C, int lower) {
  const int64_t n = (int64_t)N * N;
  const int64_t ld = 2 * (int64_t)N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / N), j = (int)(t % N);
    if (lower && j > i) continue;
    const double* r0 = G + (2 * i) * ld;
    const double* r1 = r0 + ld;
    C[t] = {r0[2 * j] + r1[2 * j + 1], r0[2 * j + 1] - r1[2 * j]};
  }
}
__global__ void k_realify_w(const cplx* W, int N, double* Wr) {
  const int64_t n = (int64_t)N * N;
  const int64_t ld = 2 * (int64_t)N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / N), m = (int)(t % N);
    const cplx w = W[t];
    Wr[(2 * k) * ld + 2 * m] = w.x;
    Wr[(2 * k) * ld + 2 * m + 1] = w.y;
    Wr[(2 * k + 1) * ld + 2 * m] = -w.y;
    Wr[(2 * k + 1) * ld + 2 * m + 1] = w.x;
  }
}

// H X ([M][N], ld N) of a complex block for the Rayleigh-Ritz products: FP64 complex, or (mixed
// with rr_precision FP32 / FP32_TC on a folded operator) the FP32 SIMT / three-term tensor-core
// apply of the real form on X rounded to FP32. Returns true when the reduced apply ran.
bool hx_complex_block(chefsi_solver_s* s, chefsi_operator_s* op, const cplx* X, int64_t ld, int N,
                      int prec, cplx* HX, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  const int rrp = s->p.rr_precision;
  if (is_mixed(prec) && (rrp == CHEFSI_PREC_FP32 || rrp == CHEFSI_PREC_FP32_TC) && op->folded) {
    chefsi_operator_s* rv = realified(op, st);
    float* xr = s->Xb32.ensure((size_t)2 * M * N);
    float* yr = s->Yb32.ensure((size_t)2 * M * N);
    const bool tc3 = rrp == CHEFSI_PREC_FP32_TC && tc_split_usable(rv, N);
    double scale = 1.0;
    if (tc3) {
      double* sc = s->scal.ensure(1);
      absmax_block_f64(reinterpret_cast<const double*>(X), 2 * ld, M, 2 * N, sc, st);
      double amax = 0.0;
      CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc, sizeof(double), cudaMemcpyDeviceToHost, st));
      CHEFSI_CUDA(cudaStreamSynchronize(st));
      if (amax > 0.0 && std::isfinite(amax))
        scale = std::ldexp(1.0, 14 - (int)std::ceil(std::log2(amax)));
    }
    complex_to_real_rows(X, ld, M, N, scale, xr, st);
    if (!(tc3 && hx_tc3(rv, xr, N, yr, N, N, 1.0 / scale, false, st)))
      hx_f32(rv, xr, N, yr, N, N, 1.0 / scale, false, st);
    real_rows_to_complex(yr, M, N, 1.0, HX, N, st);
    return true;
  }
  const int Bmax = std::max(1, std::min(s->p.wfc_block > 0 ? s->p.wfc_block : N, N));
  for (int j0 = 0; j0 < N; j0 += Bmax) {
    const int B = std::min(Bmax, N - j0);
    hx_c64(op, X + j0, ld, HX + j0, N, B, 1.0, false, st);
  }
  return false;
}

// Rayleigh-Ritz for a complex (Bloch) operator: the generalised form with Hermitian S and Hp.
int rayleigh_ritz_complex(chefsi_solver_s* s, chefsi_operator_s* op, cplx* X, int64_t ld, int N,
                          int prec, bool want_hx, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  const bool tcd = prec == CHEFSI_PREC_MIXED && dense_tc_available();
  cplx* S = reinterpret_cast<cplx*>(s->S.ensure((size_t)N * N * 2));
  cplx* Hp = reinterpret_cast<cplx*>(s->Hp.ensure((size_t)N * N * 2));
  cplx* T1 = reinterpret_cast<cplx*>(s->T1.ensure((size_t)N * N * 2));
  cplx* Z = reinterpret_cast<cplx*>(s->Z.ensure((size_t)N * N * 2));
  cplx* W = reinterpret_cast<cplx*>(s->W.ensure((size_t)N * N * 2));
  double* w = s->evals.ensure(N);
  double* Xv = reinterpret_cast<double*>(X);
  const int N2 = 2 * N;
  double* G = tcd ? s->G2.ensure((size_t)N2 * N2) : nullptr;
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  if (tcd) {
    tc_exponents<double>(Xv, 2 * ld, M, N2, s->tx, st);
    tc_split_transposed<double>(Xv, 2 * ld, M, N2, s->tx, st);
    CHEFSI_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * N2 * N2, st));
    tc_gram(s->tx, nullptr, G, N2, true, s->tcw, st);
    symmetrize_lower(G, N2, st);
    k_gram_to_complex<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(G, N, S, 1);
    CHEFSI_CHECK_LAUNCH();
  } else {
    CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(cplx) * N * N, st));
    gram_c64(X, ld, X, ld, M, N, N, S, N, true, st);
  }
  symmetrize_lower_c(S, N, st);
  if (fault_injected("not_spd")) {
    k_negate_diag0<<<1, 1, 0, st>>>(reinterpret_cast<double*>(S));
    CHEFSI_CHECK_LAUNCH();
  }
  int rc = cholesky_lower_c(S, N, st);
  if (rc != CHEFSI_OK) {
    set_last_error("overlap matrix is not positive definite (Cholesky pivot <= 0)");
    return rc;
  }
  trtri_lower_c(S, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  cplx* HX = reinterpret_cast<cplx*>(s->HX.ensure((size_t)M * N * 2));
  hx_complex_block(s, op, X, ld, N, prec, HX, st);
  double* HXv = reinterpret_cast<double*>(HX);
  if (tcd) {
    tc_exponents<double>(HXv, N2, M, N2, s->th, st);
    tc_split_transposed<double>(HXv, N2, M, N2, s->th, st);
    CHEFSI_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * N2 * N2, st));
    tc_gram(s->tx, &s->th, G, N2, true, s->tcw, st);
    k_gram_to_complex<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(G, N, Hp, 1);
    CHEFSI_CHECK_LAUNCH();
  } else {
    CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(cplx) * N * N, st));
    gram_c64(X, ld, HX, N, M, N, N, Hp, N, true, st);
  }
  symmetrize_lower_c(Hp, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  const cplx one = {1.0, 0.0}, zero = {0.0, 0.0};
  // C = L^{-1} Hp L^{-H}
  gemm_c64('N', 'N', N, N, N, one, S, N, Hp, N, zero, T1, N, st);
  gemm_c64('N', 'C', N, N, N, one, T1, N, S, N, zero, Hp, N, st);
  symmetrize_lower_c(Hp, N, st);
  rc = heevd(Hp, N, w, Z, st);
  if (rc != CHEFSI_OK) return rc;
  // W = L^{-H} Q
  gemm_c64('C', 'N', N, N, N, one, S, N, Z, N, zero, W, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  if (tcd) {
    double* Wr = s->W2.ensure((size_t)N2 * N2);
    k_realify_w<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(W, N, Wr);
    CHEFSI_CHECK_LAUNCH();
    tc_split_rows<double>(Xv, 2 * ld, M, N2, s->tx, st);
    tc_rotate(s->tx, Wr, N2, N2, Xv, 2 * ld, s->tcw, st);
    if (want_hx) {
      tc_split_rows<double>(HXv, N2, M, N2, s->th, st);
      tc_rotate(s->th, Wr, N2, N2, HXv, N2, s->tcw, st);
    }
    rc = tc_dense_check_error(s->tcw, st);
    if (rc != CHEFSI_OK) {
      set_last_error("tensor-core Rayleigh-Ritz products: a bounded device wait expired");
      return rc;
    }
  } else {
    rotate_rows_c(s, X, ld, M, N, W, st);
    if (want_hx) rotate_rows_c(s, HX, N, M, N, W, st);
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[5], st));
  return CHEFSI_OK;
}

// Spectrum-split Rayleigh-Ritz for a complex (Bloch) operator: the steps of
// rayleigh_ritz_ss_real with Hermitian products (S = X^H X = L L^H, X <- X L^{-H}, Hp = X^H H X,
// XFrac = X Q_fr). The dense products are FP64 complex GEMMs in every mode (the Bloch blocks
// are small); the mixed mode changes the H X (the real form's reduced apply, as the full
// step) and, unless ss_frac_reduced, recomputes the fractional block from an FP64 H X.
int rayleigh_ritz_ss_complex(chefsi_solver_s* s, chefsi_operator_s* op, cplx* X, int64_t ld,
                             int N, int n_occ, cplx* XF, int64_t ldf, int prec, bool want_hxf,
                             cudaStream_t st) {
  const int64_t M = op->n_dofs;
  const int nfr = N - n_occ;
  cplx* S = reinterpret_cast<cplx*>(s->S.ensure((size_t)N * N * 2));
  cplx* Hp = reinterpret_cast<cplx*>(s->Hp.ensure((size_t)N * N * 2));
  cplx* T1 = reinterpret_cast<cplx*>(s->T1.ensure((size_t)N * N * 2));
  cplx* Z = reinterpret_cast<cplx*>(s->Z.ensure((size_t)N * nfr * 2));
  cplx* W = reinterpret_cast<cplx*>(s->W.ensure((size_t)N * N * 2));
  double* w = s->evals.ensure(N);
  const cplx one = {1.0, 0.0}, zero = {0.0, 0.0};
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(cplx) * N * N, st));
  gram_c64(X, ld, X, ld, M, N, N, S, N, true, st);
  symmetrize_lower_c(S, N, st);
  int rc = cholesky_lower_c(S, N, st);
  if (rc != CHEFSI_OK) {
    set_last_error("overlap matrix is not positive definite (Cholesky pivot <= 0)");
    return rc;
  }
  trtri_lower_c(S, N, st);
  k_conj_transpose<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(S, W, N);
  CHEFSI_CHECK_LAUNCH();
  rotate_rows_c(s, X, ld, M, N, W, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  cplx* HX = reinterpret_cast<cplx*>(s->HX.ensure((size_t)M * N * 2));
  const bool reduced = hx_complex_block(s, op, X, ld, N, prec, HX, st);
  CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(cplx) * N * N, st));
  gram_c64(X, ld, HX, N, M, N, N, Hp, N, true, st);
  if (reduced && !s->p.ss_frac_reduced) {
    const int blk = std::max(1, std::min(s->p.wfc_block > 0 ? s->p.wfc_block : N, N));
    const int n_lo = (n_occ / blk) * blk;
    const int nf = N - n_lo;
    cplx* HXf = reinterpret_cast<cplx*>(s->HXf.ensure((size_t)M * nf * 2));
    for (int j0 = 0; j0 < nf; j0 += blk) {
      const int B = std::min(blk, nf - j0);
      hx_c64(op, X + n_lo + j0, ld, HXf + j0, nf, B, 1.0, false, st);
    }
    CHEFSI_CUDA(cudaMemsetAsync(T1, 0, sizeof(cplx) * nf * nf, st));
    gram_c64(X + n_lo, ld, HXf, nf, M, nf, nf, T1, nf, true, st);
    copy_block<cplx, cplx>(T1, nf, Hp + (int64_t)n_lo * N + n_lo, N, nf, nf, 1.0, st);
  }
  symmetrize_lower_c(Hp, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  rc = heevd_range(Hp, N, n_occ, nfr, w, Z, st);
  if (rc != CHEFSI_OK) return rc;
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  gemm_c64('N', 'N', M, nfr, N, one, X, ld, Z, nfr, zero, XF, ldf, st);
  if (want_hxf) {
    cplx* HXF = reinterpret_cast<cplx*>(s->HXF.ensure((size_t)M * nfr * 2));
    gemm_c64('N', 'N', M, nfr, N, one, HX, N, Z, nfr, zero, HXF, nfr, st);
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[5], st));
  return CHEFSI_OK;
}

// First-order density-matrix response for a complex operator: Hp' = X^H H' X (FP64 complex
// Gram), the recursion on the real and imaginary parts of the lower triangle, the upper
// triangle its conjugate, X <- X P'.
int dm_first_order_response_complex(chefsi_solver_s* s, chefsi_operator_s* op, cplx* X,
                                    int64_t ld, int N, const double* eig, double mu, double beta,
                                    double* dmu, int prec, cudaStream_t st) {
  const int64_t M = op->n_dofs;
  cplx* Hp = reinterpret_cast<cplx*>(s->Hp.ensure((size_t)N * N * 2));
  CHEFSI_CUDA(cudaEventRecord(s->ev[1], st));
  cplx* HX = reinterpret_cast<cplx*>(s->HX.ensure((size_t)M * N * 2));
  hx_complex_block(s, op, X, ld, N, prec, HX, st);
  CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(cplx) * N * N, st));
  gram_c64(X, ld, HX, N, M, N, N, Hp, N, true, st);
  symmetrize_lower_c(Hp, N, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[2], st));
  const double c = std::ldexp(1.0, -2 - kDmforSteps) * beta;
  double* X0 = s->T1.ensure((size_t)(2 * kDmforSteps + 1) * N);
  double* Y0 = X0 + (size_t)(kDmforSteps + 1) * N;
  k_dmfor_diag<<<(N + 127) / 128, 128, 0, st>>>(eig, N, mu, beta, c, X0, Y0, dmu);
  CHEFSI_CHECK_LAUNCH();
  k_dmfor_apply_c<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(Hp, N, c, X0, Y0);
  CHEFSI_CHECK_LAUNCH();
  CHEFSI_CUDA(cudaEventRecord(s->ev[3], st));
  rotate_rows_c(s, X, ld, M, N, Hp, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[4], st));
  return CHEFSI_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) {
    cudaGetLastError();
    return 0.f;
  }
  return ms;
}

chefsi_params default_params() {
  chefsi_params p{};
  p.chebyshev_degree = 0;
  p.cheby_wfc_block = 400;
  p.wfc_block = 400;
  p.precision = CHEFSI_PREC_FP64;
  p.lanczos_steps = 20;
  p.reproducible = 0;
  p.first_scf_degree_scale = 1.34;
  p.keep_hx = 1;
  p.rr_precision = CHEFSI_PREC_FP64;
  p.ss_frac_reduced = 0;
  p.rr_block = 0;
  p.rr_slab_rows = 0;
  p.filter_variant = 0;
  return p;
}

}  // namespace

extern "C" {

const char* chefsi_last_error(void) { return chefsi::last_error_cstr(); }
const char* chefsi_version(void) { return "chefsi-gb300 0.1 (sm_103a)"; }

uint64_t chefsi_launch_count(void) { return (uint64_t)chefsi::launch_count(); }

int32_t chefsi_chebyshev_order(double upper) {
  const unsigned ub = upper > 0 ? (unsigned)upper : 0u;
  for (const auto& e : kOrderLookup)
    if (ub <= (unsigned)e[0]) return e[1];
  return 1250;
}

int chefsi_operator_create(const chefsi_operator_desc* desc, chefsi_operator* out) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(out != nullptr, "null output handle");
  *out = nullptr;
  *out = create_operator(desc);
  CHEFSI_API_END
}

int chefsi_operator_destroy(chefsi_operator op) {
  CHEFSI_API_BEGIN
  delete op;
  CHEFSI_API_END
}

int chefsi_operator_info(chefsi_operator op, int64_t* n_dofs, int32_t* n_cells,
                         int32_t* nodes_per_cell, int32_t* is_complex) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op != nullptr, "null operator");
  if (n_dofs) *n_dofs = op->n_dofs;
  if (n_cells) *n_cells = op->n_cells;
  if (nodes_per_cell) *nodes_per_cell = op->n_e;
  if (is_complex) *is_complex = op->is_complex;
  CHEFSI_API_END
}

int chefsi_hx(chefsi_operator op, const void* src, int64_t ld_src, void* dst, int64_t ld_dst,
              int32_t n_vec, double scalar, int32_t accumulate, int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && src && dst, "null argument");
  CHEFSI_REQUIRE(n_vec >= 1 && ld_src >= n_vec && ld_dst >= n_vec, "bad block shape");
  cudaStream_t st = as_stream(stream);
  if (op->is_complex) {
    CHEFSI_REQUIRE(precision == CHEFSI_PREC_FP64, "complex operators run in FP64");
    hx_c64(op, (const cplx*)src, ld_src, (cplx*)dst, ld_dst, n_vec, scalar, accumulate != 0, st);
  } else if (precision == CHEFSI_PREC_FP64) {
    hx_f64(op, (const double*)src, ld_src, (double*)dst, ld_dst, n_vec, scalar, accumulate != 0, st);
  } else if (precision == CHEFSI_PREC_MIXED) {
    // tensor cores need a real, unconstrained operator and 16-byte aligned rows; otherwise the
    // SIMT FP32 apply serves the call
    if (!hx_tc(op, (const float*)src, ld_src, (float*)dst, ld_dst, n_vec, scalar, accumulate != 0, st)) {
      if (constrained_tc_usable(op, n_vec) && ld_src % 2 == 0 && ld_dst % 4 == 0 &&
          (reinterpret_cast<uintptr_t>(dst) & 15) == 0)
        hx_tc_constrained(op, (const float*)src, ld_src, (float*)dst, ld_dst, n_vec, scalar,
                          accumulate != 0, st);
      else
        hx_f32(op, (const float*)src, ld_src, (float*)dst, ld_dst, n_vec, scalar, accumulate != 0, st);
    }
    const int tc = tc_check_error(op, st);
    if (tc != CHEFSI_OK) throw Error(tc, "tensor-core HX: a bounded device wait expired");
  } else if (precision == CHEFSI_PREC_FP32) {
    hx_f32(op, (const float*)src, ld_src, (float*)dst, ld_dst, n_vec, scalar, accumulate != 0, st);
  } else if (precision == CHEFSI_PREC_FP32_TC) {
    // the three-term split wants max |src| < 2^15: a power-of-two scaled copy of src (undone
    // through the scalar); the SIMT FP32 apply where the tensor path does not apply
    const float* x = static_cast<const float*>(src);
    bool done = false;
    if (tc_split_usable(op, n_vec) && ld_dst % 4 == 0 &&
        (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
      DeviceBuffer<double> sc(1);
      absmax_block_f32(x, ld_src, op->n_dofs, n_vec, sc.ptr, st);
      double amax = 0.0;
      CHEFSI_CUDA(cudaMemcpyAsync(&amax, sc.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
      CHEFSI_CUDA(cudaStreamSynchronize(st));
      const double scale = (amax > 0.0 && std::isfinite(amax))
                               ? std::ldexp(1.0, 14 - (int)std::ceil(std::log2(amax)))
                               : 1.0;
      const int64_t ldx = (n_vec + 3) / 4 * 4;
      float* xs = op->ws32x.ensure((size_t)op->n_dofs * ldx);
      copy_block<float, float>(x, ld_src, xs, ldx, op->n_dofs, n_vec, scale, st);
      done = hx_tc3(op, xs, ldx, (float*)dst, ld_dst, n_vec, scalar / scale, accumulate != 0, st);
    }
    if (!done)
      hx_f32(op, x, ld_src, (float*)dst, ld_dst, n_vec, scalar, accumulate != 0, st);
    const int tc = tc_check_error(op, st);
    if (tc != CHEFSI_OK) throw Error(tc, "tensor-core HX: a bounded device wait expired");
  } else {
    throw Error(CHEFSI_ERR_INVALID, "unknown precision");
  }
  CHEFSI_API_END
}

int chefsi_overlap(chefsi_operator op, const void* X, int64_t ld, int32_t N, double* S,
                   int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && S && N >= 1 && ld >= N, "bad argument");
  cudaStream_t st = as_stream(stream);
  if (op->is_complex) {
    CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * 2 * N * N, st));
    gram_c64((const cplx*)X, ld, (const cplx*)X, ld, op->n_dofs, N, N, (cplx*)S, N, true, st);
    symmetrize_lower_c((cplx*)S, N, st);
  } else {
    CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
    gram_f64((const double*)X, ld, (const double*)X, ld, op->n_dofs, N, N, S, N, precision, true, st);
    symmetrize_lower(S, N, st);
  }
  CHEFSI_API_END
}

int chefsi_xthx(chefsi_operator op, const void* X, int64_t ld, int32_t N, double* Hp,
                int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && Hp && N >= 1 && ld >= N, "bad argument");
  cudaStream_t st = as_stream(stream);
  const int64_t M = op->n_dofs;
  if (op->is_complex) {
    DeviceBuffer<double> HX((size_t)M * N * 2);
    hx_c64(op, (const cplx*)X, ld, (cplx*)HX.ptr, N, N, 1.0, false, st);
    CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(double) * 2 * N * N, st));
    gram_c64((const cplx*)X, ld, (const cplx*)HX.ptr, N, M, N, N, (cplx*)Hp, N, true, st);
    symmetrize_lower_c((cplx*)Hp, N, st);
    CHEFSI_CUDA(cudaStreamSynchronize(st));
  } else {
    DeviceBuffer<double> HX((size_t)M * N);
    hx_all_f64(op, (const double*)X, ld, N, HX.ptr, 400, st);
    CHEFSI_CUDA(cudaMemsetAsync(Hp, 0, sizeof(double) * N * N, st));
    gram_f64((const double*)X, ld, HX.ptr, N, M, N, N, Hp, N, precision, true, st);
    symmetrize_lower(Hp, N, st);
    CHEFSI_CUDA(cudaStreamSynchronize(st));
  }
  CHEFSI_API_END
}

int chefsi_chebyshev_filter(chefsi_operator op, void* X, int64_t ld, int32_t n_vec, int32_t m,
                            double a, double b, double a0, int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && n_vec >= 1 && ld >= n_vec && m >= 1, "bad argument");
  CHEFSI_REQUIRE(b > a, "need b > a");
  cudaStream_t st = as_stream(stream);
  chefsi_solver_s tmp;
  tmp.p = default_params();
  tmp.p.cheby_wfc_block = n_vec;
  tmp.a0 = a0;
  tmp.b_low = a;
  tmp.b_up = b;
  if (op->is_complex) {
    CHEFSI_REQUIRE(ld == n_vec, "complex filter needs ld == n_vec");
    filter_all(&tmp, op, X, n_vec, m, CHEFSI_PREC_FP64, st);
  } else {
    filter_columns(&tmp, op, (double*)X, ld, 0, n_vec, m, a, b, a0, precision, st);
  }
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_syevd(int32_t N, double* A, double* w, double* Z, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(A && w && Z && N >= 1, "bad argument");
  int rc = syevd(A, N, w, Z, as_stream(stream));
  if (rc != CHEFSI_OK) return rc;
  CHEFSI_API_END
}

int chefsi_heevd(int32_t N, double* A, double* w, double* Z, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(A && w && Z && N >= 1, "bad argument");
  int rc = heevd(reinterpret_cast<cplx*>(A), N, w, reinterpret_cast<cplx*>(Z), as_stream(stream));
  if (rc != CHEFSI_OK) return rc;
  CHEFSI_API_END
}

int chefsi_lanczos_bounds(chefsi_operator op, int32_t k, int32_t reproducible, const double* v0_host,
                          uint64_t seed, double* lower, double* upper, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && lower && upper && k >= 2, "bad argument");
  cudaStream_t st = as_stream(stream);
  const int64_t M = op->n_dofs;
  // complex operators: the vectors are interleaved complex, handled as real vectors of
  // length 2M for the inner products (Re x^H y = real-view dot), which is the reference's
  // alpha = f^H v up to rounding for a Hermitian operator
  const int64_t L = op->is_complex ? 2 * M : M;
  std::vector<double> h(M);
  if (v0_host) {
    std::memcpy(h.data(), v0_host, sizeof(double) * M);
  } else {
    std::mt19937_64 gen(seed);
    std::uniform_real_distribution<double> U(0.0, 1.0);
    for (auto& x : h) x = U(gen);
  }
  std::vector<double> hv(L, 0.0);
  for (int64_t i = 0; i < M; ++i) hv[op->is_complex ? 2 * i : i] = h[i];
  DeviceBuffer<double> v(L), v0(L), f(L), sc(1);
  CHEFSI_CUDA(cudaMemcpyAsync(v.ptr, hv.data(), sizeof(double) * L, cudaMemcpyHostToDevice, st));
  auto dot = [&](const double* x, const double* y) {
    double r = 0.0;
    dot_f64(x, y, L, sc.ptr, st);
    CHEFSI_CUDA(cudaMemcpyAsync(&r, sc.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
    CHEFSI_CUDA(cudaStreamSynchronize(st));
    return r;
  };
  auto apply = [&](const double* x, double* y) {
    if (op->is_complex)
      hx_c64(op, reinterpret_cast<const cplx*>(x), 1, reinterpret_cast<cplx*>(y), 1, 1, 1.0,
             false, st);
    else
      hx_f64(op, x, 1, y, 1, 1, 1.0, false, st);
  };
  const double n0 = std::sqrt(dot(v.ptr, v.ptr));
  CHEFSI_REQUIRE(n0 > 0.0, "Lanczos start vector is zero");
  scale_block<double>(v.ptr, 1, L, 1, 1.0 / n0, st);
  apply(v.ptr, f.ptr);
  double alpha = dot(f.ptr, v.ptr);
  axpby_block<double>(v.ptr, 1, f.ptr, 1, L, 1, -alpha, 1.0, st);
  std::vector<double> T((size_t)k * k, 0.0);
  T[0] = alpha;
  for (int j = 1; j < k; ++j) {
    const double beta = std::sqrt(dot(f.ptr, f.ptr));
    CHEFSI_CUDA(cudaMemcpyAsync(v0.ptr, v.ptr, sizeof(double) * L, cudaMemcpyDeviceToDevice, st));
    copy_block<double, double>(f.ptr, 1, v.ptr, 1, L, 1, 1.0 / beta, st);
    apply(v.ptr, f.ptr);
    axpby_block<double>(v0.ptr, 1, f.ptr, 1, L, 1, -beta, 1.0, st);
    alpha = dot(f.ptr, v.ptr);
    axpby_block<double>(v.ptr, 1, f.ptr, 1, L, 1, -alpha, 1.0, st);
    T[(size_t)j * k + j - 1] = beta;
    T[(size_t)(j - 1) * k + j] = beta;
    T[(size_t)j * k + j] = alpha;
  }
  const double fn = std::sqrt(dot(f.ptr, f.ptr));
  DeviceBuffer<double> dT((size_t)k * k), dw(k), dZ((size_t)k * k);
  CHEFSI_CUDA(cudaMemcpyAsync(dT.ptr, T.data(), sizeof(double) * k * k, cudaMemcpyHostToDevice, st));
  int rc = syevd(dT.ptr, k, dw.ptr, dZ.ptr, st);
  if (rc != CHEFSI_OK) return rc;
  std::vector<double> w(k);
  CHEFSI_CUDA(cudaMemcpyAsync(w.data(), dw.ptr, sizeof(double) * k, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  std::sort(w.begin(), w.end());
  *lower = std::floor(w[0]);
  *upper = std::ceil(w[k - 1] + (reproducible ? fn : fn / 10.0));
  CHEFSI_API_END
}

int chefsi_cholesky_gs(chefsi_operator op, void* X, int64_t ld, int32_t N, int32_t precision,
                       void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && N >= 1 && ld >= N, "bad argument");
  cudaStream_t st = as_stream(stream);
  chefsi_solver_s s;
  s.p = default_params();
  if (op->is_complex) {
    cplx* S = reinterpret_cast<cplx*>(s.S.ensure((size_t)N * N * 2));
    cplx* W = reinterpret_cast<cplx*>(s.W.ensure((size_t)N * N * 2));
    CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(cplx) * N * N, st));
    gram_c64((const cplx*)X, ld, (const cplx*)X, ld, op->n_dofs, N, N, S, N, true, st);
    symmetrize_lower_c(S, N, st);
    int rc = cholesky_lower_c(S, N, st);
    if (rc != CHEFSI_OK) {
      set_last_error("overlap matrix is not positive definite (Cholesky pivot <= 0)");
      return rc;
    }
    trtri_lower_c(S, N, st);
    // X <- X L^{-H}
    k_conj_transpose<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(S, W, N);
    CHEFSI_CHECK_LAUNCH();
    rotate_rows_c(&s, (cplx*)X, ld, op->n_dofs, N, W, st);
    CHEFSI_CUDA(cudaStreamSynchronize(st));
    return CHEFSI_OK;
  }
  double* S = s.S.ensure((size_t)N * N);
  double* W = s.W.ensure((size_t)N * N);
  CHEFSI_CUDA(cudaMemsetAsync(S, 0, sizeof(double) * N * N, st));
  gram_f64((double*)X, ld, (double*)X, ld, op->n_dofs, N, N, S, N, precision, true, st);
  symmetrize_lower(S, N, st);
  int rc = cholesky_overlap(S, (const double*)X, ld, op->n_dofs, N, is_mixed(precision), st);
  if (rc != CHEFSI_OK) return rc;
  trtri_lower(S, N, st);
  // X <- X L^{-T}
  k_transpose<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(S, W, N);
  CHEFSI_CHECK_LAUNCH();
  rotate_rows(&s, (double*)X, ld, op->n_dofs, N, W, precision, st);
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_rayleigh_ritz(chefsi_operator op, void* X, int64_t ld, int32_t N, double* eig_host,
                         double* HX_out, double* W_out, int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && eig_host && N >= 1 && ld >= N, "bad argument");
  cudaStream_t st = as_stream(stream);
  chefsi_solver_s s;
  s.p = default_params();
  const int cw = op->is_complex ? 2 : 1;
  int rc = op->is_complex
               ? rayleigh_ritz_complex(&s, op, (cplx*)X, ld, N, precision, HX_out != nullptr, st)
               : rayleigh_ritz_real(&s, op, (double*)X, ld, N, precision, HX_out != nullptr, st);
  if (rc != CHEFSI_OK) return rc;
  if (HX_out)
    CHEFSI_CUDA(cudaMemcpyAsync(HX_out, s.HX.ptr, sizeof(double) * op->n_dofs * N * cw,
                                cudaMemcpyDeviceToDevice, st));
  if (W_out)
    CHEFSI_CUDA(cudaMemcpyAsync(W_out, s.W.ptr, sizeof(double) * (size_t)N * N * cw,
                                cudaMemcpyDeviceToDevice, st));
  CHEFSI_CUDA(cudaMemcpyAsync(eig_host, s.evals.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_rayleigh_ritz_spectrum_split(chefsi_operator op, void* X, int64_t ld, int32_t N,
                                        int32_t n_occ, void* XFrac, int64_t ld_frac,
                                        double* eig_host, void* HXFrac_out, int32_t precision,
                                        int32_t frac_reduced, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && XFrac && eig_host && N >= 1 && ld >= N, "bad argument");
  CHEFSI_REQUIRE(n_occ >= 0 && n_occ < N, "need 0 <= n_occ < N");
  CHEFSI_REQUIRE(ld_frac >= N - n_occ, "ld_frac below N - n_occ");
  cudaStream_t st = as_stream(stream);
  chefsi_solver_s s;
  s.p = default_params();
  s.p.rr_precision = precision == CHEFSI_PREC_MIXED ? CHEFSI_PREC_FP32_TC : CHEFSI_PREC_FP64;
  s.p.ss_frac_reduced = frac_reduced;
  const int nfr = N - n_occ;
  const int cw = op->is_complex ? 2 : 1;
  int rc = op->is_complex
               ? rayleigh_ritz_ss_complex(&s, op, (cplx*)X, ld, N, n_occ, (cplx*)XFrac, ld_frac,
                                          precision, HXFrac_out != nullptr, st)
               : rayleigh_ritz_ss_real(&s, op, (double*)X, ld, N, n_occ, (double*)XFrac,
                                       ld_frac, precision, HXFrac_out != nullptr, st);
  if (rc != CHEFSI_OK) return rc;
  if (HXFrac_out)
    CHEFSI_CUDA(cudaMemcpyAsync(HXFrac_out, s.HXF.ptr, sizeof(double) * op->n_dofs * nfr * cw,
                                cudaMemcpyDeviceToDevice, st));
  CHEFSI_CUDA(cudaMemcpyAsync(eig_host, s.evals.ptr, sizeof(double) * nfr, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_density_matrix_first_order_response(chefsi_operator op_prime, void* X, int64_t ld,
                                               int32_t N, const double* eig_host,
                                               double fermi_energy, double temperature,
                                               double* dmu_host, int32_t precision,
                                               void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op_prime && X && eig_host && dmu_host && N >= 1 && ld >= N, "bad argument");
  CHEFSI_REQUIRE(temperature > 0.0, "temperature must be positive (Kelvin)");
  cudaStream_t st = as_stream(stream);
  chefsi_solver_s s;
  s.p = default_params();
  DeviceBuffer<double> eig(N), dmu(N);
  CHEFSI_CUDA(cudaMemcpyAsync(eig.ptr, eig_host, sizeof(double) * N, cudaMemcpyHostToDevice, st));
  // beta = 1 / k_B / T, k_B in Hartree per Kelvin (include/constants.h:30)
  const double beta = 1.0 / 3.166811429e-06 / temperature;
  int rc = op_prime->is_complex
               ? dm_first_order_response_complex(&s, op_prime, (cplx*)X, ld, N, eig.ptr,
                                                 fermi_energy, beta, dmu.ptr, precision, st)
               : dm_first_order_response_real(&s, op_prime, (double*)X, ld, N, eig.ptr,
                                              fermi_energy, beta, dmu.ptr, precision, st);
  if (rc != CHEFSI_OK) return rc;
  CHEFSI_CUDA(cudaMemcpyAsync(dmu_host, dmu.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_axpby(int64_t rows, int32_t n_vec, double a, const double* x, int64_t ldx, double b,
                 double* y, int64_t ldy, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(x && y && rows >= 0 && n_vec >= 1 && ldx >= n_vec && ldy >= n_vec, "bad argument");
  axpby_block<double>(x, ldx, y, ldy, rows, n_vec, a, b, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_convert_block(int32_t src_bits, const void* src, int64_t ld_src, int32_t dst_bits,
                         void* dst, int64_t ld_dst, int64_t rows, int32_t n_vec, double scale,
                         void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(src && dst && rows >= 0 && n_vec >= 1 && ld_src >= n_vec && ld_dst >= n_vec &&
                     (src_bits == 32 || src_bits == 64) && (dst_bits == 32 || dst_bits == 64),
                 "bad argument");
  cudaStream_t st = as_stream(stream);
  if (src_bits == 64 && dst_bits == 64)
    copy_block<double, double>(static_cast<const double*>(src), ld_src, static_cast<double*>(dst),
                               ld_dst, rows, n_vec, scale, st);
  else if (src_bits == 64)
    copy_block<double, float>(static_cast<const double*>(src), ld_src, static_cast<float*>(dst),
                              ld_dst, rows, n_vec, scale, st);
  else if (dst_bits == 64)
    copy_block<float, double>(static_cast<const float*>(src), ld_src, static_cast<double*>(dst),
                              ld_dst, rows, n_vec, scale, st);
  else
    copy_block<float, float>(static_cast<const float*>(src), ld_src, static_cast<float*>(dst),
                             ld_dst, rows, n_vec, scale, st);
  CHEFSI_API_END
}

int chefsi_gemm(char ta, char tb, int64_t M, int32_t N, int32_t K, double alpha, const double* A,
                int64_t lda, const double* B, int64_t ldb, double beta, double* C, int64_t ldc,
                int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(A && B && C && M >= 0 && N >= 0 && K >= 0, "bad argument");
  gemm_f64(ta, tb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc, precision, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_assemble_cell_hamiltonians(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                      const double* shape, const double* stiffness,
                                      const double* v_jxw, double* out, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(shape && stiffness && v_jxw && out && n_cells > 0 && nodes_per_cell > 0 && n_q > 0,
                 "bad argument");
  assemble_cells(n_cells, nodes_per_cell, n_q, shape, stiffness, v_jxw, out, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_assemble_cell_hamiltonians_gga(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                          const double* shape, const double* shape_grad,
                                          const double* stiffness, const double* v_jxw,
                                          const double* gga_jxw, double* out, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(shape && shape_grad && stiffness && v_jxw && gga_jxw && out && n_cells > 0 &&
                     nodes_per_cell > 0 && n_q > 0,
                 "bad argument");
  assemble_cells_gga(n_cells, nodes_per_cell, n_q, shape, shape_grad, stiffness, v_jxw, gga_jxw,
                     out, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_assemble_cell_hamiltonians_geometry(int32_t n_cells, int32_t nodes_per_cell,
                                               int32_t n_q, const double* shape,
                                               const double* shape_grad_ref,
                                               const double* jacobian_factor,
                                               const double* v_jxw, double* out, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(shape && shape_grad_ref && jacobian_factor && v_jxw && out && n_cells > 0 &&
                     nodes_per_cell > 0 && n_q > 0,
                 "bad argument");
  assemble_cells_geometry(n_cells, nodes_per_cell, n_q, shape, shape_grad_ref, jacobian_factor,
                          v_jxw, out, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_assemble_cell_hamiltonians_bloch(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                            const double* shape, const double* shape_grad,
                                            const double* stiffness, const double* v_jxw,
                                            const double* jxw, int32_t n_k,
                                            const double* kpoints_host, void* out, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(shape && shape_grad && stiffness && v_jxw && jxw && kpoints_host && out &&
                     n_cells > 0 && nodes_per_cell > 0 && n_q > 0 && n_k > 0,
                 "bad argument");
  cudaStream_t st = as_stream(stream);
  DeviceBuffer<double> kd((size_t)3 * n_k);
  CHEFSI_CUDA(cudaMemcpyAsync(kd.ptr, kpoints_host, sizeof(double) * 3 * n_k,
                              cudaMemcpyHostToDevice, st));
  assemble_cells_bloch(n_cells, nodes_per_cell, n_q, shape, shape_grad, stiffness, v_jxw, jxw, n_k,
                       kd.ptr, (double*)out, st);
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_assemble_cell_hamiltonians_bloch_gga(int32_t n_cells, int32_t nodes_per_cell,
                                                int32_t n_q, const double* shape,
                                                const double* shape_grad, const double* stiffness,
                                                const double* v_jxw, const double* gga_jxw,
                                                const double* jxw, int32_t n_k,
                                                const double* kpoints_host, void* out,
                                                void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(shape && shape_grad && stiffness && v_jxw && gga_jxw && jxw && kpoints_host &&
                     out && n_cells > 0 && nodes_per_cell > 0 && n_q > 0 && n_k > 0,
                 "bad argument");
  cudaStream_t st = as_stream(stream);
  DeviceBuffer<double> kd((size_t)3 * n_k);
  CHEFSI_CUDA(cudaMemcpyAsync(kd.ptr, kpoints_host, sizeof(double) * 3 * n_k,
                              cudaMemcpyHostToDevice, st));
  assemble_cells_bloch(n_cells, nodes_per_cell, n_q, shape, shape_grad, stiffness, v_jxw, jxw, n_k,
                       kd.ptr, (double*)out, st, gga_jxw);
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_operator_update_cell_matrices(chefsi_operator op, const double* cell_matrices,
                                         void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && cell_matrices, "bad argument");
  update_cell_matrices(op, cell_matrices, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_cell_outer_accumulate(chefsi_operator op, const double* U, const double* V, int64_t ld,
                                 int32_t n_vec, double alpha, double* G, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && U && V && G && n_vec >= 1 && ld >= n_vec, "bad argument");
  CHEFSI_REQUIRE(!op->is_complex, "cell outer product: real operators only");
  cell_outer(op, U, V, ld, n_vec, alpha, G, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_cell_quadrature_contract(int32_t n_cells, int32_t nodes_per_cell, int32_t n_q,
                                    const double* shape, const double* G, const double* jxw,
                                    double* out, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(shape && G && out && n_cells > 0 && nodes_per_cell > 0 && n_q > 0, "bad argument");
  quad_contract(n_cells, nodes_per_cell, n_q, shape, G, jxw, out, as_stream(stream));
  CHEFSI_API_END
}

int chefsi_density(chefsi_operator op, const double* X, int64_t ld, int32_t N,
                   const double* occupation, int32_t n_q, const double* shape, const double* jxw,
                   double* rho, int32_t accumulate, int32_t precision, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && occupation && shape && rho && N >= 1 && ld >= N && n_q >= 1,
                 "bad argument");
  CHEFSI_REQUIRE(!op->is_complex, "density: real operators only");
  cudaStream_t st = as_stream(stream);
  if (precision == CHEFSI_PREC_MIXED &&
      density_tc(op, X, ld, N, occupation, n_q, shape, jxw, rho, accumulate != 0, st))
    return CHEFSI_OK;
  const size_t ng = (size_t)op->n_cells * op->n_e * op->n_e;
  double* G = op->ws64a.ensure(ng);
  CHEFSI_CUDA(cudaMemsetAsync(G, 0, sizeof(double) * ng, st));
  cell_outer(op, X, X, ld, N, 1.0, G, st, occupation);
  quad_contract(op->n_cells, op->n_e, n_q, shape, G, jxw, rho, st, accumulate != 0);
  CHEFSI_API_END
}

int chefsi_residual_norms(chefsi_operator op, const void* X, int64_t ld, int32_t N,
                          const double* eig_host, double* res_host, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(op && X && eig_host && res_host && N >= 1 && ld >= N, "bad argument");
  cudaStream_t st = as_stream(stream);
  const int64_t M = op->n_dofs;
  DeviceBuffer<double> lam(N), out(N);
  CHEFSI_CUDA(cudaMemcpyAsync(lam.ptr, eig_host, sizeof(double) * N, cudaMemcpyHostToDevice, st));
  if (op->is_complex) {
    DeviceBuffer<double> HX((size_t)M * N * 2);
    hx_c64(op, (const cplx*)X, ld, (cplx*)HX.ptr, N, N, 1.0, false, st);
    residual_norms_c64((const cplx*)X, ld, (const cplx*)HX.ptr, N, M, N, lam.ptr, out.ptr, st);
  } else {
    DeviceBuffer<double> HX((size_t)M * N);
    hx_all_f64(op, (const double*)X, ld, N, HX.ptr, 400, st);
    residual_norms_f64((const double*)X, ld, HX.ptr, N, M, N, lam.ptr, out.ptr, st);
  }
  CHEFSI_CUDA(cudaMemcpyAsync(res_host, out.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

int chefsi_set_wait_limits(uint32_t mbarrier_tries, uint32_t barrier_spins) {
  CHEFSI_API_BEGIN
  tcx::tc_set_wait_tries(mbarrier_tries);
  tcx::dense_tc_set_wait_tries(mbarrier_tries);
  dense_set_barrier_spins(barrier_spins);
  CHEFSI_API_END
}

int chefsi_solver_create(const chefsi_params* params, chefsi_solver* out) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(out != nullptr, "null output handle");
  auto* s = new chefsi_solver_s();
  s->p = params ? *params : default_params();
  if (s->p.cheby_wfc_block <= 0) s->p.cheby_wfc_block = 400;
  if (s->p.wfc_block <= 0) s->p.wfc_block = 400;
  if (s->p.lanczos_steps <= 0) s->p.lanczos_steps = s->p.reproducible ? 40 : 20;
  if (s->p.first_scf_degree_scale <= 0) s->p.first_scf_degree_scale = 1.0;
  *out = s;
  CHEFSI_API_END
}

int chefsi_solver_destroy(chefsi_solver s) {
  CHEFSI_API_BEGIN
  delete s;
  CHEFSI_API_END
}

int chefsi_solver_reinit_spectrum_bounds(chefsi_solver s, double lower_wanted,
                                         double lower_unwanted, double upper_unwanted) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s != nullptr, "null solver");
  s->a0 = lower_wanted;
  s->b_low = lower_unwanted;
  s->b_up = upper_unwanted;
  CHEFSI_API_END
}

int chefsi_solver_get_bounds(chefsi_solver s, double* a0, double* bl, double* bu, int32_t* deg) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s != nullptr, "null solver");
  if (a0) *a0 = s->a0;
  if (bl) *bl = s->b_low;
  if (bu) *bu = s->b_up;
  if (deg) *deg = s->last_degree;
  CHEFSI_API_END
}

int chefsi_solver_timings(chefsi_solver s, double* ms7) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s && ms7, "bad argument");
  for (int i = 0; i < 7; ++i) ms7[i] = s->times[i];
  CHEFSI_API_END
}

int chefsi_solver_set_profiling(chefsi_solver s, int32_t enable) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s != nullptr, "null solver");
  s->profile = enable != 0;
  CHEFSI_API_END
}

int chefsi_solver_hx_stats(chefsi_solver s, int32_t* launches, double* total_ms) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s != nullptr, "null solver");
  if (launches) *launches = s->hx_launches;
  if (total_ms) *total_ms = s->hx_ms;
  CHEFSI_API_END
}

static int degree_for(chefsi_solver_s* s, int is_first_scf) {
  int m = s->p.chebyshev_degree > 0 ? s->p.chebyshev_degree : chefsi_chebyshev_order(s->b_up);
  if (is_first_scf) m = (int)(m * s->p.first_scf_degree_scale);
  return std::max(1, m);
}

// everything of one CheFSI iteration after the filter: Rayleigh-Ritz (Cholesky-GS, X^T H X,
// projected eigensolve, rotation), residual norms, eigenvalues / residuals to the host
static int solve_after_filter(chefsi_solver_s* s, chefsi_operator_s* op, void* X, int N,
                       double* eig_host, double* res_host, int compute_residual, cudaStream_t st) {
  const int prec = s->p.precision;
  const int64_t M = op->n_dofs;
  double* res = s->resid.ensure(N);
  if (op->is_complex) {
    int rc = rayleigh_ritz_complex(s, op, (cplx*)X, N, N, prec, true, st);
    if (rc != CHEFSI_OK) return rc;
    if (compute_residual)
      residual_norms_c64((const cplx*)X, N, (const cplx*)s->HX.ptr, N, M, N, s->evals.ptr, res, st);
  } else if (rr_blocked(s, op, N, prec)) {
    int rc = rayleigh_ritz_real_blocked(s, op, (double*)X, N, N, prec,
                                        compute_residual ? res : nullptr, st);
    if (rc != CHEFSI_OK) return rc;
  } else {
    int rc = rayleigh_ritz_real(s, op, (double*)X, N, N, prec, true, st);
    if (rc != CHEFSI_OK) return rc;
    if (compute_residual) residual_norms_f64((double*)X, N, s->HX.ptr, N, M, N, s->evals.ptr, res, st);
  }
  CHEFSI_CUDA(cudaEventRecord(s->ev[6], st));
  CHEFSI_CUDA(cudaMemcpyAsync(eig_host, s->evals.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  if (compute_residual && res_host)
    CHEFSI_CUDA(cudaMemcpyAsync(res_host, res, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  s->times[0] = elapsed(s->ev[0], s->ev[1]);
  s->times[1] = elapsed(s->ev[1], s->ev[2]);
  s->times[2] = elapsed(s->ev[2], s->ev[3]);
  s->times[3] = elapsed(s->ev[3], s->ev[4]);
  s->times[4] = elapsed(s->ev[4], s->ev[5]);
  s->times[5] = elapsed(s->ev[5], s->ev[6]);
  s->times[6] = elapsed(s->ev[0], s->ev[6]);
  s->hx_collect();
  return CHEFSI_OK;
}

int chefsi_solve(chefsi_solver s, chefsi_operator op, void* X, int32_t N, double* eig_host,
                 double* res_host, int32_t compute_residual, int32_t is_first_scf, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s && op && X && eig_host && N >= 1, "bad argument");
  CHEFSI_REQUIRE(s->b_up > s->b_low, "spectrum bounds not set (call reinit_spectrum_bounds)");
  cudaStream_t st = as_stream(stream);
  const int m = degree_for(s, is_first_scf);
  s->last_degree = m;
  CHEFSI_CUDA(cudaEventRecord(s->ev[0], st));
  filter_all(s, op, X, N, m, s->p.precision, st);
  const int rc = solve_after_filter(s, op, X, N, eig_host, res_host, compute_residual, st);
  if (rc != CHEFSI_OK) return rc;
  CHEFSI_API_END
}

// One CheFSI iteration with the spectrum-split Rayleigh-Ritz step: the solve() branch taken
// when fewer eigenvalues than vectors are wanted
// (chebyshevOrthogonalizedSubspaceIterationSolverDevice.cc:584-605, residuals of the
// fractional vectors at :675-690).
int chefsi_solve_spectrum_split(chefsi_solver s, chefsi_operator op, void* X, int32_t N,
                                int32_t n_occ, void* XFrac, double* eig_host, double* res_host,
                                int32_t compute_residual, int32_t is_first_scf, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s && op && X && XFrac && eig_host && N >= 1, "bad argument");
  CHEFSI_REQUIRE(n_occ >= 0 && n_occ < N, "need 0 <= n_occ < N");
  CHEFSI_REQUIRE(s->b_up > s->b_low, "spectrum bounds not set (call reinit_spectrum_bounds)");
  cudaStream_t st = as_stream(stream);
  const int m = degree_for(s, is_first_scf);
  s->last_degree = m;
  const int nfr = N - n_occ;
  const int64_t M = op->n_dofs;
  CHEFSI_CUDA(cudaEventRecord(s->ev[0], st));
  filter_all(s, op, X, N, m, s->p.precision, st);
  int rc = op->is_complex
               ? rayleigh_ritz_ss_complex(s, op, (cplx*)X, N, N, n_occ, (cplx*)XFrac, nfr,
                                          s->p.precision, compute_residual != 0, st)
               : rayleigh_ritz_ss_real(s, op, (double*)X, N, N, n_occ, (double*)XFrac, nfr,
                                       s->p.precision, compute_residual != 0, st);
  if (rc != CHEFSI_OK) return rc;
  double* res = s->resid.ensure(nfr);
  if (compute_residual && op->is_complex)
    residual_norms_c64((const cplx*)XFrac, nfr, (const cplx*)s->HXF.ptr, nfr, M, nfr, s->evals.ptr,
                       res, st);
  else if (compute_residual)
    residual_norms_f64((const double*)XFrac, nfr, s->HXF.ptr, nfr, M, nfr, s->evals.ptr, res, st);
  CHEFSI_CUDA(cudaEventRecord(s->ev[6], st));
  CHEFSI_CUDA(cudaMemcpyAsync(eig_host, s->evals.ptr, sizeof(double) * nfr, cudaMemcpyDeviceToHost, st));
  if (compute_residual && res_host)
    CHEFSI_CUDA(cudaMemcpyAsync(res_host, res, sizeof(double) * nfr, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  for (int i = 0; i < 6; ++i) s->times[i] = elapsed(s->ev[i], s->ev[i + 1]);
  s->times[6] = elapsed(s->ev[0], s->ev[6]);
  s->hx_collect();
  CHEFSI_API_END
}

// ---------------------------------------------------------------- batched (grouped) filter
// Problems of a batch whose mixed filter runs on the tensor cores in one block are filtered
// together: per Chebyshev degree one grouped recurrence step and one persistent tensor-core
// HX launch cover every problem of a cell type (their per-problem coefficients ride in the
// kernel parameters), and the whole lockstep recurrence is captured in a CUDA graph.
namespace {

struct GroupMember {
  int idx;                     // batch entry
  chefsi_solver_s* s;
  chefsi_operator_s* op;       // the caller's operator
  chefsi_operator_s* tcop;     // the operator the tensor cores apply (op, or its real form)
  void* X;
  int N;
  int64_t rows;                // FP32 rows: n_dofs, or 2 n_dofs for the real form
  float* x;
  float* y;
  __half* hi;
  __half* lo;
  double scale;
  int m;
  float* result;
};

// Autotuner of the grouped apply: the X-ring depth and the K-blocks of gathers in flight
// (the pipeline shape of a cell tile), chosen per (cell type, work size) by timing each
// candidate on the group's own operands once; the choice is kept for the process.
std::mutex g_tune_mu;
std::map<std::pair<int, int>, TcPipeline> g_tune_cache;

TcPipeline autotune_pipeline(const std::vector<TcGroupItem>& items, cudaStream_t st) {
  int64_t pairs = 0;
  for (const auto& it : items) pairs += (int64_t)it.op->n_cells * ((it.B + 127) / 128);
  int bucket = 0;
  while ((1ll << (bucket + 1)) <= pairs) ++bucket;
  const std::pair<int, int> key{items[0].op->n_e, bucket};
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    auto f = g_tune_cache.find(key);
    if (f != g_tune_cache.end()) return f->second;
  }
  // X-ring depth x copies in flight, then the order the (cell, 128-vector chunk) pairs are
  // dealt in: a cell's chunks back to back (its tiles shared in L2 by the chunks), or tiles of
  // 8 or 64 cells with all their chunks (neighbouring cells' shared rows meet in L2)
  const TcPipeline cand[] = {{8, 6, 1}, {8, 4, 1}, {6, 4, 1}, {6, 2, 1}, {4, 2, 1},
                             {8, 6, 8}, {8, 6, 64}};
  cudaEvent_t e0, e1;
  CHEFSI_CUDA(cudaEventCreate(&e0));
  CHEFSI_CUDA(cudaEventCreate(&e1));
  TcPipeline best = cand[0];
  float best_ms = 1e30f;
  try {
    for (const TcPipeline& c : cand) {
      hx_tc_group_launch(items.data(), (int)items.size(), 2, &c, st);   // warm-up
      CHEFSI_CUDA(cudaEventRecord(e0, st));
      hx_tc_group_launch(items.data(), (int)items.size(), 2, &c, st);
      CHEFSI_CUDA(cudaEventRecord(e1, st));
      CHEFSI_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      CHEFSI_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best_ms) best_ms = ms, best = c;
    }
  } catch (...) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    throw;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune_cache[key] = best;
  return best;
}

// the filter of one group (same cell type), lockstep over the degrees, captured in a graph
void cheb_filter_group(std::vector<GroupMember*>& g, cudaStream_t st) {
  const int n = (int)g.size();
  struct Rec {
    double e, c, sigma, gamma;
  };
  std::vector<Rec> r(n);
  int mmax = 0;
  for (int i = 0; i < n; ++i) {
    chefsi_solver_s* s = g[i]->s;
    const double e = (s->b_up - s->b_low) / 2.0, c = (s->b_up + s->b_low) / 2.0;
    const double sigma = e / (s->a0 - c);
    r[i] = Rec{e, c, sigma, 2.0 / sigma};
    mmax = std::max(mmax, g[i]->m);
  }
  auto hx_items = [&](const std::vector<int>& act, const std::vector<double>& scal,
                      bool first) {
    std::vector<TcGroupItem> it;
    for (size_t k = 0; k < act.size(); ++k) {
      GroupMember* gm = g[act[k]];
      it.push_back(TcGroupItem{gm->tcop, gm->hi, gm->lo, nullptr, first ? gm->y : gm->x, gm->N,
                               gm->N, scal[k]});
    }
    return it;
  };
  // the step-1 applies, also used by the autotuner (before step 1 writes y without reading it)
  std::vector<int> all(n);
  std::iota(all.begin(), all.end(), 0);
  std::vector<double> a1(n);
  for (int i = 0; i < n; ++i) a1[i] = r[i].sigma / r[i].e;
  std::vector<TcPipeline> pipes;
  for (int i0 = 0; i0 < n; i0 += 32) {
    std::vector<int> part(all.begin() + i0, all.begin() + std::min(n, i0 + 32));
    std::vector<double> sc(a1.begin() + i0, a1.begin() + std::min(n, i0 + 32));
    pipes.push_back(autotune_pipeline(hx_items(part, sc, true), st));
  }
  // apply the active members in launches of at most 32
  auto launch = [&](const std::vector<int>& act, const std::vector<double>& scal,
                    const std::vector<double>& aa, const std::vector<double>& bb, bool first) {
    for (size_t k0 = 0; k0 < act.size(); k0 += 32) {
      const size_t k1 = std::min(act.size(), k0 + 32);
      std::vector<AxpbyGroupItem> ax;
      for (size_t k = k0; k < k1; ++k) {
        GroupMember* gm = g[act[k]];
        // step 1: y = a x, split(x); later: x = a y + b x, split(y)
        if (first)
          ax.push_back(AxpbyGroupItem{gm->x, gm->y, gm->hi, gm->lo, gm->rows * gm->N, aa[k], 0.0});
        else
          ax.push_back(AxpbyGroupItem{gm->y, gm->x, gm->hi, gm->lo, gm->rows * gm->N, aa[k], bb[k]});
      }
      axpby_split_group(ax.data(), (int)ax.size(), st);
      std::vector<int> part(act.begin() + k0, act.begin() + k1);
      std::vector<double> sc(scal.begin() + k0, scal.begin() + k1);
      const auto it = hx_items(part, sc, first);
      hx_tc_group_launch(it.data(), (int)it.size(), 2, &pipes[std::min<size_t>(k0 / 32, pipes.size() - 1)], st);
      for (size_t k = k0; k < k1; ++k) {
        GroupMember* gm = g[act[k]];
        if (gm->tcop->n_atoms)
          apply_nonlocal_f32(gm->tcop, first ? gm->x : gm->y, gm->N, first ? gm->y : gm->x, gm->N,
                             gm->N, scal[k], st);
      }
    }
  };
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  CHEFSI_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  try {
    std::vector<double> aa(n), bb(n, 0.0);
    for (int i = 0; i < n; ++i) aa[i] = a1[i] * (-r[i].c);
    launch(all, a1, aa, bb, true);
    for (int degree = 2; degree <= mmax; ++degree) {
      std::vector<int> act;
      std::vector<double> sc, ca, cb;
      for (int i = 0; i < n; ++i) {
        if (g[i]->m < degree) continue;
        const double sigma2 = 1.0 / (r[i].gamma - r[i].sigma);
        const double alpha1 = 2.0 * sigma2 / r[i].e, alpha2 = -(r[i].sigma * sigma2);
        act.push_back(i);
        sc.push_back(alpha1);
        ca.push_back(-r[i].c * alpha1);
        cb.push_back(alpha2);
        r[i].sigma = sigma2;
      }
      launch(act, sc, ca, cb, false);
      for (int i : act) std::swap(g[i]->x, g[i]->y);
    }
  } catch (...) {
    cudaStreamEndCapture(st, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  CHEFSI_CUDA(cudaStreamEndCapture(st, &graph));
  const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
  if (ie != cudaSuccess) {
    cudaGraphDestroy(graph);
    CHEFSI_CUDA(ie);
  }
  const cudaError_t le = cudaGraphLaunch(exec, st);
  const cudaError_t se = le == cudaSuccess ? cudaStreamSynchronize(st) : le;
  cudaGraphExecDestroy(exec);
  cudaGraphDestroy(graph);
  CHEFSI_CUDA(se);
  for (int i = 0; i < n; ++i) g[i]->result = g[i]->y;
}

// a batch entry whose filter can join a group: mixed precision, one block, tensor-core apply
chefsi_operator_s* group_operator(chefsi_solver_s* s, chefsi_operator_s* op, int N,
                                  cudaStream_t st) {
  if (s->p.precision != CHEFSI_PREC_MIXED) return nullptr;
  if (s->p.cheby_wfc_block > 0 && s->p.cheby_wfc_block < N) return nullptr;
  if (op->is_complex) {
    if (!op->folded) return nullptr;
    chefsi_operator_s* rv = realified(op, st);
    return tc_split_usable(rv, N) ? rv : nullptr;
  }
  return tc_split_usable(op, N) ? op : nullptr;
}

}  // namespace

int chefsi_solve_batched(int32_t count, chefsi_solver* solvers, chefsi_operator* ops, void** X,
                         const int32_t* N, double** eig_host, double** res_host,
                         int32_t compute_residual, int32_t is_first_scf, int32_t n_streams,
                         int32_t group_filter) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(count >= 0 && (count == 0 || (solvers && ops && X && N && eig_host)),
                 "bad argument");
  if (count == 0) return CHEFSI_OK;
  for (int i = 0; i < count; ++i)
    CHEFSI_REQUIRE(solvers[i] && ops[i] && X[i] && eig_host[i] && N[i] >= 1,
                   "bad argument in batch entry " + std::to_string(i));
  // distinct operators too: the entries run concurrently on several streams, and a mixed
  // filter writes its Chebyshev shift into its operator's tensor-core tiles
  for (int i = 0; i < count; ++i)
    for (int j = 0; j < i; ++j)
      CHEFSI_REQUIRE(solvers[i] != solvers[j] && ops[i] != ops[j],
                     "batch entries must use distinct solvers and operators");
  // largest first: work ~ n_dofs * N * (degree + 2) (filter) + n_dofs * N^2 (dense steps)
  std::vector<double> cost(count);
  for (int i = 0; i < count; ++i) {
    const double M = (double)ops[i]->n_dofs * (ops[i]->is_complex ? 4.0 : 1.0);
    const double deg = degree_for(solvers[i], is_first_scf) + 2.0;
    cost[i] = M * N[i] * (deg * ops[i]->n_e + N[i]);
  }
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return cost[a] > cost[b]; });
  int workers = n_streams > 0 ? n_streams : std::min(count, 8);
  workers = std::max(1, std::min(workers, count));
  int dev = 0;
  CHEFSI_CUDA(cudaGetDevice(&dev));

  // grouped filter of the entries that can share launches (two or more)
  std::vector<GroupMember> mem;
  std::vector<int> member_of(count, -1);
  {
    cudaStream_t st0 = nullptr;
    CHEFSI_CUDA(cudaStreamCreateWithFlags(&st0, cudaStreamNonBlocking));
    try {
      for (int k = 0; k < count && group_filter; ++k) {
        const int i = order[k];
        chefsi_operator_s* tcop = group_operator(solvers[i], ops[i], N[i], st0);
        if (!tcop) continue;
        GroupMember gm{};
        gm.idx = i;
        gm.s = solvers[i];
        gm.op = ops[i];
        gm.tcop = tcop;
        gm.X = X[i];
        gm.N = N[i];
        gm.rows = tcop->n_dofs;
        gm.m = degree_for(solvers[i], is_first_scf);
        mem.push_back(gm);
      }
      if (mem.size() < 2) mem.clear();
      std::vector<double> amax(mem.size(), 0.0);
      for (size_t k = 0; k < mem.size(); ++k) {
        GroupMember& gm = mem[k];
        gm.s->last_degree = gm.m;
        CHEFSI_CUDA(cudaEventRecord(gm.s->ev[0], st0));
        double* sc = gm.s->scal.ensure(1);
        const int64_t M = gm.op->n_dofs;
        if (gm.op->is_complex)
          absmax_block_f64(reinterpret_cast<const double*>(gm.X), 2 * (int64_t)gm.N, M, 2 * gm.N, sc, st0);
        else
          absmax_block_f64(reinterpret_cast<const double*>(gm.X), gm.N, M, gm.N, sc, st0);
        CHEFSI_CUDA(cudaMemcpyAsync(&amax[k], sc, sizeof(double), cudaMemcpyDeviceToHost, st0));
      }
      CHEFSI_CUDA(cudaStreamSynchronize(st0));
      std::map<int, std::vector<GroupMember*>> by_type;
      for (size_t k = 0; k < mem.size(); ++k) {
        GroupMember& gm = mem[k];
        // FP32 rows scaled by a power of two (max |x| ~ 2^8, the FP16 split's range)
        gm.scale = (amax[k] > 0.0 && std::isfinite(amax[k]))
                       ? std::ldexp(1.0, 8 - (int)std::ceil(std::log2(amax[k])))
                       : 1.0;
        const size_t n = (size_t)gm.rows * gm.N;
        gm.x = gm.s->Xb32.ensure(n);
        gm.y = gm.s->Yb32.ensure(n);
        gm.hi = gm.s->xs_hi.ensure(n);
        gm.lo = gm.s->xs_lo.ensure(n);
        if (gm.op->is_complex)
          complex_to_real_rows(reinterpret_cast<const cplx*>(gm.X), gm.N, gm.op->n_dofs, gm.N,
                               gm.scale, gm.x, st0);
        else
          copy_block<double, float>(reinterpret_cast<const double*>(gm.X), gm.N, gm.x, gm.N,
                                    gm.rows, gm.N, gm.scale, st0);
        // everything the captured launches need, allocated before the capture
        prepare_tensor_mats(gm.tcop, st0);
        if (gm.tcop->n_atoms) gm.tcop->nlW32.ensure((size_t)gm.tcop->n_atoms * gm.tcop->n_proj * gm.N);
        by_type[gm.tcop->n_e].push_back(&gm);
        member_of[gm.idx] = (int)k;
      }
      for (auto& kv : by_type) {
        cheb_filter_group(kv.second, st0);
        const int tc = tc_check_error(kv.second[0]->tcop, st0);
        if (tc != CHEFSI_OK) throw Error(tc, "tensor-core HX: a bounded device wait expired");
      }
    } catch (...) {
      cudaStreamSynchronize(st0);
      cudaStreamDestroy(st0);
      throw;
    }
    CHEFSI_CUDA(cudaStreamSynchronize(st0));
    CHEFSI_CUDA(cudaStreamDestroy(st0));
  }

  std::atomic<int> next{0};
  std::mutex mu;
  int first_rc = CHEFSI_OK;
  std::string first_msg;
  auto work = [&]() {
    cudaStream_t st = nullptr;
    if (cudaSetDevice(dev) != cudaSuccess || cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) {
      std::lock_guard<std::mutex> g(mu);
      if (first_rc == CHEFSI_OK) first_rc = CHEFSI_ERR_CUDA, first_msg = "batched solve: stream creation failed";
      return;
    }
    for (;;) {
      const int k = next.fetch_add(1);
      if (k >= count) break;
      {
        std::lock_guard<std::mutex> g(mu);
        if (first_rc != CHEFSI_OK) break;
      }
      const int i = order[k];
      int rc = CHEFSI_OK;
      std::string msg;
      if (member_of[i] >= 0) {
        // filtered in its group: back to the caller's block, then the rest of the iteration
        GroupMember& gm = mem[member_of[i]];
        try {
          if (gm.op->is_complex)
            real_rows_to_complex(gm.result, gm.op->n_dofs, gm.N, 1.0 / gm.scale,
                                 reinterpret_cast<cplx*>(gm.X), gm.N, st);
          else
            copy_block<float, double>(gm.result, gm.N, reinterpret_cast<double*>(gm.X), gm.N,
                                      gm.rows, gm.N, 1.0 / gm.scale, st);
          rc = solve_after_filter(gm.s, gm.op, gm.X, gm.N, eig_host[i],
                                  res_host ? res_host[i] : nullptr, compute_residual, st);
          if (rc != CHEFSI_OK) msg = chefsi_last_error();
        } catch (const Error& e) {
          rc = e.code, msg = e.what();
        } catch (const std::exception& e) {
          rc = CHEFSI_ERR_INVALID, msg = e.what();
        }
      } else {
        rc = chefsi_solve(solvers[i], ops[i], X[i], N[i], eig_host[i],
                          res_host ? res_host[i] : nullptr, compute_residual, is_first_scf, st);
        if (rc != CHEFSI_OK) msg = chefsi_last_error();
      }
      if (rc != CHEFSI_OK) {
        std::lock_guard<std::mutex> g(mu);
        if (first_rc == CHEFSI_OK)
          first_rc = rc, first_msg = "batch entry " + std::to_string(i) + ": " + msg;
      }
    }
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  };
  std::vector<std::thread> pool;
  for (int w = 0; w < workers; ++w) pool.emplace_back(work);
  for (auto& t : pool) t.join();
  if (first_rc != CHEFSI_OK) {
    set_last_error(first_msg);
    return first_rc;
  }
  CHEFSI_API_END
}

int chefsi_solve_no_rr(chefsi_solver s, chefsi_operator op, void* X, int32_t N, int32_t n_passes,
                       int32_t is_first_scf, void* stream) {
  CHEFSI_API_BEGIN
  CHEFSI_REQUIRE(s && op && X && N >= 1 && n_passes >= 1, "bad argument");
  CHEFSI_REQUIRE(s->b_up > s->b_low, "spectrum bounds not set");
  cudaStream_t st = as_stream(stream);
  const int m = degree_for(s, is_first_scf);
  s->last_degree = m;
  for (int p = 0; p < n_passes; ++p) filter_all(s, op, X, N, m, s->p.precision, st);
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  CHEFSI_API_END
}

}  // extern "C"
