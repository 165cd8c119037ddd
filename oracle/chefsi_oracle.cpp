// CPU oracle for the CheFSI hot path -- TEST INFRASTRUCTURE ONLY.
//
// A plain FP64 C++ restatement of DFT-FE's CPU operator apply and Chebyshev filter. It is
// the checker the GPU library is compared against and the timed CPU baseline; the product
// never links, loads or calls it.
//
// What it restates (paths inside the DFT-FE source tree):
//   * HX sequence: kohnShamDFTOperatorClass::HX, src/dftOperator/kohnShamDFTOperator.cc:952-1047
//     (scale src by M^{-1/2}, constraints.distribute, per-cell gather -> dgemm -> scatter,
//      nonlocal term, distribute_slave_to_master, scale dst by M^{-1/2}; with scaleFlag the
//      old dst is kept and scalar*HX is added to it);
//   * per-cell product: computeLocalHamiltonianTimesX,
//     src/dftOperator/matrixVectorProductImplementations.cc:99-170;
//   * nonlocal term: C diag(V) C^T summed over atoms,
//     src/dftOperator/computeNonLocalHamiltonianTimesXMemoryOpt.cc:24,268;
//   * constraints: dftUtils::constraintMatrixInfo::distribute / distribute_slave_to_master,
//     utils/constraintMatrixInfo.cc:179-418;
//   * Chebyshev filter (sigma form): linearAlgebraOperations::chebyshevFilter,
//     src/linAlg/linearAlgebraOperationsOpt.cc:276-352;
//   * residual norms: computeEigenResidualNorm, src/linAlg/linearAlgebraOperationsOpt.cc:2394-2503.
//
// Cell loop: cells are coloured so that no two cells of one colour share a dof; colours run
// one after another and the cells of a colour in parallel (OpenMP), which makes the result
// independent of the thread count (bit-reproducible).
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef std::complex<double> zdouble;

extern "C" {

struct OracleOperator {
  int64_t n_dofs;
  int32_t n_cells;
  int32_t n_e;
  int32_t is_complex;
  const int32_t* cell_map;        // [n_cells][n_e]
  const void* cell_mats;          // [n_cells][n_e][n_e] double or complex<double>, row I, col J
  const double* inv_sqrt_mass;    // [n_dofs]
  // constraints (slave rows, CSR over masters)
  int32_t n_slaves;
  const int32_t* slave_ids;
  const int32_t* slave_ptr;       // [n_slaves+1]
  const int32_t* master_ids;
  const double* weights;
  // nonlocal projectors
  int32_t n_atoms;
  int32_t n_proj;
  const int32_t* atom_ptr;        // [n_atoms+1] into atom_dofs
  const int32_t* atom_dofs;
  const double* atom_vals;        // [sum n_dofs_a][n_proj]
  const double* couplings;        // [n_atoms][n_proj]
  // colouring
  int32_t n_colours;
  const int32_t* colour_ptr;      // [n_colours+1]
  const int32_t* colour_cells;
};

// Greedy colouring of cells: no two cells of the same colour share a dof.
int oracle_colour_cells(int32_t n_cells, int32_t n_e, const int32_t* cell_map, int64_t n_dofs,
                        int32_t* colour_ptr, int32_t* colour_cells) {
  std::vector<int32_t> deg(n_dofs + 1, 0);
  for (int64_t i = 0; i < (int64_t)n_cells * n_e; ++i) deg[cell_map[i] + 1]++;
  for (int64_t d = 0; d < n_dofs; ++d) deg[d + 1] += deg[d];
  std::vector<int32_t> adj(deg[n_dofs]);
  std::vector<int32_t> fill(deg.begin(), deg.end() - 1);
  for (int32_t c = 0; c < n_cells; ++c)
    for (int32_t I = 0; I < n_e; ++I) adj[fill[cell_map[(int64_t)c * n_e + I]]++] = c;
  std::vector<int32_t> colour(n_cells, -1);
  int32_t n_col = 0;
  std::vector<int32_t> mark(64, -1);
  for (int32_t c = 0; c < n_cells; ++c) {
    for (int32_t I = 0; I < n_e; ++I) {
      int32_t d = cell_map[(int64_t)c * n_e + I];
      for (int32_t k = deg[d]; k < deg[d + 1]; ++k) {
        int32_t o = colour[adj[k]];
        if (o >= 0) {
          if (o >= (int32_t)mark.size()) mark.resize(o + 1, -1);
          mark[o] = c;
        }
      }
    }
    int32_t col = 0;
    while (col < (int32_t)mark.size() && mark[col] == c) ++col;
    colour[c] = col;
    if (col + 1 > n_col) n_col = col + 1;
    if (col >= (int32_t)mark.size()) mark.resize(col + 1, -1);
  }
  colour_ptr[0] = 0;
  for (int32_t k = 0; k < n_col; ++k) {
    int32_t cnt = 0;
    for (int32_t c = 0; c < n_cells; ++c)
      if (colour[c] == k) colour_cells[colour_ptr[k] + cnt++] = c;
    colour_ptr[k + 1] = colour_ptr[k] + cnt;
  }
  return n_col;
}

}  // extern "C"

namespace {

inline double conj_(double x) { return x; }
inline zdouble conj_(zdouble x) { return std::conj(x); }

// Y[I][b] = sum_J H[I][J] X[J][b]; X, Y are [n_e][B] with B fastest.
template <typename T>
void cell_product(const T* __restrict H, const T* __restrict X, T* __restrict Y, int n_e, int B) {
  std::fill(Y, Y + (size_t)n_e * B, T(0));
  int I = 0;
  for (; I + 4 <= n_e; I += 4) {
    T* y0 = Y + (size_t)I * B;
    T* y1 = y0 + B;
    T* y2 = y1 + B;
    T* y3 = y2 + B;
    const T* h0 = H + (size_t)I * n_e;
    for (int J = 0; J < n_e; ++J) {
      const T a0 = h0[J], a1 = h0[n_e + J], a2 = h0[2 * n_e + J], a3 = h0[3 * n_e + J];
      const T* x = X + (size_t)J * B;
      for (int b = 0; b < B; ++b) {
        const T xv = x[b];
        y0[b] += a0 * xv;
        y1[b] += a1 * xv;
        y2[b] += a2 * xv;
        y3[b] += a3 * xv;
      }
    }
  }
  for (; I < n_e; ++I) {
    T* y = Y + (size_t)I * B;
    const T* h = H + (size_t)I * n_e;
    for (int J = 0; J < n_e; ++J) {
      const T a = h[J];
      const T* x = X + (size_t)J * B;
      for (int b = 0; b < B; ++b) y[b] += a * x[b];
    }
  }
}

template <typename T>
void hx_impl(const OracleOperator* op, const T* src, T* dst, int B, double scalar, int accumulate) {
  const int64_t M = op->n_dofs;
  const int n_e = op->n_e;
  const T* mats = static_cast<const T*>(op->cell_mats);
  std::vector<T> s((size_t)M * B), y((size_t)M * B, T(0));
  // src <- M^{-1/2} src  (kohnShamDFTOperator.cc:968-975)
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i)
    for (int b = 0; b < B; ++b) s[(size_t)i * B + b] = src[(size_t)i * B + b] * op->inv_sqrt_mass[i];
  // constraints.distribute: x_s = sum_m w_sm x_m  (constraintMatrixInfo.cc:179-240)
  for (int32_t k = 0; k < op->n_slaves; ++k) {
    T* xs = &s[(size_t)op->slave_ids[k] * B];
    for (int b = 0; b < B; ++b) xs[b] = T(0);
    for (int32_t e = op->slave_ptr[k]; e < op->slave_ptr[k + 1]; ++e) {
      const T* xm = &s[(size_t)op->master_ids[e] * B];
      const double w = op->weights[e];
      for (int b = 0; b < B; ++b) xs[b] += w * xm[b];
    }
  }
  // local cell products, colour by colour (matrixVectorProductImplementations.cc:99-170)
  for (int32_t col = 0; col < op->n_colours; ++col) {
#pragma omp parallel
    {
      std::vector<T> xc((size_t)n_e * B), yc((size_t)n_e * B);
#pragma omp for schedule(dynamic, 4)
      for (int32_t k = op->colour_ptr[col]; k < op->colour_ptr[col + 1]; ++k) {
        const int32_t c = op->colour_cells[k];
        const int32_t* map = op->cell_map + (size_t)c * n_e;
        for (int I = 0; I < n_e; ++I)
          std::memcpy(&xc[(size_t)I * B], &s[(size_t)map[I] * B], sizeof(T) * B);
        cell_product<T>(mats + (size_t)c * n_e * n_e, xc.data(), yc.data(), n_e, B);
        for (int I = 0; I < n_e; ++I) {
          T* yd = &y[(size_t)map[I] * B];
          const T* ys = &yc[(size_t)I * B];
          for (int b = 0; b < B; ++b) yd[b] += ys[b];
        }
      }
    }
  }
  // nonlocal: y += C_a diag(V_a) C_a^H s  (atoms in order)
  const int P = op->n_proj;
  for (int32_t a = 0; a < op->n_atoms; ++a) {
    const int32_t d0 = op->atom_ptr[a], d1 = op->atom_ptr[a + 1];
    std::vector<T> w((size_t)P * B, T(0));
    for (int32_t r = d0; r < d1; ++r) {
      const T* xr = &s[(size_t)op->atom_dofs[r] * B];
      const double* cr = op->atom_vals + (size_t)r * P;
      for (int j = 0; j < P; ++j)
        for (int b = 0; b < B; ++b) w[(size_t)j * B + b] += cr[j] * xr[b];
    }
    for (int j = 0; j < P; ++j) {
      const double v = op->couplings[(size_t)a * P + j];
      for (int b = 0; b < B; ++b) w[(size_t)j * B + b] *= v;
    }
    for (int32_t r = d0; r < d1; ++r) {
      T* yr = &y[(size_t)op->atom_dofs[r] * B];
      const double* cr = op->atom_vals + (size_t)r * P;
      for (int j = 0; j < P; ++j)
        for (int b = 0; b < B; ++b) yr[b] += cr[j] * w[(size_t)j * B + b];
    }
  }
  // distribute_slave_to_master: x_m += w_sm x_s ; x_s = 0  (constraintMatrixInfo.cc:300-418)
  for (int32_t k = 0; k < op->n_slaves; ++k) {
    T* xs = &y[(size_t)op->slave_ids[k] * B];
    for (int32_t e = op->slave_ptr[k]; e < op->slave_ptr[k + 1]; ++e) {
      T* xm = &y[(size_t)op->master_ids[e] * B];
      const double w = op->weights[e];
      for (int b = 0; b < B; ++b) xm[b] += w * xs[b];
    }
    for (int b = 0; b < B; ++b) xs[b] = T(0);
  }
  // dst = (accumulate ? dst : 0) + scalar * M^{-1/2} y
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < M; ++i) {
    const double f = scalar * op->inv_sqrt_mass[i];
    for (int b = 0; b < B; ++b) {
      const size_t o = (size_t)i * B + b;
      dst[o] = (accumulate ? dst[o] : T(0)) + f * y[o];
    }
  }
}

// chebyshevFilter, linearAlgebraOperationsOpt.cc:276-352 (X is [M][B], filtered in place).
template <typename T>
void filter_impl(const OracleOperator* op, T* X, int B, int m, double a, double b, double a0) {
  const int64_t n = op->n_dofs * (int64_t)B;
  double e = (b - a) / 2.0, c = (b + a) / 2.0;
  double sigma = e / (a0 - c), sigma1 = sigma, gamma = 2.0 / sigma1;
  std::vector<T> Y(n, T(0));
  hx_impl<T>(op, X, Y.data(), B, 1.0, 0);
  double alpha1 = sigma1 / e, alpha2 = -c;
  // Y = alpha1 * (Y + alpha2 * X)
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) Y[i] = alpha1 * (Y[i] + alpha2 * X[i]);
  T* x = X;
  T* y = Y.data();
  for (int degree = 2; degree < m + 1; ++degree) {
    double sigma2 = 1.0 / (gamma - sigma);
    alpha1 = 2.0 * sigma2 / e;
    alpha2 = -(sigma * sigma2);
    // X = alpha2 * X - c * alpha1 * Y
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; ++i) x[i] = alpha2 * x[i] - c * alpha1 * y[i];
    // X += alpha1 * H Y
    hx_impl<T>(op, y, x, B, alpha1, 1);
    std::swap(x, y);
    sigma = sigma2;
  }
  // result is in y
  if (y != X) std::memcpy(X, y, sizeof(T) * n);
}

}  // namespace

extern "C" {

void oracle_hx(const OracleOperator* op, const void* src, void* dst, int32_t B, double scalar,
               int32_t accumulate) {
  if (op->is_complex)
    hx_impl<zdouble>(op, (const zdouble*)src, (zdouble*)dst, B, scalar, accumulate);
  else
    hx_impl<double>(op, (const double*)src, (double*)dst, B, scalar, accumulate);
}

void oracle_chebyshev_filter(const OracleOperator* op, void* X, int32_t B, int32_t m, double a,
                             double b, double a0) {
  if (op->is_complex)
    filter_impl<zdouble>(op, (zdouble*)X, B, m, a, b, a0);
  else
    filter_impl<double>(op, (double*)X, B, m, a, b, a0);
}

// residualNorm[i] = || H x_i - lambda_i x_i ||_2 over the columns of X [M][N]
// (computeEigenResidualNorm, linearAlgebraOperationsOpt.cc:2394-2503), blocked by wfc_block.
void oracle_residual_norms(const OracleOperator* op, const void* Xv, int32_t N, const double* eig,
                           int32_t wfc_block, double* out) {
  const int64_t M = op->n_dofs;
  std::vector<double> acc(N, 0.0);
  for (int32_t j0 = 0; j0 < N; j0 += wfc_block) {
    const int32_t Bb = std::min(wfc_block, N - j0);
    if (op->is_complex) {
      const zdouble* X = (const zdouble*)Xv;
      std::vector<zdouble> xb((size_t)M * Bb), hb((size_t)M * Bb);
      for (int64_t i = 0; i < M; ++i)
        for (int b = 0; b < Bb; ++b) xb[(size_t)i * Bb + b] = X[(size_t)i * N + j0 + b];
      hx_impl<zdouble>(op, xb.data(), hb.data(), Bb, 1.0, 0);
      for (int64_t i = 0; i < M; ++i)
        for (int b = 0; b < Bb; ++b) {
          const double t = std::abs(hb[(size_t)i * Bb + b] - eig[j0 + b] * xb[(size_t)i * Bb + b]);
          acc[j0 + b] += t * t;
        }
    } else {
      const double* X = (const double*)Xv;
      std::vector<double> xb((size_t)M * Bb), hb((size_t)M * Bb);
      for (int64_t i = 0; i < M; ++i)
        for (int b = 0; b < Bb; ++b) xb[(size_t)i * Bb + b] = X[(size_t)i * N + j0 + b];
      hx_impl<double>(op, xb.data(), hb.data(), Bb, 1.0, 0);
      for (int64_t i = 0; i < M; ++i)
        for (int b = 0; b < Bb; ++b) {
          const double t = hb[(size_t)i * Bb + b] - eig[j0 + b] * xb[(size_t)i * Bb + b];
          acc[j0 + b] += t * t;
        }
    }
  }
  for (int32_t i = 0; i < N; ++i) out[i] = std::sqrt(acc[i]);
}

// Cell Hamiltonian by the direct quadrature formula of hamMatrixKernelLDA (real case,
// src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:61-115):
//   H[c][I][J] = 0.5*K[I][J] + sum_q vjxw[c][q] * N[q][I] * N[q][J]
void oracle_cell_hamiltonians(int32_t n_cells, int32_t n_e, int32_t n_q, const double* K,
                              const double* N, const double* vjxw, double* H) {
#pragma omp parallel for schedule(static)
  for (int32_t c = 0; c < n_cells; ++c) {
    double* h = H + (size_t)c * n_e * n_e;
    const double* v = vjxw + (size_t)c * n_q;
    for (int I = 0; I < n_e; ++I)
      for (int J = 0; J < n_e; ++J) {
        double acc = 0.0;
        for (int q = 0; q < n_q; ++q) acc += v[q] * N[(size_t)q * n_e + I] * N[(size_t)q * n_e + J];
        h[(size_t)I * n_e + J] = 0.5 * K[(size_t)I * n_e + J] + acc;
      }
  }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
