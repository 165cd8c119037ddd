// Dense linear algebra of the CheFSI Rayleigh-Ritz step, all on the device:
//   * split-K Gram products C += A^H B over the long dof dimension (overlap X^H X and
//     projected Hamiltonian X^H (HX); fillParallelOverlapMatScalapack / XtHX in DFT-FE);
//   * a general row-major GEMM (subspace rotation X <- X Q, small N x N products);
//   * blocked Cholesky, triangular inverse (the ELPA/ScaLAPACK steps of rayleighRitzGEP);
//   * a symmetric eigensolver: Householder tridiagonalisation, Sturm-count bisection,
//     inverse iteration with re-orthogonalisation inside clusters, back-transformation;
//   * column residual norms.
// FP64 on GB300 runs at roughly 1/64 of the FP32 rate, so the mixed-precision variants of the
// Gram and rotation products compute in FP32 inside K chunks of 256 and carry FP64 across
// chunks (errors stay at FP32 rounding of each chunk, unbiased, instead of growing with K).
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace chefsi {


// ======================================================================= Gram (split K)
// C[i][j] += sum_k A[k][i] * B[k][j]. Tile 64x64, 256 threads (4x4 per thread, strided).
// Tc: compute type inside a chunk; every kChunk rows the chunk sum is added to FP64.
constexpr int GT = 64, GK = 16;

template <typename Tc>
__global__ void __launch_bounds__(256)
    gram_kernel(const double* __restrict__ A, int64_t lda, const double* __restrict__ B,
                int64_t ldb, int64_t K, int N1, int N2, double* __restrict__ C, int ldc,
                int64_t k_per_split, int ntj, int lower_only, int chunk) {
  __shared__ Tc As[GK][GT];
  __shared__ Tc Bs[GK][GT];
  const int tile = blockIdx.x;
  const int ti = tile / ntj, tj = tile % ntj;
  if (lower_only && tj > ti) return;
  const int i0 = ti * GT, j0 = tj * GT;
  const int64_t k_begin = (int64_t)blockIdx.y * k_per_split;
  const int64_t k_end = min(K, k_begin + k_per_split);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
  Tc part[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) acc[r][s] = 0.0, part[r][s] = (Tc)0;
  int since = 0;
  for (int64_t k0 = k_begin; k0 < k_end; k0 += GK) {
    for (int idx = threadIdx.x; idx < GK * GT; idx += 256) {
      const int k = idx / GT, c = idx % GT;
      const int64_t gk = k0 + k;
      As[k][c] = (gk < k_end && i0 + c < N1) ? (Tc)A[gk * lda + i0 + c] : (Tc)0;
      Bs[k][c] = (gk < k_end && j0 + c < N2) ? (Tc)B[gk * ldb + j0 + c] : (Tc)0;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GK; ++k) {
      Tc a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[k][ty + 16 * r];
#pragma unroll
      for (int s = 0; s < 4; ++s) b[s] = Bs[k][tx + 16 * s];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) part[r][s] = fma(a[r], b[s], part[r][s]);
    }
    __syncthreads();
    since += GK;
    if (since >= chunk) {
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) acc[r][s] += (double)part[r][s], part[r][s] = (Tc)0;
      since = 0;
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * s;
      if (i < N1 && j < N2) atomicAdd(&C[(int64_t)i * ldc + j], acc[r][s] + (double)part[r][s]);
    }
}

__global__ void __launch_bounds__(256)
    gram_kernel_c(const cplx* __restrict__ A, int64_t lda, const cplx* __restrict__ B, int64_t ldb,
                  int64_t K, int N1, int N2, cplx* __restrict__ C, int ldc, int64_t k_per_split,
                  int ntj, int lower_only) {
  constexpr int T = 32;
  __shared__ cplx As[GK][T];
  __shared__ cplx Bs[GK][T];
  const int tile = blockIdx.x;
  const int ti = tile / ntj, tj = tile % ntj;
  if (lower_only && tj > ti) return;
  const int i0 = ti * T, j0 = tj * T;
  const int64_t k_begin = (int64_t)blockIdx.y * k_per_split;
  const int64_t k_end = min(K, k_begin + k_per_split);
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2x2 per thread
  cplx acc[2][2];
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) acc[r][s] = {0.0, 0.0};
  for (int64_t k0 = k_begin; k0 < k_end; k0 += GK) {
    for (int idx = threadIdx.x; idx < GK * T; idx += 256) {
      const int k = idx / T, c = idx % T;
      const int64_t gk = k0 + k;
      As[k][c] = (gk < k_end && i0 + c < N1) ? A[gk * lda + i0 + c] : cplx{0.0, 0.0};
      Bs[k][c] = (gk < k_end && j0 + c < N2) ? B[gk * ldb + j0 + c] : cplx{0.0, 0.0};
    }
    __syncthreads();
    for (int k = 0; k < GK; ++k)
      for (int r = 0; r < 2; ++r)
        for (int s = 0; s < 2; ++s)
          acc[r][s] = cadd(acc[r][s], cmul(cconj(As[k][ty + 16 * r]), Bs[k][tx + 16 * s]));
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * s;
      if (i < N1 && j < N2) {
        atomicAdd(&C[(int64_t)i * ldc + j].x, acc[r][s].x);
        atomicAdd(&C[(int64_t)i * ldc + j].y, acc[r][s].y);
      }
    }
}

static int64_t choose_split(int64_t K, int tiles, int64_t min_rows) {
  int64_t want = std::max<int64_t>(1, (int64_t)kNumSMs * 4 / std::max(1, tiles));
  int64_t per = (K + want - 1) / want;
  per = std::max<int64_t>(per, min_rows);
  per = (per + GK - 1) / GK * GK;
  return per;
}

static void gemm32(bool ta, bool tb, int64_t M, int N, int64_t K, double alpha, const double* A,
                   int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, bool split,
                   bool lower_only, cudaStream_t st);

// C (N1 x N2) += A^T B with FP32 products, FP64 across chunks (split K, atomics)
static void gram32(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t K, int N1,
                   int N2, double* C, int ldc, bool lower_only, cudaStream_t st) {
  gemm32(true, false, N1, N2, K, 1.0, A, lda, B, ldb, C, ldc, true, lower_only && N1 == N2, st);
}

void gram_f64(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t K, int N1,
              int N2, double* C, int ldc, int prec, bool lower_only, cudaStream_t st) {
  const int nti = (N1 + GT - 1) / GT, ntj = (N2 + GT - 1) / GT;
  const int tiles = lower_only ? nti * (nti + 1) / 2 : nti * ntj;
  const int64_t per = choose_split(K, tiles, 256);
  const int64_t splits = (K + per - 1) / per;
  CHEFSI_REQUIRE(splits < 65536, "gram split too large");
  dim3 grid(nti * ntj, (unsigned)splits);
  if (prec == CHEFSI_PREC_FP64) {
    gram_kernel<double><<<grid, 256, 0, st>>>(A, lda, B, ldb, K, N1, N2, C, ldc, per, ntj,
                                              lower_only, 1 << 30);
    CHEFSI_CHECK_LAUNCH();
  } else if (prec == CHEFSI_PREC_MIXED && dense_tc_available()) {
    gram_tc_f64(A, lda, B, ldb, K, N1, N2, C, ldc, lower_only, st);
  } else {
    gram32(A, lda, B, ldb, K, N1, N2, C, ldc, lower_only, st);
  }
}

void gram_c64(const cplx* A, int64_t lda, const cplx* B, int64_t ldb, int64_t K, int N1, int N2,
              cplx* C, int ldc, bool lower_only, cudaStream_t st) {
  const int nti = (N1 + 31) / 32, ntj = (N2 + 31) / 32;
  const int tiles = lower_only ? nti * (nti + 1) / 2 : nti * ntj;
  const int64_t per = choose_split(K, tiles, 256);
  const int64_t splits = (K + per - 1) / per;
  CHEFSI_REQUIRE(splits < 65536, "gram split too large");
  dim3 grid(nti * ntj, (unsigned)splits);
  gram_kernel_c<<<grid, 256, 0, st>>>(A, lda, B, ldb, K, N1, N2, C, ldc, per, ntj, lower_only);
  CHEFSI_CHECK_LAUNCH();
}

// ======================================================================= GEMM
// C[M][N] = alpha op(A) op(B) + beta C, row-major. op(A)[m][k] = ta=='N' ? A[m][k] : A[k][m].
// Split K (part != nullptr): CTA z sums k in [z kc, (z+1) kc) and writes the raw sum to
// part[z][M][N]; k_splitk_reduce forms C.
template <typename Tc>
__global__ void __launch_bounds__(256)
    gemm_kernel(int ta, int tb, int64_t M, int N, int K, double alpha,
                const double* __restrict__ A, int64_t lda, const double* __restrict__ B,
                int64_t ldb, double beta, double* __restrict__ C, int64_t ldc, int chunk,
                int kc = 0, double* __restrict__ part = nullptr) {
  __shared__ Tc As[GK][GT + 1];
  __shared__ Tc Bs[GK][GT];
  const int64_t m0 = (int64_t)blockIdx.x * GT;
  const int n0 = blockIdx.y * GT;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[4][4];
  Tc partc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) acc[r][s] = 0.0, partc[r][s] = (Tc)0;
  int since = 0;
  const int kbeg = part ? blockIdx.z * kc : 0;
  const int kend = part ? min(K, kbeg + kc) : K;
  for (int k0 = kbeg; k0 < kend; k0 += GK) {
    for (int idx = threadIdx.x; idx < GK * GT; idx += 256) {
      int k, mm;
      if (ta) {  // A is [K][M]: contiguous along m
        k = idx / GT, mm = idx % GT;
      } else {  // A is [M][K]: contiguous along k
        mm = idx / GK, k = idx % GK;
      }
      const int64_t gm = m0 + mm;
      const int gk = k0 + k;
      double v = 0.0;
      if (gm < M && gk < kend) v = ta ? A[(int64_t)gk * lda + gm] : A[gm * lda + gk];
      As[k][mm] = (Tc)v;
    }
    for (int idx = threadIdx.x; idx < GK * GT; idx += 256) {
      int k, nn;
      if (tb) {  // B is [N][K]
        nn = idx / GK, k = idx % GK;
      } else {  // B is [K][N]
        k = idx / GT, nn = idx % GT;
      }
      const int gn = n0 + nn, gk = k0 + k;
      double v = 0.0;
      if (gn < N && gk < kend) v = tb ? B[(int64_t)gn * ldb + gk] : B[(int64_t)gk * ldb + gn];
      Bs[k][nn] = (Tc)v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < GK; ++k) {
      Tc a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[k][ty + 16 * r];
#pragma unroll
      for (int s = 0; s < 4; ++s) b[s] = Bs[k][tx + 16 * s];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) partc[r][s] = fma(a[r], b[s], partc[r][s]);
    }
    __syncthreads();
    since += GK;
    if (since >= chunk) {
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int s = 0; s < 4; ++s) acc[r][s] += (double)partc[r][s], partc[r][s] = (Tc)0;
      since = 0;
    }
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int64_t m = m0 + ty + 16 * r;
      const int n = n0 + tx + 16 * s;
      if (m < M && n < N) {
        if (part) {
          part[((int64_t)blockIdx.z * M + m) * N + n] = acc[r][s] + (double)partc[r][s];
        } else {
          const double v = alpha * (acc[r][s] + (double)partc[r][s]);
          double* c = &C[m * ldc + n];
          *c = (beta == 0.0) ? v : v + beta * *c;
        }
      }
    }
}

// C = alpha sum_z part[z] + beta C (fixed order over the K slices)
__global__ void k_splitk_reduce(const double* __restrict__ part, int S, int64_t M, int N,
                                double alpha, double beta, double* __restrict__ C, int64_t ldc) {
  const int64_t n = M * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int z = 0; z < S; ++z) v += part[z * n + t];
    const int64_t m = t / N;
    double* c = &C[m * ldc + (t - m * N)];
    *c = (beta == 0.0) ? alpha * v : alpha * v + beta * *c;
  }
}

void gemm_f64(char ta, char tb, int64_t M, int N, int K, double alpha, const double* A, int64_t lda,
              const double* B, int64_t ldb, double beta, double* C, int64_t ldc, int prec,
              cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((unsigned)((M + GT - 1) / GT), (N + GT - 1) / GT);
  CHEFSI_REQUIRE(grid.y < 65536, "gemm N too large");
  const int ita = (ta == 'T' || ta == 't' || ta == 'C' || ta == 'c');
  const int itb = (tb == 'T' || tb == 't' || tb == 'C' || tb == 'c');
  if (prec == CHEFSI_PREC_FP64) {
    // a 64 x 64 tile runs its whole K loop on one SM (~2 FP64 FMAs per clock): with few tiles
    // and a long K, the K range is split over CTAs and the slices are summed in fixed order
    const int64_t tiles = (int64_t)grid.x * grid.y;
    int S = 1;
    if (tiles < kNumSMs / 2 && K >= 8 * GK) {
      S = (int)std::min<int64_t>((2 * kNumSMs) / tiles, K / (4 * GK));
      S = std::max(1, std::min(S, 64));
    }
    if (S > 1) {
      const int kc = ((K + S - 1) / S + GK - 1) / GK * GK;
      S = (K + kc - 1) / kc;
      double* part = nullptr;
      CHEFSI_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&part), sizeof(double) * S * M * N, st));
      dim3 g3(grid.x, grid.y, (unsigned)S);
      gemm_kernel<double><<<g3, 256, 0, st>>>(ita, itb, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                              ldc, 1 << 30, kc, part);
      CHEFSI_CHECK_LAUNCH();
      k_splitk_reduce<<<grid_for(M * N, 256), 256, 0, st>>>(part, S, M, N, alpha, beta, C, ldc);
      CHEFSI_CHECK_LAUNCH();
      CHEFSI_CUDA(cudaFreeAsync(part, st));
      return;
    }
    gemm_kernel<double><<<grid, 256, 0, st>>>(ita, itb, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                              ldc, 1 << 30);
    CHEFSI_CHECK_LAUNCH();
  } else if (prec == CHEFSI_PREC_MIXED && alpha == 1.0 && beta == 0.0 && !itb && K >= 1 &&
             dense_tc_available()) {
    // the two shapes of the Rayleigh-Ritz step on tensor cores: A^T B over a long K (Gram)
    // and A B with a long M (rotation)
    if (ita) {
      CHEFSI_CUDA(cudaMemset2DAsync(C, sizeof(double) * ldc, 0, sizeof(double) * N, M, st));
      gram_tc_f64(A, lda, B, ldb, K, (int)M, N, C, (int)ldc, false, st);
    } else {
      rotate_tc_f64(A, lda, M, K, B, ldb, N, C, ldc, st);
    }
  } else if (beta == 0.0) {
    gemm32(ita != 0, itb != 0, M, N, K, alpha, A, lda, B, ldb, C, ldc, false, false, st);
  } else {
    gemm_kernel<float><<<grid, 256, 0, st>>>(ita, itb, M, N, K, alpha, A, lda, B, ldb, beta, C,
                                             ldc, 256);
    CHEFSI_CHECK_LAUNCH();
  }
}

// complex GEMM (FP64), 32x32 tiles, 2x2 per thread
__global__ void __launch_bounds__(256)
    gemm_kernel_c(int ta, int tb, int64_t M, int N, int K, cplx alpha, const cplx* __restrict__ A,
                  int64_t lda, const cplx* __restrict__ B, int64_t ldb, cplx beta,
                  cplx* __restrict__ C, int64_t ldc) {
  constexpr int T = 32;
  __shared__ cplx As[GK][T + 1];
  __shared__ cplx Bs[GK][T];
  const int64_t m0 = (int64_t)blockIdx.x * T;
  const int n0 = blockIdx.y * T;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  cplx acc[2][2];
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) acc[r][s] = {0.0, 0.0};
  for (int k0 = 0; k0 < K; k0 += GK) {
    for (int idx = threadIdx.x; idx < GK * T; idx += 256) {
      const int k = idx / T, mm = idx % T;
      const int64_t gm = m0 + mm;
      const int gk = k0 + k;
      cplx v = {0.0, 0.0};
      if (gm < M && gk < K) v = ta ? cconj(A[(int64_t)gk * lda + gm]) : A[gm * lda + gk];
      As[k][mm] = v;
      const int gn = n0 + mm;
      cplx w = {0.0, 0.0};
      if (gn < N && gk < K) w = tb ? cconj(B[(int64_t)gn * ldb + gk]) : B[(int64_t)gk * ldb + gn];
      Bs[k][mm] = w;
    }
    __syncthreads();
    for (int k = 0; k < GK; ++k)
      for (int r = 0; r < 2; ++r)
        for (int s = 0; s < 2; ++s)
          acc[r][s] = cadd(acc[r][s], cmul(As[k][ty + 16 * r], Bs[k][tx + 16 * s]));
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int64_t m = m0 + ty + 16 * r;
      const int n = n0 + tx + 16 * s;
      if (m < M && n < N) {
        cplx v = cmul(alpha, acc[r][s]);
        cplx* c = &C[m * ldc + n];
        if (beta.x != 0.0 || beta.y != 0.0) v = cadd(v, cmul(beta, *c));
        *c = v;
      }
    }
}

void gemm_c64(char ta, char tb, int64_t M, int N, int K, cplx alpha, const cplx* A, int64_t lda,
              const cplx* B, int64_t ldb, cplx beta, cplx* C, int64_t ldc, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  dim3 grid((unsigned)((M + 31) / 32), (N + 31) / 32);
  const int ita = (ta != 'N' && ta != 'n');
  const int itb = (tb != 'N' && tb != 'n');
  gemm_kernel_c<<<grid, 256, 0, st>>>(ita, itb, M, N, K, alpha, A, lda, B, ldb, beta, C, ldc);
  CHEFSI_CHECK_LAUNCH();
}

// ======================================================================= FP32 GEMM (mixed)
// C[M][N] (+)= alpha op(A) op(B) over the K range of this CTA, FP64 operands converted to FP32
// on load. 128x128 CTA tile, K-tile 8, 256 threads with an 8x8 register tile (two 4x4 quads
// 64 rows / columns apart, so the shared-memory reads are float4 and conflict-free), register
// double buffering of the next K-tile, FP32 products inside chunks of kChunk32 K-steps and FP64
// accumulation across chunks. split != 0: atomicAdd into C (split-K Gram products).
constexpr int kBM = 128, kBN = 128, kBK = 8, kChunk32 = 512;

template <bool TA, bool TB>
__global__ void __launch_bounds__(256, 1)
    gemm32_kernel(int64_t M, int N, int64_t K, double alpha, const double* __restrict__ A,
                  int64_t lda, const double* __restrict__ B, int64_t ldb, double* __restrict__ C,
                  int64_t ldc, int64_t k_per_split, int atomic_out, int ntn, int lower_only) {
  __shared__ __align__(16) float As[2][kBK][kBM + 4];
  __shared__ __align__(16) float Bs[2][kBK][kBN + 4];
  const int64_t tile = blockIdx.x;
  const int tn = (int)(tile % ntn);
  const int64_t tm = tile / ntn;
  if (lower_only && tn > tm) return;
  const int64_t m0 = tm * kBM;
  const int n0 = tn * kBN;
  const int64_t k_begin = (int64_t)blockIdx.y * k_per_split;
  const int64_t k_end = min(K, k_begin + k_per_split);
  const int t = threadIdx.x;
  const int tx = t % 16, ty = t / 16;

  // global -> register loads of one K-tile (4 A values, 4 B values per thread)
  double ra[4], rb[4];
  auto load = [&](int64_t k0) {
    if (TA) {  // A is [K][M]: 8 rows of 128 contiguous
      const int kk = t / 32, mm = (t % 32) * 4;
      const int64_t gk = k0 + kk;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        ra[i] = (gk < k_end && m0 + mm + i < M) ? A[gk * lda + m0 + mm + i] : 0.0;
    } else {   // A is [M][K]: 128 rows of 8 contiguous
      const int mm = t / 2, kk = (t % 2) * 4;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        ra[i] = (m0 + mm < M && k0 + kk + i < k_end) ? A[(m0 + mm) * lda + k0 + kk + i] : 0.0;
    }
    if (!TB) {  // B is [K][N]
      const int kk = t / 32, nn = (t % 32) * 4;
      const int64_t gk = k0 + kk;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        rb[i] = (gk < k_end && n0 + nn + i < N) ? B[gk * ldb + n0 + nn + i] : 0.0;
    } else {    // B is [N][K]
      const int nn = t / 2, kk = (t % 2) * 4;
#pragma unroll
      for (int i = 0; i < 4; ++i)
        rb[i] = (n0 + nn < N && k0 + kk + i < k_end) ? B[(int64_t)(n0 + nn) * ldb + k0 + kk + i] : 0.0;
    }
  };
  auto store = [&](int buf) {
    if (TA) {
      const int kk = t / 32, mm = (t % 32) * 4;
      *reinterpret_cast<float4*>(&As[buf][kk][mm]) =
          make_float4((float)ra[0], (float)ra[1], (float)ra[2], (float)ra[3]);
    } else {
      const int mm = t / 2, kk = (t % 2) * 4;
#pragma unroll
      for (int i = 0; i < 4; ++i) As[buf][kk + i][mm] = (float)ra[i];
    }
    if (!TB) {
      const int kk = t / 32, nn = (t % 32) * 4;
      *reinterpret_cast<float4*>(&Bs[buf][kk][nn]) =
          make_float4((float)rb[0], (float)rb[1], (float)rb[2], (float)rb[3]);
    } else {
      const int nn = t / 2, kk = (t % 2) * 4;
#pragma unroll
      for (int i = 0; i < 4; ++i) Bs[buf][kk + i][nn] = (float)rb[i];
    }
  };

  // FP64 chunk sums live in shared memory ([64][256], thread-fastest: conflict-free)
  extern __shared__ double acc64s[];
  float acc[8][8];
#pragma unroll
  for (int i = 0; i < 8; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.f, acc64s[(i * 8 + j) * 256 + t] = 0.0;

  int buf = 0;
  if (k_begin < k_end) {
    load(k_begin);
    store(0);
  }
  __syncthreads();
  int since = 0;
  for (int64_t k0 = k_begin; k0 < k_end; k0 += kBK) {
    const bool more = k0 + kBK < k_end;
    if (more) load(k0 + kBK);
#pragma unroll
    for (int kk = 0; kk < kBK; ++kk) {
      const float4 a0 = *reinterpret_cast<const float4*>(&As[buf][kk][ty * 4]);
      const float4 a1 = *reinterpret_cast<const float4*>(&As[buf][kk][64 + ty * 4]);
      const float4 b0 = *reinterpret_cast<const float4*>(&Bs[buf][kk][tx * 4]);
      const float4 b1 = *reinterpret_cast<const float4*>(&Bs[buf][kk][64 + tx * 4]);
      const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
      const float bv[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
    }
    if (more) store(buf ^ 1);
    __syncthreads();
    buf ^= 1;
    since += kBK;
    if (since >= kChunk32) {
#pragma unroll
      for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc64s[(i * 8 + j) * 256 + t] += (double)acc[i][j], acc[i][j] = 0.f;
      since = 0;
    }
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int64_t m = m0 + (i < 4 ? ty * 4 + i : 64 + ty * 4 + i - 4);
    if (m >= M) continue;
#pragma unroll
    for (int j = 0; j < 8; ++j) {
      const int n = n0 + (j < 4 ? tx * 4 + j : 64 + tx * 4 + j - 4);
      if (n >= N) continue;
      const double v = alpha * (acc64s[(i * 8 + j) * 256 + t] + (double)acc[i][j]);
      if (atomic_out)
        atomicAdd(&C[m * ldc + n], v);
      else
        C[m * ldc + n] = v;
    }
  }
}

// mixed-precision GEMM entry: C = alpha op(A) op(B) (atomic == false, beta = 0) or split-K
// accumulation C += alpha A^T B (gram, atomic == true)
static void gemm32(bool ta, bool tb, int64_t M, int N, int64_t K, double alpha, const double* A,
                   int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, bool split,
                   bool lower_only, cudaStream_t st) {
  const int ntn = (N + kBN - 1) / kBN;
  const int64_t ntm = (M + kBM - 1) / kBM;
  const int64_t tiles = ntm * ntn;
  int64_t per = K, splits = 1;
  if (split) {
    const int64_t live = lower_only ? ntm * (ntm + 1) / 2 : tiles;
    int64_t want = std::max<int64_t>(1, (int64_t)kNumSMs * 2 / std::max<int64_t>(1, live));
    per = std::max<int64_t>(kChunk32, (K + want - 1) / want);
    per = (per + kBK - 1) / kBK * kBK;
    splits = (K + per - 1) / per;
  }
  CHEFSI_REQUIRE(tiles < (1ll << 31) && splits < 65536, "gemm32 grid too large");
  dim3 grid((unsigned)tiles, (unsigned)splits);
  const int atomic = split ? 1 : 0;
  const int lo = lower_only ? 1 : 0;
  const size_t dyn = 64 * 256 * sizeof(double);
  static bool attr = false;
  if (!attr) {
    CHEFSI_CUDA(cudaFuncSetAttribute(gemm32_kernel<true, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    CHEFSI_CUDA(cudaFuncSetAttribute(gemm32_kernel<false, false>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    CHEFSI_CUDA(cudaFuncSetAttribute(gemm32_kernel<false, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    CHEFSI_CUDA(cudaFuncSetAttribute(gemm32_kernel<true, true>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
    attr = true;
  }
  if (ta && !tb)
    gemm32_kernel<true, false><<<grid, 256, dyn, st>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, per,
                                                       atomic, ntn, lo);
  else if (!ta && !tb)
    gemm32_kernel<false, false><<<grid, 256, dyn, st>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, per,
                                                        atomic, ntn, lo);
  else if (!ta && tb)
    gemm32_kernel<false, true><<<grid, 256, dyn, st>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, per,
                                                       atomic, ntn, lo);
  else
    gemm32_kernel<true, true><<<grid, 256, dyn, st>>>(M, N, K, alpha, A, lda, B, ldb, C, ldc, per,
                                                      atomic, ntn, lo);
  CHEFSI_CHECK_LAUNCH();
}

// ======================================================================= small helpers
__global__ void k_symmetrize_lower(double* A, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / N), j = (int)(t % N);
    if (j > i) A[t] = A[(int64_t)j * N + i];
  }
}
void symmetrize_lower(double* A, int N, cudaStream_t st) {
  k_symmetrize_lower<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(A, N);
  CHEFSI_CHECK_LAUNCH();
}
__global__ void k_symmetrize_lower_c(cplx* A, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / N), j = (int)(t % N);
    if (j > i) A[t] = cconj(A[(int64_t)j * N + i]);
    if (j == i) A[t].y = 0.0;
  }
}
void symmetrize_lower_c(cplx* A, int N, cudaStream_t st) {
  k_symmetrize_lower_c<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(A, N);
  CHEFSI_CHECK_LAUNCH();
}

// ======================================================================= Cholesky
constexpr int CB = 32;

// unblocked Cholesky of the nb x nb diagonal block at (k0, k0); flag set on a bad pivot
__global__ void k_potf2(double* A, int N, int k0, int nb, int* info) {
  __shared__ double L[CB][CB + 1];
  const int t = threadIdx.x;  // CB threads
  for (int i = 0; i < nb; ++i)
    if (t < nb) L[i][t] = A[(int64_t)(k0 + i) * N + k0 + t];
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (t == 0) {
      const double djj = L[j][j];
      if (!(djj > 0.0) || !isfinite(djj)) {
        atomicCAS(info, 0, k0 + j + 1);
        L[j][j] = 1.0;
      } else {
        L[j][j] = sqrt(djj);
      }
    }
    __syncthreads();
    if (t > j && t < nb) L[t][j] /= L[j][j];
    __syncthreads();
    // trailing update of the lower part, column by column
    if (t > j && t < nb)
      for (int i = t; i < nb; ++i) L[i][t] -= L[i][j] * L[t][j];
    __syncthreads();
  }
  for (int i = 0; i < nb; ++i)
    if (t < nb) A[(int64_t)(k0 + i) * N + k0 + t] = (t <= i) ? L[i][t] : 0.0;
}

// rows r >= k0+nb: A[r][k0:k0+nb] <- A[r][k0:k0+nb] L11^{-T}
__global__ void k_trsm_panel(double* A, int N, int k0, int nb) {
  __shared__ double L[CB][CB + 1];
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x)
    L[idx / nb][idx % nb] = A[(int64_t)(k0 + idx / nb) * N + k0 + idx % nb];
  __syncthreads();
  const int r = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  double x[CB];
  double* row = A + (int64_t)r * N + k0;
  for (int j = 0; j < nb; ++j) {
    double v = row[j];
    for (int l = 0; l < j; ++l) v -= x[l] * L[j][l];
    x[j] = v / L[j][j];
  }
  for (int j = 0; j < nb; ++j) row[j] = x[j];
}

__global__ void k_zero_upper(double* A, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    if ((int)(t % N) > (int)(t / N)) A[t] = 0.0;
}

int cholesky_lower(double* A, int N, cudaStream_t st) {
  DeviceBuffer<int> info(1);
  CHEFSI_CUDA(cudaMemsetAsync(info.ptr, 0, sizeof(int), st));
  for (int k0 = 0; k0 < N; k0 += CB) {
    const int nb = std::min(CB, N - k0);
    k_potf2<<<1, CB, 0, st>>>(A, N, k0, nb, info.ptr);
    CHEFSI_CHECK_LAUNCH();
    const int rest = N - k0 - nb;
    if (rest > 0) {
      k_trsm_panel<<<(rest + 127) / 128, 128, 0, st>>>(A, N, k0, nb);
      CHEFSI_CHECK_LAUNCH();
      // A22 -= L21 L21^T (full trailing square; the upper part is zeroed at the end)
      const int64_t off = (int64_t)(k0 + nb) * N;
      gemm_f64('N', 'T', rest, rest, nb, -1.0, A + off + k0, N, A + off + k0, N, 1.0,
               A + off + k0 + nb, N, CHEFSI_PREC_FP64, st);
    }
  }
  k_zero_upper<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(A, N);
  CHEFSI_CHECK_LAUNCH();
  int h = 0;
  CHEFSI_CUDA(cudaMemcpyAsync(&h, info.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  return h ? CHEFSI_ERR_NOT_SPD : CHEFSI_OK;
}

// ======================================================================= triangular inverse
// invert each CB x CB diagonal block of the lower-triangular L in place
__global__ void k_trtri_diag(double* L, int N) {
  __shared__ double T[CB][CB + 1];
  __shared__ double Z[CB][CB + 1];
  const int k0 = blockIdx.x * CB;
  const int nb = min(CB, N - k0);
  const int t = threadIdx.x;
  for (int i = 0; i < nb; ++i)
    if (t < nb) T[i][t] = L[(int64_t)(k0 + i) * N + k0 + t], Z[i][t] = 0.0;
  __syncthreads();
  // column t of the inverse by forward substitution
  if (t < nb) {
    for (int i = 0; i < nb; ++i) {
      double v = (i == t) ? 1.0 : 0.0;
      for (int l = t; l < i; ++l) v -= T[i][l] * Z[l][t];
      Z[i][t] = (i >= t) ? v / T[i][i] : 0.0;
    }
  }
  __syncthreads();
  for (int i = 0; i < nb; ++i)
    if (t < nb) L[(int64_t)(k0 + i) * N + k0 + t] = Z[i][t];
}

void trtri_lower(double* L, int N, cudaStream_t st) {
  const int nblk = (N + CB - 1) / CB;
  // Z = L^{-1}: first invert diagonal blocks, then block rows top-down:
  // Z[i, 0:i] = -Z_ii * (L[i, 0:i] * Z[0:i, 0:i])
  k_trtri_diag<<<nblk, CB, 0, st>>>(L, N);
  CHEFSI_CHECK_LAUNCH();
  DeviceBuffer<double> tmp((size_t)CB * N);
  for (int bi = 1; bi < nblk; ++bi) {
    const int r0 = bi * CB;
    const int nb = std::min(CB, N - r0);
    // tmp[nb][r0] = L[r0:r0+nb, 0:r0] * Z[0:r0, 0:r0]
    gemm_f64('N', 'N', nb, r0, r0, 1.0, L + (int64_t)r0 * N, N, L, N, 0.0, tmp.ptr, r0,
             CHEFSI_PREC_FP64, st);
    // L[r0:r0+nb, 0:r0] = -Z_ii * tmp
    gemm_f64('N', 'N', nb, r0, nb, -1.0, L + (int64_t)r0 * N + r0, N, tmp.ptr, r0, 0.0,
             L + (int64_t)r0 * N, N, CHEFSI_PREC_FP64, st);
  }
}

// ======================================================================= eigensolver
// The eigensolver kernels read and write the same work arrays through derived pointers; they
// carry no __restrict__ qualifiers (with them, nvcc produced wrong inverse-iteration vectors
// on sm_103a while the identical host build was exact).
// Householder step k on the symmetric row-major A (full storage maintained):
// x = A[k+1:N, k]; v = x - alpha e1 with alpha = -sign(x0) |x|; tau = 2 / v^T v.
// The reflector is kept in V[k][k+1:N] with tau[k]; d[k] = A[k][k], e[k] = alpha.
__global__ void k_hh_vector(double* A, int N, int k, double* V, double* tau, double* d, double* e) {
  __shared__ double red[32];
  const int n = N - k - 1;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double x = A[(int64_t)(k + 1 + i) * N + k];
    s += x * x;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = (threadIdx.x < (blockDim.x + 31) / 32) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) red[0] = s;
  }
  __syncthreads();
  const double nrm2 = red[0];
  const double x0 = A[(int64_t)(k + 1) * N + k];
  const double nrm = sqrt(nrm2);
  const double alpha = (x0 >= 0.0) ? -nrm : nrm;
  // v^T v = nrm2 - 2 alpha x0 + alpha^2 = 2 (nrm2 - alpha x0)
  const double vtv = 2.0 * (nrm2 - alpha * x0);
  const bool skip = !(vtv > 0.0) || nrm == 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double x = A[(int64_t)(k + 1 + i) * N + k];
    V[(int64_t)k * N + k + 1 + i] = skip ? 0.0 : (i == 0 ? x - alpha : x);
  }
  if (threadIdx.x == 0) {
    tau[k] = skip ? 0.0 : 2.0 / vtv;
    d[k] = A[(int64_t)k * N + k];
    e[k] = skip ? x0 : alpha;
  }
}

// p = tau * A22 v   (one warp per row of the trailing block)
__global__ void k_hh_symv(const double* A, int N, int k, const double* V,
                          const double* tau, double* p) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int n = N - k - 1;
  if (warp >= n) return;
  const double* row = A + (int64_t)(k + 1 + warp) * N + k + 1;
  const double* v = V + (int64_t)k * N + k + 1;
  double s = 0.0;
  for (int j = lane; j < n; j += 32) s += row[j] * v[j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) p[warp] = tau[k] * s;
}

// w = p - (tau/2)(p^T v) v   (single CTA)
__global__ void k_hh_w(int N, int k, const double* V, const double* tau,
                       double* p) {
  __shared__ double red[32];
  const int n = N - k - 1;
  const double* v = V + (int64_t)k * N + k + 1;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += p[i] * v[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = (threadIdx.x < (blockDim.x + 31) / 32) ? red[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) red[0] = s;
  }
  __syncthreads();
  const double f = 0.5 * tau[k] * red[0];
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] -= f * v[i];
}

// A22 -= v w^T + w v^T
__global__ void k_hh_rank2(double* A, int N, int k, const double* V,
                           const double* w) {
  const int n = N - k - 1;
  const int64_t tot = (int64_t)n * n;
  const double* v = V + (int64_t)k * N + k + 1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    A[(int64_t)(k + 1 + i) * N + k + 1 + j] -= v[i] * w[j] + w[i] * v[j];
  }
}

__global__ void k_tail(const double* A, int N, double* d, double* e) {
  if (threadIdx.x == 0) {
    if (N >= 2) {
      d[N - 2] = A[(int64_t)(N - 2) * N + N - 2];
      e[N - 2] = A[(int64_t)(N - 1) * N + N - 2];
    }
    d[N - 1] = A[(int64_t)(N - 1) * N + N - 1];
  }
}

// number of eigenvalues of the tridiagonal (d, e) below x (Sturm sequence)
__device__ int sturm_count(const double* d, const double* e, int n, double x, double pivmin) {
  int cnt = 0;
  double q = d[0] - x;
  if (fabs(q) < pivmin) q = -pivmin;
  if (q < 0) ++cnt;
  for (int j = 1; j < n; ++j) {
    q = d[j] - x - e[j - 1] * e[j - 1] / q;
    if (fabs(q) < pivmin) q = -pivmin;
    if (q < 0) ++cnt;
  }
  return cnt;
}

// Eigenvalue idx of the tridiagonal (d, e) by multisection: one warp per eigenvalue, the 32
// lanes evaluate Sturm counts at 32 interior points of the current interval, which then
// shrinks to the sub-interval holding eigenvalue idx (a factor 33 per step, ~11 steps to
// full precision instead of ~55 bisection steps; every Sturm count is an FP64-division chain).
// Eigenvalues idx0 .. idx0+count-1 (ascending) go to w[0 .. count).
__global__ void k_bisect_warp(const double* d, const double* e, int n, int idx0, int count,
                              double* w) {
  const int sub = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (sub >= count) return;  // uniform within the warp
  const int idx = idx0 + sub;
  double lo = 1e300, hi = -1e300, emax = 0.0;
  for (int j = lane; j < n; j += 32) {
    const double r = (j > 0 ? fabs(e[j - 1]) : 0.0) + (j < n - 1 ? fabs(e[j]) : 0.0);
    lo = fmin(lo, d[j] - r);
    hi = fmax(hi, d[j] + r);
    if (j < n - 1) emax = fmax(emax, e[j] * e[j]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    emax = fmax(emax, __shfl_xor_sync(0xffffffffu, emax, o));
  }
  const double tnorm = fmax(fabs(lo), fabs(hi));
  const double pivmin = fmax(2.2250738585072014e-308 * fmax(emax, 1.0), 1e-300);
  lo -= 2.2e-16 * tnorm + pivmin;
  hi += 2.2e-16 * tnorm + pivmin;
  for (int it = 0; it < 64; ++it) {
    if (hi - lo <= 4.0 * 2.2e-16 * fmax(fabs(lo), fabs(hi)) + pivmin) break;
    const double x = lo + (hi - lo) * ((double)(lane + 1) / 33.0);
    const unsigned above = __ballot_sync(0xffffffffu, sturm_count(d, e, n, x, pivmin) > idx);
    const int first = above ? __ffs(above) - 1 : 32;  // eigenvalue in (x[first-1], x[first]]
    const double nlo = first > 0 ? __shfl_sync(0xffffffffu, x, first - 1) : lo;
    const double nhi = first < 32 ? __shfl_sync(0xffffffffu, x, first & 31) : hi;
    if (nlo == lo && nhi == hi) break;
    lo = nlo;
    hi = nhi;
  }
  if (lane == 0) w[sub] = 0.5 * (lo + hi);
}

// Inverse iteration for the eigenvectors of the tridiagonal (d, e): Gaussian elimination with
// partial pivoting of T - lam I (the scheme of LAPACK's dlagtf / dlagts; the U factor has a
// second super-diagonal where rows were swapped), five iterations from a deterministic start
// vector, modified Gram-Schmidt against earlier members of the same cluster (eigenvalues
// closer than ortol). One thread owns a whole cluster. Workspace per vector: 5n doubles.
// w holds count eigenvalues (ascending), eigenvalues idx0 .. idx0+count-1 of the whole
// tridiagonal; their vectors go to columns 0 .. count-1 of Z. The start vector depends on the
// global index, so a subset reproduces the columns of the full solve outside clusters that
// straddle the subset's edge.
__global__ void k_inverse_iteration(const double* d, const double* e,
                                    int n, const double* w, int count, int idx0, double* Z,
                                    int ldz, double* work, unsigned char* swaps,
                                    double ortol) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= count) return;
  // only the first member of a cluster works; it handles the whole cluster sequentially
  if (idx > 0 && w[idx] - w[idx - 1] <= ortol) return;
  int last = idx;
  while (last + 1 < count && w[last + 1] - w[last] <= ortol) ++last;
  double tnorm = 0.0;
  for (int j = 0; j < n; ++j)
    tnorm = fmax(tnorm, fabs(d[j]) + (j > 0 ? fabs(e[j - 1]) : 0.0) + (j < n - 1 ? fabs(e[j]) : 0.0));
  const double eps = 2.2e-16;
  const double tiny = eps * fmax(tnorm, 1e-300);
  double* a = work + (size_t)idx * 5 * n;
  double* b = a + n;
  double* c = b + n;
  double* c2 = c + n;
  double* x = c2 + n;
  unsigned char* sw = swaps + (size_t)idx * n;
  double prev_lam = -1e300;
  for (int t = idx; t <= last; ++t) {
    double lam = w[t];
    if (t > idx && lam - prev_lam < 10.0 * eps * fabs(lam)) lam = prev_lam + 10.0 * eps * fabs(lam);
    prev_lam = lam;
    // factor T - lam I with partial pivoting; record swaps
    for (int j = 0; j < n; ++j) a[j] = d[j] - lam;
    for (int j = 0; j < n - 1; ++j) b[j] = e[j], c2[j] = 0.0;
    for (int j = 0; j < n - 1; ++j) {
      const double sub = e[j];
      if (fabs(a[j]) >= fabs(sub)) {
        if (a[j] == 0.0) a[j] = tiny;
        const double m = sub / a[j];
        c[j] = m;
        a[j + 1] -= m * b[j];
        sw[j] = 0;
      } else {
        const double m = a[j] / sub;
        const double bj = b[j];
        const double bj1 = (j + 1 < n - 1) ? b[j + 1] : 0.0;
        a[j] = sub;
        b[j] = a[j + 1];
        c2[j] = bj1;
        a[j + 1] = bj - m * b[j];
        if (j + 1 < n - 1) b[j + 1] = -m * bj1;
        c[j] = m;
        sw[j] = 1;
      }
    }
    if (a[n - 1] == 0.0) a[n - 1] = tiny;
    // deterministic start vector
    unsigned int s = 2654435761u * (unsigned)(idx0 + t + 1);
    for (int j = 0; j < n; ++j) {
      s = s * 1664525u + 1013904223u;
      x[j] = ((double)(s >> 8) / 16777216.0) - 0.5 + 1e-3;
    }
    for (int iter = 0; iter < 5; ++iter) {
      // forward: apply L^{-1} with the recorded swaps
      for (int j = 0; j < n - 1; ++j) {
        if (sw[j]) {
          const double tmp = x[j];
          x[j] = x[j + 1];
          x[j + 1] = tmp - c[j] * x[j];
        } else {
          x[j + 1] -= c[j] * x[j];
        }
      }
      // backward: U x = y, U has diag a, super b, second super c2
      x[n - 1] /= a[n - 1];
      if (n >= 2) x[n - 2] = (x[n - 2] - b[n - 2] * x[n - 1]) / a[n - 2];
      for (int j = n - 3; j >= 0; --j) x[j] = (x[j] - b[j] * x[j + 1] - c2[j] * x[j + 2]) / a[j];
      // orthogonalise against earlier members of the cluster (MGS)
      for (int q = idx; q < t; ++q) {
        double dot = 0.0;
        for (int j = 0; j < n; ++j) dot += Z[(int64_t)j * ldz + q] * x[j];
        for (int j = 0; j < n; ++j) x[j] -= dot * Z[(int64_t)j * ldz + q];
      }
      double nrm = 0.0;
      for (int j = 0; j < n; ++j) nrm += x[j] * x[j];
      nrm = sqrt(nrm);
      if (!(nrm > 0.0)) nrm = 1.0;
      for (int j = 0; j < n; ++j) x[j] /= nrm;
    }
    for (int j = 0; j < n; ++j) Z[(int64_t)j * ldz + t] = x[j];
  }
}

// r[j] = v^T Z[:, j] over rows k+1..N-1
__global__ void k_bt_dot(const double* V, int N, int k, const double* Z,
                         double* r) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const double* v = V + (int64_t)k * N;
  double s = 0.0;
  for (int i = k + 1; i < N; ++i) s += v[i] * Z[(int64_t)i * N + j];
  r[j] = s;
}
__global__ void k_bt_update(const double* V, int N, int k,
                            const double* tau, double* Z,
                            const double* r) {
  const int n = N - k - 1;
  const int64_t tot = (int64_t)n * N;
  const double* v = V + (int64_t)k * N;
  const double t = tau[k];
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < tot;
       q += (int64_t)gridDim.x * blockDim.x) {
    const int i = k + 1 + (int)(q / N), j = (int)(q % N);
    Z[(int64_t)i * N + j] -= t * v[i] * r[j];
  }
}

// ---------------------------------------------------------------- fused tridiagonalisation
// The whole Householder reduction in one cooperative launch (all CTAs co-resident) instead
// of four launches per column: per column, CTA 0 forms the reflector, all CTAs compute
// p = tau A22 v over their rows, then each CTA forms w = p - (tau/2)(v^T p) v itself and
// applies the rank-2 update to its rows; three grid barriers per column. The barrier is a
// counter plus a generation word with a bounded wait: on expiry the CTA records
// CHEFSI_ERR_TIMEOUT and every CTA leaves (the host reads the flag).
struct GridSync {
  unsigned int* count;
  unsigned int* gen;
  int* err;
};
// polls of a grid-barrier wait before it expires (lowered by chefsi_set_wait_limits in tests)
static __device__ uint32_t g_barrier_spins = 1u << 26;

__device__ __forceinline__ bool grid_barrier(const GridSync& gs, unsigned int nblocks) {
  __shared__ int fail;
  __syncthreads();
  if (threadIdx.x == 0) {
    fail = 0;
    // the limit is loaded ahead of the atomics (its latency overlaps theirs)
    const uint32_t spins = g_barrier_spins;
    const unsigned int g = atomicAdd(gs.gen, 0u);
    __threadfence();
    if (atomicAdd(gs.count, 1u) == nblocks - 1) {
      atomicExch(gs.count, 0u);
      __threadfence();
      atomicAdd(gs.gen, 1u);
    } else {
      uint32_t i = 0;
      for (; i < spins; ++i) {
        if (*reinterpret_cast<volatile unsigned int*>(gs.gen) != g) break;
        if (*reinterpret_cast<volatile int*>(gs.err) != 0) break;
        if (i > 32) __nanosleep(32);
      }
      if (i == spins) atomicExch(gs.err, CHEFSI_ERR_TIMEOUT);
    }
    __threadfence();
    fail = *reinterpret_cast<volatile int*>(gs.err) != 0;
  }
  __syncthreads();
  return fail == 0;
}

__device__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

// One cooperative launch for the whole tridiagonalisation, two grid barriers per reflector.
// Step k: every active CTA loads column k below the diagonal into shared memory and forms the
// reflector itself (norm, alpha, tau: no separate vector phase), the CTAs' warps compute
// p = tau A22 v one row per warp; after a barrier every CTA forms f = tau/2 v^T p and updates
// its rows of A22 -= v w^T + w v^T (w = p - f v); barrier. CTA 0 also stores the reflector,
// tau, d and e. A CTA leaves once the trailing size needs fewer CTAs (one row per warp), so
// the late barriers have fewer participants; every barrier is bounded.
__global__ void __launch_bounds__(256)
    k_tridiag_fused(double* A, int N, double* V, double* tau, double* d, double* e, double* p,
                    GridSync gs) {
  extern __shared__ double vs[];     // [N] the current reflector
  __shared__ double red[32];
  const int warps_per_cta = blockDim.x >> 5;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = 0; k + 2 < N; ++k) {
    const int n = N - k - 1;
    const unsigned int active =
        min(gridDim.x, (unsigned)max(1, (n + warps_per_cta - 1) / warps_per_cta));
    if (blockIdx.x >= active) return;   // never needed again: active does not grow
    // the reflector from column k (rows k+1..N-1), in every CTA
    double s = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
      const double x = A[(int64_t)(k + 1 + i) * N + k];
      vs[i] = x;
      s += x * x;
    }
    const double nrm2 = block_sum(s, red);
    const double x0 = vs[0];
    const double nrm = sqrt(nrm2);
    const double alpha = (x0 >= 0.0) ? -nrm : nrm;
    const double vtv = 2.0 * (nrm2 - alpha * x0);
    const bool skip = !(vtv > 0.0) || nrm == 0.0;
    const double tk = skip ? 0.0 : 2.0 / vtv;
    __syncthreads();
    if (threadIdx.x == 0) vs[0] = skip ? 0.0 : x0 - alpha;
    if (skip)
      for (int i = threadIdx.x + 1; i < n; i += blockDim.x) vs[i] = 0.0;
    __syncthreads();
    if (blockIdx.x == 0) {
      double* v = V + (int64_t)k * N + k + 1;
      for (int i = threadIdx.x; i < n; i += blockDim.x) v[i] = vs[i];
      if (threadIdx.x == 0) {
        tau[k] = tk;
        d[k] = A[(int64_t)k * N + k];
        e[k] = skip ? x0 : alpha;
      }
    }
    // p = tau A22 v, one warp per row
    const int nwarps = (int)active * warps_per_cta;
    for (int i = (int)blockIdx.x * warps_per_cta + wid; i < n; i += nwarps) {
      const double* row = A + (int64_t)(k + 1 + i) * N + k + 1;
      double t = 0.0;
      for (int j = lane; j < n; j += 32) t += row[j] * vs[j];
      for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
      if (lane == 0) p[i] = tk * t;
    }
    if (!grid_barrier(gs, active)) return;
    // f = (tau/2) v^T p in every CTA; A22 -= v w^T + w v^T with w = p - f v
    double q = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) q += p[i] * vs[i];
    const double f = 0.5 * tk * block_sum(q, red);
    for (int i = blockIdx.x; i < n; i += active) {
      const double vi = vs[i], wi = p[i] - f * vi;
      double* row = A + (int64_t)(k + 1 + i) * N + k + 1;
      for (int j = threadIdx.x; j < n; j += blockDim.x) {
        const double vj = vs[j], wj = p[j] - f * vj;
        row[j] -= vi * wj + wi * vj;
      }
    }
    if (!grid_barrier(gs, active)) return;
  }
}

void dense_set_barrier_spins(uint32_t spins) {
  CHEFSI_CUDA(cudaMemcpyToSymbol(g_barrier_spins, &spins, sizeof(spins)));
}

// Householder tridiagonalisation of the N x N row-major symmetric A: one cooperative launch
// when the device supports it, else the four-launch-per-column sequence.
static void tridiagonalise(double* A, int N, double* V, double* tau, double* d, double* e,
                           double* p, cudaStream_t st) {
  int dev = 0, coop = 0, sms = kNumSMs, per_sm = 0;
  CHEFSI_CUDA(cudaGetDevice(&dev));
  CHEFSI_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
  CHEFSI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  if (sizeof(double) * N > 48 * 1024)
    CHEFSI_CUDA(cudaFuncSetAttribute(k_tridiag_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(sizeof(double) * N)));
  CHEFSI_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_tridiag_fused, 256,
                                                            sizeof(double) * N));
  if (coop && per_sm > 0 && N > 2) {
    DeviceBuffer<unsigned int> sync(2);
    DeviceBuffer<int> err(1);
    CHEFSI_CUDA(cudaMemsetAsync(sync.ptr, 0, 2 * sizeof(unsigned int), st));
    CHEFSI_CUDA(cudaMemsetAsync(err.ptr, 0, sizeof(int), st));
    GridSync gs{sync.ptr, sync.ptr + 1, err.ptr};
    int blocks = std::min(sms, std::max(1, (N * 32 + 255) / 256));  // enough warps for the rows
    blocks = std::min(blocks, sms * per_sm);
    void* args[] = {&A, &N, &V, &tau, &d, &e, &p, &gs};
    CHEFSI_CUDA(cudaLaunchCooperativeKernel((const void*)k_tridiag_fused, dim3(blocks), dim3(256),
                                            args, sizeof(double) * N, st));
    CHEFSI_CHECK_LAUNCH();
    int h = 0;
    CHEFSI_CUDA(cudaMemcpyAsync(&h, err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
    CHEFSI_CUDA(cudaStreamSynchronize(st));
    if (h) throw Error(h, "tridiagonalisation: a bounded grid barrier expired");
    return;
  }
  for (int k = 0; k + 2 < N; ++k) {
    const int n = N - k - 1;
    k_hh_vector<<<1, 256, 0, st>>>(A, N, k, V, tau, d, e);
    CHEFSI_CHECK_LAUNCH();
    k_hh_symv<<<(n * 32 + 255) / 256, 256, 0, st>>>(A, N, k, V, tau, p);
    CHEFSI_CHECK_LAUNCH();
    k_hh_w<<<1, 256, 0, st>>>(N, k, V, tau, p);
    CHEFSI_CHECK_LAUNCH();
    k_hh_rank2<<<grid_for((int64_t)n * n, 256), 256, 0, st>>>(A, N, k, V, p);
    CHEFSI_CHECK_LAUNCH();
  }
}

// Compact WY form of a block of reflectors (LAPACK dlarft, forward / columnwise):
// H_k0 H_k0+1 ... H_k0+nb-1 = I - V T V^T with T upper triangular,
//   T[j][j] = tau_j,  T[0:j][j] = -tau_j T[0:j][0:j] (V^T v_j)[0:j],
// from the Gram matrix G = V^T V of the block (nb x nb). One thread per row of T.
__global__ void k_build_t(const double* G, const double* tau, int nb, double* T) {
  const int i = threadIdx.x;
  for (int j = 0; j < nb; ++j) {
    if (i < nb) {
      double v = 0.0;
      if (i < j) {
        double s = 0.0;
        for (int l = i; l < j; ++l) s += T[i * nb + l] * G[l * nb + j];
        v = -tau[j] * s;
      } else if (i == j) {
        v = tau[j];
      }
      T[i * nb + j] = v;
    }
    __syncthreads();
  }
}

__global__ void k_transpose_sq(const double* A, double* B, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    B[t] = A[(t % N) * N + t / N];
}

// Z <- H_0 H_1 ... H_{N-3} Z with the reflectors in rows of V (V[k][k+1:N], tau[k]), applied
// as compact-WY blocks of kWY reflectors, last block first: Z -= Vb (T (Vb^T Z)). Z is N x
// ncols (row-major, ld ncols): all eigenvectors, or the subset of a partial solve.
constexpr int kWY = 64;
static void back_transform_wy(const double* V, const double* tau, int N, double* Z, int ncols,
                              cudaStream_t st) {
  const int nrefl = N - 2;
  if (nrefl <= 0) return;
  DeviceBuffer<double> Vc((size_t)N * N), G((size_t)kWY * kWY), T((size_t)kWY * kWY),
      W1((size_t)kWY * ncols), W2((size_t)kWY * ncols);
  // Vc[i][k] = V[k][i]: block k0.. of reflectors is the row-major N x nb slice Vc + k0
  k_transpose_sq<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(V, Vc.ptr, N);
  CHEFSI_CHECK_LAUNCH();
  for (int end = nrefl; end > 0; end -= kWY) {
    const int k0 = std::max(0, end - kWY), nb = end - k0;
    const double* Vb = Vc.ptr + k0;
    // the two long-K products (K = N) of the block: the split-K FP64 GEMM
    gemm_f64('T', 'N', nb, nb, N, 1.0, Vb, N, Vb, N, 0.0, G.ptr, nb, CHEFSI_PREC_FP64, st);
    k_build_t<<<1, kWY, 0, st>>>(G.ptr, tau + k0, nb, T.ptr);
    CHEFSI_CHECK_LAUNCH();
    gemm_f64('T', 'N', nb, ncols, N, 1.0, Vb, N, Z, ncols, 0.0, W1.ptr, ncols, CHEFSI_PREC_FP64,
             st);                                                                       // Vb^T Z
    gemm_f64('N', 'N', nb, ncols, nb, 1.0, T.ptr, nb, W1.ptr, ncols, 0.0, W2.ptr, ncols,
             CHEFSI_PREC_FP64, st);                                                // T (Vb^T Z)
    gemm_f64('N', 'N', N, ncols, nb, -1.0, Vb, N, W2.ptr, ncols, 1.0, Z, ncols, CHEFSI_PREC_FP64,
             st);
  }
}

// Eigenpairs il .. il+count-1 (ascending order) of the symmetric row-major A (destroyed):
// tridiagonalisation, multisection for the wanted eigenvalues only, inverse iteration for
// their vectors, back-transformation of count columns. w[count], Z[N][count].
// count == N is the full solve (syevd); a partial solve is the eigenpairs_hermitian_by_index
// step of the spectrum-split Rayleigh-Ritz (the top N - Noc pairs).
int syevd_range(double* A, int N, int il, int count, double* w, double* Z, cudaStream_t st) {
  CHEFSI_REQUIRE(N >= 1, "syevd: N must be positive");
  CHEFSI_REQUIRE(il >= 0 && count >= 1 && il + count <= N, "syevd: eigenpair range out of bounds");
  DeviceBuffer<double> V((size_t)N * N), tau(N), d(N), e(N), p(N);
  CHEFSI_CUDA(cudaMemsetAsync(V.ptr, 0, sizeof(double) * N * N, st));
  CHEFSI_CUDA(cudaMemsetAsync(tau.ptr, 0, sizeof(double) * N, st));
  CHEFSI_CUDA(cudaMemsetAsync(e.ptr, 0, sizeof(double) * N, st));
  tridiagonalise(A, N, V.ptr, tau.ptr, d.ptr, e.ptr, p.ptr, st);
  k_tail<<<1, 32, 0, st>>>(A, N, d.ptr, e.ptr);
  CHEFSI_CHECK_LAUNCH();
  k_bisect_warp<<<(count + 3) / 4, 128, 0, st>>>(d.ptr, e.ptr, N, il, count, w);
  CHEFSI_CHECK_LAUNCH();
  // cluster tolerance relative to the tridiagonal's scale
  std::vector<double> hd(N), he(N);
  CHEFSI_CUDA(cudaMemcpyAsync(hd.data(), d.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaMemcpyAsync(he.data(), e.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  double tn = 0.0;
  for (int j = 0; j < N; ++j)
    tn = std::max(tn, std::fabs(hd[j]) + (j > 0 ? std::fabs(he[j - 1]) : 0.0) +
                          (j < N - 1 ? std::fabs(he[j]) : 0.0));
  const double ortol = 1e-5 * std::max(tn, 1e-300);
  DeviceBuffer<double> work((size_t)count * 5 * N);
  DeviceBuffer<unsigned char> swaps((size_t)count * N);
  k_inverse_iteration<<<(count + 31) / 32, 32, 0, st>>>(d.ptr, e.ptr, N, w, count, il, Z, count,
                                                        work.ptr, swaps.ptr, ortol);
  CHEFSI_CHECK_LAUNCH();
  back_transform_wy(V.ptr, tau.ptr, N, Z, count, st);
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  return CHEFSI_OK;
}

int syevd(double* A, int N, double* w, double* Z, cudaStream_t st) {
  return syevd_range(A, N, 0, N, w, Z, st);
}

// ======================================================================= residuals, dots
__global__ void k_resid(const double* __restrict__ X, int64_t ldx, const double* __restrict__ HX,
                        int64_t ldh, int64_t M, int N, const double* __restrict__ lam,
                        double* __restrict__ out, int64_t rows_per) {
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per;
  const int64_t r1 = min(M, r0 + rows_per);
  const double l = lam[j];
  double s = 0.0;
  for (int64_t i = r0; i < r1; ++i) {
    const double t = HX[i * ldh + j] - l * X[i * ldx + j];
    s += t * t;
  }
  atomicAdd(&out[j], s);
}
__global__ void k_resid_c(const cplx* __restrict__ X, int64_t ldx, const cplx* __restrict__ HX,
                          int64_t ldh, int64_t M, int N, const double* __restrict__ lam,
                          double* __restrict__ out, int64_t rows_per) {
  const int j = blockIdx.y * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const int64_t r0 = (int64_t)blockIdx.x * rows_per;
  const int64_t r1 = min(M, r0 + rows_per);
  const double l = lam[j];
  double s = 0.0;
  for (int64_t i = r0; i < r1; ++i) {
    const cplx h = HX[i * ldh + j], x = X[i * ldx + j];
    const double tr = h.x - l * x.x, ti = h.y - l * x.y;
    s += tr * tr + ti * ti;
  }
  atomicAdd(&out[j], s);
}
__global__ void k_sqrt(double* x, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[i] = sqrt(x[i]);
}

void residual_norms_f64(const double* X, int64_t ldx, const double* HX, int64_t ldh, int64_t M,
                        int N, const double* lam, double* out, cudaStream_t st) {
  CHEFSI_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * N, st));
  const int64_t rows_per = std::max<int64_t>(64, (M + 1023) / 1024);
  dim3 grid((unsigned)((M + rows_per - 1) / rows_per), (N + 127) / 128);
  k_resid<<<grid, 128, 0, st>>>(X, ldx, HX, ldh, M, N, lam, out, rows_per);
  CHEFSI_CHECK_LAUNCH();
  k_sqrt<<<(N + 127) / 128, 128, 0, st>>>(out, N);
  CHEFSI_CHECK_LAUNCH();
}
void residual_norms_c64(const cplx* X, int64_t ldx, const cplx* HX, int64_t ldh, int64_t M, int N,
                        const double* lam, double* out, cudaStream_t st) {
  CHEFSI_CUDA(cudaMemsetAsync(out, 0, sizeof(double) * N, st));
  const int64_t rows_per = std::max<int64_t>(64, (M + 1023) / 1024);
  dim3 grid((unsigned)((M + rows_per - 1) / rows_per), (N + 127) / 128);
  k_resid_c<<<grid, 128, 0, st>>>(X, ldx, HX, ldh, M, N, lam, out, rows_per);
  CHEFSI_CHECK_LAUNCH();
  k_sqrt<<<(N + 127) / 128, 128, 0, st>>>(out, N);
  CHEFSI_CHECK_LAUNCH();
}

__global__ void k_dot(const double* __restrict__ x, const double* __restrict__ y, int64_t n,
                      double* out) {
  double s = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    s += x[t] * y[t];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(out, s);
}
void dot_f64(const double* x, const double* y, int64_t n, double* out, cudaStream_t st) {
  CHEFSI_CUDA(cudaMemsetAsync(out, 0, sizeof(double), st));
  k_dot<<<grid_for(n, 256, kNumSMs * 4), 256, 0, st>>>(x, y, n, out);
  CHEFSI_CHECK_LAUNCH();
}

}  // namespace chefsi
