// Complex (Bloch, k-point) dense steps of the Rayleigh-Ritz step, all FP64 on the device:
//   * Cholesky S = L L^H of the Hermitian overlap and the triangular inverse L^{-1}
//     (pseudoGSDevice.cc:82-463 and rayleighRitzDevice.cc:356-819 hand these to ELPA /
//     ScaLAPACK: pzpotrf, pztrtri);
//   * the Hermitian eigensolver of the projected matrix (ELPA / zheevd in rayleighRitzGEP):
//     complex Householder tridiagonalisation A = Q T Q^H, a diagonal unitary D = diag(phi)
//     that makes T real (T = D T_r D^H with |e_j| on the off-diagonal), the real tridiagonal
//     eigensolver (multisection + inverse iteration) for T_r = Z_r diag(w) Z_r^T, and the
//     back-transformation Q D Z_r with compact-WY blocks of reflectors.
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <vector>

namespace chefsi {

namespace {

constexpr int CBc = 32;

__device__ __forceinline__ double cabs2(cplx a) { return a.x * a.x + a.y * a.y; }
__device__ __forceinline__ cplx cdiv_real(cplx a, double s) { return {a.x / s, a.y / s}; }
__device__ __forceinline__ cplx cdiv(cplx a, cplx b) {
  const double den = b.x * b.x + b.y * b.y;
  return {(a.x * b.x + a.y * b.y) / den, (a.y * b.x - a.x * b.y) / den};
}

// ---------------------------------------------------------------- Cholesky
__global__ void k_potf2_c(cplx* A, int N, int k0, int nb, int* info) {
  __shared__ cplx L[CBc][CBc + 1];
  const int t = threadIdx.x;
  for (int i = 0; i < nb; ++i)
    if (t < nb) L[i][t] = A[(int64_t)(k0 + i) * N + k0 + t];
  __syncthreads();
  for (int j = 0; j < nb; ++j) {
    if (t == 0) {
      const double djj = L[j][j].x;
      if (!(djj > 0.0) || !isfinite(djj)) {
        atomicCAS(info, 0, k0 + j + 1);
        L[j][j] = {1.0, 0.0};
      } else {
        L[j][j] = {sqrt(djj), 0.0};
      }
    }
    __syncthreads();
    if (t > j && t < nb) L[t][j] = cdiv_real(L[t][j], L[j][j].x);
    __syncthreads();
    if (t > j && t < nb)
      for (int i = t; i < nb; ++i) L[i][t] = csub(L[i][t], cmul(L[i][j], cconj(L[t][j])));
    __syncthreads();
  }
  for (int i = 0; i < nb; ++i)
    if (t < nb) A[(int64_t)(k0 + i) * N + k0 + t] = (t <= i) ? L[i][t] : cplx{0.0, 0.0};
}

// rows r >= k0+nb: A[r][k0:k0+nb] <- A[r][k0:k0+nb] L11^{-H}
__global__ void k_trsm_panel_c(cplx* A, int N, int k0, int nb) {
  __shared__ cplx L[CBc][CBc + 1];
  for (int idx = threadIdx.x; idx < nb * nb; idx += blockDim.x)
    L[idx / nb][idx % nb] = A[(int64_t)(k0 + idx / nb) * N + k0 + idx % nb];
  __syncthreads();
  const int r = k0 + nb + blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= N) return;
  cplx x[CBc];
  cplx* row = A + (int64_t)r * N + k0;
  for (int j = 0; j < nb; ++j) {
    cplx v = row[j];
    for (int l = 0; l < j; ++l) v = csub(v, cmul(x[l], cconj(L[j][l])));
    x[j] = cdiv_real(v, L[j][j].x);
  }
  for (int j = 0; j < nb; ++j) row[j] = x[j];
}

__global__ void k_zero_upper_c(cplx* A, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    if ((int)(t % N) > (int)(t / N)) A[t] = {0.0, 0.0};
}

// invert each diagonal block of the lower-triangular L in place
__global__ void k_trtri_diag_c(cplx* L, int N) {
  __shared__ cplx T[CBc][CBc + 1];
  __shared__ cplx Z[CBc][CBc + 1];
  const int k0 = blockIdx.x * CBc;
  const int nb = min(CBc, N - k0);
  const int t = threadIdx.x;
  for (int i = 0; i < nb; ++i)
    if (t < nb) T[i][t] = L[(int64_t)(k0 + i) * N + k0 + t], Z[i][t] = {0.0, 0.0};
  __syncthreads();
  if (t < nb) {
    for (int i = 0; i < nb; ++i) {
      cplx v = {(i == t) ? 1.0 : 0.0, 0.0};
      for (int l = t; l < i; ++l) v = csub(v, cmul(T[i][l], Z[l][t]));
      Z[i][t] = (i >= t) ? cdiv(v, T[i][i]) : cplx{0.0, 0.0};
    }
  }
  __syncthreads();
  for (int i = 0; i < nb; ++i)
    if (t < nb) L[(int64_t)(k0 + i) * N + k0 + t] = Z[i][t];
}

// ---------------------------------------------------------------- Hermitian eigensolver
// Householder step k on the Hermitian row-major A (full storage maintained):
// x = A[k+1:N, k]; alpha = -(x0/|x0|) |x|; v = x - alpha e1; tau = 2 / v^H v, so that
// (I - tau v v^H) x = alpha e1. d[k] = Re A[k][k], e[k] = alpha (complex).
__global__ void k_hh_vector_c(cplx* A, int N, int k, cplx* V, double* tau, double* d, cplx* e) {
  __shared__ double red[32];
  const int n = N - k - 1;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s += cabs2(A[(int64_t)(k + 1 + i) * N + k]);
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
  const double nrm = sqrt(nrm2);
  const cplx x0 = A[(int64_t)(k + 1) * N + k];
  const double ax0 = sqrt(cabs2(x0));
  const cplx ph = ax0 > 0.0 ? cdiv_real(x0, ax0) : cplx{1.0, 0.0};
  const cplx alpha = cscale(ph, -nrm);
  const double vhv = 2.0 * (nrm2 + nrm * ax0);
  const bool skip = !(vhv > 0.0) || nrm == 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cplx x = A[(int64_t)(k + 1 + i) * N + k];
    V[(int64_t)k * N + k + 1 + i] = skip ? cplx{0.0, 0.0} : (i == 0 ? csub(x, alpha) : x);
  }
  if (threadIdx.x == 0) {
    tau[k] = skip ? 0.0 : 2.0 / vhv;
    d[k] = A[(int64_t)k * N + k].x;
    e[k] = skip ? x0 : alpha;
  }
}

// p = tau A22 v   (one warp per row of the trailing block)
__global__ void k_hh_symv_c(const cplx* A, int N, int k, const cplx* V, const double* tau, cplx* p) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int n = N - k - 1;
  if (warp >= n) return;
  const cplx* row = A + (int64_t)(k + 1 + warp) * N + k + 1;
  const cplx* v = V + (int64_t)k * N + k + 1;
  double sx = 0.0, sy = 0.0;
  for (int j = lane; j < n; j += 32) {
    const cplx t = cmul(row[j], v[j]);
    sx += t.x;
    sy += t.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
  }
  if (lane == 0) p[warp] = {tau[k] * sx, tau[k] * sy};
}

// w = p - (tau/2)(v^H p) v   (single CTA)
__global__ void k_hh_w_c(int N, int k, const cplx* V, const double* tau, cplx* p) {
  __shared__ double rx[32], ry[32];
  const int n = N - k - 1;
  const cplx* v = V + (int64_t)k * N + k + 1;
  double sx = 0.0, sy = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const cplx t = cmul(cconj(v[i]), p[i]);
    sx += t.x;
    sy += t.y;
  }
  for (int o = 16; o > 0; o >>= 1) {
    sx += __shfl_xor_sync(0xffffffffu, sx, o);
    sy += __shfl_xor_sync(0xffffffffu, sy, o);
  }
  if ((threadIdx.x & 31) == 0) rx[threadIdx.x >> 5] = sx, ry[threadIdx.x >> 5] = sy;
  __syncthreads();
  if (threadIdx.x < 32) {
    const bool in = threadIdx.x < (blockDim.x + 31) / 32;
    sx = in ? rx[threadIdx.x] : 0.0;
    sy = in ? ry[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) {
      sx += __shfl_xor_sync(0xffffffffu, sx, o);
      sy += __shfl_xor_sync(0xffffffffu, sy, o);
    }
    if (threadIdx.x == 0) rx[0] = sx, ry[0] = sy;
  }
  __syncthreads();
  const cplx f = {0.5 * tau[k] * rx[0], 0.5 * tau[k] * ry[0]};
  for (int i = threadIdx.x; i < n; i += blockDim.x) p[i] = csub(p[i], cmul(f, v[i]));
}

// A22 -= v w^H + w v^H
__global__ void k_hh_rank2_c(cplx* A, int N, int k, const cplx* V, const cplx* w) {
  const int n = N - k - 1;
  const int64_t tot = (int64_t)n * n;
  const cplx* v = V + (int64_t)k * N + k + 1;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n), j = (int)(t % n);
    cplx& a = A[(int64_t)(k + 1 + i) * N + k + 1 + j];
    a = csub(a, cadd(cmul(v[i], cconj(w[j])), cmul(w[i], cconj(v[j]))));
  }
}

__global__ void k_tail_c(const cplx* A, int N, double* d, cplx* e) {
  if (threadIdx.x == 0) {
    if (N >= 2) {
      d[N - 2] = A[(int64_t)(N - 2) * N + N - 2].x;
      e[N - 2] = A[(int64_t)(N - 1) * N + N - 2];
    }
    d[N - 1] = A[(int64_t)(N - 1) * N + N - 1].x;
  }
}

// T = D T_r D^H: phi_0 = 1, phi_{j+1} = phi_j e_j / |e_j|; er[j] = |e_j|
__global__ void k_tridiag_phases(const cplx* e, int N, double* er, cplx* phi) {
  if (threadIdx.x != 0) return;
  cplx p = {1.0, 0.0};
  phi[0] = p;
  for (int j = 0; j + 1 < N; ++j) {
    const double a = sqrt(cabs2(e[j]));
    er[j] = a;
    if (a > 0.0) p = cmul(p, cdiv_real(e[j], a));
    phi[j + 1] = p;
  }
  er[N - 1] = 0.0;
}

// Z[j][t] = phi_j Zr[j][t] (N rows of ncols)
__global__ void k_phase_rows(const double* Zr, const cplx* phi, int N, int ncols, cplx* Z) {
  const int64_t n = (int64_t)N * ncols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    Z[t] = cscale(phi[t / ncols], Zr[t]);
}

// compact-WY T of a block of complex reflectors (forward, columnwise) from G = V^H V
__global__ void k_build_t_c(const cplx* G, const double* tau, int nb, cplx* T) {
  const int i = threadIdx.x;
  for (int j = 0; j < nb; ++j) {
    if (i < nb) {
      cplx v = {0.0, 0.0};
      if (i < j) {
        cplx s = {0.0, 0.0};
        for (int l = i; l < j; ++l) s = cadd(s, cmul(T[i * nb + l], G[l * nb + j]));
        v = cscale(s, -tau[j]);
      } else if (i == j) {
        v = {tau[j], 0.0};
      }
      T[i * nb + j] = v;
    }
    __syncthreads();
  }
}

__global__ void k_transpose_sq_c(const cplx* A, cplx* B, int N) {
  const int64_t n = (int64_t)N * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    B[t] = A[(t % N) * N + t / N];
}

constexpr int kWYc = 64;

// Z <- H_0 ... H_{N-3} Z with H_k = I - tau_k v_k v_k^H, v_k in row k of V; Z is N x ncols
void back_transform_wy_c(const cplx* V, const double* tau, int N, cplx* Z, int ncols,
                         cudaStream_t st) {
  const int nrefl = N - 2;
  if (nrefl <= 0) return;
  DeviceBuffer<cplx> Vc((size_t)N * N), G((size_t)kWYc * kWYc), T((size_t)kWYc * kWYc),
      W1((size_t)kWYc * ncols), W2((size_t)kWYc * ncols);
  k_transpose_sq_c<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(V, Vc.ptr, N);
  CHEFSI_CHECK_LAUNCH();
  const cplx one = {1.0, 0.0}, zero = {0.0, 0.0}, mone = {-1.0, 0.0};
  for (int end = nrefl; end > 0; end -= kWYc) {
    const int k0 = std::max(0, end - kWYc), nb = end - k0;
    const cplx* Vb = Vc.ptr + k0;
    CHEFSI_CUDA(cudaMemsetAsync(G.ptr, 0, sizeof(cplx) * nb * nb, st));
    gram_c64(Vb, N, Vb, N, N, nb, nb, G.ptr, nb, false, st);               // Vb^H Vb
    k_build_t_c<<<1, kWYc, 0, st>>>(G.ptr, tau + k0, nb, T.ptr);
    CHEFSI_CHECK_LAUNCH();
    CHEFSI_CUDA(cudaMemsetAsync(W1.ptr, 0, sizeof(cplx) * nb * ncols, st));
    gram_c64(Vb, N, Z, ncols, N, nb, ncols, W1.ptr, ncols, false, st);     // Vb^H Z
    gemm_c64('N', 'N', nb, ncols, nb, one, T.ptr, nb, W1.ptr, ncols, zero, W2.ptr, ncols, st);
    gemm_c64('N', 'N', N, ncols, nb, mone, Vb, N, W2.ptr, ncols, one, Z, ncols, st);
  }
}

}  // namespace

int cholesky_lower_c(cplx* A, int N, cudaStream_t st) {
  DeviceBuffer<int> info(1);
  CHEFSI_CUDA(cudaMemsetAsync(info.ptr, 0, sizeof(int), st));
  const cplx mone = {-1.0, 0.0}, one = {1.0, 0.0};
  for (int k0 = 0; k0 < N; k0 += CBc) {
    const int nb = std::min(CBc, N - k0);
    k_potf2_c<<<1, CBc, 0, st>>>(A, N, k0, nb, info.ptr);
    CHEFSI_CHECK_LAUNCH();
    const int rest = N - k0 - nb;
    if (rest > 0) {
      k_trsm_panel_c<<<(rest + 127) / 128, 128, 0, st>>>(A, N, k0, nb);
      CHEFSI_CHECK_LAUNCH();
      const int64_t off = (int64_t)(k0 + nb) * N;
      gemm_c64('N', 'C', rest, rest, nb, mone, A + off + k0, N, A + off + k0, N, one,
               A + off + k0 + nb, N, st);
    }
  }
  k_zero_upper_c<<<grid_for((int64_t)N * N, 256), 256, 0, st>>>(A, N);
  CHEFSI_CHECK_LAUNCH();
  int h = 0;
  CHEFSI_CUDA(cudaMemcpyAsync(&h, info.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  return h ? CHEFSI_ERR_NOT_SPD : CHEFSI_OK;
}

void trtri_lower_c(cplx* L, int N, cudaStream_t st) {
  const int nblk = (N + CBc - 1) / CBc;
  k_trtri_diag_c<<<nblk, CBc, 0, st>>>(L, N);
  CHEFSI_CHECK_LAUNCH();
  DeviceBuffer<cplx> tmp((size_t)CBc * N);
  const cplx one = {1.0, 0.0}, zero = {0.0, 0.0}, mone = {-1.0, 0.0};
  for (int bi = 1; bi < nblk; ++bi) {
    const int r0 = bi * CBc;
    const int nb = std::min(CBc, N - r0);
    gemm_c64('N', 'N', nb, r0, r0, one, L + (int64_t)r0 * N, N, L, N, zero, tmp.ptr, r0, st);
    gemm_c64('N', 'N', nb, r0, nb, mone, L + (int64_t)r0 * N + r0, N, tmp.ptr, r0, zero,
             L + (int64_t)r0 * N, N, st);
  }
}

// Eigenpairs il .. il+count-1 (ascending) of the Hermitian row-major A (destroyed); w[count],
// Z[N][count]. count == N is the full solve.
int heevd_range(cplx* A, int N, int il, int count, double* w, cplx* Z, cudaStream_t st) {
  CHEFSI_REQUIRE(N >= 1, "heevd: N must be positive");
  CHEFSI_REQUIRE(il >= 0 && count >= 1 && il + count <= N, "heevd: eigenpair range out of bounds");
  DeviceBuffer<cplx> V((size_t)N * N), e(N), p(N), phi(N);
  DeviceBuffer<double> tau(N), d(N), er(N), Zr((size_t)N * count);
  CHEFSI_CUDA(cudaMemsetAsync(V.ptr, 0, sizeof(cplx) * N * N, st));
  CHEFSI_CUDA(cudaMemsetAsync(tau.ptr, 0, sizeof(double) * N, st));
  CHEFSI_CUDA(cudaMemsetAsync(e.ptr, 0, sizeof(cplx) * N, st));
  for (int k = 0; k + 2 < N; ++k) {
    const int n = N - k - 1;
    k_hh_vector_c<<<1, 256, 0, st>>>(A, N, k, V.ptr, tau.ptr, d.ptr, e.ptr);
    CHEFSI_CHECK_LAUNCH();
    k_hh_symv_c<<<(n * 32 + 255) / 256, 256, 0, st>>>(A, N, k, V.ptr, tau.ptr, p.ptr);
    CHEFSI_CHECK_LAUNCH();
    k_hh_w_c<<<1, 256, 0, st>>>(N, k, V.ptr, tau.ptr, p.ptr);
    CHEFSI_CHECK_LAUNCH();
    k_hh_rank2_c<<<grid_for((int64_t)n * n, 256), 256, 0, st>>>(A, N, k, V.ptr, p.ptr);
    CHEFSI_CHECK_LAUNCH();
  }
  k_tail_c<<<1, 32, 0, st>>>(A, N, d.ptr, e.ptr);
  CHEFSI_CHECK_LAUNCH();
  k_tridiag_phases<<<1, 32, 0, st>>>(e.ptr, N, er.ptr, phi.ptr);
  CHEFSI_CHECK_LAUNCH();
  k_bisect_warp<<<(count + 3) / 4, 128, 0, st>>>(d.ptr, er.ptr, N, il, count, w);
  CHEFSI_CHECK_LAUNCH();
  std::vector<double> hd(N), he(N);
  CHEFSI_CUDA(cudaMemcpyAsync(hd.data(), d.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaMemcpyAsync(he.data(), er.ptr, sizeof(double) * N, cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  double tn = 0.0;
  for (int j = 0; j < N; ++j)
    tn = std::max(tn, std::fabs(hd[j]) + (j > 0 ? std::fabs(he[j - 1]) : 0.0) +
                          (j < N - 1 ? std::fabs(he[j]) : 0.0));
  const double ortol = 1e-5 * std::max(tn, 1e-300);
  DeviceBuffer<double> work((size_t)count * 5 * N);
  DeviceBuffer<unsigned char> swaps((size_t)count * N);
  k_inverse_iteration<<<(count + 31) / 32, 32, 0, st>>>(d.ptr, er.ptr, N, w, count, il, Zr.ptr,
                                                        count, work.ptr, swaps.ptr, ortol);
  CHEFSI_CHECK_LAUNCH();
  k_phase_rows<<<grid_for((int64_t)N * count, 256), 256, 0, st>>>(Zr.ptr, phi.ptr, N, count, Z);
  CHEFSI_CHECK_LAUNCH();
  back_transform_wy_c(V.ptr, tau.ptr, N, Z, count, st);
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  return CHEFSI_OK;
}

int heevd(cplx* A, int N, double* w, cplx* Z, cudaStream_t st) {
  return heevd_range(A, N, 0, N, w, Z, st);
}

}  // namespace chefsi
