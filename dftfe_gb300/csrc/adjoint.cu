// Building blocks of the local-potential adjoint and of the on-device cell Hamiltonian
// assembly (FP64 SIMT):
//   * k_assemble_cells: H_c = 1/2 K + N^T diag(v_c) N, the formula of hamMatrixKernelLDA
//     (src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:61-115), written as a
//     per-cell product over quadrature points;
//   * k_assemble_geom: the same for cells of any shape, the stiffness formed per cell from the
//     reference-cell gradients and the per-point Jacobian factors J^-1 J^-T JxW
//     (FEBasisOperations::computeCellStiffnessMatrix, utils/FEBasisOperations.cc:1133-1300);
//   * k_cell_outer: G_c[I][J] += alpha sum_b (D u)[map I][b] (D v)[map J][b] -- the
//     contraction of an adjoint pair (u = adjoint block, v = state block) with dA/dH_c, where
//     A = D H D and D = M^{-1/2};
//   * k_quad_contract: g_c(q) = jxw_c(q) sum_IJ N_qI G_c[I][J] N_qJ -- dL/dV(q) from G,
//     because dH_c[I][J]/dV_c(q) = JxW_c(q) N_qI N_qJ.
#include "internal.h"

namespace chefsi {

namespace {

constexpr int T = 32;  // output tile (I x J)

// out[c][I][J] = 0.5 K[I][J] + sum_q N[q][I] v[c][q] N[q][J]
__global__ void __launch_bounds__(256)
    k_assemble_cells(int n_cells, int n_e, int n_q, const double* __restrict__ N,
                     const double* __restrict__ K, const double* __restrict__ v,
                     double* __restrict__ out, int nt) {
  __shared__ double Ai[16][T + 1];
  __shared__ double Bj[16][T + 1];
  const int64_t blk = blockIdx.x;
  const int tj = (int)(blk % nt), ti = (int)((blk / nt) % nt);
  const int c = (int)(blk / ((int64_t)nt * nt));
  const int i0 = ti * T, j0 = tj * T;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2x2 per thread
  double acc[2][2] = {{0, 0}, {0, 0}};
  const double* vc = v + (int64_t)c * n_q;
  for (int q0 = 0; q0 < n_q; q0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * T; idx += 256) {
      const int qq = idx / T, k = idx % T;
      const int q = q0 + qq;
      const bool okq = q < n_q;
      Ai[qq][k] = (okq && i0 + k < n_e) ? N[(int64_t)q * n_e + i0 + k] * vc[q] : 0.0;
      Bj[qq][k] = (okq && j0 + k < n_e) ? N[(int64_t)q * n_e + j0 + k] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int qq = 0; qq < 16; ++qq)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int s = 0; s < 2; ++s) acc[r][s] = fma(Ai[qq][ty + 16 * r], Bj[qq][tx + 16 * s], acc[r][s]);
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int I = i0 + ty + 16 * r, J = j0 + tx + 16 * s;
      if (I < n_e && J < n_e)
        out[((int64_t)c * n_e + I) * n_e + J] = 0.5 * K[(int64_t)I * n_e + J] + acc[r][s];
    }
}

// Bloch cell Hamiltonians for n_k k-points (the k-point form of hamMatrixKernelLDA,
// src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:119-280), as the matrix applied
// to the cell vector (the transpose of the reference's flattened layout, whose complex HX
// multiplies with op = T):
//   Re out[k][c][I][J] = 0.5 K[I][J] + sum_q v[c][q] N_qI N_qJ + |k|^2/2 sum_q w[c][q] N_qI N_qJ
//   Im out[k][c][I][J] = -sum_d k_d sum_q w[c][q] N_qI dN_d[q][J]
// (w = JxW, dN_d the real-space shape-function gradients). The five cell sums are formed once
// per cell tile and combined for every k-point in the epilogue. GGA (the k-point form of
// hamMatrixKernelGGAMemOpt, :458-655) adds to the real part the gradient terms
// 2 sum_q sum_d g[c][q][d] (dN_d[q][I] N_qJ + N_qI dN_d[q][J]), g = derExcWithSigmaTimesGradRhoJxW,
// folded as for the real GGA kernel: 2 sum_d g_d dN_dI into the potential operand and three
// more operands 2 g_d N_I against the gradient operands already loaded.
template <bool GGA>
__global__ void __launch_bounds__(256)
    k_assemble_bloch(int n_cells, int n_e, int n_q, const double* __restrict__ N,
                     const double* __restrict__ dN, const double* __restrict__ K,
                     const double* __restrict__ v, const double* __restrict__ w,
                     const double* __restrict__ g, int n_k, const double* __restrict__ kpts,
                     double2* __restrict__ out, int nt) {
  __shared__ double Av[16][T + 1];
  __shared__ double Aw[16][T + 1];
  __shared__ double Bn[16][T + 1];
  __shared__ double Bd[3][16][T + 1];
  __shared__ double Ag[GGA ? 3 : 1][16][T + 1];
  const int64_t blk = blockIdx.x;
  const int tj = (int)(blk % nt), ti = (int)((blk / nt) % nt);
  const int c = (int)(blk / ((int64_t)nt * nt));
  const int i0 = ti * T, j0 = tj * T;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2x2 per thread
  double sv[2][2] = {}, sm[2][2] = {}, sg[3][2][2] = {};
  const double* vc = v + (int64_t)c * n_q;
  const double* wc = w + (int64_t)c * n_q;
  for (int q0 = 0; q0 < n_q; q0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * T; idx += 256) {
      const int qq = idx / T, k = idx % T;
      const int q = q0 + qq;
      const bool okq = q < n_q;
      const bool oki = okq && i0 + k < n_e, okj = okq && j0 + k < n_e;
      const double ni = oki ? N[(int64_t)q * n_e + i0 + k] : 0.0;
      Av[qq][k] = oki ? ni * vc[q] : 0.0;
      Aw[qq][k] = oki ? ni * wc[q] : 0.0;
      if constexpr (GGA) {
        if (oki) {
          const double* gq = g + ((int64_t)c * n_q + q) * 3;
          const int64_t iI = (int64_t)q * n_e + i0 + k, qn = (int64_t)n_q * n_e;
          for (int d = 0; d < 3; ++d) Ag[d][qq][k] = 2.0 * gq[d] * ni;
          Av[qq][k] += 2.0 * (gq[0] * dN[iI] + gq[1] * dN[qn + iI] + gq[2] * dN[2 * qn + iI]);
        } else {
          for (int d = 0; d < 3; ++d) Ag[d][qq][k] = 0.0;
        }
      }
      Bn[qq][k] = okj ? N[(int64_t)q * n_e + j0 + k] : 0.0;
      for (int d = 0; d < 3; ++d)
        Bd[d][qq][k] = okj ? dN[((int64_t)d * n_q + q) * n_e + j0 + k] : 0.0;
    }
    __syncthreads();
#pragma unroll 4
    for (int qq = 0; qq < 16; ++qq)
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        const double av = Av[qq][ty + 16 * r], aw = Aw[qq][ty + 16 * r];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int jj = tx + 16 * s;
          sv[r][s] = fma(av, Bn[qq][jj], sv[r][s]);
          sm[r][s] = fma(aw, Bn[qq][jj], sm[r][s]);
#pragma unroll
          for (int d = 0; d < 3; ++d) sg[d][r][s] = fma(aw, Bd[d][qq][jj], sg[d][r][s]);
          if constexpr (GGA) {
#pragma unroll
            for (int d = 0; d < 3; ++d) sv[r][s] = fma(Ag[d][qq][ty + 16 * r], Bd[d][qq][jj], sv[r][s]);
          }
        }
      }
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int I = i0 + ty + 16 * r, J = j0 + tx + 16 * s;
      if (I >= n_e || J >= n_e) continue;
      const double base = 0.5 * K[(int64_t)I * n_e + J] + sv[r][s];
      for (int kp = 0; kp < n_k; ++kp) {
        const double k0 = kpts[3 * kp], k1 = kpts[3 * kp + 1], k2 = kpts[3 * kp + 2];
        const double ksq = k0 * k0 + k1 * k1 + k2 * k2;
        const double re = base + 0.5 * ksq * sm[r][s];
        const double im = -(k0 * sg[0][r][s] + k1 * sg[1][r][s] + k2 * sg[2][r][s]);
        out[(((int64_t)kp * n_cells + c) * n_e + I) * n_e + J] = make_double2(re, im);
      }
    }
}

// GGA cell Hamiltonians, real (the formula of hamMatrixKernelGGAMemOpt,
// src/dftOperator/hamiltonianMatrixCalculatorFlattenedDevice.cc:283-456):
//   out[c][I][J] = 0.5 K[I][J] + sum_q ( v[c][q] N_qI N_qJ
//                  + 2 sum_d g[c][q][d] (dN_d[q][I] N_qJ + N_qI dN_d[q][J]) )
// (g = derExcWithSigmaTimesGradRhoJxW). Folded into two operand families per quadrature point:
// A0_I = v N_I + 2 sum_d g_d dN_dI against N_J, and A_d,I = 2 g_d N_I against dN_dJ.
__global__ void __launch_bounds__(256)
    k_assemble_gga(int n_cells, int n_e, int n_q, const double* __restrict__ N,
                   const double* __restrict__ dN, const double* __restrict__ K,
                   const double* __restrict__ v, const double* __restrict__ g,
                   double* __restrict__ out, int nt) {
  __shared__ double A[4][16][T + 1];
  __shared__ double Bt[4][16][T + 1];
  const int64_t blk = blockIdx.x;
  const int tj = (int)(blk % nt), ti = (int)((blk / nt) % nt);
  const int c = (int)(blk / ((int64_t)nt * nt));
  const int i0 = ti * T, j0 = tj * T;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2x2 per thread
  double acc[2][2] = {{0, 0}, {0, 0}};
  const double* vc = v + (int64_t)c * n_q;
  const double* gc = g + (int64_t)c * n_q * 3;
  for (int q0 = 0; q0 < n_q; q0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * T; idx += 256) {
      const int qq = idx / T, k = idx % T;
      const int q = q0 + qq;
      const bool okq = q < n_q;
      const bool oki = okq && i0 + k < n_e, okj = okq && j0 + k < n_e;
      const double g0 = okq ? gc[3 * q] : 0.0, g1 = okq ? gc[3 * q + 1] : 0.0,
                   g2 = okq ? gc[3 * q + 2] : 0.0;
      if (oki) {
        const int64_t iI = (int64_t)q * n_e + i0 + k;
        const int64_t qn = (int64_t)n_q * n_e;
        const double ni = N[iI];
        A[0][qq][k] = ni * vc[q] + 2.0 * (g0 * dN[iI] + g1 * dN[qn + iI] + g2 * dN[2 * qn + iI]);
        A[1][qq][k] = 2.0 * g0 * ni;
        A[2][qq][k] = 2.0 * g1 * ni;
        A[3][qq][k] = 2.0 * g2 * ni;
      } else {
        A[0][qq][k] = A[1][qq][k] = A[2][qq][k] = A[3][qq][k] = 0.0;
      }
      if (okj) {
        const int64_t iJ = (int64_t)q * n_e + j0 + k;
        const int64_t qn = (int64_t)n_q * n_e;
        Bt[0][qq][k] = N[iJ];
        Bt[1][qq][k] = dN[iJ];
        Bt[2][qq][k] = dN[qn + iJ];
        Bt[3][qq][k] = dN[2 * qn + iJ];
      } else {
        Bt[0][qq][k] = Bt[1][qq][k] = Bt[2][qq][k] = Bt[3][qq][k] = 0.0;
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int qq = 0; qq < 16; ++qq)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int ii = ty + 16 * r, jj = tx + 16 * s;
          double t = acc[r][s];
#pragma unroll
          for (int f = 0; f < 4; ++f) t = fma(A[f][qq][ii], Bt[f][qq][jj], t);
          acc[r][s] = t;
        }
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int I = i0 + ty + 16 * r, J = j0 + tx + 16 * s;
      if (I < n_e && J < n_e)
        out[((int64_t)c * n_e + I) * n_e + J] = 0.5 * K[(int64_t)I * n_e + J] + acc[r][s];
    }
}

// Cells of any shape: out[c][I][J] = sum_q ( 0.5 sum_ij dN[i][q][I] F[c][q][i][j] dN[j][q][J]
// + v[c][q] N[q][I] N[q][J] ), dN the reference-cell gradients and F the per-point Jacobian
// factor J^-1 J^-T JxW (symmetric). Per 16 quadrature points the cell's A side
// (v N_I, 0.5 sum_i dN_i F_ij) and the shared B side (N_J, dN_j) go through shared memory.
__global__ void __launch_bounds__(256)
    k_assemble_geom(int n_cells, int n_e, int n_q, const double* __restrict__ N,
                    const double* __restrict__ dN, const double* __restrict__ F,
                    const double* __restrict__ v, double* __restrict__ out, int nt) {
  __shared__ double A[4][16][T + 1];
  __shared__ double Bt[4][16][T + 1];
  const int64_t blk = blockIdx.x;
  const int tj = (int)(blk % nt), ti = (int)((blk / nt) % nt);
  const int c = (int)(blk / ((int64_t)nt * nt));
  const int i0 = ti * T, j0 = tj * T;
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;  // 2x2 per thread
  double acc[2][2] = {{0, 0}, {0, 0}};
  const double* vc = v + (int64_t)c * n_q;
  const double* Fc = F + (int64_t)c * n_q * 9;
  const int64_t qn = (int64_t)n_q * n_e;
  for (int q0 = 0; q0 < n_q; q0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * T; idx += 256) {
      const int qq = idx / T, k = idx % T;
      const int q = q0 + qq;
      const bool okq = q < n_q;
      const bool oki = okq && i0 + k < n_e, okj = okq && j0 + k < n_e;
      if (oki) {
        const int64_t iI = (int64_t)q * n_e + i0 + k;
        const double d0 = dN[iI], d1 = dN[qn + iI], d2 = dN[2 * qn + iI];
        const double* f = Fc + 9 * q;
        A[0][qq][k] = N[iI] * vc[q];
        A[1][qq][k] = 0.5 * (d0 * f[0] + d1 * f[3] + d2 * f[6]);
        A[2][qq][k] = 0.5 * (d0 * f[1] + d1 * f[4] + d2 * f[7]);
        A[3][qq][k] = 0.5 * (d0 * f[2] + d1 * f[5] + d2 * f[8]);
      } else {
        A[0][qq][k] = A[1][qq][k] = A[2][qq][k] = A[3][qq][k] = 0.0;
      }
      if (okj) {
        const int64_t iJ = (int64_t)q * n_e + j0 + k;
        Bt[0][qq][k] = N[iJ];
        Bt[1][qq][k] = dN[iJ];
        Bt[2][qq][k] = dN[qn + iJ];
        Bt[3][qq][k] = dN[2 * qn + iJ];
      } else {
        Bt[0][qq][k] = Bt[1][qq][k] = Bt[2][qq][k] = Bt[3][qq][k] = 0.0;
      }
    }
    __syncthreads();
#pragma unroll 4
    for (int qq = 0; qq < 16; ++qq)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int s = 0; s < 2; ++s) {
          const int ii = ty + 16 * r, jj = tx + 16 * s;
          double t = acc[r][s];
#pragma unroll
          for (int f = 0; f < 4; ++f) t = fma(A[f][qq][ii], Bt[f][qq][jj], t);
          acc[r][s] = t;
        }
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int I = i0 + ty + 16 * r, J = j0 + tx + 16 * s;
      if (I < n_e && J < n_e) out[((int64_t)c * n_e + I) * n_e + J] = acc[r][s];
    }
}

// G[c][I][J] += alpha * sum_b d[gI] u[gI][b] d[gJ] w[gJ][b], g = map[c][.]
__global__ void __launch_bounds__(256)
    k_cell_outer(const int* __restrict__ map, int n_e, const double* __restrict__ d,
                 const double* __restrict__ u, const double* __restrict__ w, int64_t ld, int B,
                 const double* __restrict__ wt, double alpha, double* __restrict__ G, int nt) {
  __shared__ double Ui[16][T + 1];
  __shared__ double Wj[16][T + 1];
  __shared__ int gi[T], gj[T];
  const int64_t blk = blockIdx.x;
  const int tj = (int)(blk % nt), ti = (int)((blk / nt) % nt);
  const int c = (int)(blk / ((int64_t)nt * nt));
  const int i0 = ti * T, j0 = tj * T;
  if (threadIdx.x < T) {
    gi[threadIdx.x] = i0 + threadIdx.x < n_e ? map[(int64_t)c * n_e + i0 + threadIdx.x] : -1;
    gj[threadIdx.x] = j0 + threadIdx.x < n_e ? map[(int64_t)c * n_e + j0 + threadIdx.x] : -1;
  }
  __syncthreads();
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  double acc[2][2] = {{0, 0}, {0, 0}};
  for (int b0 = 0; b0 < B; b0 += 16) {
    for (int idx = threadIdx.x; idx < 16 * T; idx += 256) {
      const int bb = idx % 16, k = idx / 16;
      const int b = b0 + bb;
      Ui[bb][k] = (b < B && gi[k] >= 0) ? u[(int64_t)gi[k] * ld + b] : 0.0;
      Wj[bb][k] = (b < B && gj[k] >= 0) ? w[(int64_t)gj[k] * ld + b] * (wt ? wt[b] : 1.0) : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int bb = 0; bb < 16; ++bb)
#pragma unroll
      for (int r = 0; r < 2; ++r)
#pragma unroll
        for (int s = 0; s < 2; ++s) acc[r][s] = fma(Ui[bb][ty + 16 * r], Wj[bb][tx + 16 * s], acc[r][s]);
    __syncthreads();
  }
  for (int r = 0; r < 2; ++r)
    for (int s = 0; s < 2; ++s) {
      const int I = ty + 16 * r, J = tx + 16 * s;
      if (i0 + I < n_e && j0 + J < n_e)
        G[((int64_t)c * n_e + i0 + I) * n_e + j0 + J] += alpha * d[gi[I]] * d[gj[J]] * acc[r][s];
    }
}

// out[c][q] = jxw[c][q] * sum_I N[q][I] sum_J G[c][I][J] N[q][J]
__global__ void k_quad_contract(int n_cells, int n_e, int n_q, const double* __restrict__ N,
                                const double* __restrict__ G, const double* __restrict__ jxw,
                                double* __restrict__ out, int accumulate) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= (int64_t)n_cells * n_q) return;
  const int c = (int)(t / n_q), q = (int)(t % n_q);
  const double* Nq = N + (int64_t)q * n_e;
  const double* Gc = G + (int64_t)c * n_e * n_e;
  double acc = 0.0;
  for (int I = 0; I < n_e; ++I) {
    double s = 0.0;
    const double* gr = Gc + (int64_t)I * n_e;
    for (int J = 0; J < n_e; ++J) s = fma(gr[J], Nq[J], s);
    acc = fma(Nq[I], s, acc);
  }
  const double v = (jxw ? jxw[t] : 1.0) * acc;
  out[t] = accumulate ? out[t] + v : v;
}

}  // namespace

void assemble_cells(int n_cells, int n_e, int n_q, const double* N, const double* K,
                    const double* v, double* out, cudaStream_t st) {
  const int nt = (n_e + T - 1) / T;
  const int64_t blocks = (int64_t)n_cells * nt * nt;
  CHEFSI_REQUIRE(blocks < (1ll << 31), "assembly grid too large");
  k_assemble_cells<<<(unsigned)blocks, 256, 0, st>>>(n_cells, n_e, n_q, N, K, v, out, nt);
  CHEFSI_CHECK_LAUNCH();
}

void assemble_cells_bloch(int n_cells, int n_e, int n_q, const double* N, const double* dN,
                          const double* K, const double* v, const double* w, int n_k,
                          const double* kpts, double* out, cudaStream_t st, const double* g) {
  const int nt = (n_e + T - 1) / T;
  const int64_t blocks = (int64_t)n_cells * nt * nt;
  CHEFSI_REQUIRE(blocks < (1ll << 31), "assembly grid too large");
  if (g)
    k_assemble_bloch<true><<<(unsigned)blocks, 256, 0, st>>>(n_cells, n_e, n_q, N, dN, K, v, w, g,
                                                           n_k, kpts,
                                                           reinterpret_cast<double2*>(out), nt);
  else
    k_assemble_bloch<false><<<(unsigned)blocks, 256, 0, st>>>(n_cells, n_e, n_q, N, dN, K, v, w,
                                                            nullptr, n_k, kpts,
                                                            reinterpret_cast<double2*>(out), nt);
  CHEFSI_CHECK_LAUNCH();
}

void assemble_cells_geometry(int n_cells, int n_e, int n_q, const double* N, const double* dN,
                             const double* F, const double* v, double* out, cudaStream_t st) {
  const int nt = (n_e + T - 1) / T;
  const int64_t blocks = (int64_t)n_cells * nt * nt;
  CHEFSI_REQUIRE(blocks < (1ll << 31), "assembly grid too large");
  k_assemble_geom<<<(unsigned)blocks, 256, 0, st>>>(n_cells, n_e, n_q, N, dN, F, v, out, nt);
  CHEFSI_CHECK_LAUNCH();
}

void assemble_cells_gga(int n_cells, int n_e, int n_q, const double* N, const double* dN,
                        const double* K, const double* v, const double* g, double* out,
                        cudaStream_t st) {
  const int nt = (n_e + T - 1) / T;
  const int64_t blocks = (int64_t)n_cells * nt * nt;
  CHEFSI_REQUIRE(blocks < (1ll << 31), "assembly grid too large");
  k_assemble_gga<<<(unsigned)blocks, 256, 0, st>>>(n_cells, n_e, n_q, N, dN, K, v, g, out, nt);
  CHEFSI_CHECK_LAUNCH();
}

void cell_outer(chefsi_operator_s* op, const double* u, const double* w, int64_t ld, int B,
                double alpha, double* G, cudaStream_t st, const double* weights) {
  const int nt = (op->n_e + T - 1) / T;
  const int64_t blocks = (int64_t)op->n_cells * nt * nt;
  CHEFSI_REQUIRE(blocks < (1ll << 31), "cell outer grid too large");
  k_cell_outer<<<(unsigned)blocks, 256, 0, st>>>(op->map.ptr, op->n_e, op->inv_sqrt_mass.ptr, u,
                                                 w, ld, B, weights, alpha, G, nt);
  CHEFSI_CHECK_LAUNCH();
}

void quad_contract(int n_cells, int n_e, int n_q, const double* N, const double* G,
                   const double* jxw, double* out, cudaStream_t st, bool accumulate) {
  const int64_t n = (int64_t)n_cells * n_q;
  k_quad_contract<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(n_cells, n_e, n_q, N, G, jxw, out,
                                                               accumulate ? 1 : 0);
  CHEFSI_CHECK_LAUNCH();
}

}  // namespace chefsi
