// The fused Chebyshev filter on tensor cores: one persistent launch per degree finishes the
// three-term recurrence inside the HX kernel's epilogue, and the nonlocal apply rides in the
// same launch as extra K columns of the cell matrices.
//
// DFT-FE's filter (linearAlgebraOperationsDevice::chebyshevFilter,
// src/linAlg/linearAlgebraOperationsDevice.cc:531-727) runs per degree an HX (gather,
// cell GEMMs, scatter; the nonlocal term by a projection, a cross-cell reduction and an apply)
// and combinedDeviceKernel (:37-104), an axpby pass over the whole block. Here, per degree j:
//   1. W = C^T x_{j-1} over the projector rows (nl projection from the split rows), written
//      as split rows n_dofs + a P + i of the same buffer, scaled by 2^t;
//   2. one launch of cell_hx_tc_kernel<FUSED> computes, for every dof row,
//        x_j = a_j (A x_{j-1} + C V W) + c_j x_{j-1} + b_j x_{j-2}
//      and writes its FP16 hi + lo split: the vectors live only as split rows, so the next
//      degree's gather reads them directly and no separate recurrence pass exists.
// Every row is reduced into an FP32 accumulator pre-set to c_j x_{j-1} + b_j x_{j-2}; the unit
// that brings a row's last contribution (counted per row and 128-vector chunk) finishes it and
// pre-sets the accumulator for the next degree (see TcFused in tc.cu).
#include "internal.h"
#include "tc_common.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace chefsi {

namespace {

constexpr int kNlChunkRows = 256;  // rows per projection chunk (the operator's chunk table)

// acc = c (hi + lo) over n entries (float4 units): the accumulators of the first degree
__global__ void k_fz_acc_init(const __half* __restrict__ hi, const __half* __restrict__ lo,
                              int64_t n, float c, float* __restrict__ acc) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n / 4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const __half2* h = reinterpret_cast<const __half2*>(hi) + 2 * t;
    const __half2* l = reinterpret_cast<const __half2*>(lo) + 2 * t;
    const float2 h0 = __half22float2(h[0]), h1 = __half22float2(h[1]);
    const float2 l0 = __half22float2(l[0]), l1 = __half22float2(l[1]);
    reinterpret_cast<float4*>(acc)[t] =
        make_float4(c * (h0.x + l0.x), c * (h0.y + l0.y), c * (h1.x + l1.x), c * (h1.y + l1.y));
  }
}

// (hi, lo) = split(scale * W) over n entries (float4 units): the W rows of the split buffer
__global__ void k_fz_w_split(const float* __restrict__ W, int64_t n, float scale,
                             __half* __restrict__ hi, __half* __restrict__ lo) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n / 4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float4 w = reinterpret_cast<const float4*>(W)[t];
    const float v[4] = {scale * w.x, scale * w.y, scale * w.z, scale * w.w};
    __half h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      h[i] = __float2half_rn(v[i]);
      l[i] = __float2half_rn(v[i] - __half2float(h[i]));
    }
    reinterpret_cast<__half2*>(hi)[2 * t] = __halves2half2(h[0], h[1]);
    reinterpret_cast<__half2*>(hi)[2 * t + 1] = __halves2half2(h[2], h[3]);
    reinterpret_cast<__half2*>(lo)[2 * t] = __halves2half2(l[0], l[1]);
    reinterpret_cast<__half2*>(lo)[2 * t + 1] = __halves2half2(l[2], l[3]);
  }
}

// the tiles' diagonal entries (cell c, node I) = split of 2^s (A_II - shift / n_I), n_I the cell
// entries of the node's dof (1 for a row of one entry); shift 0 restores the split of 2^s A_II
// exactly as the plan wrote it
__global__ void k_fz_shift(const double* __restrict__ mats, int n_cells, int n_e, int n_half,
                           int n_halves, int nkb, const int2* __restrict__ rowinfo,
                           const unsigned char* __restrict__ ncontrib, double scale, double shift,
                           __half* __restrict__ hi, __half* __restrict__ lo) {
  const int64_t n = (int64_t)n_cells * n_e;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / n_e;
    const int I = (int)(t - c * n_e);
    const int sh = rowinfo[t].y;
    const double ne = sh < 0 ? 1.0 : (double)ncontrib[sh];
    const double v = scale * (mats[(c * n_e + I) * n_e + I] - shift / ne);
    const int half = I / n_half, ri = I % n_half;
    const int64_t tix = (c * n_halves + half) * nkb + I / 32;
    const int64_t o =
        tix * n_half * 32 + tcx::sw64_offset((uint32_t)ri, 2u * (uint32_t)(I % 32)) / 2;
    const __half h = __double2half(v);
    hi[o] = h;
    lo[o] = __double2half(v - (double)__half2float(h));
  }
}

// the largest |A_II| over the cells (one block)
__global__ void k_fz_diag_max(const double* __restrict__ mats, int64_t n, int n_e,
                              double* __restrict__ out) {
  __shared__ double red[256];
  double m = 0.0;
  for (int64_t t = threadIdx.x; t < n; t += blockDim.x) {
    const int64_t c = t / n_e;
    const int I = (int)(t - c * n_e);
    m = fmax(m, fabs(mats[(c * n_e + I) * n_e + I]));
  }
  red[threadIdx.x] = m;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// (hi, lo) = split(f x) over n entries (float4 units); rewrite: x = f x as well
__global__ void k_split_scaled(float* __restrict__ x, int64_t n, float f, int rewrite,
                               __half* __restrict__ hi, __half* __restrict__ lo) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n / 4;
       t += (int64_t)gridDim.x * blockDim.x) {
    float4 v = reinterpret_cast<const float4*>(x)[t];
    v.x *= f, v.y *= f, v.z *= f, v.w *= f;
    if (rewrite) reinterpret_cast<float4*>(x)[t] = v;
    const float a[4] = {v.x, v.y, v.z, v.w};
    __half h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      h[i] = __float2half_rn(a[i]);
      l[i] = __float2half_rn(a[i] - __half2float(h[i]));
    }
    reinterpret_cast<__half2*>(hi)[2 * t] = __halves2half2(h[0], h[1]);
    reinterpret_cast<__half2*>(hi)[2 * t + 1] = __halves2half2(h[2], h[3]);
    reinterpret_cast<__half2*>(lo)[2 * t] = __halves2half2(l[0], l[1]);
    reinterpret_cast<__half2*>(lo)[2 * t + 1] = __halves2half2(l[2], l[3]);
  }
}

// x = hi + lo over n entries (float4 units)
__global__ void k_fz_join(const __half* __restrict__ hi, const __half* __restrict__ lo, int64_t n,
                          float* __restrict__ x) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n / 4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const __half2* h = reinterpret_cast<const __half2*>(hi) + 2 * t;
    const __half2* l = reinterpret_cast<const __half2*>(lo) + 2 * t;
    const float2 h0 = __half22float2(h[0]), h1 = __half22float2(h[1]);
    const float2 l0 = __half22float2(l[0]), l1 = __half22float2(l[1]);
    reinterpret_cast<float4*>(x)[t] = make_float4(h0.x + l0.x, h0.y + l0.y, h1.x + l1.x, h1.y + l1.y);
  }
}

// the projector columns of the extended tiles: entry idx[k] of the tile array receives the split
// of scale * val[k]
__global__ void k_fz_scatter(const int64_t* __restrict__ idx, const double* __restrict__ val,
                             int64_t n, double scale, __half* __restrict__ hi,
                             __half* __restrict__ lo) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double v = scale * val[t];
    const __half h = __double2half(v);
    hi[idx[t]] = h;
    lo[idx[t]] = __double2half(v - (double)__half2float(h));
  }
}

// W[a][i][b] += sum over one chunk of atom a's rows of C[r][i] x[dof_r][b], x given by its FP16
// split rows: one CTA per (row chunk, 128 vectors); 8 warps over interleaved rows, U gathered
// rows in flight per lane (4 vectors each: 8-byte hi and lo pieces), partial sums reduced in
// shared memory and added with one float4 atomic per (projector, lane). PP >= P.
template <int PP, int U>
__global__ void __launch_bounds__(256, PP <= 8 ? 4 : 2)
    k_nl_project_split(const int* __restrict__ chunk_atom, const int* __restrict__ chunk_row0,
                       const int* __restrict__ atom_ptr, const int* __restrict__ dofs,
                       const float* __restrict__ C, int P, const __half* __restrict__ xh,
                       const __half* __restrict__ xl, int64_t ld, float* __restrict__ W, int B) {
  extern __shared__ float4 red_dyn[];  // [8][P][32]
  __shared__ float Cs[kNlChunkRows * PP];
  __shared__ int Ds[kNlChunkRows];
  const int ch = blockIdx.x;
  const int a = chunk_atom[ch];
  const int r0 = chunk_row0[ch];
  const int nr = min(r0 + kNlChunkRows, atom_ptr[a + 1]) - r0;
  for (int i = threadIdx.x; i < nr * P; i += blockDim.x) Cs[i] = C[(size_t)r0 * P + i];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) Ds[i] = dofs[r0 + i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.y * 128 + lane * 4;
  float4 acc[PP];
#pragma unroll
  for (int j = 0; j < PP; ++j) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
  auto load4 = [&](int r) {
    const int64_t o = (int64_t)Ds[r] * ld + b;
    const uint2 hu = __ldg(reinterpret_cast<const uint2*>(xh + o));
    const uint2 lu = __ldg(reinterpret_cast<const uint2*>(xl + o));
    const float2 h0 = __half22float2(*reinterpret_cast<const __half2*>(&hu.x));
    const float2 h1 = __half22float2(*reinterpret_cast<const __half2*>(&hu.y));
    const float2 l0 = __half22float2(*reinterpret_cast<const __half2*>(&lu.x));
    const float2 l1 = __half22float2(*reinterpret_cast<const __half2*>(&lu.y));
    return make_float4(h0.x + l0.x, h0.y + l0.y, h1.x + l1.x, h1.y + l1.y);
  };
  if (b < B) {
    int r = warp;
    for (; r + 8 * (U - 1) < nr; r += 8 * U) {
      float4 xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) xv[u] = load4(r + 8 * u);
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < PP; ++j) {
          if (j >= P) break;
          const float cv = Cs[(r + 8 * u) * P + j];
          acc[j].x = fmaf(cv, xv[u].x, acc[j].x);
          acc[j].y = fmaf(cv, xv[u].y, acc[j].y);
          acc[j].z = fmaf(cv, xv[u].z, acc[j].z);
          acc[j].w = fmaf(cv, xv[u].w, acc[j].w);
        }
    }
    for (; r < nr; r += 8) {
      const float4 xv = load4(r);
#pragma unroll
      for (int j = 0; j < PP; ++j) {
        if (j >= P) break;
        const float cv = Cs[r * P + j];
        acc[j].x = fmaf(cv, xv.x, acc[j].x);
        acc[j].y = fmaf(cv, xv.y, acc[j].y);
        acc[j].z = fmaf(cv, xv.z, acc[j].z);
        acc[j].w = fmaf(cv, xv.w, acc[j].w);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < PP; ++j)
    if (j < P) red_dyn[(warp * P + j) * 32 + lane] = acc[j];
  __syncthreads();
  for (int t = threadIdx.x; t < P * 32; t += blockDim.x) {
    const int j = t >> 5, l = t & 31;
    float4 sum = red_dyn[j * 32 + l];
    for (int w2 = 1; w2 < 8; ++w2) {
      const float4 v = red_dyn[(w2 * P + j) * 32 + l];
      sum.x += v.x, sum.y += v.y, sum.z += v.z, sum.w += v.w;
    }
    const int bb = blockIdx.y * 128 + l * 4;
    if (bb < B) atomicAdd(reinterpret_cast<float4*>(&W[((size_t)a * P + j) * B + bb]), sum);
  }
}

template <int PP, int U>
void launch_project_split(chefsi_operator_s* op, const __half* xh, const __half* xl, int B,
                          float* W, cudaStream_t st, const float* C32 = nullptr) {
  dim3 grid(op->nl_n_chunks, (B + 127) / 128);
  const size_t red = sizeof(float4) * 8 * op->n_proj * 32;
  CHEFSI_CUDA(cudaFuncSetAttribute(k_nl_project_split<PP, U>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(float4) * 8 * PP * 32)));
  k_nl_project_split<PP, U><<<grid, 256, red, st>>>(op->nl_chunk_atom.ptr, op->nl_chunk_row0.ptr,
                                                    op->nl_ptr.ptr, op->nl_dofs.ptr,
                                                    C32 ? C32 : op->nl_vals32.ptr, op->n_proj, xh,
                                                    xl, B, W, B);
  CHEFSI_CHECK_LAUNCH();
}

// distribute on the split rows: x_s = sum_e w'_e x_m(e) for every slave row s
// (constraintMatrixInfoDevice.cc:546-594 in the folded basis), written as its FP16 split
__global__ void k_con_split_distribute(const int* __restrict__ ids, const int* __restrict__ ptr,
                                       const int* __restrict__ mas, const double* __restrict__ w,
                                       int n_con, int B, __half* hi, __half* lo) {
  const int64_t n = (int64_t)n_con * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / B), b = (int)(t - (int64_t)k * B);
    float acc = 0.f;
    for (int e = ptr[k]; e < ptr[k + 1]; ++e) {
      const int64_t o = (int64_t)mas[e] * B + b;
      acc = fmaf((float)w[e], __half2float(hi[o]) + __half2float(lo[o]), acc);
    }
    const __half h = __float2half_rn(acc);
    const int64_t o = (int64_t)ids[k] * B + b;
    hi[o] = h;
    lo[o] = __float2half_rn(acc - __half2float(h));
  }
}

// save[k] = y[slave k]; y[slave k] = 0 (the launch then reduces only its own contributions
// into the slave rows)
__global__ void k_con_stash(const int* __restrict__ ids, int n_con, float* y, int64_t ldy, int B,
                            float* __restrict__ save) {
  const int64_t n = (int64_t)n_con * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / B), b = (int)(t - (int64_t)k * B);
    float* p = y + (int64_t)ids[k] * ldy + b;
    save[t] = *p;
    *p = 0.f;
  }
}

// distribute_slave_to_master (constraintMatrixInfoDevice.cc:597-816 in the folded basis):
// y_m += w'_e y_s, then the slave row gets its saved value back
__global__ void k_con_adjoint(const int* __restrict__ ids, const int* __restrict__ ptr,
                              const int* __restrict__ mas, const double* __restrict__ w, int n_con,
                              float* y, int64_t ldy, int B, const float* __restrict__ save) {
  const int64_t n = (int64_t)n_con * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / B), b = (int)(t - (int64_t)k * B);
    float* p = y + (int64_t)ids[k] * ldy + b;
    const float v = *p;
    for (int e = ptr[k]; e < ptr[k + 1]; ++e)
      atomicAdd(y + (int64_t)mas[e] * ldy + b, (float)w[e] * v);
    *p = save[t];
  }
}

template <typename T>
std::vector<T> to_host(const DeviceBuffer<T>& b, size_t n) {
  std::vector<T> h(n);
  if (n) CHEFSI_CUDA(cudaMemcpy(h.data(), b.ptr, n * sizeof(T), cudaMemcpyDeviceToHost));
  return h;
}
template <typename T>
void to_device(DeviceBuffer<T>& b, const std::vector<T>& h) {
  b.reset(h.size());
  if (!h.empty())
    CHEFSI_CUDA(cudaMemcpy(b.ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
}

}  // namespace

// the plan's tables serve real operators of at most 512 nodes per cell on an sm_100-family
// device, with M^{-1/2} folded in by the operator or (constraint rows) by the plan itself
bool plan_usable(chefsi_operator_s* op) {
  return !op->is_complex && op->n_e <= 512 && op->n_proj <= 16 &&
         (op->folded || op->n_con > 0) && tcx::tcgen05_device();
}
bool fused_plan_usable(chefsi_operator_s* op) { return plan_usable(op) && op->folded; }
bool constrained_tc_usable(chefsi_operator_s* op, int B) {
  return plan_usable(op) && !op->folded && B % 8 == 0;
}

// The plan's tiles from the current cell matrices (on the device; the map-dependent tables
// and the projector columns' values stay): the power-of-two scale, the split of the cell
// matrices, the projector columns scattered at that scale, the diagonal bound of the shift.
static void build_plan_tiles(chefsi_operator_s* op, cudaStream_t st) {
  FusedPlan& fp = op->fz;
  const int nc = op->n_cells, ne = op->n_e;
  DeviceBuffer<double> amax(1);
  absmax_block_f64(op->mats64.ptr, ne, (int64_t)nc * ne, ne, amax.ptr, st);
  double am = 0.0;
  CHEFSI_CUDA(cudaMemcpyAsync(&am, amax.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  // constraint rows: the plan's tiles hold d_I A_IJ d_J, bounded by max|A| max(d)^2
  if (!op->folded) am *= fp.dmax2;
  am = std::max(am, fp.ext_max);
  // largest entry in [2^11, 2^12): room on the diagonals for the filter's shift (FP16 keeps
  // its 11-bit significand at every magnitude, so the headroom costs no precision)
  const int e = (am > 0 && std::isfinite(am)) ? 11 - (int)std::floor(std::log2(am)) : 0;
  const double scale = std::ldexp(1.0, e);
  fp.diag_max = 0.0;
  if (op->folded) {
    DeviceBuffer<double> dmx(1);
    k_fz_diag_max<<<1, 256, 0, st>>>(op->mats64.ptr, (int64_t)nc * ne, ne, dmx.ptr);
    CHEFSI_CHECK_LAUNCH();
    CHEFSI_CUDA(cudaMemcpyAsync(&fp.diag_max, dmx.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
    CHEFSI_CUDA(cudaStreamSynchronize(st));
  }
  fp.shift = 0.0;
  int n_half = 0, n_halves = 0;
  tc_row_split(ne, &n_half, &n_halves);
  const size_t ntile = (size_t)nc * n_halves * fp.nkb * n_half * 32;
  if (fp.hi.n != ntile) {
    fp.hi.reset(ntile);
    fp.lo.reset(ntile);
  }
  split_mats_ext(op, fp.nkb, scale, fp.hi.ptr, fp.lo.ptr, st);
  const int64_t n_ext = (int64_t)fp.ext_idx.n;
  if (n_ext) {
    k_fz_scatter<<<grid_for(n_ext, 256), 256, 0, st>>>(fp.ext_idx.ptr, fp.ext_val.ptr, n_ext,
                                                       scale, fp.hi.ptr, fp.lo.ptr);
    CHEFSI_CHECK_LAUNCH();
  }
  fp.scale = (float)scale;
  fp.tiles_ready = true;
}

void prepare_fused_plan(chefsi_operator_s* op, cudaStream_t st) {
  FusedPlan& fp = op->fz;
  if (fp.ready) {
    if (!fp.tiles_ready) build_plan_tiles(op, st);
    return;
  }
  CHEFSI_REQUIRE(plan_usable(op), "tensor-core plan: operator not supported");
  const int nc = op->n_cells, ne = op->n_e;
  const int64_t M = op->n_dofs;
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  const std::vector<int> map = to_host(op->map, (size_t)nc * ne);
  // cell entries per dof (CSR) and the shared-row numbering
  std::vector<int64_t> eptr(M + 1, 0);
  for (int v : map) ++eptr[v + 1];
  for (int64_t d = 0; d < M; ++d) eptr[d + 1] += eptr[d];
  std::vector<int> ent(eptr[M]);
  {
    std::vector<int64_t> fill(eptr.begin(), eptr.end() - 1);
    for (int64_t k = 0; k < (int64_t)map.size(); ++k) ent[fill[map[k]]++] = (int)k;  // c * ne + I
  }
  std::vector<int> sidx(M, -1);
  std::vector<unsigned char> ncontrib;
  int64_t n_shared = 0;
  for (int64_t d = 0; d < M; ++d) {
    const int64_t cnt = eptr[d + 1] - eptr[d];
    CHEFSI_REQUIRE(cnt <= 255, "fused filter step: a dof with more than 255 cell entries");
    if (cnt > 1) {
      sidx[d] = (int)n_shared++;
      ncontrib.push_back((unsigned char)cnt);
    }
  }
  std::vector<int> rowinfo((size_t)nc * ne * 2);
  for (size_t k = 0; k < map.size(); ++k) {
    rowinfo[2 * k] = map[k];
    rowinfo[2 * k + 1] = sidx[map[k]];
  }
  // projector (atom, dof) pairs -> cell entries, atoms -> per-cell slots
  const int P = op->n_atoms ? op->n_proj : 0;
  std::vector<std::vector<int>> slots(nc);
  auto slot_of = [&](int c, int a) {
    const auto& v = slots[c];
    for (size_t i = 0; i < v.size(); ++i)
      if (v[i] == a) return (int)i;
    return -1;
  };
  std::vector<int> nptr, ndofs;
  std::vector<double> C, V;
  if (P) {
    nptr = to_host(op->nl_ptr, (size_t)op->n_atoms + 1);
    ndofs = to_host(op->nl_dofs, (size_t)op->nl_nnz);
    C = to_host(op->nl_vals64, (size_t)op->nl_nnz * P);
    if (!op->folded) {
      // constraint rows: the operator keeps C unscaled; the plan folds M^{-1/2} in (and keeps
      // an FP32 copy for the projection from the split rows)
      const std::vector<double> d = to_host(op->inv_sqrt_mass, (size_t)M);
      std::vector<float> c32((size_t)op->nl_nnz * P);
      for (int64_t r = 0; r < op->nl_nnz; ++r)
        for (int j = 0; j < P; ++j) {
          C[(size_t)r * P + j] *= d[ndofs[r]];
          c32[(size_t)r * P + j] = (float)C[(size_t)r * P + j];
        }
      to_device(fp.nl_c32, c32);
    }
    V = to_host(op->couplings, (size_t)op->n_atoms * P);
    // rows owned by one cell entry fix their cell; the others join a cell of theirs that has
    // the atom already, else the one with the fewest atoms
    for (int a = 0; a < op->n_atoms; ++a)
      for (int r = nptr[a]; r < nptr[a + 1]; ++r) {
        const int d = ndofs[r];
        if (eptr[d + 1] - eptr[d] != 1) continue;
        const int c = ent[eptr[d]] / ne;
        if (slot_of(c, a) < 0) slots[c].push_back(a);
      }
    for (int a = 0; a < op->n_atoms; ++a)
      for (int r = nptr[a]; r < nptr[a + 1]; ++r) {
        const int d = ndofs[r];
        bool have = false;
        int best = -1;
        for (int64_t k = eptr[d]; k < eptr[d + 1]; ++k) {
          const int c = ent[k] / ne;
          if (slot_of(c, a) >= 0) {
            have = true;
            break;
          }
          if (best < 0 || slots[c].size() < slots[best].size()) best = c;
        }
        if (!have) slots[best].push_back(a);
      }
  }
  int max_slots = 0;
  for (const auto& v : slots) max_slots = std::max(max_slots, (int)v.size());
  const int kstride = (ne + P * max_slots + 31) / 32 * 32;
  const int nkb = kstride / 32;
  std::vector<int> mapk((size_t)nc * kstride, -1);
  for (int c = 0; c < nc; ++c) {
    for (int I = 0; I < ne; ++I) mapk[(size_t)c * kstride + I] = map[(size_t)c * ne + I];
    for (size_t sl = 0; sl < slots[c].size(); ++sl)
      for (int j = 0; j < P; ++j)
        mapk[(size_t)c * kstride + ne + sl * P + j] = (int)(M + (int64_t)slots[c][sl] * P + j);
  }
  CHEFSI_REQUIRE(M + (int64_t)op->n_atoms * P < (1ll << 31),
                 "fused filter step: too many rows for 32-bit map entries");
  // scales: 2^t W with max |x| <= 2^9 stays below 2^15; the tiles hold 2^s A and 2^(s-t) C V
  double wscale = 1.0, ext_max = 0.0;
  if (P) {
    double n1max = 0.0;
    for (int a = 0; a < op->n_atoms; ++a)
      for (int j = 0; j < P; ++j) {
        double n1 = 0.0;
        for (int r = nptr[a]; r < nptr[a + 1]; ++r) n1 += std::fabs(C[(size_t)r * P + j]);
        n1max = std::max(n1max, n1);
      }
    if (n1max > 0.0 && std::isfinite(n1max)) wscale = std::ldexp(1.0, (int)std::floor(6.0 - std::log2(n1max)));
    for (int a = 0; a < op->n_atoms; ++a)
      for (int r = nptr[a]; r < nptr[a + 1]; ++r)
        for (int j = 0; j < P; ++j)
          ext_max = std::max(ext_max, std::fabs(C[(size_t)r * P + j] * V[(size_t)a * P + j]) / wscale);
  }
  fp.dmax2 = 1.0;
  if (!op->folded) {
    // the plan's tiles hold d_I A_IJ d_J: bound their largest entry by max|A| max(d)^2, and
    // rescale the constraint weights for the folded basis: x_s = sum (w d_m / d_s) x_m
    DeviceBuffer<double> dm(1);
    absmax_block_f64(op->inv_sqrt_mass.ptr, 1, M, 1, dm.ptr, st);
    double dmax = 0.0;
    CHEFSI_CUDA(cudaMemcpyAsync(&dmax, dm.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
    CHEFSI_CUDA(cudaStreamSynchronize(st));
    fp.dmax2 = dmax * dmax;
    const std::vector<double> d = to_host(op->inv_sqrt_mass, (size_t)M);
    const std::vector<int> ids = to_host(op->con_ids, (size_t)op->n_con);
    const std::vector<int> ptr = to_host(op->con_ptr, (size_t)op->n_con + 1);
    const std::vector<int> mas = to_host(op->con_master, (size_t)ptr[op->n_con]);
    std::vector<double> w = to_host(op->con_w, (size_t)ptr[op->n_con]);
    for (int k = 0; k < op->n_con; ++k)
      for (int e = ptr[k]; e < ptr[k + 1]; ++e) w[e] *= d[mas[e]] / d[ids[k]];
    to_device(fp.con_wp, w);
  }
  fp.ext_max = ext_max;
  int n_half = 0, n_halves = 0;
  tc_row_split(ne, &n_half, &n_halves);
  if (P) {
    std::vector<int64_t> idx;
    std::vector<double> val;
    idx.reserve((size_t)op->nl_nnz * P);
    val.reserve((size_t)op->nl_nnz * P);
    for (int a = 0; a < op->n_atoms; ++a)
      for (int r = nptr[a]; r < nptr[a + 1]; ++r) {
        const int d = ndofs[r];
        int entry = -1, sl = -1;
        for (int64_t k = eptr[d]; k < eptr[d + 1] && entry < 0; ++k) {
          const int s2 = slot_of(ent[k] / ne, a);
          if (s2 >= 0) entry = ent[k], sl = s2;
        }
        CHEFSI_REQUIRE(entry >= 0, "fused filter step: projector row without a cell");
        const int c = entry / ne, I = entry % ne;
        const int half = I / n_half, ri = I % n_half;
        for (int j = 0; j < P; ++j) {
          const int J = ne + sl * P + j;
          const int64_t tix = ((int64_t)c * n_halves + half) * nkb + J / 32;
          idx.push_back(tix * n_half * 32 + tcx::sw64_offset((uint32_t)ri, 2u * (uint32_t)(J % 32)) / 2);
          val.push_back(C[(size_t)r * P + j] * V[(size_t)a * P + j] / wscale);
        }
      }
    to_device(fp.ext_idx, idx);
    to_device(fp.ext_val, val);
  }
  to_device(fp.mapk, mapk);
  to_device(fp.rowinfo, rowinfo);
  to_device(fp.ncontrib, ncontrib);
  fp.nkb = nkb;
  fp.kstride = kstride;
  fp.max_slots = max_slots;
  fp.n_shared = n_shared;
  fp.rows = M + (int64_t)op->n_atoms * P;
  fp.wscale = (float)wscale;
  build_plan_tiles(op, st);
  fp.ready = true;
}

void nl_project_to_split(chefsi_operator_s* op, const float* x, int B, float* W, __half* hi,
                         __half* lo, cudaStream_t st, double f) {
  if (op->n_atoms == 0) return;
  const FusedPlan& fp = op->fz;
  nl_project_f32(op, x, B, W, B, st);   // zeroes W first
  const int64_t nw = (int64_t)op->n_atoms * op->n_proj * B;
  const int64_t off = op->n_dofs * (int64_t)B;
  k_fz_w_split<<<grid_for(nw / 4, 256), 256, 0, st>>>(W, nw, (float)(fp.wscale * f), hi + off,
                                                      lo + off);
  CHEFSI_CHECK_LAUNCH();
}

bool set_tile_shift(chefsi_operator_s* op, double shift, cudaStream_t st) {
  FusedPlan& fp = op->fz;
  CHEFSI_REQUIRE(fp.ready && fp.tiles_ready, "tile shift: plan not prepared");
  if (shift == fp.shift) return true;
  if (!op->folded) return false;
  // |A_II - shift / n_I| <= max |A_II| + |shift| must stay inside FP16's range once scaled
  if (!(((double)fp.scale) * (fp.diag_max + std::fabs(shift)) < 60000.0)) return false;
  int n_half = 0, n_halves = 0;
  tc_row_split(op->n_e, &n_half, &n_halves);
  const int64_t n = (int64_t)op->n_cells * op->n_e;
  k_fz_shift<<<grid_for(n, 256), 256, 0, st>>>(
      op->mats64.ptr, op->n_cells, op->n_e, n_half, n_halves, fp.nkb,
      reinterpret_cast<const int2*>(fp.rowinfo.ptr), fp.ncontrib.ptr, (double)fp.scale, shift,
      fp.hi.ptr, fp.lo.ptr);
  CHEFSI_CHECK_LAUNCH();
  fp.shift = shift;
  return true;
}

void split_scaled_f32(float* x, int64_t n, double f, bool rewrite, __half* hi, __half* lo,
                      cudaStream_t st) {
  CHEFSI_REQUIRE(n % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(hi) & 7) == 0 &&
                     (reinterpret_cast<uintptr_t>(lo) & 7) == 0,
                 "scaled split: 16-byte aligned block, a multiple of 4 entries");
  k_split_scaled<<<grid_for(n / 4, 256), 256, 0, st>>>(x, n, (float)f, rewrite ? 1 : 0, hi, lo);
  CHEFSI_CHECK_LAUNCH();
}

void hx_tc_constrained_split(chefsi_operator_s* op, __half* hi, __half* lo, float* dst,
                             int64_t ldd, int B, double scalar, float* W, float* save,
                             cudaStream_t st) {
  prepare_fused_plan(op, st);
  const FusedPlan& fp = op->fz;
  const int64_t nc = (int64_t)op->n_con * B;
  k_con_split_distribute<<<grid_for(nc, 256), 256, 0, st>>>(
      op->con_ids.ptr, op->con_ptr.ptr, op->con_master.ptr, fp.con_wp.ptr, op->n_con, B, hi, lo);
  CHEFSI_CHECK_LAUNCH();
  if (op->n_atoms) {
    const int64_t nw = (int64_t)op->n_atoms * op->n_proj * B;
    CHEFSI_CUDA(cudaMemsetAsync(W, 0, sizeof(float) * nw, st));
    if (op->n_proj <= 4)
      launch_project_split<4, 8>(op, hi, lo, B, W, st, fp.nl_c32.ptr);
    else if (op->n_proj <= 8)
      launch_project_split<8, 4>(op, hi, lo, B, W, st, fp.nl_c32.ptr);
    else
      launch_project_split<16, 4>(op, hi, lo, B, W, st, fp.nl_c32.ptr);
    const int64_t off = op->n_dofs * (int64_t)B;
    k_fz_w_split<<<grid_for(nw / 4, 256), 256, 0, st>>>(W, nw, fp.wscale, hi + off, lo + off);
    CHEFSI_CHECK_LAUNCH();
  }
  k_con_stash<<<grid_for(nc, 256), 256, 0, st>>>(op->con_ids.ptr, op->n_con, dst, ldd, B, save);
  CHEFSI_CHECK_LAUNCH();
  hx_tc_folded_launch(op, hi, lo, dst, ldd, B, scalar, st);
  k_con_adjoint<<<grid_for(nc, 256), 256, 0, st>>>(op->con_ids.ptr, op->con_ptr.ptr,
                                                   op->con_master.ptr, fp.con_wp.ptr, op->n_con,
                                                   dst, ldd, B, save);
  CHEFSI_CHECK_LAUNCH();
}

void hx_tc_constrained(chefsi_operator_s* op, const float* src, int64_t lds, float* dst,
                       int64_t ldd, int B, double scalar, bool accumulate, cudaStream_t st) {
  CHEFSI_REQUIRE(constrained_tc_usable(op, B) && lds % 2 == 0 && ldd % 4 == 0 &&
                     (reinterpret_cast<uintptr_t>(dst) & 15) == 0,
                 "constrained tensor-core HX: real operator, B a multiple of 8, aligned rows");
  prepare_fused_plan(op, st);
  const size_t rows = (size_t)op->fz.rows;
  __half* hi = op->xs_hi.ensure(rows * B);
  __half* lo = op->xs_lo.ensure(rows * B);
  float* W = op->n_atoms ? op->nlW32.ensure((size_t)op->n_atoms * op->n_proj * B) : nullptr;
  float* save = op->ws32x.ensure((size_t)op->n_con * B);
  split_rows_f32(src, lds, op->n_dofs, B, hi, lo, st);
  if (!accumulate) scale_block<float>(dst, ldd, op->n_dofs, B, 0.0, st);
  hx_tc_constrained_split(op, hi, lo, dst, ldd, B, scalar, W, save, st);
}

// The filter of one block: X [M][B] FP32 in (scaled so that max |x| ~ 2^8), p_m(A) X out.
// Coefficients of the sigma-scaled recurrence (linearAlgebraOperationsDevice.cc:531-727):
//   x_1 = alpha1 (A - c) x_0, alpha1 = sigma1 / e;
//   x_j = alpha1_j (A - c) x_{j-1} + alpha2_j x_{j-2}, sigma2 = 1 / (gamma - sigma),
//   alpha1_j = 2 sigma2 / e, alpha2_j = -sigma sigma2.
void cheb_filter_fused(chefsi_operator_s* op, FusedWork& w, float* X, int64_t M, int B, int m,
                       double a, double b, double a0, const std::function<void()>& mark,
                       cudaStream_t st) {
  prepare_fused_plan(op, st);
  const FusedPlan& fp = op->fz;
  const int n_chunks = (B + 127) / 128;
  const size_t nrows = (size_t)fp.rows * B;
  __half* h[2] = {w.hi[0].ensure(nrows), w.hi[1].ensure(nrows)};
  __half* l[2] = {w.lo[0].ensure(nrows), w.lo[1].ensure(nrows)};
  float* acc = w.acc.ensure((size_t)M * B);
  unsigned* counter = w.counter.ensure(std::max<size_t>(1, (size_t)fp.n_shared * n_chunks));
  float* W = op->n_atoms ? w.W.ensure((size_t)op->n_atoms * op->n_proj * B) : nullptr;
  CHEFSI_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned) * (size_t)fp.n_shared * n_chunks, st));
  // coefficients a_j, c_j, b_j for j = 1..m
  std::vector<double> ca(m + 2, 0.0), cc(m + 2, 0.0), cb(m + 2, 0.0);
  {
    const double e = (b - a) / 2.0, c = (b + a) / 2.0;
    double sigma = e / (a0 - c);
    const double sigma1 = sigma, gamma = 2.0 / sigma1;
    ca[1] = sigma1 / e;
    cc[1] = -c * ca[1];
    for (int j = 2; j <= m; ++j) {
      const double sigma2 = 1.0 / (gamma - sigma);
      ca[j] = 2.0 * sigma2 / e;
      cc[j] = -c * ca[j];
      cb[j] = -(sigma * sigma2);
      sigma = sigma2;
    }
  }
  split_rows_f32(X, B, M, B, h[0], l[0], st);
  k_fz_acc_init<<<grid_for(M * B / 4, 256), 256, 0, st>>>(h[0], l[0], M * B, (float)cc[1], acc);
  CHEFSI_CHECK_LAUNCH();
  for (int j = 1; j <= m; ++j) {
    const int in = (j - 1) & 1, out = j & 1;
    mark();
    if (op->n_atoms) {
      const size_t nw = (size_t)op->n_atoms * op->n_proj * B;
      CHEFSI_CUDA(cudaMemsetAsync(W, 0, sizeof(float) * nw, st));
      if (op->n_proj <= 4)
        launch_project_split<4, 8>(op, h[in], l[in], B, W, st);
      else if (op->n_proj <= 8)
        launch_project_split<8, 4>(op, h[in], l[in], B, W, st);
      else
        launch_project_split<16, 4>(op, h[in], l[in], B, W, st);
      k_fz_w_split<<<grid_for((int64_t)nw / 4, 256), 256, 0, st>>>(W, (int64_t)nw, fp.wscale,
                                                                   h[in] + M * B, l[in] + M * B);
      CHEFSI_CHECK_LAUNCH();
    }
    TcFusedLaunch f{};
    f.op = op;
    f.xhi = h[in];
    f.xlo = l[in];
    f.ohi = h[out];
    f.olo = l[out];
    f.acc = acc;
    f.counter = counter;
    f.B = B;
    f.a = ca[j];
    f.c = cc[j];
    f.b = cb[j];
    f.has_next = j < m;
    f.cn = cc[j + 1];
    f.bn = cb[j + 1];
    hx_tc_fused_launch(f, st);
    mark();
  }
  k_fz_join<<<grid_for(M * B / 4, 256), 256, 0, st>>>(h[m & 1], l[m & 1], M * B, X);
  CHEFSI_CHECK_LAUNCH();
}

}  // namespace chefsi
