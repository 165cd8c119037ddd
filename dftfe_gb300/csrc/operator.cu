// Kohn-Sham operator on the device: creation (maps, cell matrices, mass scaling, nonlocal
// projectors, constraints) and the SIMT operator apply HX for FP64, FP32 and complex FP64.
//
// The apply is DFT-FE's cell-matrix formulation (src/dftOperator/
// matrixVectorProductImplementationsDevice.cc:27-117): gather the cell's dofs, multiply by
// the dense cell matrix, scatter-add. Here the three steps are one kernel: a CTA owns one
// (cell, row tile, vector tile), gathers its X rows straight into shared memory through the
// cell->dof map, runs the register-tiled product and scatter-adds with atomics, so the
// reference's n_cells x n_e x B cell-vector arrays are never materialised. When the operator
// has no constraint rows (periodicity folded into the map), M^{-1/2} is folded into the cell
// matrices and projectors at creation, so HX needs no scaling passes.
#include "internal.h"
#include "pow2.cuh"

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <atomic>
#include <mutex>
#include <type_traits>

namespace chefsi {

// ------------------------------------------------------------------ status & allocation
static thread_local std::string g_last_error;
void set_last_error(const std::string& msg) { g_last_error = msg; }
const char* last_error_cstr() { return g_last_error.c_str(); }

static std::atomic<unsigned long long> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

bool fault_injected(const char* what) {
  const char* v = std::getenv("CHEFSI_FAULT_INJECT");
  return v && std::strcmp(v, what) == 0;
}

void* dmalloc(size_t bytes) {
  if (fault_injected("alloc"))
    throw Error(CHEFSI_ERR_ALLOC, "device allocation refused by CHEFSI_FAULT_INJECT=alloc");
  void* p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    throw Error(CHEFSI_ERR_ALLOC, std::string("cudaMalloc(") + std::to_string(bytes) +
                                      ") failed: " + cudaGetErrorString(e));
  }
  return p;
}
void dfree(void* p) { cudaFree(p); }

// ------------------------------------------------------------------ scalar traits
__device__ __forceinline__ cplx operator+(cplx a, cplx b) { return {a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cplx operator*(cplx a, cplx b) {
  return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
__device__ __forceinline__ cplx operator*(double s, cplx a) { return {s * a.x, s * a.y}; }

template <typename T> struct Tr;
template <> struct Tr<double> {
  __device__ static double zero() { return 0.0; }
  __device__ static void fma(double& acc, double a, double b) { acc = ::fma(a, b, acc); }
  __device__ static void atomic_add(double* p, double v) { atomicAdd(p, v); }
  __device__ static double scale(double s, double v) { return s * v; }
};
template <> struct Tr<float> {
  __device__ static float zero() { return 0.f; }
  __device__ static void fma(float& acc, float a, float b) { acc = fmaf(a, b, acc); }
  __device__ static void atomic_add(float* p, float v) { atomicAdd(p, v); }
  __device__ static float scale(double s, float v) { return (float)s * v; }
};
template <> struct Tr<cplx> {
  __device__ static cplx zero() { return {0.0, 0.0}; }
  __device__ static void fma(cplx& acc, cplx a, cplx b) {
    acc.x = ::fma(a.x, b.x, ::fma(-a.y, b.y, acc.x));
    acc.y = ::fma(a.x, b.y, ::fma(a.y, b.x, acc.y));
  }
  __device__ static void atomic_add(cplx* p, cplx v) {
    atomicAdd(&p->x, v.x);
    atomicAdd(&p->y, v.y);
  }
  __device__ static cplx scale(double s, cplx v) { return {s * v.x, s * v.y}; }
};

// ------------------------------------------------------------------ fused cell HX (SIMT)
// CTA tile: TI cell rows x TB vectors; thread (tx, ty) owns rows ty + r*(TI/RI) and vectors
// tx + s*(TB/RB). Linear block id -> (vector tile fastest, row tile, cell) so CTAs working on
// one cell run together and share its matrix and X rows through L2.
constexpr int kMaxNodesPerCell = 512;

template <typename T, int TI, int TB, int RI, int RB, int TK>
__global__ void __launch_bounds__((TI / RI) * (TB / RB))
    cell_hx_simt(const T* __restrict__ mats, const int* __restrict__ map, int n_e,
                 const T* __restrict__ src, int64_t lds, T* __restrict__ dst, int64_t ldd, int B,
                 double scalar, int n_itiles, int n_btiles) {
  constexpr int NX = TB / RB;  // threads along vectors
  constexpr int NY = TI / RI;  // threads along rows
  constexpr int NT = NX * NY;
  __shared__ T As[TK][TI + 1];
  __shared__ T Xs[TK][TB];
  __shared__ int rows[kMaxNodesPerCell];

  const int64_t lin = blockIdx.x;
  const int bt = (int)(lin % n_btiles);
  const int it = (int)((lin / n_btiles) % n_itiles);
  const int c = (int)(lin / ((int64_t)n_btiles * n_itiles));
  const int i0 = it * TI, b0 = bt * TB;
  const int tid = threadIdx.x;
  const int tx = tid % NX, ty = tid / NX;
  const T* Ac = mats + (size_t)c * n_e * n_e;

  for (int k = tid; k < n_e; k += NT) rows[k] = map[(size_t)c * n_e + k];
  __syncthreads();

  T acc[RI][RB];
#pragma unroll
  for (int r = 0; r < RI; ++r)
#pragma unroll
    for (int s = 0; s < RB; ++s) acc[r][s] = Tr<T>::zero();

  for (int k0 = 0; k0 < n_e; k0 += TK) {
    for (int idx = tid; idx < TI * TK; idx += NT) {
      const int i = idx / TK, k = idx % TK;
      const int gi = i0 + i, gk = k0 + k;
      As[k][i] = (gi < n_e && gk < n_e) ? Ac[(size_t)gi * n_e + gk] : Tr<T>::zero();
    }
    for (int idx = tid; idx < TK * TB; idx += NT) {
      const int k = idx / TB, b = idx % TB;
      const int gk = k0 + k, gb = b0 + b;
      Xs[k][b] = (gk < n_e && gb < B) ? src[(int64_t)rows[gk] * lds + gb] : Tr<T>::zero();
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < TK; ++k) {
      T a[RI], x[RB];
#pragma unroll
      for (int r = 0; r < RI; ++r) a[r] = As[k][ty + r * NY];
#pragma unroll
      for (int s = 0; s < RB; ++s) x[s] = Xs[k][tx + s * NX];
#pragma unroll
      for (int r = 0; r < RI; ++r)
#pragma unroll
        for (int s = 0; s < RB; ++s) Tr<T>::fma(acc[r][s], a[r], x[s]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < RI; ++r) {
    const int gi = i0 + ty + r * NY;
    if (gi >= n_e) continue;
    T* drow = dst + (int64_t)rows[gi] * ldd;
#pragma unroll
    for (int s = 0; s < RB; ++s) {
      const int gb = b0 + tx + s * NX;
      if (gb < B) Tr<T>::atomic_add(drow + gb, Tr<T>::scale(scalar, acc[r][s]));
    }
  }
}

template <typename T, int TI, int TB, int RI, int RB, int TK>
static void launch_cell_hx(const T* mats, const int* map, int n_cells, int n_e, const T* src,
                           int64_t lds, T* dst, int64_t ldd, int B, double scalar,
                           cudaStream_t st) {
  const int nit = (n_e + TI - 1) / TI, nbt = (B + TB - 1) / TB;
  const int64_t blocks = (int64_t)n_cells * nit * nbt;
  CHEFSI_REQUIRE(blocks < (1ll << 31), "cell HX grid too large");
  cell_hx_simt<T, TI, TB, RI, RB, TK><<<(unsigned)blocks, (TI / RI) * (TB / RB), 0, st>>>(
      mats, map, n_e, src, lds, dst, ldd, B, scalar, nit, nbt);
  CHEFSI_CHECK_LAUNCH();
}

// ------------------------------------------------------------------ nonlocal projectors
// Rows of every atom are cut into chunks of kNlChunk rows. project: W[a][j][b] += sum_rows
// C[r][j] x[dof_r][b]; apply: y[dof_r][b] += scalar * sum_j C[r][j] V[a][j] W[a][j][b].
constexpr int kNlChunk = 256;
constexpr int kMaxProj = 16;

template <typename T>
__global__ void nl_project(const int* __restrict__ chunk_atom, const int* __restrict__ chunk_row0,
                           const int* __restrict__ atom_ptr, const int* __restrict__ dofs,
                           const T* __restrict__ C, int P, const T* __restrict__ src, int64_t lds,
                           T* __restrict__ W, int B) {
  __shared__ T Cs[kNlChunk * kMaxProj];
  __shared__ int Ds[kNlChunk];
  const int ch = blockIdx.x;
  const int a = chunk_atom[ch];
  const int r0 = chunk_row0[ch];
  const int r1 = min(r0 + kNlChunk, atom_ptr[a + 1]);
  const int nr = r1 - r0;
  for (int i = threadIdx.x; i < nr * P; i += blockDim.x) Cs[i] = C[(size_t)r0 * P + i];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) Ds[i] = dofs[r0 + i];
  __syncthreads();
  const int b = blockIdx.y * blockDim.x + threadIdx.x;
  if (b >= B) return;
  T acc[kMaxProj];
  for (int j = 0; j < kMaxProj; ++j) acc[j] = Tr<T>::zero();
  for (int r = 0; r < nr; ++r) {
    const T x = src[(int64_t)Ds[r] * lds + b];
    for (int j = 0; j < P; ++j) Tr<T>::fma(acc[j], Cs[r * P + j], x);
  }
  for (int j = 0; j < P; ++j) Tr<T>::atomic_add(&W[((size_t)a * P + j) * B + b], acc[j]);
}

template <typename T>
__global__ void nl_apply(const int* __restrict__ chunk_atom, const int* __restrict__ chunk_row0,
                         const int* __restrict__ atom_ptr, const int* __restrict__ dofs,
                         const T* __restrict__ C, int P, const double* __restrict__ V,
                         const T* __restrict__ W, T* __restrict__ dst, int64_t ldd, int B,
                         double scalar) {
  __shared__ T Cs[kNlChunk * kMaxProj];
  __shared__ int Ds[kNlChunk];
  const int ch = blockIdx.x;
  const int a = chunk_atom[ch];
  const int r0 = chunk_row0[ch];
  const int r1 = min(r0 + kNlChunk, atom_ptr[a + 1]);
  const int nr = r1 - r0;
  for (int i = threadIdx.x; i < nr * P; i += blockDim.x) Cs[i] = C[(size_t)r0 * P + i];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) Ds[i] = dofs[r0 + i];
  __syncthreads();
  const int b = blockIdx.y * blockDim.x + threadIdx.x;
  if (b >= B) return;
  T w[kMaxProj];
  for (int j = 0; j < P; ++j)
    w[j] = Tr<T>::scale(scalar * V[(size_t)a * P + j], W[((size_t)a * P + j) * B + b]);
  for (int r = 0; r < nr; ++r) {
    T acc = Tr<T>::zero();
    for (int j = 0; j < P; ++j) Tr<T>::fma(acc, Cs[r * P + j], w[j]);
    Tr<T>::atomic_add(&dst[(int64_t)Ds[r] * ldd + b], acc);
  }
}

template <typename T>
static void apply_nonlocal(chefsi_operator_s* op, const T* C, T* W, const T* src, int64_t lds,
                           T* dst, int64_t ldd, int B, double scalar, cudaStream_t st) {
  if (op->n_atoms == 0) return;
  const size_t wn = (size_t)op->n_atoms * op->n_proj * B;
  CHEFSI_CUDA(cudaMemsetAsync(W, 0, wn * sizeof(T), st));
  const int threads = 128;
  dim3 grid(op->nl_n_chunks, (B + threads - 1) / threads);
  nl_project<T><<<grid, threads, 0, st>>>(op->nl_chunk_atom.ptr, op->nl_chunk_row0.ptr,
                                          op->nl_ptr.ptr, op->nl_dofs.ptr, C, op->n_proj, src,
                                          lds, W, B);
  CHEFSI_CHECK_LAUNCH();
  nl_apply<T><<<grid, threads, 0, st>>>(op->nl_chunk_atom.ptr, op->nl_chunk_row0.ptr,
                                        op->nl_ptr.ptr, op->nl_dofs.ptr, C, op->n_proj,
                                        op->couplings.ptr, W, dst, ldd, B, scalar);
  CHEFSI_CHECK_LAUNCH();
}

// ------------------------------------------------------------------ constraints
// distribute: x_s = sum_m w x_m (constraintMatrixInfoDevice.cc:33-230)
template <typename T>
__global__ void con_distribute(const int* __restrict__ ids, const int* __restrict__ ptr,
                               const int* __restrict__ mas, const double* __restrict__ w,
                               int n_con, T* x, int64_t ld, int B) {
  const int64_t n = (int64_t)n_con * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / B), b = (int)(t % B);
    T acc = Tr<T>::zero();
    for (int e = ptr[k]; e < ptr[k + 1]; ++e) {
      const T xm = x[(int64_t)mas[e] * ld + b];
      acc = acc + Tr<T>::scale(w[e], xm);
    }
    x[(int64_t)ids[k] * ld + b] = acc;
  }
}
// distribute_slave_to_master: x_m += w x_s ; x_s = 0 (constraintMatrixInfoDevice.cc:237-330)
template <typename T>
__global__ void con_slave_to_master(const int* __restrict__ ids, const int* __restrict__ ptr,
                                    const int* __restrict__ mas, const double* __restrict__ w,
                                    int n_con, T* x, int64_t ld, int B) {
  const int64_t n = (int64_t)n_con * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int k = (int)(t / B), b = (int)(t % B);
    T* xs = &x[(int64_t)ids[k] * ld + b];
    const T v = *xs;
    for (int e = ptr[k]; e < ptr[k + 1]; ++e)
      Tr<T>::atomic_add(&x[(int64_t)mas[e] * ld + b], Tr<T>::scale(w[e], v));
    *xs = Tr<T>::zero();
  }
}

// ------------------------------------------------------------------ elementwise kernels
template <typename T>
__global__ void k_scale_rows(const T* __restrict__ src, int64_t lds, T* __restrict__ dst,
                             int64_t ldd, const double* __restrict__ d, int64_t rows, int B) {
  const int64_t n = rows * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / B;
    const int b = (int)(t % B);
    dst[i * ldd + b] = Tr<T>::scale(d[i], src[i * lds + b]);
  }
}

// dst = (acc ? dst : 0) + scalar * d[i] * y
template <typename T>
__global__ void k_finish(const T* __restrict__ y, int64_t ldy, T* __restrict__ dst, int64_t ldd,
                         const double* __restrict__ d, int64_t rows, int B, double scalar,
                         int acc) {
  const int64_t n = rows * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / B;
    const int b = (int)(t % B);
    const T v = Tr<T>::scale(scalar * d[i], y[i * ldy + b]);
    dst[i * ldd + b] = acc ? dst[i * ldd + b] + v : v;
  }
}

template <typename T>
__global__ void k_axpby(const T* __restrict__ x, int64_t ldx, T* __restrict__ y, int64_t ldy,
                        int64_t rows, int B, double a, double b_) {
  const int64_t n = rows * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / B;
    const int b = (int)(t % B);
    y[i * ldy + b] = Tr<T>::scale(a, x[i * ldx + b]) + Tr<T>::scale(b_, y[i * ldy + b]);
  }
}

// ---- streaming block kernels: dst = s * src (with precision conversion), x *= s, max |x|.
// A scale s = 2^k is applied exactly on the bit patterns (pow2.cuh); any other s multiplies in
// the destination's precision. Contiguous blocks run as flat float4-wide passes; strided
// blocks run rows x columns with no integer division per entry (tpr threads per row, a
// power of two).
struct Scale {
  double s;
  int k;     // s == 2^k when p2
  bool p2;
};
inline Scale make_scale(double s) {
  Scale r{s, 0, false};
  int e = 0;
  const double f = std::frexp(s, &e);
  if (f == 0.5 && e - 1 >= -1000 && e - 1 <= 1000) r.k = e - 1, r.p2 = true;
  return r;
}
template <typename Ts, typename Td> struct Conv;
template <> struct Conv<float, float> {
  __device__ static float f(float x, const Scale& c) {
    return c.p2 ? ldexpf_exact(x, c.k) : (float)c.s * x;
  }
};
template <> struct Conv<double, float> {
  __device__ static float f(double x, const Scale& c) {
    return c.p2 ? narrow_ldexp(x, c.k) : (float)(c.s * x);
  }
};
template <> struct Conv<float, double> {
  __device__ static double f(float x, const Scale& c) {
    return c.p2 ? widen_ldexp(x, c.k) : c.s * widen_ldexp(x, 0);
  }
};
template <> struct Conv<double, double> {
  __device__ static double f(double x, const Scale& c) { return c.p2 ? ldexp_exact(x, c.k) : c.s * x; }
};
template <> struct Conv<cplx, cplx> {
  __device__ static cplx f(cplx x, const Scale& c) {
    return {Conv<double, double>::f(x.x, c), Conv<double, double>::f(x.y, c)};
  }
};

// four consecutive entries as one or two 16-byte accesses
template <typename T> struct Quad { T v[4]; };
template <typename T>
__device__ __forceinline__ Quad<T> load_quad(const T* p) {
  Quad<T> q;
  if constexpr (sizeof(T) == 4) {
    const float4 a = *reinterpret_cast<const float4*>(p);
    q.v[0] = a.x, q.v[1] = a.y, q.v[2] = a.z, q.v[3] = a.w;
  } else if constexpr (sizeof(T) == 8) {
    const double2 a = reinterpret_cast<const double2*>(p)[0];
    const double2 b = reinterpret_cast<const double2*>(p)[1];
    q.v[0] = a.x, q.v[1] = a.y, q.v[2] = b.x, q.v[3] = b.y;
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) q.v[i] = p[i];
  }
  return q;
}
template <typename T>
__device__ __forceinline__ void store_quad(T* p, const Quad<T>& q) {
  if constexpr (sizeof(T) == 4) {
    *reinterpret_cast<float4*>(p) = make_float4(q.v[0], q.v[1], q.v[2], q.v[3]);
  } else if constexpr (sizeof(T) == 8) {
    reinterpret_cast<double2*>(p)[0] = make_double2(q.v[0], q.v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(q.v[2], q.v[3]);
  } else {
#pragma unroll
    for (int i = 0; i < 4; ++i) p[i] = q.v[i];
  }
}

// flat pass over n entries (n % 4 == 0, both pointers 16-byte aligned)
template <typename Ts, typename Td>
__global__ void k_copy_flat(const Ts* __restrict__ src, Td* __restrict__ dst, int64_t n4, Scale c) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const Quad<Ts> a = load_quad(src + 4 * t);
    Quad<Td> b;
#pragma unroll
    for (int i = 0; i < 4; ++i) b.v[i] = Conv<Ts, Td>::f(a.v[i], c);
    store_quad(dst + 4 * t, b);
  }
}
// strided rows: block of 256 threads = (256 / tpr) rows x tpr columns
template <typename Ts, typename Td>
__global__ void k_copy_strided(const Ts* __restrict__ src, int64_t lds, Td* __restrict__ dst,
                            int64_t ldd, int64_t rows, int B, int log_tpr, Scale c) {
  const int tpr = 1 << log_tpr;
  const int col0 = threadIdx.x & (tpr - 1);
  const int rpb = blockDim.x >> log_tpr;
  for (int64_t r = (int64_t)blockIdx.x * rpb + (threadIdx.x >> log_tpr); r < rows;
       r += (int64_t)gridDim.x * rpb)
    for (int j = col0; j < B; j += tpr) dst[r * ldd + j] = Conv<Ts, Td>::f(src[r * lds + j], c);
}

template <typename T>
__global__ void k_scale_flat(T* __restrict__ x, int64_t n4, Scale c, bool zero) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    Quad<T> a;
    if (zero) {
#pragma unroll
      for (int i = 0; i < 4; ++i) a.v[i] = Tr<T>::zero();
    } else {
      a = load_quad(x + 4 * t);
#pragma unroll
      for (int i = 0; i < 4; ++i) a.v[i] = Conv<T, T>::f(a.v[i], c);
    }
    store_quad(x + 4 * t, a);
  }
}
template <typename T>
__global__ void k_scale_strided(T* __restrict__ x, int64_t ld, int64_t rows, int B, int log_tpr,
                                Scale c, bool zero) {
  const int tpr = 1 << log_tpr;
  const int col0 = threadIdx.x & (tpr - 1);
  const int rpb = blockDim.x >> log_tpr;
  for (int64_t r = (int64_t)blockIdx.x * rpb + (threadIdx.x >> log_tpr); r < rows;
       r += (int64_t)gridDim.x * rpb)
    for (int j = col0; j < B; j += tpr)
      x[r * ld + j] = zero ? Tr<T>::zero() : Conv<T, T>::f(x[r * ld + j], c);
}

// max |x| as the largest key of |x| (non-negative doubles order like their bit patterns)
__device__ __forceinline__ void absmax_commit(unsigned long long m, unsigned long long* out) {
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}
// |x| keys: FP64 on the bit patterns; FP32 maxima taken in FP32 (exact) and keyed at the end
__device__ __forceinline__ unsigned long long key_of(double x) { return abs_key(x); }
__device__ __forceinline__ unsigned long long key_of(float x) { return abs_key((double)fabsf(x)); }
__device__ __forceinline__ void key_max(unsigned long long& m, double x) { m = max(m, abs_key(x)); }
__device__ __forceinline__ void key_max(float& m, float x) { m = fmaxf(m, fabsf(x)); }
__device__ __forceinline__ unsigned long long key_final(unsigned long long m) { return m; }
__device__ __forceinline__ unsigned long long key_final(float m) { return key_of(m); }
template <typename T>
using KeyAcc = typename std::conditional<std::is_same<T, float>::value, float, unsigned long long>::type;

template <typename T>
__global__ void k_absmax_flat(const T* __restrict__ x, int64_t n4, unsigned long long* out) {
  KeyAcc<T> m = 0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const Quad<T> q = load_quad(x + 4 * t);
#pragma unroll
    for (int i = 0; i < 4; ++i) key_max(m, q.v[i]);
  }
  absmax_commit(key_final(m), out);
}
template <typename T>
__global__ void k_absmax_strided(const T* __restrict__ x, int64_t ld, int64_t rows, int B,
                                 int log_tpr, unsigned long long* out) {
  const int tpr = 1 << log_tpr;
  const int col0 = threadIdx.x & (tpr - 1);
  const int rpb = blockDim.x >> log_tpr;
  KeyAcc<T> m = 0;
  for (int64_t r = (int64_t)blockIdx.x * rpb + (threadIdx.x >> log_tpr); r < rows;
       r += (int64_t)gridDim.x * rpb)
    for (int j = col0; j < B; j += tpr) key_max(m, x[r * ld + j]);
  absmax_commit(key_final(m), out);
}

// threads per row for the strided kernels: the power of two >= B, at most 256
inline int log_threads_per_row(int B) {
  int l = 0;
  while (l < 8 && (1 << l) < B) ++l;
  return l;
}
inline bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }
inline int rows_grid(int64_t rows, int log_tpr) {
  return grid_for((rows + (256 >> log_tpr) - 1) / (256 >> log_tpr), 1);
}

template <typename T>
void scale_block(T* x, int64_t ld, int64_t rows, int B, double s, cudaStream_t st) {
  if (rows <= 0 || B <= 0) return;
  const Scale c = make_scale(s);
  const int64_t n = rows * B;
  if ((ld == B || rows == 1) && n % 4 == 0 && aligned16(x)) {
    k_scale_flat<T><<<grid_for(n / 4, 256), 256, 0, st>>>(x, n / 4, c, s == 0.0);
  } else {
    const int l = log_threads_per_row(B);
    k_scale_strided<T><<<rows_grid(rows, l), 256, 0, st>>>(x, ld, rows, B, l, c, s == 0.0);
  }
  CHEFSI_CHECK_LAUNCH();
}
template void scale_block<double>(double*, int64_t, int64_t, int, double, cudaStream_t);
template void scale_block<float>(float*, int64_t, int64_t, int, double, cudaStream_t);
template void scale_block<cplx>(cplx*, int64_t, int64_t, int, double, cudaStream_t);

template <typename T>
void axpby_block(const T* x, int64_t ldx, T* y, int64_t ldy, int64_t rows, int B, double a,
                 double b, cudaStream_t st) {
  k_axpby<T><<<grid_for(rows * B, 256), 256, 0, st>>>(x, ldx, y, ldy, rows, B, a, b);
  CHEFSI_CHECK_LAUNCH();
}
template void axpby_block<double>(const double*, int64_t, double*, int64_t, int64_t, int, double,
                                  double, cudaStream_t);
template void axpby_block<float>(const float*, int64_t, float*, int64_t, int64_t, int, double,
                                 double, cudaStream_t);
template void axpby_block<cplx>(const cplx*, int64_t, cplx*, int64_t, int64_t, int, double,
                                double, cudaStream_t);

template <typename Ts, typename Td>
void copy_block(const Ts* src, int64_t lds, Td* dst, int64_t ldd, int64_t rows, int B, double s,
                cudaStream_t st) {
  if (rows <= 0 || B <= 0) return;
  const Scale c = make_scale(s);
  const int64_t n = rows * B;
  if (((lds == B && ldd == B) || rows == 1) && n % 4 == 0 && aligned16(src) && aligned16(dst)) {
    k_copy_flat<Ts, Td><<<grid_for(n / 4, 256), 256, 0, st>>>(src, dst, n / 4, c);
  } else {
    const int l = log_threads_per_row(B);
    k_copy_strided<Ts, Td><<<rows_grid(rows, l), 256, 0, st>>>(src, lds, dst, ldd, rows, B, l, c);
  }
  CHEFSI_CHECK_LAUNCH();
}
template void copy_block<double, double>(const double*, int64_t, double*, int64_t, int64_t, int,
                                         double, cudaStream_t);
template void copy_block<double, float>(const double*, int64_t, float*, int64_t, int64_t, int,
                                        double, cudaStream_t);
template void copy_block<float, double>(const float*, int64_t, double*, int64_t, int64_t, int,
                                        double, cudaStream_t);
template void copy_block<float, float>(const float*, int64_t, float*, int64_t, int64_t, int,
                                       double, cudaStream_t);
template void copy_block<cplx, cplx>(const cplx*, int64_t, cplx*, int64_t, int64_t, int, double,
                                     cudaStream_t);

template <typename T>
static void absmax_block(const T* x, int64_t ld, int64_t rows, int B, double* out_dev,
                         cudaStream_t st) {
  CHEFSI_CUDA(cudaMemsetAsync(out_dev, 0, sizeof(double), st));
  if (rows <= 0 || B <= 0) return;
  unsigned long long* out = reinterpret_cast<unsigned long long*>(out_dev);
  const int64_t n = rows * B;
  if ((ld == B || rows == 1) && n % 4 == 0 && aligned16(x)) {
    k_absmax_flat<T><<<grid_for(n / 4, 256, kNumSMs * 8), 256, 0, st>>>(x, n / 4, out);
  } else {
    const int l = log_threads_per_row(B);
    k_absmax_strided<T><<<std::min(rows_grid(rows, l), kNumSMs * 8), 256, 0, st>>>(x, ld, rows, B,
                                                                                   l, out);
  }
  CHEFSI_CHECK_LAUNCH();
}
void absmax_block_f64(const double* x, int64_t ld, int64_t rows, int B, double* out_dev,
                      cudaStream_t st) {
  absmax_block<double>(x, ld, rows, B, out_dev, st);
}
void absmax_block_f32(const float* x, int64_t ld, int64_t rows, int B, double* out_dev,
                      cudaStream_t st) {
  absmax_block<float>(x, ld, rows, B, out_dev, st);
}

// ------------------------------------------------------------------ operator apply
template <typename T>
static void hx_generic(chefsi_operator_s* op, const T* mats, const T* nlC, T* nlW, const T* src,
                       int64_t lds, T* dst, int64_t ldd, int B, double scalar, bool accumulate,
                       cudaStream_t st, void (*cell)(const T*, const int*, int, int, const T*,
                                                     int64_t, T*, int64_t, int, double,
                                                     cudaStream_t)) {
  const int64_t M = op->n_dofs;
  if (op->folded) {
    if (!accumulate) scale_block<T>(dst, ldd, M, B, 0.0, st);
    cell(mats, op->map.ptr, op->n_cells, op->n_e, src, lds, dst, ldd, B, scalar, st);
    apply_nonlocal<T>(op, nlC, nlW, src, lds, dst, ldd, B, scalar, st);
    return;
  }
  // DFT-FE's sequence with explicit scaling and constraint rows
  // (kohnShamDFTOperatorDevice.cc:3767-3860)
  const size_t need = (size_t)M * B * (sizeof(T) / sizeof(double) + (sizeof(T) < 8 ? 1 : 0));
  T* xs = reinterpret_cast<T*>(op->ws64a.ensure(need));
  T* ys = reinterpret_cast<T*>(op->ws64b.ensure(need));
  k_scale_rows<T><<<grid_for(M * B, 256), 256, 0, st>>>(src, lds, xs, B, op->inv_sqrt_mass.ptr,
                                                        M, B);
  CHEFSI_CHECK_LAUNCH();
  if (op->n_con) {
    con_distribute<T><<<grid_for((int64_t)op->n_con * B, 256), 256, 0, st>>>(
        op->con_ids.ptr, op->con_ptr.ptr, op->con_master.ptr, op->con_w.ptr, op->n_con, xs, B, B);
    CHEFSI_CHECK_LAUNCH();
  }
  scale_block<T>(ys, B, M, B, 0.0, st);
  cell(mats, op->map.ptr, op->n_cells, op->n_e, xs, B, ys, B, B, 1.0, st);
  apply_nonlocal<T>(op, nlC, nlW, xs, B, ys, B, B, 1.0, st);
  if (op->n_con) {
    con_slave_to_master<T><<<grid_for((int64_t)op->n_con * B, 256), 256, 0, st>>>(
        op->con_ids.ptr, op->con_ptr.ptr, op->con_master.ptr, op->con_w.ptr, op->n_con, ys, B, B);
    CHEFSI_CHECK_LAUNCH();
  }
  k_finish<T><<<grid_for(M * B, 256), 256, 0, st>>>(ys, B, dst, ldd, op->inv_sqrt_mass.ptr, M, B,
                                                    scalar, accumulate ? 1 : 0);
  CHEFSI_CHECK_LAUNCH();
}

static void cell_f64(const double* m, const int* map, int nc, int ne, const double* s, int64_t lds,
                     double* d, int64_t ldd, int B, double sc, cudaStream_t st) {
  if (B <= 16)
    launch_cell_hx<double, 64, 16, 4, 1, 16>(m, map, nc, ne, s, lds, d, ldd, B, sc, st);
  else
    launch_cell_hx<double, 64, 32, 4, 2, 16>(m, map, nc, ne, s, lds, d, ldd, B, sc, st);
}
static void cell_f32(const float* m, const int* map, int nc, int ne, const float* s, int64_t lds,
                     float* d, int64_t ldd, int B, double sc, cudaStream_t st) {
  if (B <= 16)
    launch_cell_hx<float, 64, 16, 4, 1, 16>(m, map, nc, ne, s, lds, d, ldd, B, sc, st);
  else
    launch_cell_hx<float, 128, 64, 8, 4, 16>(m, map, nc, ne, s, lds, d, ldd, B, sc, st);
}
static void cell_c64(const cplx* m, const int* map, int nc, int ne, const cplx* s, int64_t lds,
                     cplx* d, int64_t ldd, int B, double sc, cudaStream_t st) {
  if (B <= 16)
    launch_cell_hx<cplx, 32, 16, 2, 1, 16>(m, map, nc, ne, s, lds, d, ldd, B, sc, st);
  else
    launch_cell_hx<cplx, 64, 32, 4, 2, 8>(m, map, nc, ne, s, lds, d, ldd, B, sc, st);
}

void hx_f64(chefsi_operator_s* op, const double* src, int64_t lds, double* dst, int64_t ldd, int B,
            double scalar, bool accumulate, cudaStream_t st) {
  CHEFSI_REQUIRE(!op->is_complex, "hx_f64 on a complex operator");
  double* W = op->n_atoms ? op->nlW64.ensure((size_t)op->n_atoms * op->n_proj * B) : nullptr;
  hx_generic<double>(op, op->mats64.ptr, op->nl_vals64.ptr, W, src, lds, dst, ldd, B, scalar,
                     accumulate, st, cell_f64);
}

void hx_f32(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd, int B,
            double scalar, bool accumulate, cudaStream_t st) {
  CHEFSI_REQUIRE(!op->is_complex, "hx_f32 on a complex operator");
  CHEFSI_REQUIRE(op->mats32.ptr != nullptr, "operator has no FP32 cell matrices");
  float* W = op->n_atoms ? op->nlW32.ensure((size_t)op->n_atoms * op->n_proj * B) : nullptr;
  hx_generic<float>(op, op->mats32.ptr, op->nl_vals32.ptr, W, src, lds, dst, ldd, B, scalar,
                    accumulate, st, cell_f32);
}

// W[a][j][b] += sum over one kNlChunk-row chunk of atom a of C[r][j] x[dof_r][b]: one CTA per
// (row chunk, 128-vector tile). The chunk's C rows and dofs are staged in shared memory, the 8
// warps take interleaved rows with U gathered float4 loads in flight per lane, the warps'
// partial sums are reduced in shared memory and added to W with one float4 atomic per
// (projector, lane). Many more CTAs than atoms x tiles, so the gather has enough loads in
// flight to approach the memory bandwidth. PP >= P is the compile-time projector capacity: the
// accumulators are PP float4 registers, so a small PP keeps four CTAs resident per SM.
template <int PP, int U>
__global__ void __launch_bounds__(256, PP <= 8 ? 4 : 2)
    nl_project_chunk4(const int* __restrict__ chunk_atom, const int* __restrict__ chunk_row0,
                      const int* __restrict__ atom_ptr, const int* __restrict__ dofs,
                      const float* __restrict__ C, int P, const float* __restrict__ src,
                      int64_t lds, float* __restrict__ W, int B) {
  extern __shared__ float4 red_dyn[];                 // [8][P][32]
  __shared__ float Cs[kNlChunk * PP];
  __shared__ int Ds[kNlChunk];
  const int ch = blockIdx.x;
  const int a = chunk_atom[ch];
  const int r0 = chunk_row0[ch];
  const int nr = min(r0 + kNlChunk, atom_ptr[a + 1]) - r0;
  for (int i = threadIdx.x; i < nr * P; i += blockDim.x) Cs[i] = C[(size_t)r0 * P + i];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) Ds[i] = dofs[r0 + i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int b = blockIdx.y * 128 + lane * 4;
  float4 acc[PP];
#pragma unroll
  for (int j = 0; j < PP; ++j) acc[j] = make_float4(0.f, 0.f, 0.f, 0.f);
  if (b < B) {
    int r = warp;
    for (; r + 8 * (U - 1) < nr; r += 8 * U) {
      float4 xv[U];
#pragma unroll
      for (int u = 0; u < U; ++u)
        xv[u] = __ldg(reinterpret_cast<const float4*>(src + (int64_t)Ds[r + 8 * u] * lds + b));
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
      const float4 xv = __ldg(reinterpret_cast<const float4*>(src + (int64_t)Ds[r] * lds + b));
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
static void launch_nl_project_chunk4(chefsi_operator_s* op, const float* x, int64_t ldx, float* W,
                                     int B, cudaStream_t st) {
  dim3 grid(op->nl_n_chunks, (B + 127) / 128);
  const size_t red = sizeof(float4) * 8 * op->n_proj * 32;
  CHEFSI_CUDA(cudaFuncSetAttribute(nl_project_chunk4<PP, U>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)(sizeof(float4) * 8 * PP * 32)));
  nl_project_chunk4<PP, U><<<grid, 256, red, st>>>(op->nl_chunk_atom.ptr, op->nl_chunk_row0.ptr,
                                                   op->nl_ptr.ptr, op->nl_dofs.ptr,
                                                   op->nl_vals32.ptr, op->n_proj, x, ldx, W, B);
}

void nl_project_f32(chefsi_operator_s* op, const float* x, int64_t ldx, float* W, int B,
                    cudaStream_t st) {
  if (op->n_atoms == 0) return;
  const bool vec = (B % 4 == 0) && (ldx % 4 == 0) && ((reinterpret_cast<uintptr_t>(x) & 15) == 0);
  if (vec) {
    CHEFSI_CUDA(cudaMemsetAsync(W, 0, sizeof(float) * (size_t)op->n_atoms * op->n_proj * B, st));
    if (op->n_proj <= 4)
      launch_nl_project_chunk4<4, 8>(op, x, ldx, W, B, st);
    else if (op->n_proj <= 8)
      launch_nl_project_chunk4<8, 4>(op, x, ldx, W, B, st);
    else
      launch_nl_project_chunk4<kMaxProj, 4>(op, x, ldx, W, B, st);
  } else {
    CHEFSI_CUDA(cudaMemsetAsync(W, 0, sizeof(float) * (size_t)op->n_atoms * op->n_proj * B, st));
    const int threads = 128;
    dim3 grid(op->nl_n_chunks, (B + threads - 1) / threads);
    nl_project<float><<<grid, threads, 0, st>>>(op->nl_chunk_atom.ptr, op->nl_chunk_row0.ptr,
                                                op->nl_ptr.ptr, op->nl_dofs.ptr, op->nl_vals32.ptr,
                                                op->n_proj, x, ldx, W, B);
  }
  CHEFSI_CHECK_LAUNCH();
}

// y[dof_r][b..b+3] += scalar * sum_j C[r][j] V[a][j] W[a][j][b..b+3] (float4 atomics); PP >= P
// is the compile-time projector capacity (PP float4 registers of scaled W per thread)
template <int PP>
__global__ void __launch_bounds__(128, PP <= 8 ? 8 : 4)
    nl_apply_v4(const int* __restrict__ chunk_atom, const int* __restrict__ chunk_row0,
                const int* __restrict__ atom_ptr, const int* __restrict__ dofs,
                const float* __restrict__ C, int P, const double* __restrict__ V,
                const float* __restrict__ W, float* __restrict__ dst, int64_t ldd, int B,
                float scalar) {
  __shared__ float Cs[kNlChunk * PP];
  __shared__ int Ds[kNlChunk];
  const int ch = blockIdx.x;
  const int a = chunk_atom[ch];
  const int r0 = chunk_row0[ch];
  const int r1 = min(r0 + kNlChunk, atom_ptr[a + 1]);
  const int nr = r1 - r0;
  for (int i = threadIdx.x; i < nr * P; i += blockDim.x) Cs[i] = C[(size_t)r0 * P + i];
  for (int i = threadIdx.x; i < nr; i += blockDim.x) Ds[i] = dofs[r0 + i];
  __syncthreads();
  const int b = (blockIdx.y * blockDim.x + threadIdx.x) * 4;
  if (b >= B) return;
  float4 w[PP];
#pragma unroll
  for (int j = 0; j < PP; ++j) {
    if (j >= P) break;
    const float f = scalar * (float)V[(size_t)a * P + j];
    const float4 x = *reinterpret_cast<const float4*>(&W[((size_t)a * P + j) * B + b]);
    w[j] = make_float4(f * x.x, f * x.y, f * x.z, f * x.w);
  }
  for (int r = 0; r < nr; ++r) {
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int j = 0; j < PP; ++j) {
      if (j >= P) break;
      const float cv = Cs[r * P + j];
      acc.x = fmaf(cv, w[j].x, acc.x);
      acc.y = fmaf(cv, w[j].y, acc.y);
      acc.z = fmaf(cv, w[j].z, acc.z);
      acc.w = fmaf(cv, w[j].w, acc.w);
    }
    atomicAdd(reinterpret_cast<float4*>(dst + (int64_t)Ds[r] * ldd + b), acc);
  }
}

void apply_nonlocal_f32(chefsi_operator_s* op, const float* src, int64_t lds, float* dst,
                        int64_t ldd, int B, double scalar, cudaStream_t st) {
  if (op->n_atoms == 0) return;
  float* W = op->nlW32.ensure((size_t)op->n_atoms * op->n_proj * B);
  const bool vec = (B % 4 == 0) && (lds % 4 == 0) && (ldd % 4 == 0) &&
                   ((reinterpret_cast<uintptr_t>(src) & 15) == 0) &&
                   ((reinterpret_cast<uintptr_t>(dst) & 15) == 0);
  if (!vec) {
    apply_nonlocal<float>(op, op->nl_vals32.ptr, W, src, lds, dst, ldd, B, scalar, st);
    return;
  }
  nl_project_f32(op, src, lds, W, B, st);
  const int threads = 128;
  dim3 grid(op->nl_n_chunks, (B / 4 + threads - 1) / threads);
  auto launch = [&](auto kernel) {
    kernel<<<grid, threads, 0, st>>>(op->nl_chunk_atom.ptr, op->nl_chunk_row0.ptr, op->nl_ptr.ptr,
                                     op->nl_dofs.ptr, op->nl_vals32.ptr, op->n_proj,
                                     op->couplings.ptr, W, dst, ldd, B, (float)scalar);
  };
  if (op->n_proj <= 4)
    launch(nl_apply_v4<4>);
  else if (op->n_proj <= 8)
    launch(nl_apply_v4<8>);
  else
    launch(nl_apply_v4<kMaxProj>);
  CHEFSI_CHECK_LAUNCH();
}

void hx_c64(chefsi_operator_s* op, const cplx* src, int64_t lds, cplx* dst, int64_t ldd, int B,
            double scalar, bool accumulate, cudaStream_t st) {
  CHEFSI_REQUIRE(op->is_complex, "hx_c64 on a real operator");
  CHEFSI_REQUIRE(op->n_atoms == 0, "complex operators with projectors are not supported");
  hx_generic<cplx>(op, reinterpret_cast<const cplx*>(op->mats64.ptr), nullptr, nullptr, src, lds,
                   dst, ldd, B, scalar, accumulate, st, cell_c64);
}

// ------------------------------------------------------------------ creation
// fold: A_e[I][J] = d[map I] * H_e[I][J] * d[map J]
template <typename T>
__global__ void k_fold_mats(T* mats, const int* __restrict__ map, const double* __restrict__ d,
                            int n_cells, int n_e) {
  const int64_t n = (int64_t)n_cells * n_e * n_e;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / ((int64_t)n_e * n_e);
    const int r = (int)(t % ((int64_t)n_e * n_e));
    const int I = r / n_e, J = r % n_e;
    const double f = d[map[c * n_e + I]] * d[map[c * n_e + J]];
    mats[t] = Tr<T>::scale(f, mats[t]);
  }
}

__global__ void k_fold_proj(double* C, const int* __restrict__ dofs, const double* __restrict__ d,
                            int64_t nnz, int P) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nnz * P;
       t += (int64_t)gridDim.x * blockDim.x)
    C[t] *= d[dofs[t / P]];
}

__global__ void k_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    b[t] = (float)a[t];
}

void update_cell_matrices(chefsi_operator_s* op, const double* mats_dev, cudaStream_t st) {
  CHEFSI_REQUIRE(!op->is_complex, "update_cell_matrices: real operators only");
  const int64_t nc = op->n_cells, ne = op->n_e;
  const size_t nm = (size_t)nc * ne * ne;
  CHEFSI_CUDA(cudaMemcpyAsync(op->mats64.ptr, mats_dev, nm * sizeof(double),
                              cudaMemcpyDeviceToDevice, st));
  if (op->folded) {
    k_fold_mats<double><<<grid_for((int64_t)nm, 256), 256, 0, st>>>(op->mats64.ptr, op->map.ptr,
                                                                    op->inv_sqrt_mass.ptr, nc, ne);
    CHEFSI_CHECK_LAUNCH();
  }
  k_to_f32<<<grid_for((int64_t)nm, 256), 256, 0, st>>>(op->mats64.ptr, op->mats32.ptr, nm);
  CHEFSI_CHECK_LAUNCH();
  op->tc.ready = false;  // the FP16 split is rebuilt on the next tensor-core apply
  op->fz.tiles_ready = false;  // and so are the filter plan's tiles (its tables stay)
}

// real form of the complex cell matrices: row (I, p), column (J, q), p/q = 0 real part,
// 1 imaginary part: [[Re A, -Im A], [Im A, Re A]] interleaved node by node
__global__ void k_realify_cells(const cplx* __restrict__ mats, int64_t nc, int ne,
                                double* __restrict__ out) {
  const int ne2 = 2 * ne;
  const int64_t n = nc * ne2 * ne2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / ((int64_t)ne2 * ne2);
    const int r = (int)(t % ((int64_t)ne2 * ne2));
    const int R = r / ne2, Q = r % ne2;
    const int p = R & 1, q = Q & 1;
    const cplx a = mats[(c * ne + (R >> 1)) * ne + (Q >> 1)];
    out[t] = (p == q) ? a.x : (p == 0 ? -a.y : a.y);
  }
}
__global__ void k_realify_map(const int* __restrict__ map, int64_t n, int* __restrict__ out) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < 2 * n;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = 2 * map[t >> 1] + (int)(t & 1);
}

chefsi_operator_s* realified(chefsi_operator_s* op, cudaStream_t st) {
  if (op->rv) return op->rv.get();
  CHEFSI_REQUIRE(op->is_complex && op->folded,
                 "real form: folded complex operators only (no constraint rows)");
  auto rv = std::make_unique<chefsi_operator_s>();
  rv->n_dofs = 2 * op->n_dofs;
  rv->n_cells = op->n_cells;
  rv->n_e = 2 * op->n_e;
  rv->is_complex = 0;
  rv->folded = true;
  const int64_t nc = op->n_cells;
  const size_t nm = (size_t)nc * rv->n_e * rv->n_e;
  rv->map.reset((size_t)nc * rv->n_e);
  k_realify_map<<<grid_for(nc * op->n_e * 2, 256), 256, 0, st>>>(op->map.ptr, nc * op->n_e,
                                                                  rv->map.ptr);
  CHEFSI_CHECK_LAUNCH();
  rv->mats64.reset(nm);
  k_realify_cells<<<grid_for((int64_t)nm, 256), 256, 0, st>>>(
      reinterpret_cast<const cplx*>(op->mats64.ptr), nc, op->n_e, rv->mats64.ptr);
  CHEFSI_CHECK_LAUNCH();
  rv->mats32.reset(nm);
  k_to_f32<<<grid_for((int64_t)nm, 256), 256, 0, st>>>(rv->mats64.ptr, rv->mats32.ptr, nm);
  CHEFSI_CHECK_LAUNCH();
  op->rv = std::move(rv);
  return op->rv.get();
}

__global__ void k_complex_to_rows(const cplx* __restrict__ X, int64_t ld, int64_t M, int B,
                                  double s, float* __restrict__ out) {
  const int64_t n = 2 * M * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = t / B;
    const int j = (int)(t % B);
    const cplx v = X[(row >> 1) * ld + j];
    out[t] = (float)(s * ((row & 1) ? v.y : v.x));
  }
}
__global__ void k_rows_to_complex(const float* __restrict__ in, int64_t M, int B, double s,
                                  cplx* __restrict__ X, int64_t ld) {
  const int64_t n = M * B;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t g = t / B;
    const int j = (int)(t % B);
    X[g * ld + j] = {s * (double)in[(2 * g) * B + j], s * (double)in[(2 * g + 1) * B + j]};
  }
}
void complex_to_real_rows(const cplx* X, int64_t ld, int64_t M, int B, double s, float* out,
                          cudaStream_t st) {
  k_complex_to_rows<<<grid_for(2 * M * B, 256), 256, 0, st>>>(X, ld, M, B, s, out);
  CHEFSI_CHECK_LAUNCH();
}
void real_rows_to_complex(const float* in, int64_t M, int B, double s, cplx* X, int64_t ld,
                          cudaStream_t st) {
  k_rows_to_complex<<<grid_for(M * B, 256), 256, 0, st>>>(in, M, B, s, X, ld);
  CHEFSI_CHECK_LAUNCH();
}

template <typename T>
static void upload(DeviceBuffer<T>& buf, const T* host, size_t n) {
  buf.reset(n);
  if (n) CHEFSI_CUDA(cudaMemcpy(buf.ptr, host, n * sizeof(T), cudaMemcpyHostToDevice));
}

static bool all_finite(const double* p, size_t n) {
  for (size_t i = 0; i < n; ++i)
    if (!std::isfinite(p[i])) return false;
  return true;
}

chefsi_operator_s* create_operator(const chefsi_operator_desc* d) {
  CHEFSI_REQUIRE(d != nullptr, "null operator description");
  CHEFSI_REQUIRE(d->n_dofs > 0 && d->n_cells > 0 && d->nodes_per_cell > 0, "empty operator");
  CHEFSI_REQUIRE(d->nodes_per_cell <= kMaxNodesPerCell, "nodes_per_cell > 512 is not supported");
  CHEFSI_REQUIRE(d->n_dofs < (1ll << 31), "n_dofs must fit in int32 indices");
  CHEFSI_REQUIRE(d->cell_dof_map && d->cell_matrices && d->sqrt_mass && d->inv_sqrt_mass,
                 "missing operator arrays");
  const int64_t nc = d->n_cells, ne = d->nodes_per_cell;
  for (int64_t i = 0; i < nc * ne; ++i)
    CHEFSI_REQUIRE(d->cell_dof_map[i] >= 0 && d->cell_dof_map[i] < d->n_dofs,
                   "cell_dof_map entry out of range");
  const size_t nm = (size_t)nc * ne * ne * (d->is_complex ? 2 : 1);
  if (fault_injected("nan") || !all_finite((const double*)d->cell_matrices, nm) ||
      !all_finite(d->inv_sqrt_mass, d->n_dofs) || !all_finite(d->sqrt_mass, d->n_dofs))
    throw Error(CHEFSI_ERR_NAN, "non-finite value in the operator inputs");
  if (d->n_constrained) {
    CHEFSI_REQUIRE(d->constrained_ids && d->constraint_ptr && d->master_ids && d->master_weights,
                   "missing constraint arrays");
    for (int k = 0; k < d->n_constrained; ++k) {
      CHEFSI_REQUIRE(d->constrained_ids[k] >= 0 && d->constrained_ids[k] < d->n_dofs,
                     "constrained id out of range");
      CHEFSI_REQUIRE(d->constraint_ptr[k + 1] >= d->constraint_ptr[k], "constraint_ptr not monotone");
    }
    for (int e = 0; e < d->constraint_ptr[d->n_constrained]; ++e)
      CHEFSI_REQUIRE(d->master_ids[e] >= 0 && d->master_ids[e] < d->n_dofs, "master id out of range");
  }
  if (d->n_atoms) {
    CHEFSI_REQUIRE(!d->is_complex, "projectors on complex operators are not supported");
    CHEFSI_REQUIRE(d->n_proj >= 1 && d->n_proj <= kMaxProj, "n_proj must be in [1, 16]");
    CHEFSI_REQUIRE(d->atom_dof_ptr && d->atom_dofs && d->atom_proj && d->couplings,
                   "missing projector arrays");
    for (int a = 0; a < d->n_atoms; ++a)
      CHEFSI_REQUIRE(d->atom_dof_ptr[a + 1] >= d->atom_dof_ptr[a], "atom_dof_ptr not monotone");
    for (int64_t r = 0; r < d->atom_dof_ptr[d->n_atoms]; ++r)
      CHEFSI_REQUIRE(d->atom_dofs[r] >= 0 && d->atom_dofs[r] < d->n_dofs, "atom dof out of range");
  }

  auto* op = new chefsi_operator_s();
  try {
    op->n_dofs = d->n_dofs;
    op->n_cells = d->n_cells;
    op->n_e = d->nodes_per_cell;
    op->is_complex = d->is_complex;
    op->folded = d->n_constrained == 0;
    upload(op->map, d->cell_dof_map, (size_t)nc * ne);
    upload(op->mats64, (const double*)d->cell_matrices, nm);
    upload(op->sqrt_mass, d->sqrt_mass, d->n_dofs);
    upload(op->inv_sqrt_mass, d->inv_sqrt_mass, d->n_dofs);
    if (op->folded) {
      if (d->is_complex)
        k_fold_mats<cplx><<<grid_for((int64_t)nc * ne * ne, 256), 256>>>(
            reinterpret_cast<cplx*>(op->mats64.ptr), op->map.ptr, op->inv_sqrt_mass.ptr, nc, ne);
      else
        k_fold_mats<double><<<grid_for((int64_t)nc * ne * ne, 256), 256>>>(
            op->mats64.ptr, op->map.ptr, op->inv_sqrt_mass.ptr, nc, ne);
      CHEFSI_CHECK_LAUNCH();
    }
    if (!d->is_complex) {
      op->mats32.reset(nm);
      k_to_f32<<<grid_for(nm, 256), 256>>>(op->mats64.ptr, op->mats32.ptr, nm);
      CHEFSI_CHECK_LAUNCH();
    }
    if (d->n_constrained) {
      op->n_con = d->n_constrained;
      upload(op->con_ids, d->constrained_ids, d->n_constrained);
      upload(op->con_ptr, d->constraint_ptr, d->n_constrained + 1);
      const int nnz = d->constraint_ptr[d->n_constrained];
      upload(op->con_master, d->master_ids, nnz);
      upload(op->con_w, d->master_weights, nnz);
    }
    if (d->n_atoms) {
      op->n_atoms = d->n_atoms;
      op->n_proj = d->n_proj;
      op->nl_nnz = d->atom_dof_ptr[d->n_atoms];
      upload(op->nl_ptr, d->atom_dof_ptr, d->n_atoms + 1);
      upload(op->nl_dofs, d->atom_dofs, op->nl_nnz);
      upload(op->nl_vals64, d->atom_proj, (size_t)op->nl_nnz * d->n_proj);
      upload(op->couplings, d->couplings, (size_t)d->n_atoms * d->n_proj);
      if (op->folded) {
        k_fold_proj<<<grid_for(op->nl_nnz * d->n_proj, 256), 256>>>(
            op->nl_vals64.ptr, op->nl_dofs.ptr, op->inv_sqrt_mass.ptr, op->nl_nnz, d->n_proj);
        CHEFSI_CHECK_LAUNCH();
      }
      op->nl_vals32.reset((size_t)op->nl_nnz * d->n_proj);
      k_to_f32<<<grid_for(op->nl_nnz * d->n_proj, 256), 256>>>(
          op->nl_vals64.ptr, op->nl_vals32.ptr, op->nl_nnz * d->n_proj);
      CHEFSI_CHECK_LAUNCH();
      // chunks of kNlChunk rows of one atom, ordered by their smallest dof: with spatially
      // ordered dofs, the chunks of overlapping projector supports then run at about the same
      // time and the rows they share (1.4 supports per row in dense wells) are re-read and
      // re-reduced in L2 instead of HBM
      std::vector<std::pair<int, std::pair<int, int>>> chunks;
      for (int a = 0; a < d->n_atoms; ++a)
        for (int r = d->atom_dof_ptr[a]; r < d->atom_dof_ptr[a + 1]; r += kNlChunk) {
          const int r1 = std::min(r + kNlChunk, d->atom_dof_ptr[a + 1]);
          int dmin = d->atom_dofs[r];
          for (int i = r + 1; i < r1; ++i) dmin = std::min(dmin, d->atom_dofs[i]);
          chunks.push_back({dmin, {a, r}});
        }
      std::stable_sort(chunks.begin(), chunks.end(),
                       [](const auto& x, const auto& y) { return x.first < y.first; });
      std::vector<int> ca, cr;
      for (const auto& c : chunks) {
        ca.push_back(c.second.first);
        cr.push_back(c.second.second);
      }
      op->nl_n_chunks = (int)ca.size();
      upload(op->nl_chunk_atom, ca.data(), ca.size());
      upload(op->nl_chunk_row0, cr.data(), cr.size());
      if (op->nl_n_chunks == 0) op->n_atoms = 0;
    }
    CHEFSI_CUDA(cudaDeviceSynchronize());
  } catch (...) {
    delete op;
    throw;
  }
  return op;
}

}  // namespace chefsi
