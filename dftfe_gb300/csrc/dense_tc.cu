// Tensor-core dense products of the mixed-precision Rayleigh-Ritz step on GB300:
//   * Gram products C += A^T B over the long dof dimension: the overlap S = X^T X and the
//     projected Hamiltonian X^T (HX) (DFT-FE: fillParallelOverlapMatScalapack,
//     src/linAlg/linearAlgebraOperationsDevice.cc:3079-3240, and XtHX,
//     src/dftOperator/kohnShamDFTOperatorDevice.cc:4003-4157);
//   * the subspace rotation X <- X W (subspaceRotationScalapack,
//     src/linAlg/linearAlgebraOperationsDevice.cc:1833-2240, which DFT-FE runs in FP32 under
//     useMixedPrecSubspaceRotRR).
//
// Arithmetic: every operand column is scaled by a power of two 2^e so that its largest entry
// lies in [2^14, 2^15), then split into FP16 hi + lo (22 significant bits). tcgen05.mma
// kind::f16 forms hi*hi + hi*lo + lo*hi (the lo*lo term is below 2^-22 relative) with FP32
// accumulation in tensor memory; the power-of-two scalings are undone exactly in FP64.
//   * Gram: 128 x 128 output tiles. The K (dof) range of a tile is split over k-slices of
//     CTAs; inside a CTA each chunk of 128 dofs accumulates in tensor memory (FP32, 8 MMA
//     steps) and is then added by the epilogue warps into an unevaluated FP32 pair (TwoSum,
//     ~48 bits; the high parts in registers, the low parts in 128 spare tensor-memory
//     columns) while the MMAs of the next chunks run in the other two accumulators. The
//     tensor core's FP32 accumulation truncates, so its error grows with the number of steps
//     in one direction for sums of equal-sign terms (the diagonal of X^T X): 2048-dof chunks
//     left a relative bias of ~6e-6, 128-dof chunks keep it near 2e-7. FP64 adds in the
//     epilogue would not keep up (FP64 runs at ~2 FMA/clk/SM on GB300). Each CTA writes its
//     FP64 partial tile; a reduction kernel adds the k-slices in a fixed order.
//   * Rotation: Y^T = W'^T X'^T with W' = diag(2^-e) W (each row of W absorbs the scale of
//     the matching X column, exactly), the output column scale of W' taken out per row of
//     Y^T. Tiles are 128 output columns x 256 dofs, persistent CTAs, double-buffered
//     accumulators; the epilogue writes FP64 rows of Y with 256-byte coalesced stores. The
//     FP16 copy of X is read, so Y may be X itself (in-place rotation).
// The split kernels store every operand as tiles (128 or 256 rows x 32 K entries) that are
// already the 64-byte-swizzled, K-major shared-memory image the MMA descriptors read, so a
// K-block stage is a few bulk copies (cp.async.bulk) through an mbarrier ring. Tensor-map
// (TMA tensor) loads of the same boxes fetch 128 or 256 rows of 64 bytes each; for a 1.7M-row
// operand those rows lie 3.5 MB apart, one 2 MB page each, and a Gram took 28 ms instead of
// 7.6 ms with the contiguous tiles. One lane issues the MMAs. Every wait is bounded: on expiry the CTA records
// CHEFSI_ERR_TIMEOUT, waits (bounded) for its own copies, frees its tensor memory and returns.
#include "internal.h"
#include "tc_common.cuh"
#include "pow2.cuh"

#include <algorithm>
#include <cmath>
#include <type_traits>

namespace chefsi {

using namespace tcx;

namespace {

constexpr int kKB = 32;                 // halves per K-block (64-byte rows)
constexpr int kRows8K = 128 * kKB * 2;  // one 128-row operand tile: 8 KB

// ======================================================================= conversions
// column maxima of |X| as order-preserving keys (FP32 maxima in FP32, FP64 ones on the bit
// patterns: no FP64 arithmetic per entry)
__device__ __forceinline__ void col_max(float x, float& m) { m = fmaxf(m, fabsf(x)); }
__device__ __forceinline__ void col_max(double x, unsigned long long& m) { m = max(m, abs_key(x)); }
__device__ __forceinline__ unsigned long long col_key(float m) { return abs_key((double)m); }
__device__ __forceinline__ unsigned long long col_key(unsigned long long m) { return m; }
template <typename T>
__global__ void k_col_absmax(const T* __restrict__ X, int64_t ld, int64_t M, int N,
                             unsigned long long* __restrict__ out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  typename std::conditional<std::is_same<T, float>::value, float, unsigned long long>::type m = 0;
  for (int64_t r = blockIdx.y; r < M; r += gridDim.y) col_max(X[r * ld + j], m);
  atomicMax(&out[j], col_key(m));
}

// e[j]: m 2^e in [2^14, 2^15) for the column maximum m (clamped to keep 2^e a normal double);
// sc[j] = 2^e[j]
__global__ void k_col_exponent(const unsigned long long* __restrict__ bits, int N,
                               int* __restrict__ e, double* __restrict__ sc) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= N) return;
  const double m = __longlong_as_double((long long)bits[j]);
  int ex = 0, ej = 0;
  if (m > 0.0 && isfinite(m)) {
    frexp(m, &ex);  // m = f 2^ex, f in [0.5, 1)
    ej = min(max(15 - ex, -1000), 1000);
  }
  e[j] = ej;
  sc[j] = ldexp(1.0, ej);
}

__device__ __forceinline__ void split_half(double v, __half& h, __half& l) {
  h = __double2half(v);
  l = __double2half(v - (double)__half2float(h));
}
// the same split from an FP32 value (the FP32 rounding keeps 24 bits, the split 22): the
// column scale 2^e is applied exactly on the bit patterns, (float)(x 2^e) with one rounding,
// and the split runs on the FP32 pipe
__device__ __forceinline__ float scaled_f32(double x, int e) { return narrow_ldexp(x, e); }
__device__ __forceinline__ float scaled_f32(float x, int e) { return ldexpf_exact(x, e); }
__device__ __forceinline__ void split_half_f32(float v, __half& h, __half& l) {
  h = __float2half_rn(v);
  l = __float2half_rn(v - __half2float(h));
}

// [M][N] (ld) -> hi/lo, column j scaled by 2^ex[j], zero padding to Np columns and Kp dofs,
// stored as tiles of 128 columns x 32 dofs ([Np / 128][Kp / 32][4096 halves]), each tile the
// 64-byte-swizzled shared-memory image of a K-major operand (one bulk copy per tile)
template <typename T>
__global__ void __launch_bounds__(256)
    k_split_t(const T* __restrict__ X, int64_t ld, int64_t M, int N, const int* __restrict__ ex,
              int64_t Kp, __half* __restrict__ hi, __half* __restrict__ lo) {
  __shared__ float tile[64][65];  // [column][dof]
  const int64_t k0 = (int64_t)blockIdx.x * 64;
  const int j0 = blockIdx.y * 64;
  for (int idx = threadIdx.x; idx < 64 * 64; idx += 256) {
    const int r = idx >> 6, c = idx & 63;
    const int64_t k = k0 + r;
    const int j = j0 + c;
    float v = 0.f;
    if (k < M && j < N) v = scaled_f32(X[k * ld + j], ex[j]);
    tile[c][r] = v;
  }
  __syncthreads();
  for (int idx = threadIdx.x; idx < 64 * 32; idx += 256) {
    const int c = idx >> 5, p = idx & 31;
    __half h0, l0, h1, l1;
    split_half_f32(tile[c][2 * p], h0, l0);
    split_half_f32(tile[c][2 * p + 1], h1, l1);
    // tile (panel of 128 columns, K-block of 32 dofs), 64-byte-swizzled image, 4096 halves
    const int jj = j0 + c;
    const int64_t k = k0 + 2 * p;
    const int64_t o = (((int64_t)(jj >> 7) * (Kp / 32) + (k >> 5)) << 12) +
                      (sw64_offset((uint32_t)(jj & 127), 2u * (uint32_t)(k & 31)) >> 1);
    *reinterpret_cast<__half2*>(hi + o) = __halves2half2(h0, h1);
    *reinterpret_cast<__half2*>(lo + o) = __halves2half2(l0, l1);
  }
}

// [M][N] (ld) -> hi/lo, column j scaled by 2^ex[j], columns zero-padded to Kr (Kr % 32 == 0)
// and rows to Mp (a multiple of 256), stored as tiles of 256 rows x 32 columns
// ([Mp / 256][Kr / 32][8192 halves]), each the 64-byte-swizzled shared-memory image of a
// K-major rotation operand. A warp handles 4 rows x one 32-column K-block per step (lane =
// row 4 + 4-column quad): it writes 4 whole 64-byte tile rows, 256 contiguous bytes.
template <typename T>
__global__ void k_split_r(const T* __restrict__ X, int64_t ld, int64_t M, int64_t Mp, int N,
                          const int* __restrict__ ex, int Kr, __half* __restrict__ hi,
                          __half* __restrict__ lo) {
  const int lane = threadIdx.x & 31;
  const int rr = lane >> 3, qq = lane & 7;
  const int nkb = Kr / 32;
  const int64_t items = (Mp / 4) * nkb;
  const int64_t wstep = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t w = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < items;
       w += wstep) {
    const int64_t rb = w / nkb;
    const int kb = (int)(w - rb * nkb);
    const int64_t r = rb * 4 + rr;
    const int j = kb * 32 + qq * 4;
    __half h[4], l[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
      split_half_f32(r < M && j + i < N ? scaled_f32(X[r * ld + j + i], ex[j + i]) : 0.f, h[i], l[i]);
    __half2 hv[2] = {__halves2half2(h[0], h[1]), __halves2half2(h[2], h[3])};
    __half2 lv[2] = {__halves2half2(l[0], l[1]), __halves2half2(l[2], l[3])};
    const int64_t o = (((r >> 8) * nkb + kb) << 13) +
                      (sw64_offset((uint32_t)(r & 255), 8u * (uint32_t)qq) >> 1);
    *reinterpret_cast<uint2*>(hi + o) = *reinterpret_cast<const uint2*>(hv);
    *reinterpret_cast<uint2*>(lo + o) = *reinterpret_cast<const uint2*>(lv);
  }
}

// Rotation operand: Wt[m][k] = W[k][m] 2^(t_m - e_k) as FP16 hi/lo tiles of 128 m x 32 k
// ([Mp / 128][Kr / 32][4096 halves], swizzled shared-memory images; W is K x n_out),
// with t_m the exponent that puts column m of diag(2^-e) W into [2^14, 2^15). One block per
// output column.
__global__ void __launch_bounds__(256)
    k_prep_rotation(const double* __restrict__ W, int64_t ldw, int K, int n_out,
                    const int* __restrict__ e, int Kr, int* __restrict__ t_out,
                    __half* __restrict__ hi, __half* __restrict__ lo) {
  __shared__ double red[256];
  __shared__ int tm_s;
  const int m = blockIdx.x;
  double mx = 0.0;
  if (m < n_out)
    for (int k = threadIdx.x; k < K; k += 256) mx = fmax(mx, fabs(ldexp(W[(int64_t)k * ldw + m], -e[k])));
  red[threadIdx.x] = mx;
  __syncthreads();
  for (int s = 128; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    int ex = 0;
    const double v = red[0];
    if (v > 0.0 && isfinite(v)) frexp(v, &ex);
    tm_s = (v > 0.0 && isfinite(v)) ? 15 - ex : 0;
    t_out[m] = tm_s;
  }
  __syncthreads();
  const int tm = tm_s;
  for (int k = threadIdx.x; k < Kr; k += 256) {
    const double v = (m < n_out && k < K) ? ldexp(W[(int64_t)k * ldw + m], tm - e[k]) : 0.0;
    __half h, l;
    split_half(v, h, l);
    // tile (128 output columns, 32 k), 64-byte-swizzled image of 4096 halves
    const int64_t o = (((int64_t)(m >> 7) * (Kr / 32) + (k >> 5)) << 12) +
                      (sw64_offset((uint32_t)(m & 127), 2u * (uint32_t)(k & 31)) >> 1);
    hi[o] = h;
    lo[o] = l;
  }
}

// ======================================================================= Gram kernel
struct GramArgs {
  int n_tiles;   // output tiles in the enumeration
  int tiles_j;   // tiles along j (full enumeration)
  int lower;     // enumerate tiles with tj <= ti only
  int same;      // B is A: diagonal tiles load A once
  int kslices;   // CTAs per tile (K split)
  int nkb;       // K-blocks of 32 dofs
  int kc;        // K-blocks per tensor-memory chunk (4 accumulators in rotation)
  int stages;
  int n1, n2;    // valid output rows / columns
  double* part;  // [kslices][padded n1][ldp = padded n2], scaled units
  const __half* a_hi;  // operand tiles [panel][K-block][4096 halves]
  const __half* a_lo;
  const __half* b_hi;
  const __half* b_lo;
  int64_t ldp, pstride;
  int* err;
};

constexpr int kGramEpiWarps = 16;  // four per tensor-memory lane quarter, 32 columns each
constexpr int kGramThreads = 64 + 32 * kGramEpiWarps;  // warp 0 copies, warp 1 MMA, then epilogue
constexpr int kGramAcc = 3;        // chunk accumulators (128 columns each); columns 384.. hold
                                   // the TwoSum low parts
constexpr int kGramStage = 4 * kRows8K;

__device__ __forceinline__ void gram_tile(int t, const GramArgs& a, int& ti, int& tj) {
  if (a.lower) {
    int i = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while ((i + 1) * (i + 2) / 2 <= t) ++i;
    while (i * (i + 1) / 2 > t) --i;
    ti = i;
    tj = t - i * (i + 1) / 2;
  } else {
    ti = t / a.tiles_j;
    tj = t % a.tiles_j;
  }
}

__global__ void __launch_bounds__(kGramThreads, 1)
    gram_tc_kernel(GramArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = a.stages;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * kGramStage);
  uint64_t* full = bars;                 // [S] stage bytes landed
  uint64_t* empty = bars + S;            // [S] MMAs done reading the stage
  uint64_t* acc_full = bars + 2 * S;     // [kGramAcc]
  uint64_t* acc_empty = bars + 2 * S + 4;  // [kGramAcc] one arrival per epilogue warp
  uint64_t* mma_done = bars + 2 * S + 8;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 9);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 2 * S + 10);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tile = blockIdx.x % a.n_tiles, slice = blockIdx.x / a.n_tiles;
  int ti, tj;
  gram_tile(tile, a, ti, tj);
  const bool diag = a.same && ti == tj;
  const int n_chunks = (a.nkb + a.kc - 1) / a.kc;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < kGramAcc; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kGramEpiWarps);   // one arrival per epilogue warp
    }
    mbar_init(mma_done, 1);
    *abort_flag = wait_limit_init(a.err);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, 512);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int64_t g = 0;
      int s = 0;
      uint32_t r = 0;
      bool ok = true;
      for (int c = slice; c < n_chunks && ok; c += a.kslices) {
        const int kb1 = min(a.nkb, (c + 1) * a.kc);
        for (int kb = c * a.kc; kb < kb1; ++kb) {
          if (!mbar_wait(&empty[s], (r & 1) ^ 1, a.err, abort_flag)) {
            ok = false;
            break;
          }
          uint8_t* st = smem + s * kGramStage;
          mbar_arrive_expect_tx(&full[s], diag ? 2 * kRows8K : 4 * kRows8K);
          const int64_t ta = ((int64_t)ti * a.nkb + kb) * (kRows8K / 2);
          bulk_load(st, a.a_hi + ta, kRows8K, &full[s]);
          bulk_load(st + kRows8K, a.a_lo + ta, kRows8K, &full[s]);
          if (!diag) {
            const int64_t tb = ((int64_t)tj * a.nkb + kb) * (kRows8K / 2);
            bulk_load(st + 2 * kRows8K, a.b_hi + tb, kRows8K, &full[s]);
            bulk_load(st + 3 * kRows8K, a.b_lo + tb, kRows8K, &full[s]);
          }
          ++g;
          if (++s == S) s = 0, ++r;
        }
      }
      if (*abort_flag) {
        for (int64_t h = (g > S ? g - S : 0); h < g; ++h) {
          const int s = (int)(h % S);
          const uint32_t r = (uint32_t)(h / S);
          for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(&full[s], r & 1); ++i)
            __nanosleep(128);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_f16(128, 128);
      int s = 0;
      uint32_t r = 0;
      int it = 0;
      bool ok = true;
      for (int c = slice; c < n_chunks && ok; c += a.kslices, ++it) {
        const int buf = it % kGramAcc;
        const uint32_t ph = (uint32_t)((it / kGramAcc) & 1);
        if (!mbar_wait(&acc_empty[buf], ph ^ 1, a.err, abort_flag)) break;
        fence_after();
        const uint32_t d = tmem + buf * 128;
        const int kb0 = c * a.kc, kb1 = min(a.nkb, kb0 + a.kc);
        for (int kb = kb0; kb < kb1; ++kb) {
          if (!mbar_wait(&full[s], r & 1, a.err, abort_flag)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t st = smem_u32(smem + s * kGramStage);
          const uint32_t ahi = st, alo = st + kRows8K;
          const uint32_t bhi = diag ? ahi : st + 2 * kRows8K;
          const uint32_t blo = diag ? alo : st + 3 * kRows8K;
#pragma unroll
          for (int ks = 0; ks < kKB / 16; ++ks) {
            const uint32_t koff = ks * 32;
            const uint32_t acc0 = (kb > kb0 || ks > 0) ? 1u : 0u;
            mma_f16(d, smem_desc_sw64(ahi + koff), smem_desc_sw64(bhi + koff), idesc, acc0);
            mma_f16(d, smem_desc_sw64(ahi + koff), smem_desc_sw64(blo + koff), idesc, 1u);
            mma_f16(d, smem_desc_sw64(alo + koff), smem_desc_sw64(bhi + koff), idesc, 1u);
          }
          mma_commit(&empty[s]);
          if (++s == S) s = 0, ++r;
        }
        if (ok) mma_commit(&acc_full[buf]);
      }
      mma_commit(mma_done);
      for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(mma_done, 0); ++i) __nanosleep(128);
    }
  } else {
    // epilogue: warp w owns tensor-memory lanes 32*(w%4).. (row i) and accumulator columns
    // 32*((w-2)/4).. It keeps the sum of its 32 entries as FP32 pairs (sh + sl, TwoSum: the
    // exact error of every addition goes to sl): sh in registers, sl in tensor memory. Four
    // warps share a lane quarter, so their tensor-memory round trips overlap.
    const int q = warp & 3, hcol = (warp - 2) >> 2;
    constexpr int kCols = 128 / (kGramEpiWarps / 4);
    const uint32_t lane_off = (uint32_t)(q * 32) << 16;
    const uint32_t tl = tmem + 128 * kGramAcc + hcol * kCols + lane_off;
    float sh[kCols];
#pragma unroll
    for (int c = 0; c < kCols; ++c) sh[c] = 0.f;
    {
      const uint32_t z[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
      for (int c0 = 0; c0 < kCols; c0 += 8) tmem_st8(tl + c0, z);
      tmem_wait_st();
    }
    bool ok = true;
    int it = 0;
    for (int c = slice; c < n_chunks; c += a.kslices, ++it) {
      const int buf = it % kGramAcc;
      const uint32_t ph = (uint32_t)((it / kGramAcc) & 1);
      ok = __all_sync(0xffffffffu, mbar_wait(&acc_full[buf], ph, a.err, abort_flag));
      if (!ok) break;
      fence_after();
      const uint32_t tv = tmem + buf * 128 + hcol * kCols + lane_off;
#pragma unroll
      for (int c0 = 0; c0 < kCols; c0 += 16) {
        uint32_t rv[16], rl[16];
        tmem_ld16_async(tv + c0, rv);
        tmem_ld16_async(tl + c0, rl);
        tmem_wait_ld();
#pragma unroll
        for (int u = 0; u < 16; ++u) {
          const float v = __uint_as_float(rv[u]);
          const float h = sh[c0 + u];
          const float s = __fadd_rn(h, v);
          const float bp = __fsub_rn(s, h);
          const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bp)), __fsub_rn(v, bp));
          sh[c0 + u] = s;
          rl[u] = __float_as_uint(__fadd_rn(__uint_as_float(rl[u]), err));
        }
        tmem_st16(tl + c0, rl);
      }
      tmem_wait_st();
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[buf]);
    }
    // the partial in scaled units over the whole (padded) tile; the reduction reads the
    // valid part and undoes the column scalings
    const int i = ti * 128 + q * 32 + lane;
    double* prow =
        a.part + (int64_t)slice * a.pstride + (int64_t)i * a.ldp + tj * 128 + hcol * kCols;
#pragma unroll
    for (int c0 = 0; c0 < kCols; c0 += 8) {
      uint32_t rl[8];
      tmem_ld8_async(tl + c0, rl);
      tmem_wait_ld();
#pragma unroll
      for (int u = 0; u < 8; ++u)
        prow[c0 + u] = ok ? (double)sh[c0 + u] + (double)__uint_as_float(rl[u]) : 0.0;
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, 512);
  }
}

__global__ void k_gram_reduce(const double* __restrict__ part, int kslices, int64_t pstride,
                              int64_t ldp, int n1, int n2, int lower, const int* __restrict__ ea,
                              const int* __restrict__ eb, double* __restrict__ C, int64_t ldc) {
  const int64_t n = (int64_t)n1 * n2;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(t / n2), j = (int)(t % n2);
    if (lower && (j >> 7) > (i >> 7)) continue;
    double s = 0.0;
    for (int k = 0; k < kslices; ++k) s += part[k * pstride + (int64_t)i * ldp + j];
    C[(int64_t)i * ldc + j] += ldexp(s, -(ea[i] + eb[j]));
  }
}

// ======================================================================= rotation kernel
struct RotArgs {
  int m_tiles;      // 128-column tiles of the output
  int64_t n_tiles;  // ceil(M / 256) * m_tiles
  int nkb;          // K-blocks of 32 along the input columns
  int stages;
  int64_t M;
  int N;            // output columns
  const int* et;    // exponent of each output column
  double* Y;
  int64_t ldy;
  int* err;
  const __half* w_hi;  // W' tiles [m panel][K-block][4096 halves]
  const __half* w_lo;
  const __half* x_hi;  // X row-split tiles [256-row panel][K-block][8192 halves]
  const __half* x_lo;
};

constexpr int kRotThreads = 192;  // warp 0 copies, warp 1 MMA, warps 2..5 epilogue
constexpr int kRotStage = 2 * kRows8K + 4 * kRows8K;  // A hi/lo (128 rows), B hi/lo (256 rows)

__global__ void __launch_bounds__(kRotThreads, 1)
    rotate_tc_kernel(RotArgs a) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = a.stages;
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + S * kRotStage);
  uint64_t* full = bars;
  uint64_t* empty = bars + S;
  uint64_t* acc_full = bars + 2 * S;
  uint64_t* acc_empty = bars + 2 * S + 2;  // 4 epilogue-warp arrivals
  uint64_t* mma_done = bars + 2 * S + 4;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 2 * S + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 2 * S + 6);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t first = blockIdx.x, step = gridDim.x;
  const int64_t my_tiles = first < a.n_tiles ? (a.n_tiles - first + step - 1) / step : 0;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], 4);   // one arrival per epilogue warp
    }
    mbar_init(mma_done, 1);
    *abort_flag = wait_limit_init(a.err);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, 512);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      int64_t g = 0;
      int s = 0;
      uint32_t r = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        const int64_t t = first + it * step;
        const int nt = (int)(t / a.m_tiles), mt = (int)(t % a.m_tiles);
        for (int kb = 0; kb < a.nkb; ++kb) {
          if (!mbar_wait(&empty[s], (r & 1) ^ 1, a.err, abort_flag)) {
            ok = false;
            break;
          }
          uint8_t* st = smem + s * kRotStage;
          mbar_arrive_expect_tx(&full[s], kRotStage);
          // one bulk copy per operand tile (swizzled shared-memory images)
          const int64_t tw = ((int64_t)mt * a.nkb + kb) * (kRows8K / 2);
          const int64_t tx = ((int64_t)nt * a.nkb + kb) * kRows8K;
          bulk_load(st, a.w_hi + tw, kRows8K, &full[s]);
          bulk_load(st + kRows8K, a.w_lo + tw, kRows8K, &full[s]);
          bulk_load(st + 2 * kRows8K, a.x_hi + tx, 2 * kRows8K, &full[s]);
          bulk_load(st + 4 * kRows8K, a.x_lo + tx, 2 * kRows8K, &full[s]);
          ++g;
          if (++s == S) s = 0, ++r;
        }
      }
      if (*abort_flag) {
        for (int64_t h = (g > S ? g - S : 0); h < g; ++h) {
          const int s = (int)(h % S);
          const uint32_t r = (uint32_t)(h / S);
          for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(&full[s], r & 1); ++i)
            __nanosleep(128);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      const uint32_t idesc = idesc_f16(128, 256);
      int s = 0;
      uint32_t r = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_tiles && ok; ++it) {
        const int buf = (int)(it & 1);
        const uint32_t ph = (uint32_t)((it >> 1) & 1);
        if (!mbar_wait(&acc_empty[buf], ph ^ 1, a.err, abort_flag)) break;
        fence_after();
        const uint32_t d = tmem + buf * 256;
        for (int kb = 0; kb < a.nkb; ++kb) {
          if (!mbar_wait(&full[s], r & 1, a.err, abort_flag)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t st = smem_u32(smem + s * kRotStage);
          const uint32_t whi = st, wlo = st + kRows8K;
          const uint32_t xhi = st + 2 * kRows8K, xlo = st + 4 * kRows8K;
#pragma unroll
          for (int ks = 0; ks < kKB / 16; ++ks) {
            const uint32_t koff = ks * 32;
            const uint32_t acc0 = (kb > 0 || ks > 0) ? 1u : 0u;
            mma_f16(d, smem_desc_sw64(whi + koff), smem_desc_sw64(xhi + koff), idesc, acc0);
            mma_f16(d, smem_desc_sw64(whi + koff), smem_desc_sw64(xlo + koff), idesc, 1u);
            mma_f16(d, smem_desc_sw64(wlo + koff), smem_desc_sw64(xhi + koff), idesc, 1u);
          }
          mma_commit(&empty[s]);
          if (++s == S) s = 0, ++r;
        }
        if (ok) mma_commit(&acc_full[buf]);
      }
      mma_commit(mma_done);
      for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(mma_done, 0); ++i) __nanosleep(128);
    }
  } else {
    // epilogue warps 2..5: tensor-memory lane = output column m, accumulator column = dof
    const int q = warp & 3;
    for (int64_t it = 0; it < my_tiles; ++it) {
      const int buf = (int)(it & 1);
      const uint32_t ph = (uint32_t)((it >> 1) & 1);
      const bool ok = __all_sync(0xffffffffu, mbar_wait(&acc_full[buf], ph, a.err, abort_flag));
      if (!ok) break;
      fence_after();
      const int64_t t = first + it * step;
      const int64_t n0 = (t / a.m_tiles) * 256;
      const int m = (int)(t % a.m_tiles) * 128 + q * 32 + lane;
      const bool mok = m < a.N;
      const double sc = mok ? ldexp(1.0, -a.et[m]) : 0.0;
      double* ycol = a.Y + m;
      const uint32_t tq = tmem + buf * 256 + ((uint32_t)(q * 32) << 16);
      for (int c0 = 0; c0 < 256; c0 += 16) {
        float v[16];
        tmem_ld16(tq + c0, v);
        if (mok) {
#pragma unroll
          for (int u = 0; u < 16; ++u) {
            const int64_t n = n0 + c0 + u;
            if (n < a.M) ycol[n * a.ldy] = (double)v[u] * sc;
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acc_empty[buf]);
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, 512);
  }
}

int gram_smem(int stages) { return stages * kGramStage + 8 * (2 * stages + 12) + 1024; }
int rot_smem(int stages) { return stages * kRotStage + 8 * (2 * stages + 8) + 1024; }

}  // namespace

int device_sms() {
  int dev = 0, sms = kNumSMs;
  CHEFSI_CUDA(cudaGetDevice(&dev));
  CHEFSI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  return sms;
}

// ======================================================================= host API
bool dense_tc_available() { return tcgen05_device(); }

template <typename T>
void tc_exponents(const T* X, int64_t ld, int64_t M, int N, TcOperand& op, cudaStream_t st) {
  op.bits.ensure(N);
  op.e.ensure(N);
  op.sc.ensure(N);
  CHEFSI_CUDA(cudaMemsetAsync(op.bits.ptr, 0, sizeof(unsigned long long) * N, st));
  const int64_t ysplit = std::max<int64_t>(1, std::min<int64_t>(M, 2048));
  dim3 grid((N + 255) / 256, (unsigned)ysplit);
  k_col_absmax<T><<<grid, 256, 0, st>>>(X, ld, M, N, op.bits.ptr);
  CHEFSI_CHECK_LAUNCH();
  k_col_exponent<<<(N + 255) / 256, 256, 0, st>>>(op.bits.ptr, N, op.e.ptr, op.sc.ptr);
  CHEFSI_CHECK_LAUNCH();
}

template <typename T>
void tc_split_transposed(const T* X, int64_t ld, int64_t M, int N, TcOperand& op, cudaStream_t st) {
  op.rows = M;
  op.cols = N;
  op.transposed = true;
  op.ld = (M + 63) / 64 * 64;                 // Kp: dofs, zero-padded
  op.padded = (N + 127) / 128 * 128;          // Np: columns, zero-padded
  const size_t n = (size_t)op.padded * op.ld;
  op.hi.ensure(n);
  op.lo.ensure(n);
  CHEFSI_REQUIRE(op.ld / 64 < (1ll << 31), "tensor-core split: too many rows");
  dim3 grid((unsigned)(op.ld / 64), (unsigned)(op.padded / 64));
  k_split_t<T><<<grid, 256, 0, st>>>(X, ld, M, N, op.e.ptr, op.ld, op.hi.ptr, op.lo.ptr);
  CHEFSI_CHECK_LAUNCH();
}

template <typename T>
void tc_split_rows(const T* X, int64_t ld, int64_t M, int N, TcOperand& op, cudaStream_t st) {
  op.rows = M;
  op.cols = N;
  op.transposed = false;
  op.ld = (N + 63) / 64 * 64;                 // Kr: columns, zero-padded
  op.padded = (int)op.ld;
  const int64_t Mp = (M + 255) / 256 * 256;   // rows, zero-padded to whole 256-row tiles
  const size_t n = (size_t)Mp * op.ld;
  op.hi.ensure(n);
  op.lo.ensure(n);
  const int64_t items = (Mp / 4) * (op.ld / 32);   // one per warp step (8 warps a block)
  k_split_r<T><<<grid_for((items + 7) / 8, 1), 256, 0, st>>>(X, ld, M, Mp, N, op.e.ptr,
                                                              (int)op.ld, op.hi.ptr, op.lo.ptr);
  CHEFSI_CHECK_LAUNCH();
}

template void tc_exponents<double>(const double*, int64_t, int64_t, int, TcOperand&, cudaStream_t);
template void tc_exponents<float>(const float*, int64_t, int64_t, int, TcOperand&, cudaStream_t);
template void tc_split_transposed<double>(const double*, int64_t, int64_t, int, TcOperand&, cudaStream_t);
template void tc_split_transposed<float>(const float*, int64_t, int64_t, int, TcOperand&, cudaStream_t);
template void tc_split_rows<double>(const double*, int64_t, int64_t, int, TcOperand&, cudaStream_t);
template void tc_split_rows<float>(const float*, int64_t, int64_t, int, TcOperand&, cudaStream_t);

void tc_gram(const TcOperand& A, const TcOperand* B, double* C, int64_t ldc, bool lower,
             TcDenseWork& w, cudaStream_t st) {
  const TcOperand& Bo = B ? *B : A;
  CHEFSI_REQUIRE(A.transposed && Bo.transposed && A.ld == Bo.ld && A.rows == Bo.rows,
                 "tensor-core Gram: operands must be transposed splits of the same rows");
  const bool same = (B == nullptr) || (B == &A);
  const int n1 = A.cols, n2 = Bo.cols;
  lower = lower && n1 == n2;
  const int ti_n = A.padded / 128, tj_n = Bo.padded / 128;
  const int n_tiles = lower ? ti_n * (ti_n + 1) / 2 : ti_n * tj_n;
  const int sms = device_sms();
  const int nkb = (int)(A.ld / kKB);
  const int kc = 4;  // 128 dofs per tensor-memory chunk
  const int n_chunks = (nkb + kc - 1) / kc;
  int kslices = std::max(1, std::min(sms / std::max(1, n_tiles), n_chunks));
  if (!w.err.ptr) {
    w.err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(w.err.ptr, 0, sizeof(int), st));
  }
  const int64_t ldp = Bo.padded;
  const int64_t pstride = (int64_t)A.padded * ldp;
  double* part = w.part.ensure((size_t)kslices * pstride);

  GramArgs g{};
  g.a_hi = A.hi.ptr;
  g.a_lo = A.lo.ptr;
  g.b_hi = Bo.hi.ptr;
  g.b_lo = Bo.lo.ptr;
  g.n_tiles = n_tiles;
  g.tiles_j = tj_n;
  g.lower = lower ? 1 : 0;
  g.same = same ? 1 : 0;
  g.kslices = kslices;
  g.nkb = nkb;
  g.kc = kc;
  g.stages = 6;
  g.n1 = n1;
  g.n2 = n2;
  g.part = part;
  g.ldp = ldp;
  g.pstride = pstride;
  g.err = w.err.ptr;
  const int smem = gram_smem(g.stages);
  CHEFSI_CUDA(cudaFuncSetAttribute(gram_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int64_t grid = (int64_t)n_tiles * kslices;
  CHEFSI_REQUIRE(grid < (1ll << 31), "tensor-core Gram: grid too large");
  gram_tc_kernel<<<(unsigned)grid, kGramThreads, smem, st>>>(g);
  CHEFSI_CHECK_LAUNCH();
  k_gram_reduce<<<grid_for((int64_t)n1 * n2, 256), 256, 0, st>>>(
      part, kslices, pstride, ldp, n1, n2, lower ? 1 : 0, A.e.ptr, Bo.e.ptr, C, ldc);
  CHEFSI_CHECK_LAUNCH();
}

void tc_rotate(const TcOperand& Xr, const double* W, int64_t ldw, int n_out, double* Y,
               int64_t ldy, TcDenseWork& w, cudaStream_t st) {
  CHEFSI_REQUIRE(!Xr.transposed, "tensor-core rotation: operand must be a row split");
  CHEFSI_REQUIRE(Y != nullptr && W != nullptr && n_out >= 1, "tensor-core rotation: bad argument");
  if (Xr.rows <= 0) return;
  const int N = n_out;
  const int Kr = (int)Xr.ld;
  const int Mp = (N + 127) / 128 * 128;
  if (!w.err.ptr) {
    w.err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(w.err.ptr, 0, sizeof(int), st));
  }
  w.whi.ensure((size_t)Mp * Kr);
  w.wlo.ensure((size_t)Mp * Kr);
  w.et.ensure(Mp);
  k_prep_rotation<<<Mp, 256, 0, st>>>(W, ldw, Xr.cols, N, Xr.e.ptr, Kr, w.et.ptr, w.whi.ptr,
                                      w.wlo.ptr);
  CHEFSI_CHECK_LAUNCH();

  RotArgs r{};
  r.w_hi = w.whi.ptr;
  r.w_lo = w.wlo.ptr;
  r.x_hi = Xr.hi.ptr;
  r.x_lo = Xr.lo.ptr;
  r.m_tiles = Mp / 128;
  r.n_tiles = ((Xr.rows + 255) / 256) * r.m_tiles;
  r.nkb = Kr / kKB;
  r.stages = 4;
  r.M = Xr.rows;
  r.N = N;
  r.et = w.et.ptr;
  r.Y = Y;
  r.ldy = ldy;
  r.err = w.err.ptr;
  const int smem = rot_smem(r.stages);
  CHEFSI_CUDA(cudaFuncSetAttribute(rotate_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  const int64_t grid = std::min<int64_t>(device_sms(), r.n_tiles);
  rotate_tc_kernel<<<(unsigned)grid, kRotThreads, smem, st>>>(r);
  CHEFSI_CHECK_LAUNCH();
}

namespace tcx {
void dense_tc_set_wait_tries(uint32_t tries) {
  CHEFSI_CUDA(cudaMemcpyToSymbol(g_wait_tries, &tries, sizeof(tries)));
}
}  // namespace tcx

int tc_dense_check_error(TcDenseWork& w, cudaStream_t st) {
  if (!w.err.ptr) return CHEFSI_OK;
  int h = 0;
  CHEFSI_CUDA(cudaMemcpyAsync(&h, w.err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  if (h) CHEFSI_CUDA(cudaMemsetAsync(w.err.ptr, 0, sizeof(int), st));
  return h;
}

// C (N1 x N2) += A^T B through the tensor-core Gram (temporaries owned by the call)
void gram_tc_f64(const double* A, int64_t lda, const double* B, int64_t ldb, int64_t K, int N1,
                 int N2, double* C, int ldc, bool lower_only, cudaStream_t st) {
  TcOperand a, b;
  TcDenseWork w;
  tc_exponents<double>(A, lda, K, N1, a, st);
  tc_split_transposed<double>(A, lda, K, N1, a, st);
  const bool same = (A == B) && (lda == ldb) && (N1 == N2);
  if (!same) {
    tc_exponents<double>(B, ldb, K, N2, b, st);
    tc_split_transposed<double>(B, ldb, K, N2, b, st);
  }
  tc_gram(a, same ? nullptr : &b, C, ldc, lower_only, w, st);
  const int rc = tc_dense_check_error(w, st);
  if (rc != CHEFSI_OK) throw Error(rc, "tensor-core Gram: a bounded device wait expired");
}

// Y[M][n_out] = X[M][K] W[K][n_out] through the tensor-core rotation (temporaries owned by
// the call); Y may be X when n_out == K
void rotate_tc_f64(const double* X, int64_t ld, int64_t M, int K, const double* W, int64_t ldw,
                   int n_out, double* Y, int64_t ldy, cudaStream_t st) {
  if (M <= 0) return;
  TcOperand x;
  TcDenseWork w;
  tc_exponents<double>(X, ld, M, K, x, st);
  tc_split_rows<double>(X, ld, M, K, x, st);
  tc_rotate(x, W, ldw, n_out, Y, ldy, w, st);
  const int rc = tc_dense_check_error(w, st);
  if (rc != CHEFSI_OK) throw Error(rc, "tensor-core rotation: a bounded device wait expired");
}

}  // namespace chefsi
