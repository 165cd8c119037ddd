// Tensor-core filter HX on GB300: tcgen05 MMAs with FP16-split operands, FP32 accumulation
// in tensor memory, fused gather / scatter through the cell -> dof map.
//
// DFT-FE's local HX (src/dftOperator/matrixVectorProductImplementationsDevice.cc:27-117)
// gathers X into n_cells x n_e x B cell blocks, calls gemmStridedBatched and scatter-adds.
// Here one CTA owns one (cell, 128-vector chunk):
//   * warp 0 (one lane) streams K-blocks of the cell matrix (FP16 hi and lo parts, 64-byte
//     rows, 64B-swizzled) into shared memory with TMA;
//   * warps 2..5 gather the chunk's X rows (FP32) straight from the global block through the
//     cell's dof map, split each value into FP16 hi + lo and write them K-major with the same
//     swizzle (one thread per vector, so the global loads coalesce along the vectors);
//   * warp 1 (one lane) issues tcgen05.mma kind::f16 with M = 128 vectors, N = the cell's
//     rows (one or two MMAs of N <= 256), K = 16:
//       D += Xhi Ahi^T + Xhi Alo^T + Xlo Ahi^T           (the lo*lo term is below 2^-22)
//     and the accumulator D[vector][row] (FP32) stays in tensor memory;
//   * warps 2..5 then read D with tcgen05.ld (lane = vector) and scatter-add
//     scalar * D / 2^s into the output rows with red.global.add.f32 -- for every cell row the
//     32 lanes of a warp hit 32 consecutive floats, so each atomic instruction is one 128-byte
//     line.
// A 3..4-stage mbarrier pipeline overlaps TMA, the X split and the MMAs. Every mbarrier wait
// is bounded: on expiry the CTA records CHEFSI_ERR_TIMEOUT in a device flag, waits (bounded)
// for its own TMA copies, frees its tensor memory and returns.
#include "internal.h"
#include "tc_common.cuh"

#include <cuda.h>

#include <algorithm>
#include <cmath>
#include <mutex>
#include <vector>

namespace chefsi {

using namespace tcx;

namespace {

constexpr int kVec = 128;          // vectors per CTA (MMA M)
constexpr int kKB = 32;            // halves per K-block (64-byte rows)
constexpr int kRowBytes = kKB * 2; // 64
struct TcArgs {
  const float* src;
  int64_t lds;
  float* dst;
  int64_t ldd;
  const int* map;
  int n_e;
  int nkb;         // K-blocks of 32 columns
  int B;
  int n_chunks;    // 128-vector chunks
  int n_half;      // cell rows per work unit (= MMA N)
  int n_halves;    // row halves per cell (1 or 2)
  int buf_stride;  // tensor-memory column offset of accumulator 1
  int tmem_cols;
  int stages;
  int64_t n_units; // n_cells * n_chunks * n_halves
  float out_scale; // scalar / 2^s
  int* err;
};

// shared memory carve-up (offsets from a 1024-byte aligned base)
constexpr int kXStages = 4;                    // cp.async staging depth for the X gather
constexpr int kXStageBytes = kKB * kVec * 4;    // [32 rows][128 vectors] FP32 = 16 KB

struct Layout {
  int x_tile;   // 128 rows x 64 B = 8 KB
  int a_tile;   // n_half rows x 64 B, rounded to 1 KB
  int stage;    // xhi, xlo, ahi, alo
  int xstage;   // FP32 staging ring of the gathered rows
  int bars;     // barrier block
  int total;
};
__host__ __device__ inline Layout make_layout(int n_half, int stages) {
  Layout L;
  L.x_tile = kVec * kRowBytes;
  L.a_tile = ((n_half * kRowBytes + 1023) / 1024) * 1024;
  L.stage = 2 * L.x_tile + 2 * L.a_tile;
  L.xstage = stages * L.stage;
  L.bars = L.xstage + kXStages * kXStageBytes;
  L.total = L.bars + 8 * (3 * stages + 8);
  return L;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
// named barrier among the 128 X-producer threads (barrier 0 is __syncthreads)
__device__ __forceinline__ void producers_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }
// the same barrier with an OR-reduction, so the producers take stop decisions together
__device__ __forceinline__ bool producers_sync_or(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.or.pred po, 1, 128, pi;\n"
      " selp.u32 %0, 1, 0, po;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v)
      : "memory");
  return r != 0;
}

struct Unit {
  int cell, chunk, half;
};
// The CTA's it-th unit: (cell, chunk) pairs are dealt round-robin over the CTAs and a CTA
// runs both row halves of its pair back to back, so the second gather of the chunk's X rows
// comes from L2.
__device__ __forceinline__ Unit unit_at(int64_t it, int64_t first, int64_t step,
                                        const TcArgs& a) {
  Unit w;
  w.half = (int)(it % a.n_halves);
  const int64_t cc = first + (it / a.n_halves) * step;
  w.chunk = (int)(cc % a.n_chunks);
  w.cell = (int)(cc / a.n_chunks);
  return w;
}

// Persistent warp-specialised kernel, one CTA per SM. Work unit = (cell, 128-vector chunk,
// row half); (cell, chunk) pairs are dealt round-robin so the CTAs of the GPU sweep the cells
// in order (a cell's matrix halves are re-read from L2, not HBM), and each CTA runs the two
// halves of its pair back to back (the second gather of the pair's X rows hits L2).
//   warp 0        TMA of the cell-matrix K-blocks (hi, lo) into the stage ring
//   warp 1        tcgen05.mma issue (one lane), two tensor-memory accumulators
//   warps 2..5    X gather (one thread per vector, next K-block prefetched in registers),
//                 FP16 hi/lo split, 64B-swizzled K-major stores
//   warps 6..9    epilogue: tcgen05.ld of a finished accumulator, red.global.add.f32 scatter,
//                 overlapped with the MMAs of the next unit
constexpr int kThreads2 = 320;

__global__ void __launch_bounds__(kThreads2, 1)
    cell_hx_tc_kernel(const __grid_constant__ CUtensorMap tm_hi,
                      const __grid_constant__ CUtensorMap tm_lo, TcArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = args.stages;
  const Layout L = make_layout(args.n_half, S);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.bars);
  uint64_t* tma_full = bars;            // [S] TMA bytes landed
  uint64_t* x_full = bars + S;          // [S] 128 producer arrivals
  uint64_t* empty = bars + 2 * S;       // [S] MMA finished reading the stage
  uint64_t* acc_full = bars + 3 * S;    // [2] accumulator ready for the epilogue
  uint64_t* acc_empty = bars + 3 * S + 2;  // [2] accumulator drained (128 arrivals)
  uint64_t* mma_done = bars + 3 * S + 4;   // final MMA completion
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bars + 3 * S + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(bars + 3 * S + 6);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t first = blockIdx.x;
  const int64_t step = gridDim.x;
  const int64_t n_pairs = args.n_units / args.n_halves;   // (cell, chunk) pairs
  const int64_t my_units =
      first < n_pairs ? ((n_pairs - first + step - 1) / step) * args.n_halves : 0;
  const int nkb = args.nkb;
  const int64_t my_blocks = my_units * nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&tma_full[s], 1);
      mbar_init(&x_full[s], kVec);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kVec);
    }
    mbar_init(mma_done, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(args.tmem_cols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- TMA producer
    if (lane == 0) {
      const uint32_t bytes = 2u * args.n_half * kRowBytes;
      int64_t issued = 0;
      for (int64_t g = 0; g < my_blocks; ++g) {
        const Unit w = unit_at(g / nkb, first, step, args);
        const int kb = (int)(g % nkb);
        const int s = (int)(g % S);
        const uint32_t r = (uint32_t)(g / S);
        if (!mbar_wait(&empty[s], (r & 1) ^ 1, args.err, abort_flag)) break;
        uint8_t* st = smem + s * L.stage;
        mbar_arrive_expect_tx(&tma_full[s], bytes);
        tma_load_3d(st + 2 * L.x_tile, &tm_hi, kb * kKB, w.half * args.n_half, w.cell, &tma_full[s]);
        tma_load_3d(st + 2 * L.x_tile + L.a_tile, &tm_lo, kb * kKB, w.half * args.n_half, w.cell,
                    &tma_full[s]);
        issued = g + 1;
      }
      if (*abort_flag) {
        for (int64_t g = (issued > S ? issued - S : 0); g < issued; ++g) {
          const int s = (int)(g % S);
          const uint32_t r = (uint32_t)(g / S);
          for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(&tma_full[s], r & 1); ++i)
            __nanosleep(128);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_f16(kVec, args.n_half);
      bool ok = true;
      for (int64_t it = 0; it < my_units && ok; ++it) {
        const int buf = (int)(it & 1);
        const uint32_t ph = (uint32_t)((it >> 1) & 1);
        if (!mbar_wait(&acc_empty[buf], ph ^ 1, args.err, abort_flag)) break;
        fence_after();
        const uint32_t d = tmem + buf * args.buf_stride;
        for (int kb = 0; kb < nkb; ++kb) {
          const int64_t g = it * nkb + kb;
          const int s = (int)(g % S);
          const uint32_t r = (uint32_t)(g / S);
          if (!mbar_wait(&tma_full[s], r & 1, args.err, abort_flag) ||
              !mbar_wait(&x_full[s], r & 1, args.err, abort_flag)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t st = smem_u32(smem + s * L.stage);
          const uint32_t xhi = st, xlo = st + L.x_tile;
          const uint32_t ahi = st + 2 * L.x_tile, alo = ahi + L.a_tile;
#pragma unroll
          for (int ks = 0; ks < kKB / 16; ++ks) {
            const uint32_t koff = ks * 32;  // 16 halves = 32 bytes along K
            const uint32_t acc0 = (kb > 0 || ks > 0) ? 1u : 0u;
            mma_f16(d, smem_desc_sw64(xhi + koff), smem_desc_sw64(ahi + koff), idesc, acc0);
            mma_f16(d, smem_desc_sw64(xhi + koff), smem_desc_sw64(alo + koff), idesc, 1u);
            mma_f16(d, smem_desc_sw64(xlo + koff), smem_desc_sw64(ahi + koff), idesc, 1u);
          }
          mma_commit(&empty[s]);
        }
        if (ok) mma_commit(&acc_full[buf]);
      }
      // every MMA must be complete before tensor memory is freed, also on the abort path
      mma_commit(mma_done);
      for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(mma_done, 0); ++i) __nanosleep(128);
    }
  } else if (warp < 6) {
    // ---------------- X producers: cp.async gather into an FP32 staging ring (kXStages deep,
    // so ~64 KB of rows are in flight per SM), then FP16 hi/lo split into the stage ring
    const int t = threadIdx.x - 64;          // 0..127
    const int v = (warp & 3) * 32 + lane;    // vector row this thread converts
    uint8_t* xst = smem + L.xstage;
    // the dof-map entries of a K-block are loaded one issue ahead, so the cp.async of a block
    // never waits on a dependent map load
    int mnext[8];
    auto load_map = [&](int64_t g, int* mv) {
      if (g < my_blocks) {
        const Unit w = unit_at(g / nkb, first, step, args);
        const int kb = (int)(g % nkb);
        const int* mrow = args.map + (int64_t)w.cell * args.n_e;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int J = kb * kKB + ((i * 128 + t) >> 5);
          mv[i] = J < args.n_e ? __ldg(mrow + J) : -1;
        }
      }
    };
    auto issue = [&](int64_t g) {
      uint8_t* slot = xst + (int)(g % kXStages) * kXStageBytes;
      int mv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) mv[i] = mnext[i];
      load_map(g + 1, mnext);
      if (g < my_blocks) {
        const Unit w = unit_at(g / nkb, first, step, args);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int q = i * 128 + t;             // 16-byte chunk of the [32][128] slot
          const int j = q >> 5, c4 = (q & 31) * 4;
          const int gb = w.chunk * kVec + c4;
          const bool ok = (mv[i] >= 0) && (gb < args.B);
          const float* src = ok ? args.src + (int64_t)mv[i] * args.lds + gb : args.src;
          cp_async16(slot + j * (kVec * 4) + c4 * 4, src, ok);
        }
      }
      cp_async_commit();
    };
    load_map(0, mnext);
#pragma unroll
    for (int i = 0; i < kXStages - 1; ++i) issue(i);
    bool stop = false;
    for (int64_t g = 0; g < my_blocks; ++g) {
      issue(g + kXStages - 1);
      cp_async_wait<kXStages - 1>();
      // block g's rows landed for all producer threads; a stop seen by any thread ends all
      if (producers_sync_or(stop)) break;
      const float* slot = reinterpret_cast<const float*>(xst + (int)(g % kXStages) * kXStageBytes);
      float cur[kKB];
#pragma unroll
      for (int j = 0; j < kKB; ++j) cur[j] = slot[j * kVec + v];
      producers_sync();                       // slot may be refilled by the next issue
      const int s = (int)(g % S);
      const uint32_t r = (uint32_t)(g / S);
      if (!mbar_wait(&empty[s], (r & 1) ^ 1, args.err, abort_flag)) {
        stop = true;
        continue;
      }
      uint8_t* st = smem + s * L.stage;
      uint8_t* rhi = st + v * kRowBytes;
      uint8_t* rlo = st + L.x_tile + v * kRowBytes;
      const int sw = (v >> 1) & 3;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        uint32_t hv[4], lv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const float a0 = cur[c * 8 + 2 * u], a1 = cur[c * 8 + 2 * u + 1];
          const __half2 h = __floats2half2_rn(a0, a1);
          const float2 hf = __half22float2(h);
          const __half2 l = __floats2half2_rn(a0 - hf.x, a1 - hf.y);
          hv[u] = *reinterpret_cast<const uint32_t*>(&h);
          lv[u] = *reinterpret_cast<const uint32_t*>(&l);
        }
        const int pc = (c ^ sw) * 16;
        *reinterpret_cast<uint4*>(rhi + pc) = make_uint4(hv[0], hv[1], hv[2], hv[3]);
        *reinterpret_cast<uint4*>(rlo + pc) = make_uint4(lv[0], lv[1], lv[2], lv[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&x_full[s]);
    }
    cp_async_wait<0>();
  } else {
    // ---------------- epilogue warps 6..9
    const int q = warp & 3;                  // tensor-memory lane quarter of this warp
    const int v = q * 32 + lane;
    for (int64_t it = 0; it < my_units; ++it) {
      const int buf = (int)(it & 1);
      const uint32_t ph = (uint32_t)((it >> 1) & 1);
      const bool ok = __all_sync(0xffffffffu, mbar_wait(&acc_full[buf], ph, args.err, abort_flag));
      if (!ok) break;
      fence_after();
      const Unit w = unit_at(it, first, step, args);
      const int gb = w.chunk * kVec + v;
      const bool vok = gb < args.B;
      const int* mrow = args.map + (int64_t)w.cell * args.n_e + w.half * args.n_half;
      const int nrows = min(args.n_half, args.n_e - w.half * args.n_half);
      float* dstb = args.dst + gb;
      const uint32_t tq = tmem + buf * args.buf_stride + ((uint32_t)(q * 32) << 16);
      for (int c0 = 0; c0 < args.n_half; c0 += 16) {
        float vals[16];
        tmem_ld16(tq + c0, vals);
        if (vok) {
#pragma unroll
          for (int i = 0; i < 16; ++i) {
            const int I = c0 + i;
            if (I < nrows)
              atomicAdd(dstb + (int64_t)__ldg(mrow + I) * args.ldd, args.out_scale * vals[i]);
          }
        }
      }
      fence_before();
      mbar_arrive(&acc_empty[buf]);
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(args.tmem_cols));
  }
}

// ---------------------------------------------------------------- host side
__global__ void k_split_mats(const double* __restrict__ mats, int n_cells, int n_e, int npad,
                             double scale, __half* __restrict__ hi, __half* __restrict__ lo) {
  const int64_t n = (int64_t)n_cells * npad * npad;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t / ((int64_t)npad * npad);
    const int r = (int)(t % ((int64_t)npad * npad));
    const int I = r / npad, J = r % npad;
    double v = 0.0;
    if (I < n_e && J < n_e) v = scale * mats[(c * n_e + I) * n_e + J];
    const __half h = __double2half(v);
    hi[t] = h;
    lo[t] = __double2half(v - (double)__half2float(h));
  }
}

void make_map(CUtensorMap* m, __half* base, int n_cells, int npad, int box_rows) {
  EncodeTiledFn enc = get_encode();
  if (!enc) throw Error(CHEFSI_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  cuuint64_t dims[3] = {(cuuint64_t)npad, (cuuint64_t)npad, (cuuint64_t)n_cells};
  cuuint64_t strides[2] = {(cuuint64_t)npad * 2, (cuuint64_t)npad * npad * 2};
  cuuint32_t box[3] = {(cuuint32_t)kKB, (cuuint32_t)box_rows, 1};
  cuuint32_t estr[3] = {1, 1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 3, base, dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(CHEFSI_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

struct TcPlan {
  int npad, n_half, n_halves, buf_stride, tmem_cols, stages, smem;
};

TcPlan plan_for(int n_e) {
  TcPlan p{};
  p.npad = (n_e + 31) / 32 * 32;
  if (p.npad <= 256) {
    p.n_halves = 1;
    p.n_half = p.npad;
  } else {
    p.n_halves = 2;
    p.n_half = p.npad / 2;  // multiple of 16
  }
  p.buf_stride = p.n_half <= 128 ? 128 : 256;
  p.tmem_cols = 2 * p.buf_stride;
  const int budget = 220 * 1024;
  p.stages = 8;
  while (p.stages > 2 && make_layout(p.n_half, p.stages).total + 1024 > budget) --p.stages;
  p.smem = make_layout(p.n_half, p.stages).total + 1024;
  return p;
}

}  // namespace

namespace tcx {
EncodeTiledFn get_encode() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                         &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
    else
      cudaGetLastError();
  });
  return fn;
}

void make_map_2d(CUtensorMap* m, const __half* base, int64_t inner, int64_t rows, int64_t ld,
                 int box_inner, int box_rows) {
  EncodeTiledFn enc = get_encode();
  if (!enc) throw Error(CHEFSI_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  CHEFSI_REQUIRE((reinterpret_cast<uintptr_t>(base) & 15) == 0 && (ld * 2) % 16 == 0 &&
                     (box_inner * 2) % 16 == 0 && box_rows <= 256 && box_inner <= 256,
                 "tensor map: unaligned base, row stride or box");
  cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
  cuuint32_t box[2] = {(cuuint32_t)box_inner, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT16, 2, const_cast<__half*>(base), dims, strides,
                   box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS)
    throw Error(CHEFSI_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

bool tcgen05_device() {
  if (!get_encode()) return false;
  int dev = 0, major = 0;
  CHEFSI_CUDA(cudaGetDevice(&dev));
  CHEFSI_CUDA(cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev));
  return major == 10;  // sm_100 family (GB300 = 10.3)
}
}  // namespace tcx

void prepare_tensor_mats(chefsi_operator_s* op, cudaStream_t st) {
  auto& tc = op->tc;
  if (tc.ready || op->is_complex || !op->folded) return;
  const int n_e = op->n_e;
  const TcPlan p = plan_for(n_e);
  CHEFSI_REQUIRE(p.n_half <= 256 && p.n_half % 16 == 0, "cell too large for the tensor path");
  // power-of-two scale: largest |A_e| -> [2^14, 2^15)
  DeviceBuffer<double> amax(1);
  absmax_block_f64(op->mats64.ptr, n_e, (int64_t)op->n_cells * n_e, n_e, amax.ptr, st);
  double h = 0.0;
  CHEFSI_CUDA(cudaMemcpyAsync(&h, amax.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  const int e = (h > 0 && std::isfinite(h)) ? 14 - (int)std::floor(std::log2(h)) : 0;
  tc.scale = (float)std::ldexp(1.0, e);
  tc.npad = p.npad;
  tc.kpad = p.npad;
  const size_t n = (size_t)op->n_cells * p.npad * p.npad;
  tc.hi.reset(n);
  tc.lo.reset(n);
  k_split_mats<<<grid_for((int64_t)n, 256), 256, 0, st>>>(op->mats64.ptr, op->n_cells, n_e, p.npad,
                                                          std::ldexp(1.0, e), tc.hi.ptr, tc.lo.ptr);
  CHEFSI_CHECK_LAUNCH();
  tc.ready = true;
}

bool tc_usable(chefsi_operator_s* op) {
  if (op->is_complex || !op->folded || op->n_e > 512) return false;
  return tcgen05_device();
}

// launch the persistent tensor-core kernel (a.out_scale set by the caller)
static void launch_tc(chefsi_operator_s* op, TcArgs& a, const float* src, int64_t lds, float* dst,
                      int64_t ldd, int B, cudaStream_t st) {
  prepare_tensor_mats(op, st);
  const TcPlan p = plan_for(op->n_e);
  if (!op->tc_err.ptr) {
    op->tc_err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(op->tc_err.ptr, 0, sizeof(int), st));
  }
  CUtensorMap mhi, mlo;
  make_map(&mhi, op->tc.hi.ptr, op->n_cells, p.npad, p.n_half);
  make_map(&mlo, op->tc.lo.ptr, op->n_cells, p.npad, p.n_half);
  a.src = src;
  a.lds = lds;
  a.dst = dst;
  a.ldd = ldd;
  a.map = op->map.ptr;
  a.n_e = op->n_e;
  a.nkb = p.npad / kKB;
  a.B = B;
  a.n_chunks = (B + kVec - 1) / kVec;
  a.n_half = p.n_half;
  a.n_halves = p.n_halves;
  a.buf_stride = p.buf_stride;
  a.tmem_cols = p.tmem_cols;
  a.stages = p.stages;
  a.n_units = (int64_t)op->n_cells * a.n_chunks * p.n_halves;
  a.err = op->tc_err.ptr;
  CHEFSI_CUDA(cudaFuncSetAttribute(cell_hx_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   227 * 1024));
  int dev = 0, sms = kNumSMs;
  CHEFSI_CUDA(cudaGetDevice(&dev));
  CHEFSI_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t grid = std::min<int64_t>(sms, a.n_units / p.n_halves);
  cell_hx_tc_kernel<<<(unsigned)grid, kThreads2, p.smem, st>>>(mhi, mlo, a);
  CHEFSI_CHECK_LAUNCH();
}

// the X gather copies 16-byte pieces: rows must start 16-byte aligned
static bool gather_aligned(const float* src, int64_t lds, int B) {
  return (B % 4 == 0) && (lds % 4 == 0) && ((reinterpret_cast<uintptr_t>(src) & 15) == 0);
}

bool hx_tc(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd, int B,
           double scalar, bool accumulate, cudaStream_t st) {
  if (!tc_usable(op) || !gather_aligned(src, lds, B)) return false;
  if (!accumulate) scale_block<float>(dst, ldd, op->n_dofs, B, 0.0, st);
  prepare_tensor_mats(op, st);
  TcArgs a{};
  a.out_scale = (float)(scalar / op->tc.scale);
  launch_tc(op, a, src, lds, dst, ldd, B, st);
  apply_nonlocal_f32(op, src, lds, dst, ldd, B, scalar, st);
  return true;
}

int tc_check_error(chefsi_operator_s* op, cudaStream_t st) {
  if (!op->tc_err.ptr) return CHEFSI_OK;
  int h = 0;
  CHEFSI_CUDA(cudaMemcpyAsync(&h, op->tc_err.ptr, sizeof(int), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  if (h) CHEFSI_CUDA(cudaMemsetAsync(op->tc_err.ptr, 0, sizeof(int), st));
  return h;
}

}  // namespace chefsi
