// Tensor-core filter HX on GB300: tcgen05 MMAs with FP16-split operands, FP32 accumulation
// in tensor memory, fused gather / scatter through the cell -> dof map.
//
// DFT-FE's local HX (src/dftOperator/matrixVectorProductImplementationsDevice.cc:27-117)
// gathers X into n_cells x n_e x B cell blocks, calls gemmStridedBatched and scatter-adds.
// Here no cell block is materialised, and one CTA owns one (cell, 128-vector chunk, half of
// the cell's rows) at a time:
//   * producer warps copy the chunk's X rows through the cell's dof map (cp.async, 16-byte
//     pieces) into a 128B-swizzled, MN-major tile: either FP16 hi + lo rows the caller split
//     (the Rayleigh-Ritz apply, the unshifted filter variants) or, for the default filter step
//     (F32X), FP32 rows staged per thread and split by the producers themselves; one bulk copy
//     per split term loads the cell-matrix K-block (FP16 hi and lo of 2^s A_e, stored tile by
//     tile as the K-major, 64B-swizzled shared-memory image);
//   * one lane issues tcgen05.mma kind::f16 with M = 128 vectors, N = the half's rows
//     (<= 256), K = 16:  D += Xhi Ahi^T + Xhi Alo^T + Xlo Ahi^T  (lo*lo is below 2^-22);
//   * the epilogue warps read D with tcgen05.ld (lane = vector) and scatter-add
//     scalar * D / 2^s into the output rows with red.global.add.f32 -- for every cell row the
//     32 lanes of a warp hit 32 consecutive floats, one 128-byte line per instruction. The
//     scatter's instruction stream is the kernel's critical path (per-role cycle counters
//     show the epilogue busy ~95% of the time), so two warps share each tensor-memory lane
//     quarter and drain half of the columns each (8 epilogue warps: 1.10x faster than 4).
//     Measured and rejected: float4 reductions after a lane-quad transpose (1.6x slower),
//     plain load + store for the rows only one cell touches (more latency on the same
//     critical path, 1.08x slower), L2 prefetch of the output rows (1.07x slower), rows
//     staged in shared memory 16 at a time and added by the bulk-copy unit
//     (cp.reduce.async.bulk .add.f32, one 512-byte row segment per instruction: 1.15x
//     slower), and loading the rows of one cell entry a 16-row group ahead and storing them
//     instead of reducing (1.6x slower).
// An mbarrier pipeline of up to 8 stages overlaps the copies, the MMAs and the scatter of the
// previous unit. Every mbarrier wait is bounded: on expiry the CTA records
// CHEFSI_ERR_TIMEOUT in a device flag, waits (bounded) for its own bulk copies, frees its
// tensor memory and returns.
#include "internal.h"
#include "tc_common.cuh"

#include <algorithm>
#include <cmath>
#include <vector>

namespace chefsi {

using namespace tcx;

namespace {

constexpr int kVec = 128;          // vectors per work unit (MMA M)
constexpr int kKB = 32;            // cell nodes per K-block
constexpr int kRowBytes = kKB * 2; // 64: one K-major row of the cell-matrix tile

// shared-memory descriptor of an MN-major, 128-byte-swizzled operand: atoms of 64 elements
// (128 B) along M x 8 rows along K (1 KB); lbo = byte step between atoms along M, sbo =
// byte step between 8-row groups along K
__device__ __forceinline__ uint64_t smem_desc_mn_sw128(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;  // SWIZZLE_128B
  return d;
}

// X tile of one K-block: 2 atoms along the 128 vectors x 4 groups of 8 nodes
constexpr uint32_t kXAtomM = 1024;   // byte step between the two 64-vector atoms
constexpr uint32_t kXGroupK = 2048;  // byte step between 8-node groups
constexpr int kXTile = 8192;         // 32 nodes x 128 vectors x 2 B

// One operator applied to one block of vectors. A launch takes a group of these (operators of
// the same cell type: the same n_e and tile shapes), so many Hamiltonians of uneven mesh and
// block sizes share one persistent launch; a single apply is a group of one.
struct TcProblem {
  const __half* xhi;   // split rows [rows][ldx]
  const __half* xlo;
  const __half* xlo3;  // third term of the three-term split (NS == 3)
  float* dst;          // output rows [rows][ldd]
  const int* map;      // [n_cells][n_e]
  const __half* ahi;   // cell-matrix tiles in their shared-memory image (see TensorCellMats)
  const __half* alo;
  const __half* alo3;
  int64_t ldx;         // halves
  int64_t ldd;
  int64_t pair_begin;  // first (cell, chunk) pair of this problem in the group's enumeration
  int B;               // vectors
  int n_chunks;        // 128-vector chunks
  float out_scale;     // scalar / 2^s
  int a_shared;        // 1: one matrix for every cell (the density's shape functions)
  const float* occ;    // density: per-vector weights (occupations, scales folded in)
  float* rho;          // density: [n_cells][n_rows] sums of occ_v D[v][row]^2
};
constexpr int kMaxGroup = 32;

// The fused filter step (one problem): the epilogue finishes the three-term recurrence
//   x_j = out_scale D + cj x_{j-1} + bj x_{j-2}
// instead of only scatter-adding D. Every row's FP32 accumulator is pre-set to
// cj x_{j-1} + bj x_{j-2} (by the previous degree); the drain warps reduce D into it. Once the
// unit's reductions are performed, the finalizer warps count the unit's arrival on each shared
// row (acquire-release atomics per row and 128-vector chunk); the unit that brings a row's last
// contribution (always, for rows of one cell entry) writes the row's FP16 split of x_j and
// pre-sets its accumulator for the next degree: cn x_j + bn x_{j-1}.
struct TcFused {
  const int* mapk;                 // [n_cells][kstride] split row feeding K index J (-1: zero)
  int kstride;
  int has_next;
  const int2* rowinfo;             // [n_cells][n_e] {dof, shared index or -1}
  __half* ohi;                     // output split rows (x_j)
  __half* olo;
  float* acc;                      // [n_dofs][B] accumulators
  unsigned* counter;               // [n_shared][n_chunks] arrivals
  const unsigned char* ncontrib;   // [n_shared] cell entries per shared row
  float cj, bj, cn, bn;
};

struct TcArgs {
  TcProblem prob[kMaxGroup];
  int n_probs;
  int64_t n_pairs; // (cell, chunk) pairs over the group
  int n_e;
  int n_rows;      // matrix rows (= n_e for H; quadrature points for the density)
  int nkb;         // K-blocks of 32 nodes
  int n_half;      // cell rows per work unit (= MMA N)
  int n_halves;    // row halves per cell (1 or 2)
  int buf_stride;  // tensor-memory column offset of accumulator 1
  int tmem_cols;
  int stages;      // cell-matrix ring depth
  int xstages;     // X ring depth
  int lookahead;   // K-blocks of X copies in flight per producer thread
  int cell_tile;   // > 1: (cell, chunk) pairs dealt as tiles of cell_tile cells, every chunk of
                   // a tile's cells before the next tile; <= 1: a cell's chunks back to back
  // F32X launches: X given as FP32 rows x32 [rows][ldx] (rows >= w_row: the projector
  // coefficients), split into FP16 hi + lo by the producer warps after scaling by xf (dof rows)
  // or wf (projector rows); sstages FP32 staging slots per producer thread ring
  const float* x32;
  float xf, wf;
  int64_t w_row;
  int sstages;
  int* err;
  TcFused fz;      // FUSED launches only
};
static_assert(sizeof(TcArgs) <= 4096, "kernel parameters above 4 KB");

// Two rings: the X tiles (xhi, xlo [, xlo3]: 8 KB each a stage) and the cell-matrix tiles
// (ahi, alo [, alo3]). The X ring is the deeper one, since its rows come through the gather
// from HBM / L2 while a cell's matrix halves are shared by the eight chunks processed at about
// the same time (L2). ns = number of split terms (2 or 3).
struct Layout {
  int a_tile;   // n_half rows x 64 B, rounded to 1 KB
  int xstage;   // ns X tiles
  int astage;   // ns matrix tiles
  int aoff;     // start of the matrix ring
  int soff;     // start of the FP32 staging ring (F32X: 32 nodes x 128 vectors a slot)
  int bars;     // barrier block
  int offs;     // epilogue row offsets: 2 x 256 int64 (one table per accumulator)
  int queue;    // fused step: two queues of finished shared rows (count + 256 entries each)
  int total;
};
constexpr int kQueueStride = 264;  // ints per queue (count, 256 entries, padding)
constexpr int kStageF32 = 32 * 128 * 4;  // bytes of one FP32 staging slot
__host__ __device__ inline Layout make_layout(int n_half, int stages, int xstages, int ns,
                                              bool fused = false, int sstages = 0) {
  Layout L;
  L.a_tile = ((n_half * kRowBytes + 1023) / 1024) * 1024;
  L.xstage = ns * kXTile;
  L.astage = ns * L.a_tile;
  L.aoff = xstages * L.xstage;
  L.soff = L.aoff + stages * L.astage;
  L.bars = L.soff + sstages * kStageF32;
  L.offs = L.bars + 8 * (2 * stages + 2 * xstages + 12);
  L.queue = L.offs + 2 * 256 * 8;
  L.total = L.queue + (fused ? 2 * kQueueStride * 4 : 0);
  return L;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src, bool valid) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(dst), "l"(src),
               "r"(valid ? 16 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_n(int n) {
  // wait until at most n of this thread's groups are pending (n is small and warp-uniform)
  switch (n) {
    case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
    case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
    case 2: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
    case 3: asm volatile("cp.async.wait_group 3;" ::: "memory"); break;
    case 4: asm volatile("cp.async.wait_group 4;" ::: "memory"); break;
    case 5: asm volatile("cp.async.wait_group 5;" ::: "memory"); break;
    default: asm volatile("cp.async.wait_group 6;" ::: "memory"); break;
  }
}

// epilogue warps: two per tensor-memory lane quarter, each draining half of the columns
constexpr int kEpiWarps = 8;

// named barrier 2 among the epilogue threads with an AND-reduction of v
__device__ __forceinline__ bool epilogue_sync_and(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, 2, %2, pi;\n"
      " selp.u32 %0, 1, 0, po;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kEpiWarps * 32)
      : "memory");
  return r != 0;
}

// named barrier 2 among the epilogue threads
__device__ __forceinline__ void epilogue_sync() {
  asm volatile("bar.sync 2, %0;" ::"n"(kEpiWarps * 32) : "memory");
}
// arrival on a shared row's counter: release of this CTA's reductions (ordered before by the
// epilogue barrier) and acquire of the other contributors' ones
__device__ __forceinline__ unsigned atom_add_acq_rel_gpu(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v)
               : "memory");
  return old;
}
// fire-and-forget FP32 reduction at L2 (no returned value)
__device__ __forceinline__ void red_add_f32(float* p, float v) {
  asm volatile("red.global.add.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
}
// 16-byte load at L2 (the reductions of other SMs live there; never an L1 copy)
__device__ __forceinline__ float4 ld_cg_f4(const float* p) {
  float4 v;
  asm volatile("ld.global.cg.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(p)
               : "memory");
  return v;
}

// FP32 -> FP16 hi + lo (22 significant bits; the vectors are pre-scaled into FP16's range)
__device__ __forceinline__ void split_f32(float a, __half& h, __half& l) {
  h = __float2half_rn(a);
  l = __float2half_rn(a - __half2float(h));
}

struct Unit {
  int cell, chunk, half, p;
};
// The CTA's it-th unit: (cell, chunk) pairs are dealt round-robin over the CTAs and a CTA
// runs both row halves of its pair back to back, so the second gather of the chunk's X rows
// comes from L2.
__device__ __forceinline__ Unit unit_at(int64_t it, int64_t first, int64_t step,
                                        const TcArgs& a) {
  Unit w;
  w.half = (int)(it % a.n_halves);
  const int64_t cc = first + (it / a.n_halves) * step;
  int p = 0;
  for (int q = 1; q < a.n_probs; ++q)
    if (cc >= a.prob[q].pair_begin) p = q;   // problems in ascending pair order
  const int64_t lc = cc - a.prob[p].pair_begin;
  const int nch = a.prob[p].n_chunks;
  const int G = a.cell_tile;
  if (G <= 1 || nch == 1) {
    w.chunk = (int)(lc % nch);
    w.cell = (int)(lc / nch);
  } else {
    // tile t holds cells [t G, t G + g) (g = G but for the last tile), chunk-major inside
    const int64_t span = (int64_t)G * nch;
    const int64_t t = lc / span;
    const int64_t r = lc - t * span;
    const int64_t pairs = (p + 1 < a.n_probs ? a.prob[p + 1].pair_begin : a.n_pairs) -
                          a.prob[p].pair_begin;
    const int g = (int)min((int64_t)G, pairs / nch - t * G);
    w.chunk = (int)(r / g);
    w.cell = (int)(t * G + r % g);
  }
  w.p = p;
  return w;
}

// Persistent warp-specialised kernel, one CTA per SM. Work unit = (cell, 128-vector chunk,
// row half of the cell matrix). The filter keeps its vectors also as FP16 hi + lo rows
// [dof][vectors], which are exactly the rows of an MN-major A operand (M = vectors):
//   warp 0        bulk copies of the cell-matrix K-block tiles (hi, lo; K-major, 64B-swizzled)
//   warp 1        tcgen05.mma issue (one lane): D[vector][row] += Xhi Ahi + Xhi Alo + Xlo Ahi,
//                 M = 128 vectors, N = the half's rows, K = 16; two accumulators in tensor
//                 memory
//   warps 2..5    X rows: cp.async of 16-byte pieces of the hi and lo rows of the K-block's
//                 32 dofs (dof-map entries loaded one K-block ahead) straight into the
//                 128B-swizzled MN-major tile, `lookahead` K-blocks in flight; no conversion
//   warps 6..13   epilogue: tcgen05.ld of a finished accumulator (lane = vector) and
//                 red.global.add.f32 into the output rows (one 128-byte line per warp
//                 instruction; row offsets staged in shared memory once per unit),
//                 overlapped with the MMAs of the next unit
constexpr int kThreads3 = 192 + 32 * kEpiWarps;
// the fused step adds a warpgroup of finalizer warps (the recurrence of finished rows)
constexpr int kFinWarps = 8;
constexpr int kThreadsFused = kThreads3 + 32 * kFinWarps;
// named barrier 3 among the finalizer warps, with an AND-reduction of v
__device__ __forceinline__ bool fin_sync_and(bool v) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred pi, po;\n setp.ne.u32 pi, %1, 0;\n bar.red.and.pred po, 3, %2, pi;\n"
      " selp.u32 %0, 1, 0, po;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)v), "n"(kFinWarps * 32)
      : "memory");
  return r != 0;
}
__device__ __forceinline__ void fin_sync() {
  asm volatile("bar.sync 3, %0;" ::"n"(kFinWarps * 32) : "memory");
}

// NS = 2: the filter's split (hi + lo, 22 bits), products Xhi Ahi + Xhi Alo + Xlo Ahi.
// NS = 3: hi + lo + lo3 (33 bits: an FP32 vector exactly, the cell matrix to 2^-33), products
//         down to 2^-22 relative: + Xhi Alo3 + Xlo3 Ahi + Xlo Alo.
// KCHUNK: every K-block (32 nodes) accumulates in a fresh tensor-memory accumulator and the
//         epilogue adds the K-block results in FP32 registers (round to nearest) before the
//         scatter. The tensor core's own FP32 accumulation over the ~130 MMA steps of a unit
//         leaves errors ~5x those of an FP32 SIMT apply; over the 12 steps of one K-block it
//         does not. Needs at most kChunkCols accumulator columns per epilogue warp.
constexpr int kChunkCols = 96;
// DENS: the density mode. The matrix is the shape-function matrix N[q][node] (one for all
//       cells, rows = quadrature points in parts of n_half), so D[v][q] = psi_v(x_q) for the
//       gathered vectors; the epilogue adds occ_v D[v][q]^2 over the vectors into rho[c][q]
//       (warp butterfly reduction, one FP32 atomic per quadrature point and warp).
// FUSED: the fused filter step (see TcFused): the K side gathers through the extended map
//        (the cell's nodes, then its projector coefficients W), the epilogue finishes the
//        recurrence.
// F32X: the X rows come as FP32 (args.x32), copied into a per-thread staging ring and split by
//       the producer warps themselves (no separate split pass over the vectors).
template <int NS, bool KCHUNK, bool DENS = false, bool FUSED = false, bool F32X = false>
__global__ void __launch_bounds__(FUSED ? kThreadsFused : kThreads3, 1)
    cell_hx_tc_kernel(TcArgs args) {
  extern __shared__ uint8_t smem_raw[];
  uint8_t* smem = reinterpret_cast<uint8_t*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int S = args.stages, SX = args.xstages;
  const Layout L = make_layout(args.n_half, S, SX, NS, FUSED, F32X ? args.sstages : 0);
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem + L.bars);
  uint64_t* tma_full = bars;            // [S] cell-matrix tile bytes landed
  uint64_t* a_empty = bars + S;         // [S] MMA finished reading the matrix stage
  uint64_t* x_full = bars + 2 * S;      // [SX] 4 producer-warp arrivals (their copies landed)
  uint64_t* x_empty = bars + 2 * S + SX;   // [SX] MMA finished reading the X stage
  uint64_t* acc_full = bars + 2 * S + 2 * SX;       // [2] accumulator ready for the epilogue
  uint64_t* acc_empty = acc_full + 2;               // [2] accumulator drained (one arrival per epilogue warp)
  uint64_t* mma_done = acc_full + 4;                // final MMA completion
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(acc_full + 5);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(acc_full + 6);
  uint64_t* rows_ready = acc_full + 7;    // [2] fused: a unit's reductions are performed
  uint64_t* rows_empty = acc_full + 9;    // [2] fused: the finalizers are done with the slot

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t first = blockIdx.x;
  const int64_t step = gridDim.x;
  const int64_t n_pairs = args.n_pairs;   // (cell, chunk) pairs over the group
  const int64_t my_units =
      first < n_pairs ? ((n_pairs - first + step - 1) / step) * args.n_halves : 0;
  const int nkb = args.nkb;
  const int64_t my_blocks = my_units * nkb;

  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&tma_full[s], 1);
      mbar_init(&a_empty[s], 1);
    }
    for (int s = 0; s < SX; ++s) {
      mbar_init(&x_full[s], 4);      // one arrival per producer warp
      mbar_init(&x_empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&acc_full[b], 1);
      mbar_init(&acc_empty[b], kEpiWarps);   // one arrival per epilogue warp
    }
    mbar_init(mma_done, 1);
    if (FUSED) {
      for (int b = 0; b < 2; ++b) {
        mbar_init(&rows_ready[b], 1);
        mbar_init(&rows_empty[b], kFinWarps);
      }
    }
    *abort_flag = wait_limit_init(args.err);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) tmem_alloc(tmem_slot, args.tmem_cols);
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    // ---------------- bulk-copy producer of the cell-matrix K-blocks
    if (lane == 0) {
      const uint32_t bytes = (uint32_t)NS * args.n_half * kRowBytes;
      int64_t issued = 0;
      int s = 0;
      uint32_t r = 0;
      bool ok = true;
      for (int64_t it = 0; it < my_units && ok; ++it) {
        const Unit w = unit_at(it, first, step, args);
        for (int kb = 0; kb < nkb; ++kb) {
          if (!mbar_wait(&a_empty[s], (r & 1) ^ 1, args.err, abort_flag)) {
            ok = false;
            break;
          }
          uint8_t* st = smem + L.aoff + s * L.astage;
          mbar_arrive_expect_tx(&tma_full[s], bytes);
          // one contiguous block per split term: the (cell, half, K-block) tile, stored in
          // its swizzled shared-memory image
          const TcProblem& pa = args.prob[w.p];
          const int64_t tix = ((int64_t)(pa.a_shared ? 0 : w.cell) * args.n_halves + w.half) * nkb + kb;
          const int64_t toff = tix * (args.n_half * (kRowBytes / 2));
          const TcProblem& pr = args.prob[w.p];
          bulk_load(st, pr.ahi + toff, bytes / NS, &tma_full[s]);
          bulk_load(st + L.a_tile, pr.alo + toff, bytes / NS, &tma_full[s]);
          if (NS == 3) bulk_load(st + 2 * L.a_tile, pr.alo3 + toff, bytes / NS, &tma_full[s]);
          ++issued;
          if (++s == S) s = 0, ++r;
        }
      }
      if (*abort_flag) {
        for (int64_t h = (issued > S ? issued - S : 0); h < issued; ++h) {
          const int sh = (int)(h % S);
          const uint32_t rh = (uint32_t)(h / S);
          for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(&tma_full[sh], rh & 1); ++i)
            __nanosleep(128);
        }
      }
    }
  } else if (warp == 1) {
    // ---------------- MMA issuer
    if (lane == 0) {
      const uint32_t idesc = idesc_f16(kVec, args.n_half) | (1u << 15);  // A MN-major
      bool ok = true;
      int s = 0, sx = 0;            // ring positions of the next K-block
      uint32_t r = 0, rx = 0;       // and their phases
      int64_t g = 0;                // K-blocks issued (KCHUNK: accumulator sequence)
      for (int64_t it = 0; it < my_units && ok; ++it) {
        int buf = (int)(it & 1);
        uint32_t ph = (uint32_t)((it >> 1) & 1);
        if (!KCHUNK) {
          if (!mbar_wait(&acc_empty[buf], ph ^ 1, args.err, abort_flag)) break;
          fence_after();
        }
        uint32_t d = tmem + buf * args.buf_stride;
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          if (KCHUNK) {
            buf = (int)(g & 1);
            ph = (uint32_t)((g >> 1) & 1);
            if (!mbar_wait(&acc_empty[buf], ph ^ 1, args.err, abort_flag)) {
              ok = false;
              break;
            }
            fence_after();
            d = tmem + buf * args.buf_stride;
          }
          if (!mbar_wait(&tma_full[s], r & 1, args.err, abort_flag) ||
              !mbar_wait(&x_full[sx], rx & 1, args.err, abort_flag)) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t xhi = smem_u32(smem + sx * L.xstage), xlo = xhi + kXTile;
          const uint32_t ahi = smem_u32(smem + L.aoff + s * L.astage), alo = ahi + L.a_tile;
          if (NS == 2) {
#pragma unroll
            for (int ks = 0; ks < kKB / 16; ++ks) {
              const uint32_t xoff = ks * 2 * kXGroupK;  // 16 nodes = two 8-node groups
              const uint32_t koff = ks * 32;            // 16 halves of a K-major row
              const uint32_t acc0 = ((!KCHUNK && kb > 0) || ks > 0) ? 1u : 0u;
              mma_f16(d, smem_desc_mn_sw128(xhi + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(ahi + koff), idesc, acc0);
              mma_f16(d, smem_desc_mn_sw128(xhi + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(alo + koff), idesc, 1u);
              mma_f16(d, smem_desc_mn_sw128(xlo + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(ahi + koff), idesc, 1u);
            }
          } else {
            // small products of both K-steps first, the two hi * hi products last, so that
            // the truncating FP32 accumulation adds few terms at the large magnitude
            const uint32_t xlo3 = xhi + 2 * kXTile, alo3 = ahi + 2 * L.a_tile;
#pragma unroll
            for (int ks = 0; ks < kKB / 16; ++ks) {
              const uint32_t xoff = ks * 2 * kXGroupK;
              const uint32_t koff = ks * 32;
              const uint32_t acc0 = ((!KCHUNK && kb > 0) || ks > 0) ? 1u : 0u;
              mma_f16(d, smem_desc_mn_sw128(xlo + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(alo + koff), idesc, acc0);
              mma_f16(d, smem_desc_mn_sw128(xhi + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(alo3 + koff), idesc, 1u);
              mma_f16(d, smem_desc_mn_sw128(xlo3 + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(ahi + koff), idesc, 1u);
              mma_f16(d, smem_desc_mn_sw128(xhi + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(alo + koff), idesc, 1u);
              mma_f16(d, smem_desc_mn_sw128(xlo + xoff, kXAtomM, kXGroupK),
                      smem_desc_sw64(ahi + koff), idesc, 1u);
            }
#pragma unroll
            for (int ks = 0; ks < kKB / 16; ++ks)
              mma_f16(d, smem_desc_mn_sw128(xhi + ks * 2 * kXGroupK, kXAtomM, kXGroupK),
                      smem_desc_sw64(ahi + ks * 32), idesc, 1u);
          }
          mma_commit(&a_empty[s]);
          mma_commit(&x_empty[sx]);
          if (KCHUNK) mma_commit(&acc_full[buf]);
          if (++s == S) s = 0, ++r;
          if (++sx == SX) sx = 0, ++rx;
        }
        if (!KCHUNK && ok) mma_commit(&acc_full[buf]);
      }
      // every MMA must be complete before tensor memory is freed, also on the abort path
      mma_commit(mma_done);
      for (uint32_t i = 0; i < kWaitLimit && !mbar_try_wait(mma_done, 0); ++i) __nanosleep(128);
    }
  } else if (warp < 6) {
    // ---------------- X producers. Thread t copies 16-byte piece cc = t % 16 (8 vectors) of
    // the hi and lo rows of the K-block's nodes 8 j + t / 16 (j = 0..3). Element (vector m,
    // node k) of the tile sits in atom (m / 64, k / 8), row k % 8, 16-byte chunk
    // (m % 64) / 8 XOR k % 8.
    // F32X: the thread's FP32 pieces of a K-block (4 rows x 8 vectors, 32 B each) go to
    // its staging slot, row r at r x 512 B, vectors 8 cc..8 cc + 7 as 16-byte chunks
    // 2 cc + (h XOR (cc / 4) % 2) (the XOR spreads a warp's read-back over all banks); the
    // thread splits its own pieces into the tile once they landed, so staging needs no barrier.
    const int t = threadIdx.x - 64;
    const int cc = t & 15, rsub = t >> 4;
    const int mi = cc >> 3, c = cc & 7;
    const uint32_t dst_base = mi * kXAtomM + rsub * 128 + ((uint32_t)(c ^ rsub) << 4);
    const int D = F32X ? args.sstages - 1 : args.lookahead;
    const uint32_t sw = (uint32_t)(cc >> 2) & 1u;
    const uint32_t s_base = smem_u32(smem + L.soff) + (uint32_t)rsub * 512u + (uint32_t)cc * 32u;
    uint32_t wmask = 0;   // F32X: bit 4 slot + j = row j of the slot is a projector row
    // cursor over this CTA's K-blocks (no per-block divisions): unit it, K-block kb
    int64_t c_it = 0;
    int c_kb = 0;
    Unit c_w = my_units > 0 ? unit_at(0, first, step, args) : Unit{0, 0, 0, 0};
    struct Pending {
      int rows[4];
      int vb;
      int p;
      bool valid;
    } nxt;
    // dof-map entries of the cursor's K-block (one K-block ahead of the copies)
    auto load_next = [&]() {
      nxt.valid = c_it < my_units;
      if (nxt.valid) {
        // the extended K side (the cell's nodes, then its projector columns) for the fused step
        // and for a single apply with the nonlocal term folded in
        const bool kext = FUSED || args.fz.mapk != nullptr;
        const int kst = kext ? args.fz.kstride : args.n_e;
        const int* mrow = (kext ? args.fz.mapk : args.prob[c_w.p].map) + (int64_t)c_w.cell * kst;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int J = c_kb * kKB + j * 8 + rsub;
          nxt.rows[j] = J < kst ? __ldg(mrow + J) : -1;
        }
        nxt.vb = c_w.chunk * kVec + cc * 8;
        nxt.p = c_w.p;
        if (++c_kb == nkb) {
          c_kb = 0;
          if (++c_it < my_units) c_w = unit_at(c_it, first, step, args);
        }
      }
    };
    int s_iss = 0;
    uint32_t r_iss = 0;
    // issue the copies of the next K-block into its X stage (waits for the stage to be free)
    auto issue = [&]() -> bool {
      const Pending cur = nxt;
      load_next();
      if (F32X) {
        // into staging slot s_iss (free: its previous block was split by this thread)
        if (cur.valid) {
          const TcProblem& pr = args.prob[cur.p];
          const bool vok = cur.vb < pr.B;
          const uint32_t st = s_base + (uint32_t)s_iss * kStageF32;
          wmask &= ~(15u << (4 * s_iss));
#pragma unroll
          for (int j = 0; j < 4; ++j) {
            const bool ok = vok && cur.rows[j] >= 0;
            const int64_t off = ok ? (int64_t)cur.rows[j] * pr.ldx + cur.vb : 0;
            const uint32_t d = st + (uint32_t)j * 8u * 512u;
            cp_async16(d + (sw << 4), args.x32 + off, ok);
            cp_async16(d + ((sw ^ 1u) << 4), args.x32 + off + 4, ok);
            if (ok && cur.rows[j] >= args.w_row) wmask |= 1u << (4 * s_iss + j);
          }
        }
        cp_async_commit();
        if (++s_iss == D + 1) s_iss = 0;
        return true;
      }
      if (cur.valid) {
        // warp-uniform decision: the warp arrives on x_full as one
        if (!__all_sync(0xffffffffu, mbar_wait(&x_empty[s_iss], (r_iss & 1) ^ 1, args.err, abort_flag)))
          return false;
        const TcProblem& pr = args.prob[cur.p];
        const bool vok = cur.vb < pr.B;
        const uint32_t st = smem_u32(smem + s_iss * L.xstage);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const bool ok = vok && cur.rows[j] >= 0;
          const int64_t off = ok ? (int64_t)cur.rows[j] * pr.ldx + cur.vb : 0;
          const uint32_t d = st + dst_base + j * kXGroupK;
          cp_async16(d, pr.xhi + off, ok);
          cp_async16(d + kXTile, pr.xlo + off, ok);
          if (NS == 3) cp_async16(d + 2 * kXTile, pr.xlo3 + off, ok);
        }
      }
      cp_async_commit();
      if (++s_iss == SX) s_iss = 0, ++r_iss;
      return true;
    };
    load_next();
    bool ok = true;
    for (int i = 0; i < D && ok; ++i) ok = issue();
    int s_arr = 0;
    uint32_t r_arr = 0;
    int s_cv = 0;   // F32X: staging slot of block g
    for (int64_t g = 0; g < my_blocks && ok; ++g) {
      ok = issue();
      cp_async_wait_n(D);                      // this thread's copies of block g landed
      if (F32X) {
        // split the staged block into X stage s_arr once the MMA has released it
        if (!__all_sync(0xffffffffu, mbar_wait(&x_empty[s_arr], (r_arr & 1) ^ 1, args.err, abort_flag))) {
          ok = false;
          break;
        }
        const uint32_t sb = s_base + (uint32_t)s_cv * kStageF32;
        const uint32_t tb = smem_u32(smem + s_arr * L.xstage) + dst_base;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const float f = (wmask >> (4 * s_cv + j)) & 1u ? args.wf : args.xf;
          float v[8];
          asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                       : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
                       : "r"(sb + (uint32_t)j * 8u * 512u + (sw << 4)));
          asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                       : "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                       : "r"(sb + (uint32_t)j * 8u * 512u + ((sw ^ 1u) << 4)));
          // the split of split_f32, two values per conversion
          uint32_t h[4], l[4];
#pragma unroll
          for (int i = 0; i < 4; ++i) {
            const float a0 = f * v[2 * i], a1 = f * v[2 * i + 1];
            const __half2 h2 = __floats2half2_rn(a0, a1);
            const float2 hf = __half22float2(h2);
            const __half2 l2 = __floats2half2_rn(a0 - hf.x, a1 - hf.y);
            h[i] = *reinterpret_cast<const uint32_t*>(&h2);
            l[i] = *reinterpret_cast<const uint32_t*>(&l2);
          }
          const uint32_t d = tb + (uint32_t)j * kXGroupK;
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(d), "r"(h[0]), "r"(h[1]),
                       "r"(h[2]), "r"(h[3])
                       : "memory");
          asm volatile("st.shared.v4.b32 [%0], {%1, %2, %3, %4};" ::"r"(d + kXTile), "r"(l[0]),
                       "r"(l[1]), "r"(l[2]), "r"(l[3])
                       : "memory");
        }
        if (++s_cv == D + 1) s_cv = 0;
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) mbar_arrive(&x_full[s_arr]);
      if (++s_arr == SX) s_arr = 0, ++r_arr;
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
  } else if (FUSED && warp >= 6 + kEpiWarps) {
    // ---------------- fused step: finalizer warps, one unit behind the drain. For each unit:
    // arrivals on the shared rows (acquire-release; the unit that brings a row's last
    // contribution finishes it), then for every finished row (single rows always) and the
    // unit's 128-vector chunk, a warp at a time with 16-byte accesses:
    //   x_j = acc;  split(x_j) -> output rows;  acc <- cn x_j + bn x_{j-1}  (next degree)
    const TcFused& fz = args.fz;
    const TcProblem& pr = args.prob[0];
    const int f = threadIdx.x - (192 + 32 * kEpiWarps);   // finalizer thread 0..255
    const int fw = f >> 5;
    int* lists = reinterpret_cast<int*>(smem + L.queue);
    const int64_t ld = pr.ldx;
    constexpr int kBatch = 4;
    for (int64_t it = 0; it < my_units; ++it) {
      const int slot = (int)(it & 1);
      const uint32_t ph = (uint32_t)((it >> 1) & 1);
      const bool okw = __all_sync(0xffffffffu, mbar_wait(&rows_ready[slot], ph, args.err, abort_flag));
      int* list = lists + slot * kQueueStride;
      if (f == 0) list[0] = 0;
      if (!fin_sync_and(okw)) break;
      const Unit w = unit_at(it, first, step, args);
      const int nrows = min(args.n_half, args.n_e - w.half * args.n_half);
      const int2* rinfo = reinterpret_cast<const int2*>(smem + L.offs) + slot * 256;
      for (int I = f; I < nrows; I += 32 * kFinWarps) {
        const int2 r = rinfo[I];
        bool last = r.y < 0;
        if (!last) {
          const unsigned old = atom_add_acq_rel_gpu(fz.counter + (int64_t)r.y * pr.n_chunks + w.chunk, 1u);
          last = (old + 1u) % (unsigned)__ldg(fz.ncontrib + r.y) == 0u;
        }
        if (last) list[1 + atomicAdd(list, 1)] = I;
      }
      fin_sync();
      const int n = list[0];
      const int v0 = w.chunk * kVec + lane * 4;
      if (v0 < pr.B) {
        for (int k0 = fw; k0 < n; k0 += kFinWarps * kBatch) {
          float4 a[kBatch];
          uint2 xh[kBatch], xl[kBatch];
          int64_t o[kBatch];
#pragma unroll
          for (int b = 0; b < kBatch; ++b) {
            const int k = k0 + b * kFinWarps;
            o[b] = k < n ? (int64_t)rinfo[list[1 + k]].x * ld + v0 : -1;
            if (o[b] >= 0) {
              a[b] = ld_cg_f4(fz.acc + o[b]);
              if (fz.has_next) {
                xh[b] = __ldg(reinterpret_cast<const uint2*>(pr.xhi + o[b]));
                xl[b] = __ldg(reinterpret_cast<const uint2*>(pr.xlo + o[b]));
              }
            }
          }
#pragma unroll
          for (int b = 0; b < kBatch; ++b) {
            if (o[b] < 0) continue;
            __half h[4], l[4];
            split_f32(a[b].x, h[0], l[0]);
            split_f32(a[b].y, h[1], l[1]);
            split_f32(a[b].z, h[2], l[2]);
            split_f32(a[b].w, h[3], l[3]);
            __half2 hh[2] = {__halves2half2(h[0], h[1]), __halves2half2(h[2], h[3])};
            __half2 ll[2] = {__halves2half2(l[0], l[1]), __halves2half2(l[2], l[3])};
            *reinterpret_cast<uint2*>(fz.ohi + o[b]) = *reinterpret_cast<uint2*>(hh);
            *reinterpret_cast<uint2*>(fz.olo + o[b]) = *reinterpret_cast<uint2*>(ll);
            if (fz.has_next) {
              const float2 h01 = __half22float2(*reinterpret_cast<const __half2*>(&xh[b].x));
              const float2 h23 = __half22float2(*reinterpret_cast<const __half2*>(&xh[b].y));
              const float2 l01 = __half22float2(*reinterpret_cast<const __half2*>(&xl[b].x));
              const float2 l23 = __half22float2(*reinterpret_cast<const __half2*>(&xl[b].y));
              float4 nx;
              nx.x = fmaf(fz.bn, h01.x + l01.x, fz.cn * a[b].x);
              nx.y = fmaf(fz.bn, h01.y + l01.y, fz.cn * a[b].y);
              nx.z = fmaf(fz.bn, h23.x + l23.x, fz.cn * a[b].z);
              nx.w = fmaf(fz.bn, h23.y + l23.y, fz.cn * a[b].w);
              *reinterpret_cast<float4*>(fz.acc + o[b]) = nx;
            }
          }
        }
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&rows_empty[slot]);
    }
  } else {
    // ---------------- epilogue warps 6..6 + kEpiWarps - 1
    const int q = warp & 3;                  // tensor-memory lane quarter of this warp
    // this warp's 16-column groups of the accumulator: part (warp - 6) / 4 of kEpiWarps / 4
    const int ng = args.n_half >> 4, part = (warp - 6) >> 2, nparts = kEpiWarps / 4;
    const int c_beg = (ng * part / nparts) * 16, c_end = (ng * (part + 1) / nparts) * 16;
    if (KCHUNK) {
      // per unit: stage the row offsets, then add the unit's nkb K-block accumulators into
      // registers (this warp's columns [c_beg, c_end), at most kChunkCols), then scatter
      int64_t g = 0;
      bool okp = true;
      for (int64_t it = 0; it < my_units; ++it) {
        const Unit w = unit_at(it, first, step, args);
        const TcProblem& pr = args.prob[w.p];
        const int* mrow = pr.map + (int64_t)w.cell * args.n_e + w.half * args.n_half;
        const int nrows = min(args.n_half, args.n_e - w.half * args.n_half);
        int64_t* offs = reinterpret_cast<int64_t*>(smem + L.offs) + (it & 1) * 256;
        for (int I = (warp - 6) * 32 + lane; I < args.n_half; I += kEpiWarps * 32)
          offs[I] = I < nrows ? (int64_t)__ldg(mrow + I) * pr.ldd : -1;
        if (!epilogue_sync_and(okp)) break;
        float sum[kChunkCols];
#pragma unroll
        for (int i = 0; i < kChunkCols; ++i) sum[i] = 0.f;
        bool ok = true;
        for (int kb = 0; kb < nkb; ++kb, ++g) {
          const int buf = (int)(g & 1);
          const uint32_t ph = (uint32_t)((g >> 1) & 1);
          if (!__all_sync(0xffffffffu, mbar_wait(&acc_full[buf], ph, args.err, abort_flag))) {
            ok = false;
            break;
          }
          fence_after();
          const uint32_t tq = tmem + buf * args.buf_stride + ((uint32_t)(q * 32) << 16);
#pragma unroll
          for (int gi = 0; gi < kChunkCols / 16; ++gi) {
            if (c_beg + 16 * gi < c_end) {
              float v[16];
              tmem_ld16(tq + c_beg + 16 * gi, v);
#pragma unroll
              for (int i = 0; i < 16; ++i) sum[16 * gi + i] += v[i];
            }
          }
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acc_empty[buf]);
        }
        okp = ok;
        const int gb = w.chunk * kVec + q * 32 + lane;
        if (ok && gb < pr.B) {
          float* dstb = pr.dst + gb;
          const float osc = pr.out_scale;
#pragma unroll
          for (int gi = 0; gi < kChunkCols / 16; ++gi) {
            if (c_beg + 16 * gi < c_end) {
#pragma unroll
              for (int i = 0; i < 16; ++i) {
                const int64_t o = offs[c_beg + 16 * gi + i];
                if (o >= 0) atomicAdd(dstb + o, osc * sum[16 * gi + i]);
              }
            }
          }
        }
      }
    } else if (FUSED) {
      // ---- the fused step's drain: every row of the unit is reduced into its FP32 accumulator
      // (pre-set to c x_{j-1} + b x_{j-2}); at the start of the next unit the warps fence
      // their reductions (gpu scope) and hand the unit to the finalizer warps
      const TcProblem& pr = args.prob[0];
      const int e = threadIdx.x - 192;          // drain thread 0..255
      bool ok = true;
      int64_t it = 0;
      for (; it < my_units; ++it) {
        const int buf = (int)(it & 1);
        const uint32_t ph = (uint32_t)((it >> 1) & 1);
        bool okw = mbar_wait(&acc_full[buf], ph, args.err, abort_flag);
        // the slot's row table was last read by the finalizers for unit it - 2
        okw = okw && mbar_wait(&rows_empty[buf], ph ^ 1, args.err, abort_flag);
        okw = __all_sync(0xffffffffu, okw);
        fence_after();
        const Unit w = unit_at(it, first, step, args);
        const int nrows = min(args.n_half, args.n_e - w.half * args.n_half);
        int2* rinfo = reinterpret_cast<int2*>(smem + L.offs) + buf * 256;
        if (okw)
          for (int I = e; I < args.n_half; I += kEpiWarps * 32)
            rinfo[I] = I < nrows ? __ldg(args.fz.rowinfo + (int64_t)w.cell * args.n_e +
                                         w.half * args.n_half + I)
                                 : make_int2(-1, -1);
        // the previous unit's reductions are performed at gpu scope before it is handed over
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        if (!epilogue_sync_and(okw)) {
          ok = false;
          break;
        }
        if (it > 0 && e == 0) mbar_arrive(&rows_ready[(it - 1) & 1]);
        const int gb = w.chunk * kVec + q * 32 + lane;
        const bool vok = gb < pr.B;
        float* accb = args.fz.acc + gb;
        const float osc = pr.out_scale;
        const uint32_t tq = tmem + buf * args.buf_stride + ((uint32_t)(q * 32) << 16);
        for (int c0 = c_beg; c0 < c_end; c0 += 16) {
          float vals[16];
          tmem_ld16(tq + c0, vals);
          if (vok) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const int d = rinfo[c0 + i].x;
              if (d >= 0) red_add_f32(accb + (int64_t)d * pr.ldx, osc * vals[i]);
            }
          }
        }
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[buf]);
      }
      if (ok && it > 0) {
        asm volatile("fence.acq_rel.gpu;" ::: "memory");
        epilogue_sync();
        if (e == 0) mbar_arrive(&rows_ready[(it - 1) & 1]);
      }
    } else if (DENS) {
      for (int64_t it = 0; it < my_units; ++it) {
        const int buf = (int)(it & 1);
        const uint32_t ph = (uint32_t)((it >> 1) & 1);
        const bool okw = __all_sync(0xffffffffu, mbar_wait(&acc_full[buf], ph, args.err, abort_flag));
        fence_after();
        if (!epilogue_sync_and(okw)) break;
        const Unit w = unit_at(it, first, step, args);
        const TcProblem& pr = args.prob[w.p];
        const int nrows = min(args.n_half, args.n_rows - w.half * args.n_half);
        const int gb = w.chunk * kVec + q * 32 + lane;
        const float f = gb < pr.B ? __ldg(pr.occ + gb) : 0.f;
        float* rrow = pr.rho + (int64_t)w.cell * args.n_rows + w.half * args.n_half;
        const uint32_t tq = tmem + buf * args.buf_stride + ((uint32_t)(q * 32) << 16);
        for (int c0 = c_beg; c0 < c_end; c0 += 16) {
          float v[16];
          tmem_ld16(tq + c0, v);
#pragma unroll
          for (int i = 0; i < 16; ++i) v[i] = f * v[i] * v[i];
          // butterfly: each step a lane keeps half of its values and adds its partner's
          // matching half; after offsets 16, 8, 4, 2 lane l holds value (l >> 1) & 15 summed
          // over 16 lanes, the last exchange adds the other 16
#pragma unroll
          for (int sh = 4, half = 8; sh >= 1; --sh, half >>= 1) {
            const bool up = (lane >> sh) & 1;
#pragma unroll
            for (int j = 0; j < half; ++j) {
              const float send = up ? v[j] : v[j + half];
              const float keep = up ? v[j + half] : v[j];
              v[j] = keep + __shfl_xor_sync(0xffffffffu, send, 1 << sh);
            }
          }
          const float tot = v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
          const int col = c0 + ((lane >> 1) & 15);
          if ((lane & 1) == 0 && col < nrows) atomicAdd(rrow + col, tot);
        }
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[buf]);
      }
    } else {
      for (int64_t it = 0; it < my_units; ++it) {
        const int buf = (int)(it & 1);
        const uint32_t ph = (uint32_t)((it >> 1) & 1);
        const bool okw = __all_sync(0xffffffffu, mbar_wait(&acc_full[buf], ph, args.err, abort_flag));
        fence_after();
        const Unit w = unit_at(it, first, step, args);
        const TcProblem& pr = args.prob[w.p];
        const int* mrow = pr.map + (int64_t)w.cell * args.n_e + w.half * args.n_half;
        const int nrows = min(args.n_half, args.n_e - w.half * args.n_half);
        // the unit's output-row offsets (dof * ldd), staged once by the epilogue warps; rows
        // past nrows get an offset no lane uses (they are skipped)
        int64_t* offs = reinterpret_cast<int64_t*>(smem + L.offs) + buf * 256;
        if (okw)
          for (int I = (warp - 6) * 32 + lane; I < args.n_half; I += kEpiWarps * 32)
            offs[I] = I < nrows ? (int64_t)__ldg(mrow + I) * pr.ldd : -1;
        // the epilogue warps continue or stop together (a named barrier with an AND-reduction)
        if (!epilogue_sync_and(okw)) break;
        const int gb = w.chunk * kVec + q * 32 + lane;
        const bool vok = gb < pr.B;
        float* dstb = pr.dst + gb;
        const float osc = pr.out_scale;
        const uint32_t tq = tmem + buf * args.buf_stride + ((uint32_t)(q * 32) << 16);
        for (int c0 = c_beg; c0 < c_end; c0 += 16) {
          float vals[16];
          tmem_ld16(tq + c0, vals);
          if (vok) {
#pragma unroll
            for (int i = 0; i < 16; ++i) {
              const int64_t o = offs[c0 + i];
              if (o >= 0) atomicAdd(dstb + o, osc * vals[i]);
            }
          }
        }
        fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&acc_empty[buf]);
      }
    }
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    tmem_dealloc(tmem, args.tmem_cols);
  }
}

// ---------------------------------------------------------------- host side
// Tensor-core copy of the cell matrices, tile by tile: tile (cell, half, kb) holds rows
// [half n_half, (half + 1) n_half) and columns [32 kb, 32 kb + 32) of 2^s A_e (zero outside
// n_e) as n_half rows of 64 bytes in the 64-byte-swizzled shared-memory image, so that the
// kernel loads a K-block with one bulk copy. Entry t of the array (in storage order) maps to
// (cell c, row I, column J) of the padded matrix:
__device__ __forceinline__ void tile_entry(int64_t t, int n_half, int n_halves, int nkb, int& c,
                                           int& I, int& J) {
  const int64_t tile_elems = (int64_t)n_half * 32;
  const int64_t tix = t / tile_elems;
  const uint32_t p = (uint32_t)(t - tix * tile_elems);
  const uint32_t o = sw64_offset(0, 2 * p);  // the swizzle is its own inverse
  const int kb = (int)(tix % nkb);
  const int64_t ch = tix / nkb;
  I = (int)(ch % n_halves) * n_half + (int)(o / 64);
  J = kb * 32 + (int)(o % 64) / 2;
  c = (int)(ch / n_halves);
}
__global__ void k_split_mats(const double* __restrict__ mats, int n_cells, int n_e, int n_half,
                             int n_halves, double scale, __half* __restrict__ hi,
                             __half* __restrict__ lo) {
  const int nkb = n_half * n_halves / 32;
  const int64_t n = (int64_t)n_cells * n_half * n_halves * n_half * n_halves;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int c, I, J;
    tile_entry(t, n_half, n_halves, nkb, c, I, J);
    double v = 0.0;
    if (I < n_e && J < n_e) v = scale * mats[((int64_t)c * n_e + I) * n_e + J];
    const __half h = __double2half(v);
    hi[t] = h;
    lo[t] = __double2half(v - (double)__half2float(h));
  }
}

// the fused step's tiles: (cell, half, K-block) tiles over nkb K-blocks; nodes J < n_e from the
// cell matrices, the projector columns (J >= n_e) left zero here and scattered afterwards
// (d, map non-null: the cell matrices are unscaled and D = diag(d) is folded in here,
// d[map I] A_IJ d[map J], as for the operators with constraint rows)
__global__ void k_split_mats_ext(const double* __restrict__ mats, int n_cells, int n_e, int n_half,
                                 int n_halves, int nkb, double scale, const double* __restrict__ d,
                                 const int* __restrict__ map, __half* __restrict__ hi,
                                 __half* __restrict__ lo) {
  const int64_t n = (int64_t)n_cells * n_halves * nkb * n_half * 32;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int c, I, J;
    tile_entry(t, n_half, n_halves, nkb, c, I, J);
    double v = 0.0;
    if (I < n_e && J < n_e) {
      v = scale * mats[((int64_t)c * n_e + I) * n_e + J];
      if (d) v *= d[map[(int64_t)c * n_e + I]] * d[map[(int64_t)c * n_e + J]];
    }
    const __half h = __double2half(v);
    hi[t] = h;
    lo[t] = __double2half(v - (double)__half2float(h));
  }
}

// third term of the three-term split of the cell matrices: lo3 = fp16(v - hi - lo) with
// v = 2^s A_e, hi = fp16(v), lo = fp16(v - hi) (the two-term arrays), in the same tile layout
__global__ void k_split_mats_lo3(const double* __restrict__ mats, int n_cells, int n_e, int n_half,
                                 int n_halves, double scale, __half* __restrict__ lo3) {
  const int nkb = n_half * n_halves / 32;
  const int64_t n = (int64_t)n_cells * n_half * n_halves * n_half * n_halves;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    int c, I, J;
    tile_entry(t, n_half, n_halves, nkb, c, I, J);
    double v = 0.0;
    if (I < n_e && J < n_e) v = scale * mats[((int64_t)c * n_e + I) * n_e + J];
    const double h = (double)__half2float(__double2half(v));
    const double l = (double)__half2float(__double2half(v - h));
    lo3[t] = __double2half(v - h - l);
  }
}

// FP32 -> FP16 hi + lo + lo3, exact: x - hi and (x - hi) - lo are exact in FP32 and the last
// term holds the remaining <= 2 significant bits of the 24
__device__ __forceinline__ void split3_f32(float a, __half& h, __half& l, __half& l3) {
  h = __float2half_rn(a);
  const float r = a - __half2float(h);
  l = __float2half_rn(r);
  l3 = __float2half_rn(r - __half2float(l));
}
// (hi, lo, lo3)[r][j] = split3(x[r][j]) for a [M][B] block (x leading dimension ldx, splits ld B)
__global__ void k_split_rows3(const float* __restrict__ x, int64_t ldx, int64_t M, int B,
                              __half* __restrict__ hi, __half* __restrict__ lo,
                              __half* __restrict__ lo3) {
  const int64_t n = M * (int64_t)(B / 2);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / (B / 2);
    const int j = (int)(t % (B / 2)) * 2;
    const float2 v = *reinterpret_cast<const float2*>(x + r * ldx + j);
    __half h0, l0, m0, h1, l1, m1;
    split3_f32(v.x, h0, l0, m0);
    split3_f32(v.y, h1, l1, m1);
    *reinterpret_cast<__half2*>(hi + r * B + j) = __halves2half2(h0, h1);
    *reinterpret_cast<__half2*>(lo + r * B + j) = __halves2half2(l0, l1);
    *reinterpret_cast<__half2*>(lo3 + r * B + j) = __halves2half2(m0, m1);
  }
}

// (hi, lo)[r][j] = split(x[r][j]) for a [M][B] block (x leading dimension ldx, splits ld B)
__global__ void k_split_rows(const float* __restrict__ x, int64_t ldx, int64_t M, int B,
                             __half* __restrict__ hi, __half* __restrict__ lo) {
  const int64_t n = M * (int64_t)(B / 2);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / (B / 2);
    const int j = (int)(t % (B / 2)) * 2;
    const float2 v = *reinterpret_cast<const float2*>(x + r * ldx + j);
    __half h0, l0, h1, l1;
    split_f32(v.x, h0, l0);
    split_f32(v.y, h1, l1);
    *reinterpret_cast<__half2*>(hi + r * B + j) = __halves2half2(h0, h1);
    *reinterpret_cast<__half2*>(lo + r * B + j) = __halves2half2(l0, l1);
  }
}

// y = a x + b y on a contiguous [M][B] block (b == 0: y = a x, y not read), and
// (hi, lo) = split(x) (the step of the Chebyshev recurrence that reads the vector the next HX
// multiplies)
__global__ void k_axpby_split(const float* __restrict__ x, float* __restrict__ y, int64_t n,
                              float a, float b, __half* __restrict__ hi, __half* __restrict__ lo) {
  const bool read_y = b != 0.f;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n / 4;
       t += (int64_t)gridDim.x * blockDim.x) {
    const float4 xv = reinterpret_cast<const float4*>(x)[t];
    float4 yv = read_y ? reinterpret_cast<float4*>(y)[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    yv.x = a * xv.x + b * yv.x;
    yv.y = a * xv.y + b * yv.y;
    yv.z = a * xv.z + b * yv.z;
    yv.w = a * xv.w + b * yv.w;
    reinterpret_cast<float4*>(y)[t] = yv;
    __half h[4], l[4];
    split_f32(xv.x, h[0], l[0]);
    split_f32(xv.y, h[1], l[1]);
    split_f32(xv.z, h[2], l[2]);
    split_f32(xv.w, h[3], l[3]);
    reinterpret_cast<__half2*>(hi)[2 * t] = __halves2half2(h[0], h[1]);
    reinterpret_cast<__half2*>(hi)[2 * t + 1] = __halves2half2(h[2], h[3]);
    reinterpret_cast<__half2*>(lo)[2 * t] = __halves2half2(l[0], l[1]);
    reinterpret_cast<__half2*>(lo)[2 * t + 1] = __halves2half2(l[2], l[3]);
  }
}

// The recurrence step for a group of blocks (up to 32): y_i = a_i x_i + b_i y_i and
// (hi_i, lo_i) = split(x_i), over the concatenation of the blocks in float4 units; the block of
// an index is found by binary search over the ascending begins.
struct AxpbyItem {
  const float* x;
  float* y;
  __half* hi;
  __half* lo;
  int64_t n4;      // float4 entries
  int64_t begin4;  // first float4 index of this block in the concatenation
  float a, b;
};
struct AxpbyGroupArgs {
  AxpbyItem it[kMaxGroup];
  int n;
  int64_t total4;
};
static_assert(sizeof(AxpbyGroupArgs) <= 4096, "kernel parameters above 4 KB");

__global__ void k_axpby_split_group(const __grid_constant__ AxpbyGroupArgs g) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < g.total4;
       t += (int64_t)gridDim.x * blockDim.x) {
    int lo = 0, hi = g.n - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (t >= g.it[mid].begin4) lo = mid; else hi = mid - 1;
    }
    const AxpbyItem& it = g.it[lo];
    const int64_t u = t - it.begin4;
    const float4 xv = reinterpret_cast<const float4*>(it.x)[u];
    float4 yv = it.b != 0.f ? reinterpret_cast<float4*>(it.y)[u] : make_float4(0.f, 0.f, 0.f, 0.f);
    yv.x = it.a * xv.x + it.b * yv.x;
    yv.y = it.a * xv.y + it.b * yv.y;
    yv.z = it.a * xv.z + it.b * yv.z;
    yv.w = it.a * xv.w + it.b * yv.w;
    reinterpret_cast<float4*>(it.y)[u] = yv;
    __half h[4], l[4];
    split_f32(xv.x, h[0], l[0]);
    split_f32(xv.y, h[1], l[1]);
    split_f32(xv.z, h[2], l[2]);
    split_f32(xv.w, h[3], l[3]);
    reinterpret_cast<__half2*>(it.hi)[2 * u] = __halves2half2(h[0], h[1]);
    reinterpret_cast<__half2*>(it.hi)[2 * u + 1] = __halves2half2(h[2], h[3]);
    reinterpret_cast<__half2*>(it.lo)[2 * u] = __halves2half2(l[0], l[1]);
    reinterpret_cast<__half2*>(it.lo)[2 * u + 1] = __halves2half2(l[2], l[3]);
  }
}

struct TcPlan {
  int npad, n_half, n_halves, buf_stride, tmem_cols, stages, xstages, smem;
};

TcPlan plan_for(int n_e, int ns, bool fused = false) {
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
  // three matrix stages, then as many X stages as fit (at most 8, at least 3); two matrix
  // stages when three leave no room for three X stages
  const int budget = 220 * 1024;
  p.stages = 3;
  p.xstages = 8;
  auto total = [&] { return make_layout(p.n_half, p.stages, p.xstages, ns, fused).total + 1024; };
  while (p.xstages > 3 && total() > budget) --p.xstages;
  if (total() > budget) p.stages = 2;
  p.smem = total();
  return p;
}

}  // namespace

namespace tcx {
void tc_set_wait_tries(uint32_t tries) {
  CHEFSI_CUDA(cudaMemcpyToSymbol(g_wait_tries, &tries, sizeof(tries)));
}
bool tcgen05_device() {
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
  const TcPlan p = plan_for(n_e, 2);
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
  k_split_mats<<<grid_for((int64_t)n, 256), 256, 0, st>>>(op->mats64.ptr, op->n_cells, n_e, p.n_half,
                                                          p.n_halves, std::ldexp(1.0, e), tc.hi.ptr,
                                                          tc.lo.ptr);
  CHEFSI_CHECK_LAUNCH();
  tc.ready = true;
  tc.lo3_ready = false;
}

// the third split term of the cell matrices, for the three-term apply
static void prepare_tensor_mats_lo3(chefsi_operator_s* op, cudaStream_t st) {
  prepare_tensor_mats(op, st);
  auto& tc = op->tc;
  if (tc.lo3_ready) return;
  const size_t n = (size_t)op->n_cells * tc.npad * tc.npad;
  tc.lo3.reset(n);
  const TcPlan p = plan_for(op->n_e, 2);
  k_split_mats_lo3<<<grid_for((int64_t)n, 256), 256, 0, st>>>(
      op->mats64.ptr, op->n_cells, op->n_e, p.n_half, p.n_halves, (double)tc.scale, tc.lo3.ptr);
  CHEFSI_CHECK_LAUNCH();
  tc.lo3_ready = true;
}

bool tc_usable(chefsi_operator_s* op) {
  if (op->is_complex || !op->folded || op->n_e > 512) return false;
  return tcgen05_device();
}

// Launch the persistent tensor-core kernel over a group of applies of operators with the same
// cell type: dst_i += scalar_i A_i src_i for the split rows (xhi, xlo [, xlo3]: [rows][B_i]
// FP16) of each item; ns = number of split terms (2, or 3 with xlo3). pipe (optional)
// overrides the X-ring depth and the copy lookahead of the default plan.
void hx_tc_group_launch(const TcGroupItem* items, int n, int ns, const TcPipeline* pipe,
                        cudaStream_t st) {
  CHEFSI_REQUIRE(n >= 1 && n <= kMaxGroup, "tensor-core HX group: 1.." + std::to_string(kMaxGroup) + " items");
  CHEFSI_REQUIRE(ns == 2 || ns == 3, "tensor-core HX: two or three split terms");
  chefsi_operator_s* op0 = items[0].op;
  const int n_e = op0->n_e;
  TcPlan p = plan_for(n_e, ns);
  TcArgs a{};
  a.n_probs = n;
  a.n_e = n_e;
  a.n_rows = n_e;
  a.nkb = p.npad / kKB;
  a.n_half = p.n_half;
  a.n_halves = p.n_halves;
  a.buf_stride = p.buf_stride;
  a.tmem_cols = p.tmem_cols;
  a.stages = p.stages;
  a.xstages = p.xstages;
  a.lookahead = std::max(1, std::min(p.xstages - 2, 6));
  if (pipe) a.cell_tile = pipe->cell_tile;
  if (pipe && pipe->xstages >= 3 && pipe->xstages <= p.xstages) {
    a.xstages = pipe->xstages;
    p.smem = make_layout(p.n_half, p.stages, a.xstages, ns).total + 1024;
    a.lookahead = std::max(1, std::min(pipe->lookahead, a.xstages - 2));
  }
  if (!op0->tc_err.ptr) {
    op0->tc_err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(op0->tc_err.ptr, 0, sizeof(int), st));
  }
  a.err = op0->tc_err.ptr;
  int64_t pairs = 0;
  for (int i = 0; i < n; ++i) {
    const TcGroupItem& it = items[i];
    chefsi_operator_s* op = it.op;
    CHEFSI_REQUIRE(op->n_e == n_e && tc_usable(op), "tensor-core HX group: operators of one cell type");
    CHEFSI_REQUIRE(op->n_dofs < (1ll << 31), "tensor-core HX: too many dofs for 32-bit map entries");
    const __half* x3 = ns == 3 ? it.xlo3 : it.xlo;
    CHEFSI_REQUIRE((reinterpret_cast<uintptr_t>(it.xhi) & 15) == 0 &&
                       (reinterpret_cast<uintptr_t>(it.xlo) & 15) == 0 &&
                       (reinterpret_cast<uintptr_t>(x3) & 15) == 0 && it.B % 8 == 0 &&
                       it.ldd % 4 == 0 && (reinterpret_cast<uintptr_t>(it.dst) & 15) == 0,
                   "tensor-core HX: split rows and output rows must be 16-byte aligned");
    if (ns == 3)
      prepare_tensor_mats_lo3(op, st);
    else
      prepare_tensor_mats(op, st);
    TcProblem& pr = a.prob[i];
    pr.xhi = it.xhi;
    pr.xlo = it.xlo;
    pr.xlo3 = x3;
    pr.dst = it.dst;
    pr.map = op->map.ptr;
    pr.ahi = op->tc.hi.ptr;
    pr.alo = op->tc.lo.ptr;
    pr.alo3 = ns == 3 ? op->tc.lo3.ptr : op->tc.lo.ptr;
    pr.ldx = it.B;
    pr.ldd = it.ldd;
    pr.B = it.B;
    pr.n_chunks = (it.B + kVec - 1) / kVec;
    pr.out_scale = (float)(it.scalar / op->tc.scale);
    pr.pair_begin = pairs;
    pairs += (int64_t)op->n_cells * pr.n_chunks;
  }
  a.n_pairs = pairs;
  auto kernel = ns == 3 ? cell_hx_tc_kernel<3, true> : cell_hx_tc_kernel<2, false>;
  CHEFSI_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
  const int64_t grid = std::min<int64_t>(device_sms(), pairs);
  kernel<<<(unsigned)grid, kThreads3, p.smem, st>>>(a);
  CHEFSI_CHECK_LAUNCH();
}

void tc_row_split(int n_e, int* n_half, int* n_halves) {
  const TcPlan p = plan_for(n_e, 2, true);
  *n_half = p.n_half;
  *n_halves = p.n_halves;
}

void split_mats_ext(chefsi_operator_s* op, int nkb, double scale, __half* hi, __half* lo,
                    cudaStream_t st) {
  const TcPlan p = plan_for(op->n_e, 2, true);
  const int64_t n = (int64_t)op->n_cells * p.n_halves * nkb * p.n_half * 32;
  const bool fold = !op->folded;   // constraint rows: fold M^{-1/2} into this copy
  k_split_mats_ext<<<grid_for(n, 256), 256, 0, st>>>(
      op->mats64.ptr, op->n_cells, op->n_e, p.n_half, p.n_halves, nkb, scale,
      fold ? op->inv_sqrt_mass.ptr : nullptr, fold ? op->map.ptr : nullptr, hi, lo);
  CHEFSI_CHECK_LAUNCH();
}

// dst += scalar (A + C V C^T) x for one operator: the split rows xhi / xlo [plan rows][B] hold x
// in rows [0, n_dofs) and 2^t C^T x in the projector rows after them; the nonlocal apply runs
// on the tensor cores as the plan's extra K columns of the cell matrices
void hx_tc_folded_launch(chefsi_operator_s* op, const __half* xhi, const __half* xlo, float* dst,
                         int64_t ldd, int B, double scalar, cudaStream_t st, double shift) {
  const FusedPlan& fp = op->fz;
  CHEFSI_REQUIRE(fp.ready && fp.tiles_ready, "folded nonlocal HX: tables not prepared");
  CHEFSI_REQUIRE(set_tile_shift(op, shift, st), "folded nonlocal HX: shift out of the tiles' range");
  const int n_e = op->n_e;
  const TcPlan p = plan_for(n_e, 2);
  CHEFSI_REQUIRE(B % 8 == 0 && ldd % 4 == 0 && (reinterpret_cast<uintptr_t>(xhi) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(xlo) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(dst) & 15) == 0,
                 "folded nonlocal HX: 16-byte aligned rows, B a multiple of 8");
  TcArgs a{};
  a.n_probs = 1;
  a.n_e = n_e;
  a.n_rows = n_e;
  a.nkb = fp.nkb;
  a.n_half = p.n_half;
  a.n_halves = p.n_halves;
  a.buf_stride = p.buf_stride;
  a.tmem_cols = p.tmem_cols;
  a.stages = p.stages;
  a.xstages = p.xstages;
  a.lookahead = std::max(1, std::min(p.xstages - 2, 6));
  if (!op->tc_err.ptr) {
    op->tc_err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(op->tc_err.ptr, 0, sizeof(int), st));
  }
  a.err = op->tc_err.ptr;
  TcProblem& pr = a.prob[0];
  pr.xhi = xhi;
  pr.xlo = xlo;
  pr.xlo3 = xlo;
  pr.dst = dst;
  pr.map = op->map.ptr;
  pr.ahi = fp.hi.ptr;
  pr.alo = fp.lo.ptr;
  pr.alo3 = fp.lo.ptr;
  pr.ldx = B;
  pr.ldd = ldd;
  pr.B = B;
  pr.n_chunks = (B + kVec - 1) / kVec;
  pr.out_scale = (float)(scalar / fp.scale);
  pr.pair_begin = 0;
  a.n_pairs = (int64_t)op->n_cells * pr.n_chunks;
  a.fz.mapk = fp.mapk.ptr;
  a.fz.kstride = fp.kstride;
  auto kernel = cell_hx_tc_kernel<2, false>;
  CHEFSI_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
  const int64_t grid = std::min<int64_t>(device_sms(), a.n_pairs);
  kernel<<<(unsigned)grid, kThreads3, p.smem, st>>>(a);
  CHEFSI_CHECK_LAUNCH();
}

// dst += scalar (A - shift I + C V C^T) (xf x) with x given as FP32 rows x32 [plan rows][B]
// (rows [0, n_dofs) the vectors, the projector rows after them C^T x unscaled): the producer
// warps split xf x (and 2^t xf C^T x) into FP16 hi + lo themselves
void hx_tc_folded_f32_launch(chefsi_operator_s* op, const float* x32, float* dst, int64_t ldd,
                             int B, double scalar, double xf, cudaStream_t st, double shift) {
  const FusedPlan& fp = op->fz;
  CHEFSI_REQUIRE(fp.ready && fp.tiles_ready, "folded nonlocal HX: tables not prepared");
  CHEFSI_REQUIRE(set_tile_shift(op, shift, st), "folded nonlocal HX: shift out of the tiles' range");
  const int n_e = op->n_e;
  TcPlan p = plan_for(n_e, 2);
  CHEFSI_REQUIRE(B % 8 == 0 && ldd % 4 == 0 && (reinterpret_cast<uintptr_t>(x32) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(dst) & 15) == 0,
                 "folded nonlocal HX: 16-byte aligned rows, B a multiple of 8");
  // X ring of split tiles (at least 3 stages) and the FP32 staging ring (at most 8 slots: its
  // depth - 1 K-blocks of copies in flight per producer thread)
  int xs = 4, ss = 7;
  auto total = [&] { return make_layout(p.n_half, p.stages, xs, 2, false, ss).total + 1024; };
  while (ss > 4 && total() > 220 * 1024) --ss;
  while (xs > 3 && total() > 220 * 1024) --xs;
  while (ss > 3 && total() > 220 * 1024) --ss;
  CHEFSI_REQUIRE(total() <= 227 * 1024, "folded nonlocal HX: shared memory");
  TcArgs a{};
  a.n_probs = 1;
  a.n_e = n_e;
  a.n_rows = n_e;
  a.nkb = fp.nkb;
  a.n_half = p.n_half;
  a.n_halves = p.n_halves;
  a.buf_stride = p.buf_stride;
  a.tmem_cols = p.tmem_cols;
  a.stages = p.stages;
  a.xstages = xs;
  a.sstages = ss;
  a.lookahead = ss - 1;
  a.x32 = x32;
  a.xf = (float)xf;
  a.wf = (float)(xf * fp.wscale);
  a.w_row = op->n_dofs;
  if (!op->tc_err.ptr) {
    op->tc_err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(op->tc_err.ptr, 0, sizeof(int), st));
  }
  a.err = op->tc_err.ptr;
  TcProblem& pr = a.prob[0];
  pr.dst = dst;
  pr.map = op->map.ptr;
  pr.ahi = fp.hi.ptr;
  pr.alo = fp.lo.ptr;
  pr.alo3 = fp.lo.ptr;
  pr.ldx = B;
  pr.ldd = ldd;
  pr.B = B;
  pr.n_chunks = (B + kVec - 1) / kVec;
  pr.out_scale = (float)(scalar / fp.scale);
  pr.pair_begin = 0;
  a.n_pairs = (int64_t)op->n_cells * pr.n_chunks;
  a.fz.mapk = fp.mapk.ptr;
  a.fz.kstride = fp.kstride;
  auto kernel = cell_hx_tc_kernel<2, false, false, false, true>;
  CHEFSI_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
  const int64_t grid = std::min<int64_t>(device_sms(), a.n_pairs);
  kernel<<<(unsigned)grid, kThreads3, total(), st>>>(a);
  CHEFSI_CHECK_LAUNCH();
}

void hx_tc_fused_launch(const TcFusedLaunch& f, cudaStream_t st) {
  chefsi_operator_s* op = f.op;
  const FusedPlan& fp = op->fz;
  CHEFSI_REQUIRE(fp.ready && fp.tiles_ready, "fused filter step: tables not prepared");
  CHEFSI_REQUIRE(set_tile_shift(op, 0.0, st), "fused filter step: tiles not restored");
  const int n_e = op->n_e;
  const TcPlan p = plan_for(n_e, 2, true);
  CHEFSI_REQUIRE(f.B % 8 == 0 && (reinterpret_cast<uintptr_t>(f.xhi) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(f.xlo) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(f.ohi) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(f.olo) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(f.acc) & 15) == 0,
                 "fused filter step: 16-byte aligned rows, B a multiple of 8");
  TcArgs a{};
  a.n_probs = 1;
  a.n_e = n_e;
  a.n_rows = n_e;
  a.nkb = fp.nkb;
  a.n_half = p.n_half;
  a.n_halves = p.n_halves;
  a.buf_stride = p.buf_stride;
  a.tmem_cols = p.tmem_cols;
  a.stages = p.stages;
  a.xstages = p.xstages;
  a.lookahead = std::max(1, std::min(p.xstages - 2, 6));
  if (!op->tc_err.ptr) {
    op->tc_err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(op->tc_err.ptr, 0, sizeof(int), st));
  }
  a.err = op->tc_err.ptr;
  TcProblem& pr = a.prob[0];
  pr.xhi = f.xhi;
  pr.xlo = f.xlo;
  pr.xlo3 = f.xlo;
  pr.dst = nullptr;
  pr.map = op->map.ptr;
  pr.ahi = fp.hi.ptr;
  pr.alo = fp.lo.ptr;
  pr.alo3 = fp.lo.ptr;
  pr.ldx = f.B;
  pr.ldd = f.B;
  pr.B = f.B;
  pr.n_chunks = (f.B + kVec - 1) / kVec;
  pr.out_scale = (float)(f.a / fp.scale);
  pr.pair_begin = 0;
  a.n_pairs = (int64_t)op->n_cells * pr.n_chunks;
  TcFused& z = a.fz;
  z.mapk = fp.mapk.ptr;
  z.kstride = fp.kstride;
  z.has_next = f.has_next;
  z.rowinfo = reinterpret_cast<const int2*>(fp.rowinfo.ptr);
  z.ohi = f.ohi;
  z.olo = f.olo;
  z.acc = f.acc;
  z.counter = f.counter;
  z.ncontrib = fp.ncontrib.ptr;
  z.cj = (float)f.c;
  z.bj = (float)f.b;
  z.cn = (float)f.cn;
  z.bn = (float)f.bn;
  auto kernel = cell_hx_tc_kernel<2, false, false, true>;
  CHEFSI_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
  const int64_t grid = std::min<int64_t>(device_sms(), a.n_pairs);
  kernel<<<(unsigned)grid, kThreadsFused, p.smem, st>>>(a);
  CHEFSI_CHECK_LAUNCH();
}

// one apply: a group of one
static void launch_tc(chefsi_operator_s* op, const __half* xhi, const __half* xlo,
                      const __half* xlo3, float* dst, int64_t ldd, int B, double scalar, int ns,
                      cudaStream_t st) {
  TcGroupItem it{op, xhi, xlo, xlo3, dst, ldd, B, scalar};
  hx_tc_group_launch(&it, 1, ns, nullptr, st);
}

bool tc_split_usable(chefsi_operator_s* op, int B) { return tc_usable(op) && B % 8 == 0; }

void split_rows_f32(const float* x, int64_t ldx, int64_t M, int B, __half* hi, __half* lo,
                    cudaStream_t st) {
  CHEFSI_REQUIRE(B % 2 == 0 && ldx % 2 == 0, "split rows: even widths only");
  k_split_rows<<<grid_for(M * (B / 2), 256), 256, 0, st>>>(x, ldx, M, B, hi, lo);
  CHEFSI_CHECK_LAUNCH();
}

void axpby_split_group(const AxpbyGroupItem* items, int n, cudaStream_t st) {
  CHEFSI_REQUIRE(n >= 1 && n <= kMaxGroup, "grouped recurrence step: 1..32 blocks");
  AxpbyGroupArgs g{};
  g.n = n;
  int64_t total = 0;
  for (int i = 0; i < n; ++i) {
    const AxpbyGroupItem& it = items[i];
    CHEFSI_REQUIRE(it.n % 4 == 0 && (reinterpret_cast<uintptr_t>(it.x) & 15) == 0 &&
                       (reinterpret_cast<uintptr_t>(it.y) & 15) == 0 &&
                       (reinterpret_cast<uintptr_t>(it.hi) & 7) == 0 &&
                       (reinterpret_cast<uintptr_t>(it.lo) & 7) == 0,
                   "grouped recurrence step: 16-byte aligned blocks with a multiple of 4 entries");
    g.it[i] = AxpbyItem{it.x, it.y, it.hi, it.lo, it.n / 4, total, (float)it.a, (float)it.b};
    total += it.n / 4;
  }
  g.total4 = total;
  if (total == 0) return;
  k_axpby_split_group<<<grid_for(total, 256), 256, 0, st>>>(g);
  CHEFSI_CHECK_LAUNCH();
}

void axpby_split_f32(const float* x, float* y, int64_t M, int B, double a, double b, __half* hi,
                     __half* lo, cudaStream_t st) {
  const int64_t n = M * B;
  CHEFSI_REQUIRE(n % 4 == 0 && (reinterpret_cast<uintptr_t>(x) & 15) == 0 &&
                     (reinterpret_cast<uintptr_t>(y) & 15) == 0,
                 "axpby split: 16-byte aligned blocks with a multiple of 4 entries");
  k_axpby_split<<<grid_for(n / 4, 256), 256, 0, st>>>(x, y, n, (float)a, (float)b, hi, lo);
  CHEFSI_CHECK_LAUNCH();
}

bool hx_tc_split(chefsi_operator_s* op, const __half* xhi, const __half* xlo, const float* src,
                 int64_t lds, float* dst, int64_t ldd, int B, double scalar, bool accumulate,
                 cudaStream_t st) {
  // the scatter adds float4 pieces: output rows 16-byte aligned
  if (!tc_split_usable(op, B) || ldd % 4 != 0 || (reinterpret_cast<uintptr_t>(dst) & 15) != 0)
    return false;
  if (!accumulate) scale_block<float>(dst, ldd, op->n_dofs, B, 0.0, st);
  launch_tc(op, xhi, xlo, nullptr, dst, ldd, B, scalar, 2, st);
  apply_nonlocal_f32(op, src, lds, dst, ldd, B, scalar, st);
  return true;
}

bool hx_tc(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd, int B,
           double scalar, bool accumulate, cudaStream_t st) {
  if (!tc_split_usable(op, B) || lds % 2 != 0 || ldd % 4 != 0 ||
      (reinterpret_cast<uintptr_t>(dst) & 15) != 0)
    return false;
  __half* hi = op->xs_hi.ensure((size_t)op->n_dofs * B);
  __half* lo = op->xs_lo.ensure((size_t)op->n_dofs * B);
  split_rows_f32(src, lds, op->n_dofs, B, hi, lo, st);
  return hx_tc_split(op, hi, lo, src, lds, dst, ldd, B, scalar, accumulate, st);
}

bool hx_tc3(chefsi_operator_s* op, const float* src, int64_t lds, float* dst, int64_t ldd, int B,
            double scalar, bool accumulate, cudaStream_t st) {
  if (!tc_split_usable(op, B) || lds % 2 != 0 || ldd % 4 != 0 ||
      (reinterpret_cast<uintptr_t>(dst) & 15) != 0)
    return false;
  // the K-block-chunked epilogue holds each warp's accumulator columns in registers
  const int ng = plan_for(op->n_e, 3).n_half / 16;
  if ((ng + kEpiWarps / 4 - 1) / (kEpiWarps / 4) * 16 > kChunkCols) return false;
  const size_t n = (size_t)op->n_dofs * B;
  __half* hi = op->xs_hi.ensure(n);
  __half* lo = op->xs_lo.ensure(n);
  __half* lo3 = op->xs_lo3.ensure(n);
  k_split_rows3<<<grid_for(op->n_dofs * (B / 2), 256), 256, 0, st>>>(src, lds, op->n_dofs, B, hi,
                                                                      lo, lo3);
  CHEFSI_CHECK_LAUNCH();
  if (!accumulate) {
    if (ldd == B)
      CHEFSI_CUDA(cudaMemsetAsync(dst, 0, sizeof(float) * n, st));
    else
      scale_block<float>(dst, ldd, op->n_dofs, B, 0.0, st);
  }
  launch_tc(op, hi, lo, lo3, dst, ldd, B, scalar, 3, st);
  apply_nonlocal_f32(op, src, lds, dst, ldd, B, scalar, st);
  return true;
}

// ---------------------------------------------------------------- density on tensor cores
// (hi, lo)[r][j] = split(fp32(x[r][j]) * fp32(d[r] 2^s)): the vectors M^{-1/2} x, scaled into
// the FP16 split's range
__global__ void k_split_rows_dscaled(const double* __restrict__ x, int64_t ldx, int64_t M, int B,
                                     const double* __restrict__ d, double s,
                                     __half* __restrict__ hi, __half* __restrict__ lo) {
  const int64_t n = M * (int64_t)(B / 2);
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / (B / 2);
    const int j = (int)(t % (B / 2)) * 2;
    const float dr = (float)(d[r] * s);
    __half h0, l0, h1, l1;
    split_f32((float)x[r * ldx + j] * dr, h0, l0);
    split_f32((float)x[r * ldx + j + 1] * dr, h1, l1);
    *reinterpret_cast<__half2*>(hi + r * B + j) = __halves2half2(h0, h1);
    *reinterpret_cast<__half2*>(lo + r * B + j) = __halves2half2(l0, l1);
  }
}

// shape-function tiles: part h, K-block kb = rows [h n_half, ...) x nodes [32 kb, ...) of
// 2^s N, zero outside (n_q, n_e), each tile the 64B-swizzled K-major shared-memory image
__global__ void k_split_shape(const double* __restrict__ N, int n_q, int n_e, int n_half,
                              int n_parts, int nkb, double s, __half* __restrict__ hi,
                              __half* __restrict__ lo) {
  const int64_t tile_elems = (int64_t)n_half * 32;
  const int64_t n = (int64_t)n_parts * nkb * tile_elems;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t tix = t / tile_elems;
    const uint32_t o = sw64_offset(0, 2u * (uint32_t)(t - tix * tile_elems));
    const int kb = (int)(tix % nkb), h = (int)(tix / nkb);
    const int I = h * n_half + (int)(o / 64), J = kb * 32 + (int)(o % 64) / 2;
    const double v = (I < n_q && J < n_e) ? s * N[(int64_t)I * n_e + J] : 0.0;
    const __half hh = __double2half(v);
    hi[t] = hh;
    lo[t] = __double2half(v - (double)__half2float(hh));
  }
}

__global__ void k_density_weights(const double* __restrict__ occ, int B, double s,
                                  float* __restrict__ w) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j < B) w[j] = (float)(occ[j] * s);
}

// rho[t] (+)= jxw[t] * r32[t]
__global__ void k_density_finish(const float* __restrict__ r32, const double* __restrict__ jxw,
                                 int64_t n, int accumulate, double* __restrict__ rho) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const double v = (jxw ? jxw[t] : 1.0) * (double)r32[t];
    rho[t] = accumulate ? rho[t] + v : v;
  }
}

bool density_tc(chefsi_operator_s* op, const double* X, int64_t ld, int B, const double* occ,
                int n_q, const double* shape, const double* jxw, double* rho, bool accumulate,
                cudaStream_t st) {
  if (!tc_usable(op) || B % 8 != 0) return false;
  const int n_e = op->n_e;
  const int npad_k = (n_e + 31) / 32 * 32;
  const int nkb = npad_k / kKB;
  const int n_parts = (n_q + 255) / 256;
  const int n_half = ((n_q + n_parts - 1) / n_parts + 15) / 16 * 16;
  const int64_t M = op->n_dofs;
  // scales: max |M^{-1/2} x| <= max|x| max|d| -> 2^8, max |N| -> [2^14, 2^15)
  DeviceBuffer<double> mx(2);
  absmax_block_f64(X, ld, M, B, mx.ptr, st);
  absmax_block_f64(op->inv_sqrt_mass.ptr, 1, M, 1, mx.ptr + 1, st);
  double h[2] = {0.0, 0.0};
  CHEFSI_CUDA(cudaMemcpyAsync(h, mx.ptr, 2 * sizeof(double), cudaMemcpyDeviceToHost, st));
  DeviceBuffer<double> nmax(1);
  absmax_block_f64(shape, n_e, n_q, n_e, nmax.ptr, st);
  double hn = 0.0;
  CHEFSI_CUDA(cudaMemcpyAsync(&hn, nmax.ptr, sizeof(double), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  const double amax = h[0] * h[1];
  const int ex = (amax > 0 && std::isfinite(amax)) ? 8 - (int)std::ceil(std::log2(amax)) : 0;
  const int en = (hn > 0 && std::isfinite(hn)) ? 14 - (int)std::floor(std::log2(hn)) : 0;
  const size_t nx = (size_t)M * B;
  __half* xh = op->xs_hi.ensure(nx);
  __half* xl = op->xs_lo.ensure(nx);
  k_split_rows_dscaled<<<grid_for(M * (B / 2), 256), 256, 0, st>>>(
      X, ld, M, B, op->inv_sqrt_mass.ptr, std::ldexp(1.0, ex), xh, xl);
  CHEFSI_CHECK_LAUNCH();
  const int64_t nt = (int64_t)n_parts * nkb * n_half * 32;
  DeviceBuffer<__half> sh(nt), sl(nt);
  k_split_shape<<<grid_for(nt, 256), 256, 0, st>>>(shape, n_q, n_e, n_half, n_parts, nkb,
                                                    std::ldexp(1.0, en), sh.ptr, sl.ptr);
  CHEFSI_CHECK_LAUNCH();
  DeviceBuffer<float> w(B);
  k_density_weights<<<(B + 255) / 256, 256, 0, st>>>(occ, B, std::ldexp(1.0, -2 * (ex + en)), w.ptr);
  CHEFSI_CHECK_LAUNCH();
  const int64_t nr = (int64_t)op->n_cells * n_q;
  DeviceBuffer<float> r32(nr);
  CHEFSI_CUDA(cudaMemsetAsync(r32.ptr, 0, sizeof(float) * nr, st));
  // the launch: rows = quadrature points in n_parts parts of n_half
  TcArgs a{};
  a.n_probs = 1;
  a.n_e = n_e;
  a.n_rows = n_q;
  a.nkb = nkb;
  a.n_half = n_half;
  a.n_halves = n_parts;
  a.buf_stride = n_half <= 128 ? 128 : 256;
  a.tmem_cols = 2 * a.buf_stride;
  a.stages = 3;
  a.xstages = 8;
  while (a.xstages > 3 && make_layout(n_half, a.stages, a.xstages, 2).total + 1024 > 220 * 1024)
    --a.xstages;
  a.lookahead = std::max(1, std::min(a.xstages - 2, 6));
  const int smem = make_layout(n_half, a.stages, a.xstages, 2).total + 1024;
  if (!op->tc_err.ptr) {
    op->tc_err.reset(1);
    CHEFSI_CUDA(cudaMemsetAsync(op->tc_err.ptr, 0, sizeof(int), st));
  }
  a.err = op->tc_err.ptr;
  TcProblem& pr = a.prob[0];
  pr.xhi = xh;
  pr.xlo = xl;
  pr.xlo3 = xl;
  pr.dst = nullptr;
  pr.map = op->map.ptr;
  pr.ahi = sh.ptr;
  pr.alo = sl.ptr;
  pr.alo3 = sl.ptr;
  pr.ldx = B;
  pr.ldd = B;
  pr.B = B;
  pr.n_chunks = (B + kVec - 1) / kVec;
  pr.out_scale = 1.f;
  pr.a_shared = 1;
  pr.occ = w.ptr;
  pr.rho = r32.ptr;
  pr.pair_begin = 0;
  a.n_pairs = (int64_t)op->n_cells * pr.n_chunks;
  auto kernel = cell_hx_tc_kernel<2, false, true>;
  CHEFSI_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
  const int64_t grid = std::min<int64_t>(device_sms(), a.n_pairs);
  kernel<<<(unsigned)grid, kThreads3, smem, st>>>(a);
  CHEFSI_CHECK_LAUNCH();
  k_density_finish<<<grid_for(nr, 256), 256, 0, st>>>(r32.ptr, jxw, nr, accumulate ? 1 : 0, rho);
  CHEFSI_CHECK_LAUNCH();
  const int tc = tc_check_error(op, st);   // synchronises: the temporaries live until here
  if (tc != CHEFSI_OK) throw Error(tc, "tensor-core density: a bounded device wait expired");
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
