// chefsi_syevd_noalloc: the projected eigensolver without any device allocation.
//
// Some callers cannot call cudaMalloc while they solve: a host application that hands the
// GPU's memory to its own pool allocator up front (the way DFT-FE pre-sizes its
// MemoryStorage buffers, or a framework whose caching allocator has already reserved the
// HBM) would see such an allocation fail or fragment its pool, and a caller driving other
// streams cannot afford the device-wide synchronisation cudaFree implies. chefsi_syevd
// allocates its workspace on every call; this variant keeps the same workspace in one
// file-scope device array instead, sized for N <= kNoAllocMaxN.
//
// The array's name is a host-side stand-in in host code, so its device address is looked up
// with cudaGetSymbolAddress on the current device, and that address is what the kernels
// receive. The CUDA runtime loads this library's device code lazily: the first look-up on a
// device loads the module and places the array in device memory there (about 3.3 MB, kept
// until the process exits), so a caller whose pool allocator takes the device memory makes
// one warm-up call first. The look-up is repeated on every call (it is a host-side query once
// the module is loaded), so the address stays right after a cudaDeviceReset. Every call shares
// the array and it keeps the previous call's contents; everything that must start at zero is
// cleared on each call. Calls that overlap on the GPU (different streams, or different
// threads on one device) race on the array and must be serialised by the caller.
#include "internal.h"

namespace chefsi {

namespace {

constexpr int kNoAllocMaxN = 256;
constexpr size_t kN2 = (size_t)kNoAllocMaxN * kNoAllocMaxN;
// V [N][N] reflectors, inverse-iteration work [5][N][N], swap flags [N][N] bytes,
// tau / d / e / p [N] each, and one slot for the cluster tolerance
constexpr size_t kOffV = 0;
constexpr size_t kOffWork = kOffV + kN2;
constexpr size_t kOffSwaps = kOffWork + 5 * kN2;
constexpr size_t kOffTau = kOffSwaps + kN2 / sizeof(double);
constexpr size_t kOffD = kOffTau + kNoAllocMaxN;
constexpr size_t kOffE = kOffD + kNoAllocMaxN;
constexpr size_t kOffP = kOffE + kNoAllocMaxN;
constexpr size_t kOffTol = kOffP + kNoAllocMaxN;
constexpr size_t kScratchDoubles = kOffTol + 32;

static __device__ __align__(256) double g_syevd_scratch[kScratchDoubles];

// device address of g_syevd_scratch on the current device (the first look-up on a device
// loads the module there)
double* scratch_on_current_device() {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_syevd_scratch);
  if (e != cudaSuccess || p == nullptr) {
    cudaGetLastError();
    throw Error(CHEFSI_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch) failed: ") +
                                     cudaGetErrorString(e));
  }
  return static_cast<double*>(p);
}

// cluster tolerance 1e-5 * max_j (|d_j| + |e_{j-1}| + |e_j|), computed on the device
__global__ void k_cluster_tol(const double* d, const double* e, int n, double* out) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double tn = 0.0;
  for (int j = 0; j < n; ++j)
    tn = fmax(tn, fabs(d[j]) + (j > 0 ? fabs(e[j - 1]) : 0.0) + (j < n - 1 ? fabs(e[j]) : 0.0));
  *out = 1e-5 * fmax(tn, 1e-300);
}

int syevd_noalloc(double* A, int N, double* w, double* Z, cudaStream_t st) {
  if (N < 1 || N > kNoAllocMaxN)
    throw Error(CHEFSI_ERR_INVALID, "chefsi_syevd_noalloc: N = " + std::to_string(N) +
                                        " outside [1, " + std::to_string(kNoAllocMaxN) + "]");
  double* base = scratch_on_current_device();
  double* V = base + kOffV;
  double* work = base + kOffWork;
  unsigned char* swaps = reinterpret_cast<unsigned char*>(base + kOffSwaps);
  double* tau = base + kOffTau;
  double* d = base + kOffD;
  double* e = base + kOffE;
  double* p = base + kOffP;
  double* tol = base + kOffTol;
  // state left by the previous call: clear what the algorithm expects to start at zero
  CHEFSI_CUDA(cudaMemsetAsync(V, 0, sizeof(double) * (size_t)N * N, st));
  CHEFSI_CUDA(cudaMemsetAsync(tau, 0, sizeof(double) * N, st));
  CHEFSI_CUDA(cudaMemsetAsync(e, 0, sizeof(double) * N, st));
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
  k_tail<<<1, 32, 0, st>>>(A, N, d, e);
  CHEFSI_CHECK_LAUNCH();
  k_bisect_warp<<<(N + 3) / 4, 128, 0, st>>>(d, e, N, 0, N, w);
  CHEFSI_CHECK_LAUNCH();
  k_cluster_tol<<<1, 32, 0, st>>>(d, e, N, tol);
  CHEFSI_CHECK_LAUNCH();
  double ortol = 0.0;
  CHEFSI_CUDA(cudaMemcpyAsync(&ortol, tol, sizeof(double), cudaMemcpyDeviceToHost, st));
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  k_inverse_iteration<<<(N + 63) / 64, 64, 0, st>>>(d, e, N, w, N, 0, Z, N, work, swaps, ortol);
  CHEFSI_CHECK_LAUNCH();
  for (int k = N - 3; k >= 0; --k) {
    k_bt_dot<<<(N + 127) / 128, 128, 0, st>>>(V, N, k, Z, p);
    CHEFSI_CHECK_LAUNCH();
    k_bt_update<<<grid_for((int64_t)(N - k - 1) * N, 256), 256, 0, st>>>(V, N, k, tau, Z, p);
    CHEFSI_CHECK_LAUNCH();
  }
  CHEFSI_CUDA(cudaStreamSynchronize(st));
  return CHEFSI_OK;
}

}  // namespace

}  // namespace chefsi

extern "C" int chefsi_syevd_noalloc(int32_t N, double* A, double* w, double* Z, void* stream) {
  try {
    if (!A || !w || !Z) throw chefsi::Error(CHEFSI_ERR_INVALID, "chefsi_syevd_noalloc: null pointer");
    return chefsi::syevd_noalloc(A, N, w, Z, chefsi::as_stream(stream));
  } catch (const chefsi::Error& e) {
    chefsi::set_last_error(e.what());
    return e.code;
  } catch (const std::exception& e) {
    chefsi::set_last_error(e.what());
    return CHEFSI_ERR_INVALID;
  } catch (...) {
    chefsi::set_last_error("unknown error");
    return CHEFSI_ERR_INVALID;
  }
}
