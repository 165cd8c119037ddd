// A C++17 program that drives CheFSI on the GPU through include/chefsi.hpp (the C++ host
// layer shaped like DFT-FE's operator and solver classes), the way DFT-FE's
// kohnShamEigenSpaceCompute (src/dft/kohnShamEigenSolve.cc:296-501) calls the solver per
// (k-point, spin):
//   * the first solve is the first filtering call (Lanczos bounds, the first-call bLow);
//   * later solves get a0 = lowest Ritz value, bLow = highest, b = the returned upper bound;
//   * the last solves ask for fewer eigenvalues than vectors, which takes the spectrum-split
//     branch (XFrac receives the fractional Ritz vectors).
// Built and run by tests/test_gpu_cpp_layer.py. Usage: solve_gpu <dir> <mixed 0|1>; <dir>
// holds meta.txt and the operator's arrays as raw binary files; out.txt receives, per solve,
// "iter a0 bLow b n ev[0..n) res[0..n)".
#include <cuda_runtime.h>

#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "chefsi.hpp"

template <typename T>
static std::vector<T> read_bin(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  if (!f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(n * sizeof(T))))
    throw std::runtime_error("cannot read " + path);
  return v;
}

static void cuda_check(cudaError_t e, const char* what) {
  if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

int main(int argc, char** argv) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <dir> <mixed 0|1>\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const bool mixed = std::string(argv[2]) == "1";
  try {
    long long n_dofs = 0;
    int n_cells = 0, n_e = 0, n_atoms = 0, n_proj = 0, nnz = 0, N = 0, n_full = 0, n_split = 0,
        n_core = 0, degree = 0;
    {
      std::ifstream m(dir + "/meta.txt");
      if (!(m >> n_dofs >> n_cells >> n_e >> n_atoms >> n_proj >> nnz >> N >> n_full >> n_split >>
            n_core >> degree))
        throw std::runtime_error("bad meta.txt");
    }
    const size_t M = static_cast<size_t>(n_dofs);
    auto cell_map = read_bin<int32_t>(dir + "/cell_map.bin", (size_t)n_cells * n_e);
    auto cell_mats = read_bin<double>(dir + "/cell_mats.bin", (size_t)n_cells * n_e * n_e);
    auto sqrt_mass = read_bin<double>(dir + "/sqrt_mass.bin", M);
    auto inv_sqrt_mass = read_bin<double>(dir + "/inv_sqrt_mass.bin", M);
    auto atom_ptr = read_bin<int32_t>(dir + "/atom_ptr.bin", (size_t)n_atoms + 1);
    auto atom_dofs = read_bin<int32_t>(dir + "/atom_dofs.bin", (size_t)nnz);
    auto atom_proj = read_bin<double>(dir + "/atom_proj.bin", (size_t)nnz * n_proj);
    auto couplings = read_bin<double>(dir + "/couplings.bin", (size_t)n_atoms * n_proj);
    auto X0 = read_bin<double>(dir + "/X0.bin", M * N);

    chefsi_operator_desc d{};
    d.n_dofs = n_dofs;
    d.n_cells = n_cells;
    d.nodes_per_cell = n_e;
    d.is_complex = 0;
    d.cell_dof_map = cell_map.data();
    d.cell_matrices = cell_mats.data();
    d.sqrt_mass = sqrt_mass.data();
    d.inv_sqrt_mass = inv_sqrt_mass.data();
    d.n_atoms = n_atoms;
    d.n_proj = n_proj;
    d.atom_dof_ptr = atom_ptr.data();
    d.atom_dofs = atom_dofs.data();
    d.atom_proj = atom_proj.data();
    d.couplings = couplings.data();
    chefsi::KohnShamOperator op(d);

    double* dX = nullptr;
    double* dXF = nullptr;
    cuda_check(cudaMalloc(&dX, sizeof(double) * M * N), "cudaMalloc X");
    cuda_check(cudaMalloc(&dXF, sizeof(double) * M * N), "cudaMalloc XFrac");
    cuda_check(cudaMemcpy(dX, X0.data(), sizeof(double) * M * N, cudaMemcpyHostToDevice), "H2D");

    chefsi_params p{};
    p.chebyshev_degree = degree;
    p.cheby_wfc_block = N;
    p.wfc_block = N;
    p.precision = CHEFSI_PREC_MIXED;
    p.lanczos_steps = 20;
    p.first_scf_degree_scale = 1.0;
    p.keep_hx = 1;
    p.rr_precision = CHEFSI_PREC_FP32_TC;
    chefsi::ChebyshevOrthogonalizedSubspaceIterationSolver solver(0.0, 0.0, 0.0, p);

    std::FILE* out = std::fopen((dir + "/out.txt").c_str(), "w");
    if (!out) throw std::runtime_error("cannot write out.txt");
    double a0_full = 0.0;
    for (int it = 0; it < n_full + n_split; ++it) {
      const bool split = it >= n_full;
      std::vector<double> eig(split ? N - n_core : N), res;
      const double b = solver.solve(op, dX, split ? dXF : nullptr, N, eig, res, it == 0, true,
                                    mixed);
      std::fprintf(out, "%d %.17g %.17g %.17g %zu", it, solver.lowerBoundWantedSpectrum(),
                   solver.lowerBoundUnWantedSpectrum(), b, eig.size());
      for (double v : eig) std::fprintf(out, " %.17g", v);
      for (double v : res) std::fprintf(out, " %.17g", v);
      std::fprintf(out, "\n");
      if (!split) a0_full = eig.front();
      solver.reinitSpectrumBounds(split ? a0_full : eig.front(), eig.back(), b);
    }
    std::fclose(out);
    cudaFree(dX);
    cudaFree(dXF);
  } catch (const chefsi::Error& e) {
    std::fprintf(stderr, "chefsi::Error %d: %s\n", e.code(), e.what());
    return 1;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "error: %s\n", e.what());
    return 1;
  }
  return 0;
}
