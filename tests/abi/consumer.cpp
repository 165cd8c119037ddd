// A C++17 consumer of include/chefsi.hpp (the C++ host layer), compiled, linked and run by
// tests/test_abi.py on a machine without a GPU: it checks the host logic only (first-call
// bound, error translation); the adaptor-shaped function is compiled but not run.
#include <cmath>
#include <cstdio>
#include <vector>

#include "chefsi.hpp"

// the calls DFT-FE's kohnShamEigenSpaceCompute makes per (k-point, spin) through the layer
double adaptor(chefsi::ChebyshevOrthogonalizedSubspaceIterationSolver& s,
               chefsi::KohnShamOperator& op, double* d_X, double* d_XFrac, int N, int n_core,
               bool first, bool mixed, void* stream) {
  std::vector<double> eig(N - n_core), res;
  const double b = s.solve(op, d_X, d_XFrac, N, eig, res, first, true, mixed, first, stream);
  s.reinitSpectrumBounds(eig.front(), eig.back(), b);
  return b;
}

int main() {
  int failures = 0;
  const double bl = chefsi::first_call_lower_unwanted(-1.0, 9.0, 96, 64000, false);
  if (std::fabs(bl - 2.0) > 1e-12) ++failures;
  const double blr = chefsi::first_call_lower_unwanted(-1.0, 9.0, 96, 64000, true);
  if (std::fabs(blr + 0.85) > 1e-12) ++failures;
  chefsi_params p{};
  p.precision = CHEFSI_PREC_MIXED;
  chefsi::ChebyshevOrthogonalizedSubspaceIterationSolver s(-1.0, 2.0, 9.0, p);
  s.reinitSpectrumBounds(-2.0, 1.0, 8.0);
  if (s.lowerBoundWantedSpectrum() != -2.0 || s.upperBoundUnWantedSpectrum() != 8.0) ++failures;
  chefsi_operator_desc d{};
  try {
    chefsi::KohnShamOperator op(d);
    ++failures;  // an empty description must be rejected
  } catch (const chefsi::Error& e) {
    if (e.code() != CHEFSI_ERR_INVALID) ++failures;
    std::printf("%s\n", e.what());
  }
  std::printf("failures=%d\n", failures);
  return failures == 0 ? 0 : 1;
}
