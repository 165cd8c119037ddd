/*
 * chefsi.hpp -- C++ host layer over the C ABI (chefsi.h), shaped like DFT-FE's classes so an
 * adaptor inside DFT-FE reads like the code it replaces:
 *
 *   chefsi::KohnShamOperator
 *       operatorDFTDeviceClass (include/operatorDevice.h:43-420): HX (:176-185, scaleFlag and
 *       scalar), XtHX (:230-241), the overlap of fillParallelOverlapMatScalapack;
 *   chefsi::ChebyshevOrthogonalizedSubspaceIterationSolver
 *       chebyshevOrthogonalizedSubspaceIterationSolverDevice
 *       (include/chebyshevOrthogonalizedSubspaceIterationSolverDevice.h:37-166): the constructor
 *       with the three spectrum bounds, solve (first-call Lanczos bounds, the spectrum-split
 *       branch when fewer eigenvalues than vectors are asked for, the upper bound returned),
 *       solveNoRR, densityMatrixEigenBasisFirstOrderResponse, reinitSpectrumBounds.
 *
 * Header-only; every call goes through the C ABI. Failures raise chefsi::Error (the C++ side
 * of the reference raises dealii::ExcMessage through AssertThrow); nothing throws across the C
 * ABI itself. Vectors are device pointers in the Loewdin basis (scaled by M^{1/2}), as the C
 * ABI takes them.
 */
#ifndef CHEFSI_GB300_HPP
#define CHEFSI_GB300_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "chefsi.h"

namespace chefsi {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& what) : std::runtime_error(what), code_(code) {}
  int code() const noexcept { return code_; }

 private:
  int code_;
};

inline void check(int rc, const char* where) {
  if (rc != CHEFSI_OK) {
    const char* msg = chefsi_last_error();
    throw Error(rc, std::string(where) + ": " + (msg ? msg : "unknown error"));
  }
}

/* lowerBoundUnWantedSpectrum of the first filtering call
   (chebyshevOrthogonalizedSubspaceIterationSolverDevice.cc:241-263):
   a0 + (b - a0) N / M (10 with reproducible output, else 200) */
inline double first_call_lower_unwanted(double a0, double b, int n_vectors, int64_t n_dofs,
                                        bool reproducible) {
  return a0 + (b - a0) * n_vectors / static_cast<double>(n_dofs) * (reproducible ? 10.0 : 200.0);
}

class KohnShamOperator {
 public:
  explicit KohnShamOperator(const chefsi_operator_desc& desc) {
    check(chefsi_operator_create(&desc, &h_), "chefsi_operator_create");
    int32_t nc = 0, ne = 0, cplx = 0;
    check(chefsi_operator_info(h_, &n_dofs_, &nc, &ne, &cplx), "chefsi_operator_info");
    is_complex_ = cplx != 0;
  }
  ~KohnShamOperator() {
    if (h_) chefsi_operator_destroy(h_);
  }
  KohnShamOperator(const KohnShamOperator&) = delete;
  KohnShamOperator& operator=(const KohnShamOperator&) = delete;
  KohnShamOperator(KohnShamOperator&& o) noexcept
      : h_(std::exchange(o.h_, nullptr)), n_dofs_(o.n_dofs_), is_complex_(o.is_complex_) {}

  chefsi_operator handle() const { return h_; }
  int64_t n_dofs() const { return n_dofs_; }
  bool is_complex() const { return is_complex_; }

  /* dst = (scaleFlag ? dst : 0) + scalar A src over n_vectors columns (ld = n_vectors) */
  void HX(const void* src, int n_vectors, bool scaleFlag, double scalar, void* dst,
          int precision = CHEFSI_PREC_FP64, void* stream = nullptr) {
    check(chefsi_hx(h_, src, n_vectors, dst, n_vectors, n_vectors, scalar, scaleFlag ? 1 : 0,
                    precision, stream),
          "HX");
  }
  /* Hp = X^H A X (device N x N) */
  void XtHX(const void* X, int N, double* Hp, int precision = CHEFSI_PREC_FP64,
            void* stream = nullptr) {
    check(chefsi_xthx(h_, X, N, N, Hp, precision, stream), "XtHX");
  }
  /* S = X^H X (device N x N) */
  void overlap(const void* X, int N, double* S, int precision = CHEFSI_PREC_FP64,
               void* stream = nullptr) {
    check(chefsi_overlap(h_, X, N, N, S, precision, stream), "overlap");
  }
  void updateCellMatrices(const double* cell_matrices_device, void* stream = nullptr) {
    check(chefsi_operator_update_cell_matrices(h_, cell_matrices_device, stream),
          "updateCellMatrices");
  }

 private:
  chefsi_operator h_ = nullptr;
  int64_t n_dofs_ = 0;
  bool is_complex_ = false;
};

class ChebyshevOrthogonalizedSubspaceIterationSolver {
 public:
  /* params.precision is the mixed mode used when useMixedPrecOverall is set */
  ChebyshevOrthogonalizedSubspaceIterationSolver(double lowerBoundWantedSpectrum,
                                                 double lowerBoundUnWantedSpectrum,
                                                 double upperBoundUnWantedSpectrum,
                                                 const chefsi_params& params,
                                                 bool reuseLanczosUpperBoundFromFirstCall = false)
      : a0_(lowerBoundWantedSpectrum),
        b_low_(lowerBoundUnWantedSpectrum),
        b_up_(upperBoundUnWantedSpectrum),
        params_(params),
        reuse_upper_(reuseLanczosUpperBoundFromFirstCall) {}
  ~ChebyshevOrthogonalizedSubspaceIterationSolver() {
    for (chefsi_solver s : solvers_)
      if (s) chefsi_solver_destroy(s);
  }
  ChebyshevOrthogonalizedSubspaceIterationSolver(
      const ChebyshevOrthogonalizedSubspaceIterationSolver&) = delete;
  ChebyshevOrthogonalizedSubspaceIterationSolver& operator=(
      const ChebyshevOrthogonalizedSubspaceIterationSolver&) = delete;

  void reinitSpectrumBounds(double lowerBoundWantedSpectrum, double lowerBoundUnWantedSpectrum,
                            double upperBoundUnWantedSpectrum) {
    a0_ = lowerBoundWantedSpectrum;
    b_low_ = lowerBoundUnWantedSpectrum;
    b_up_ = upperBoundUnWantedSpectrum;
  }

  /* One CheFSI iteration on X ([n_dofs][N] device). eigenValues.size() == N: the full
     Rayleigh-Ritz step; a smaller size N - Noc: the spectrum-split step, XFrac
     ([n_dofs][N - Noc] device) receiving the fractional Ritz vectors. residualNorms is resized
     to eigenValues.size(). Returns the upper bound of the unwanted spectrum. */
  double solve(KohnShamOperator& op, void* X, void* XFrac, int N,
               std::vector<double>& eigenValues, std::vector<double>& residualNorms,
               bool isFirstFilteringCall, bool computeResidual, bool useMixedPrecOverall = false,
               bool isFirstScf = false, void* stream = nullptr) {
    if (eigenValues.empty() || static_cast<int>(eigenValues.size()) > N)
      throw Error(CHEFSI_ERR_INVALID, "solve: eigenValues must hold 1..N entries");
    if (isFirstFilteringCall || !reuse_upper_) {
      double lo = 0.0, up = 0.0;
      const int k = params_.lanczos_steps > 0 ? params_.lanczos_steps
                                               : (params_.reproducible ? 40 : 20);
      check(chefsi_lanczos_bounds(op.handle(), k, params_.reproducible, nullptr, 0, &lo, &up,
                                  stream),
            "lanczosLowerUpperBoundEigenSpectrum");
      b_up_ = up;
      if (isFirstFilteringCall) {
        a0_ = lo;
        b_low_ = first_call_lower_unwanted(lo, up, N, op.n_dofs(), params_.reproducible != 0);
      }
    }
    chefsi_solver s = solver(useMixedPrecOverall);
    check(chefsi_solver_reinit_spectrum_bounds(s, a0_, b_low_, b_up_), "reinitSpectrumBounds");
    const int n_eig = static_cast<int>(eigenValues.size());
    residualNorms.assign(n_eig, 0.0);
    if (n_eig < N) {
      if (!XFrac) throw Error(CHEFSI_ERR_INVALID, "solve: the spectrum-split step needs XFrac");
      check(chefsi_solve_spectrum_split(s, op.handle(), X, N, N - n_eig, XFrac,
                                        eigenValues.data(), residualNorms.data(),
                                        computeResidual ? 1 : 0, isFirstScf ? 1 : 0, stream),
            "solve (spectrum split)");
    } else {
      check(chefsi_solve(s, op.handle(), X, N, eigenValues.data(), residualNorms.data(),
                         computeResidual ? 1 : 0, isFirstScf ? 1 : 0, stream),
            "solve");
    }
    return b_up_;
  }

  void solveNoRR(KohnShamOperator& op, void* X, int N, int numberPasses,
                 bool useMixedPrecOverall = false, bool isFirstScf = false,
                 void* stream = nullptr) {
    chefsi_solver s = solver(useMixedPrecOverall);
    check(chefsi_solver_reinit_spectrum_bounds(s, a0_, b_low_, b_up_), "reinitSpectrumBounds");
    check(chefsi_solve_no_rr(s, op.handle(), X, N, numberPasses, isFirstScf ? 1 : 0, stream),
          "solveNoRR");
  }

  /* operatorPrime applies the first-order potential only; X becomes X P'. Returns
     densityMatDerFermiEnergy. */
  std::vector<double> densityMatrixEigenBasisFirstOrderResponse(
      KohnShamOperator& operatorPrime, void* X, const std::vector<double>& eigenValues,
      double fermiEnergy, double TVal, bool useMixedPrec = false, void* stream = nullptr) {
    std::vector<double> dmu(eigenValues.size());
    const int N = static_cast<int>(eigenValues.size());
    check(chefsi_density_matrix_first_order_response(
              operatorPrime.handle(), X, N, N, eigenValues.data(), fermiEnergy, TVal, dmu.data(),
              useMixedPrec ? params_.precision : CHEFSI_PREC_FP64, stream),
          "densityMatrixEigenBasisFirstOrderResponse");
    return dmu;
  }

  double lowerBoundWantedSpectrum() const { return a0_; }
  double lowerBoundUnWantedSpectrum() const { return b_low_; }
  double upperBoundUnWantedSpectrum() const { return b_up_; }

 private:
  chefsi_solver solver(bool mixed) {
    chefsi_solver& s = solvers_[mixed ? 1 : 0];
    if (!s) {
      chefsi_params p = params_;
      if (!mixed) p.precision = CHEFSI_PREC_FP64;
      check(chefsi_solver_create(&p, &s), "chefsi_solver_create");
    }
    return s;
  }

  double a0_, b_low_, b_up_;
  chefsi_params params_;
  bool reuse_upper_;
  chefsi_solver solvers_[2] = {nullptr, nullptr};
};

}  // namespace chefsi

#endif  // CHEFSI_GB300_HPP
