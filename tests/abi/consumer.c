/* A C consumer of include/chefsi.h, compiled as C99 and as C++17 by tests/test_abi.py: the
   header must be usable from both (cgo / ctypes / JNI bindings see the C form, the DFT-FE
   adaptor the C++ form). main() calls only the host-side entry points; the adaptor-shaped
   functions below are compiled and linked but not run (they need a GPU). */
#include <stdio.h>
#include <string.h>

#include "chefsi.h"

/* the calls the DFT-FE adaptor makes per (k-point, spin), in its order */
int adaptor_solve(chefsi_solver s, chefsi_operator h, double* d_X, int N, double* eig,
                  double* res, int is_first_scf, void* stream) {
  int rc = chefsi_solve(s, h, d_X, N, eig, res, 1, is_first_scf, stream);
  if (rc != CHEFSI_OK) return rc;
  double a0, bl, bu;
  int deg;
  return chefsi_solver_get_bounds(s, &a0, &bl, &bu, &deg);
}

int adaptor_spectrum_split(chefsi_solver s, chefsi_operator h, double* d_X, int N, int n_core,
                           double* d_XFrac, double* eig, double* res, void* stream) {
  return chefsi_solve_spectrum_split(s, h, d_X, N, n_core, d_XFrac, eig, res, 1, 0, stream);
}

int adaptor_response(chefsi_operator h_prime, double* d_X, int N, const double* eig, double mu,
                     double T, double* dmu, void* stream) {
  return chefsi_density_matrix_first_order_response(h_prime, d_X, N, N, eig, mu, T, dmu,
                                                    CHEFSI_PREC_FP64, stream);
}

int main(void) {
  chefsi_params p;
  memset(&p, 0, sizeof p);
  p.precision = CHEFSI_PREC_MIXED;
  p.rr_precision = CHEFSI_PREC_FP32_TC;
  const char* v = chefsi_version();
  const int m = chefsi_chebyshev_order(400.0);
  const int rc = chefsi_operator_create(NULL, NULL);
  printf("%s|%d|%d|%d\n", v, m, rc == CHEFSI_ERR_INVALID, (int)sizeof(chefsi_params));
  return (v != NULL && m == 24 && rc == CHEFSI_ERR_INVALID) ? 0 : 1;
}
