// Test-only C entry points to the library's host eigensolvers (votca_gb300/csrc/host_eig.cpp),
// compiled with the host compiler by tests/test_host_eig.py.
#include <cstdint>
#include <vector>

#include "host_eig.hpp"

extern "C" {

int shim_sym_eig(int64_t n, const double *A, double *evals, double *V) {
  std::vector<double> e, v;
  if (!vgb::sym_eig(n, A, e, v)) return 1;
  for (int64_t i = 0; i < n; ++i) evals[i] = e[i];
  for (int64_t i = 0; i < n * n; ++i) V[i] = v[i];
  return 0;
}

int shim_gen_eig(int64_t n, const double *T, const double *B, double *wr, double *wi, double *V) {
  std::vector<double> r, im, v;
  if (!vgb::gen_eig(n, T, B, r, im, v)) return 1;
  for (int64_t i = 0; i < n; ++i) {
    wr[i] = r[i];
    wi[i] = im[i];
  }
  for (int64_t i = 0; i < n * n; ++i) V[i] = v[i];
  return 0;
}
}
