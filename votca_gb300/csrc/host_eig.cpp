// Small dense eigensolvers (see host_eig.hpp).
#include "host_eig.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <numeric>

namespace vgb {

namespace {

inline double sgn(double a, double b) { return b >= 0.0 ? std::fabs(a) : -std::fabs(a); }

// Householder reduction of a symmetric matrix to tridiagonal form.
// a: n x n column-major (overwritten).  On return d = diagonal, e[i] = T(i+1, i)
// for i < n-1, and Q (column-major) with A = Q T Q^T.
void tridiagonalize(int64_t n, std::vector<double> &a, std::vector<double> &d,
                    std::vector<double> &e, std::vector<double> &Q) {
  Q.assign(n * n, 0.0);
  for (int64_t i = 0; i < n; ++i) Q[i + n * i] = 1.0;
  std::vector<double> v(n), p(n), w(n);
  auto A = [&](int64_t r, int64_t c) -> double & { return a[r + n * c]; };
  for (int64_t k = 0; k + 2 < n; ++k) {
    // x = A[k+1:, k]
    double scale = 0.0;
    for (int64_t i = k + 1; i < n; ++i) scale += std::fabs(A(i, k));
    if (scale == 0.0) continue;
    double sig = 0.0;
    for (int64_t i = k + 1; i < n; ++i) {
      v[i] = A(i, k) / scale;
      sig += v[i] * v[i];
    }
    const double alpha = -sgn(std::sqrt(sig), v[k + 1]);
    v[k + 1] -= alpha;
    double vn = 0.0;
    for (int64_t i = k + 1; i < n; ++i) vn += v[i] * v[i];
    if (vn == 0.0) continue;
    vn = std::sqrt(vn);
    for (int64_t i = k + 1; i < n; ++i) v[i] /= vn;
    // p = A22 v
    for (int64_t i = k + 1; i < n; ++i) p[i] = 0.0;
    for (int64_t c = k + 1; c < n; ++c) {
      const double vc = v[c];
      for (int64_t r = k + 1; r < n; ++r) p[r] += A(r, c) * vc;
    }
    double vp = 0.0;
    for (int64_t i = k + 1; i < n; ++i) vp += v[i] * p[i];
    for (int64_t i = k + 1; i < n; ++i) w[i] = p[i] - vp * v[i];
    // A22 <- A22 - 2 v w^T - 2 w v^T
    for (int64_t c = k + 1; c < n; ++c) {
      const double vc = 2.0 * v[c], wc = 2.0 * w[c];
      for (int64_t r = k + 1; r < n; ++r) A(r, c) -= v[r] * wc + w[r] * vc;
    }
    A(k + 1, k) = alpha * scale;
    A(k, k + 1) = alpha * scale;
    for (int64_t i = k + 2; i < n; ++i) A(i, k) = A(k, i) = 0.0;
    // Q <- Q H,  H = I - 2 v v^T on rows/cols k+1..n-1
    for (int64_t r = 0; r < n; ++r) {
      double s = 0.0;
      for (int64_t c = k + 1; c < n; ++c) s += Q[r + n * c] * v[c];
      s *= 2.0;
      for (int64_t c = k + 1; c < n; ++c) Q[r + n * c] -= s * v[c];
    }
  }
  d.resize(n);
  e.assign(n, 0.0);
  for (int64_t i = 0; i < n; ++i) d[i] = A(i, i);
  for (int64_t i = 0; i + 1 < n; ++i) e[i] = A(i + 1, i);
}

// Implicit-shift QL on the symmetric tridiagonal (d, e), rotations applied to
// the columns of Z (n x n column-major).
bool tridiagonal_ql(int64_t n, std::vector<double> &d, std::vector<double> &e,
                    std::vector<double> &Z) {
  const double eps = std::numeric_limits<double>::epsilon();
  for (int64_t l = 0; l < n; ++l) {
    int iter = 0;
    while (true) {
      int64_t m = l;
      for (; m + 1 < n; ++m) {
        const double dd = std::fabs(d[m]) + std::fabs(d[m + 1]);
        if (std::fabs(e[m]) <= eps * dd) break;
      }
      if (m == l) break;
      if (++iter > 200) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + sgn(r, g));
      double s = 1.0, c = 1.0, p = 0.0;
      int64_t i = m - 1;
      bool deflated = false;
      for (; i >= l; --i) {
        double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {
          d[i + 1] -= p;
          e[m] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        double *zi = Z.data() + n * i, *zi1 = Z.data() + n * (i + 1);
        for (int64_t k = 0; k < n; ++k) {
          f = zi1[k];
          zi1[k] = s * zi[k] + c * f;
          zi[k] = c * zi[k] - s * f;
        }
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  return true;
}

}  // namespace

bool sym_eig(int64_t n, const double *A, std::vector<double> &evals, std::vector<double> &V) {
  if (n <= 0) { evals.clear(); V.clear(); return true; }
  std::vector<double> a(A, A + n * n);
  // symmetrise against round-off in the projected matrix
  for (int64_t c = 0; c < n; ++c)
    for (int64_t r = c + 1; r < n; ++r) {
      const double m = 0.5 * (a[r + n * c] + a[c + n * r]);
      a[r + n * c] = a[c + n * r] = m;
    }
  std::vector<double> d, e, Q;
  tridiagonalize(n, a, d, e, Q);
  if (!tridiagonal_ql(n, d, e, Q)) return false;
  std::vector<int64_t> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  std::stable_sort(idx.begin(), idx.end(), [&](int64_t x, int64_t y) { return d[x] < d[y]; });
  evals.resize(n);
  V.resize(n * n);
  for (int64_t j = 0; j < n; ++j) {
    evals[j] = d[idx[j]];
    std::copy(Q.begin() + n * idx[j], Q.begin() + n * (idx[j] + 1), V.begin() + n * j);
  }
  return true;
}

bool gen_eig(int64_t, const double *, const double *, std::vector<double> &, std::vector<double> &,
             std::vector<double> &) {
  return false;
}

}  // namespace vgb
