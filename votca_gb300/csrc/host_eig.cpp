// Small dense eigensolvers (see host_eig.hpp).
#include "host_eig.hpp"

#include <algorithm>
#include <cmath>
#include <complex>
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
// the columns of Z (n x n column-major).  This is the published QL algorithm with
// implicit Wilkinson shifts of Bowdler, Martin, Reinsch and Wilkinson ("The QR and QL
// algorithms for symmetric matrices", Numer. Math. 11 (1968) 293-306; EISPACK's tql2):
// deflate where |e_m| <= eps (|d_m| + |d_m+1|), shift by the eigenvalue of the leading
// 2 x 2 block closer to d_l, chase the bulge with plane rotations.
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

namespace {

// LU factorisation with partial pivoting of the n x n column-major matrix a (in place).
bool lu_factor(int64_t n, std::vector<double> &a, std::vector<int64_t> &piv) {
  piv.resize(n);
  double amax = 0.0;
  for (double v : a) amax = std::max(amax, std::fabs(v));
  const double tiny = amax * 1e-300 + 1e-300;
  for (int64_t k = 0; k < n; ++k) {
    int64_t p = k;
    double best = std::fabs(a[k + n * k]);
    for (int64_t i = k + 1; i < n; ++i)
      if (std::fabs(a[i + n * k]) > best) { best = std::fabs(a[i + n * k]); p = i; }
    piv[k] = p;
    if (best <= tiny) return false;
    if (p != k)
      for (int64_t j = 0; j < n; ++j) std::swap(a[k + n * j], a[p + n * j]);
    const double inv = 1.0 / a[k + n * k];
    for (int64_t i = k + 1; i < n; ++i) a[i + n * k] *= inv;
    for (int64_t j = k + 1; j < n; ++j) {
      const double f = a[k + n * j];
      if (f == 0.0) continue;
      for (int64_t i = k + 1; i < n; ++i) a[i + n * j] -= a[i + n * k] * f;
    }
  }
  return true;
}

// Solve (LU) x = b in place for a column-major right-hand side block b (n x m).
void lu_solve(int64_t n, const std::vector<double> &lu, const std::vector<int64_t> &piv,
              double *b, int64_t m) {
  for (int64_t c = 0; c < m; ++c) {
    double *x = b + n * c;
    for (int64_t k = 0; k < n; ++k) std::swap(x[k], x[piv[k]]);
    for (int64_t k = 0; k < n; ++k)
      for (int64_t i = k + 1; i < n; ++i) x[i] -= lu[i + n * k] * x[k];
    for (int64_t k = n - 1; k >= 0; --k) {
      x[k] /= lu[k + n * k];
      for (int64_t i = 0; i < k; ++i) x[i] -= lu[i + n * k] * x[k];
    }
  }
}

// Householder reduction of a general matrix to upper Hessenberg form (in place).
void hessenberg(int64_t n, std::vector<double> &a) {
  auto A = [&](int64_t r, int64_t c) -> double & { return a[r + n * c]; };
  std::vector<double> v(n);
  for (int64_t k = 0; k + 2 < n; ++k) {
    double scale = 0.0;
    for (int64_t i = k + 1; i < n; ++i) scale += std::fabs(A(i, k));
    if (scale == 0.0) continue;
    double sig = 0.0;
    for (int64_t i = k + 1; i < n; ++i) { v[i] = A(i, k) / scale; sig += v[i] * v[i]; }
    const double alpha = -sgn(std::sqrt(sig), v[k + 1]);
    v[k + 1] -= alpha;
    double vn = 0.0;
    for (int64_t i = k + 1; i < n; ++i) vn += v[i] * v[i];
    if (vn == 0.0) continue;
    vn = std::sqrt(vn);
    for (int64_t i = k + 1; i < n; ++i) v[i] /= vn;
    // A <- H A H with H = I - 2 v v^T acting on rows/cols k+1..n-1
    for (int64_t c = 0; c < n; ++c) {
      double s = 0.0;
      for (int64_t i = k + 1; i < n; ++i) s += v[i] * A(i, c);
      s *= 2.0;
      for (int64_t i = k + 1; i < n; ++i) A(i, c) -= s * v[i];
    }
    for (int64_t r = 0; r < n; ++r) {
      double s = 0.0;
      for (int64_t i = k + 1; i < n; ++i) s += A(r, i) * v[i];
      s *= 2.0;
      for (int64_t i = k + 1; i < n; ++i) A(r, i) -= s * v[i];
    }
    for (int64_t i = k + 2; i < n; ++i) A(i, k) = 0.0;
  }
}

// Eigenvalues of an upper Hessenberg matrix by the Francis double-shift QR
// iteration with deflation (the classical real-arithmetic algorithm).
bool hessenberg_qr(int64_t n, std::vector<double> &h, std::vector<double> &wr,
                   std::vector<double> &wi) {
  auto a = [&](int64_t r, int64_t c) -> double & { return h[r + n * c]; };
  wr.assign(n, 0.0);
  wi.assign(n, 0.0);
  double anorm = 0.0;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = std::max<int64_t>(i - 1, 0); j < n; ++j) anorm += std::fabs(a(i, j));
  int64_t nn = n - 1;
  double t = 0.0;
  while (nn >= 0) {
    int its = 0;
    int64_t l;
    do {
      for (l = nn; l >= 1; --l) {
        double s = std::fabs(a(l - 1, l - 1)) + std::fabs(a(l, l));
        if (s == 0.0) s = anorm;
        if (std::fabs(a(l, l - 1)) + s == s) {
          a(l, l - 1) = 0.0;
          break;
        }
      }
      double x = a(nn, nn);
      if (l == nn) {  // one root
        wr[nn] = x + t;
        wi[nn] = 0.0;
        --nn;
      } else {
        double y = a(nn - 1, nn - 1);
        double w = a(nn, nn - 1) * a(nn - 1, nn);
        if (l == nn - 1) {  // two roots
          const double p = 0.5 * (y - x);
          const double q = p * p + w;
          double z = std::sqrt(std::fabs(q));
          x += t;
          if (q >= 0.0) {
            z = p + sgn(z, p);
            wr[nn - 1] = wr[nn] = x + z;
            if (z != 0.0) wr[nn] = x - w / z;
            wi[nn - 1] = wi[nn] = 0.0;
          } else {
            wr[nn - 1] = wr[nn] = x + p;  // pair stored with the positive imaginary part first
            wi[nn - 1] = z;
            wi[nn] = -z;
          }
          nn -= 2;
        } else {  // no roots found yet: one double-shift step
          if (its == 60) return false;
          if (its == 10 || its == 20) {  // exceptional shift
            t += x;
            for (int64_t i = 0; i <= nn; ++i) a(i, i) -= x;
            const double s = std::fabs(a(nn, nn - 1)) + std::fabs(a(nn - 1, nn - 2));
            y = x = 0.75 * s;
            w = -0.4375 * s * s;
          }
          ++its;
          int64_t m;
          double p = 0, q = 0, r = 0, z;
          for (m = nn - 2; m >= l; --m) {
            z = a(m, m);
            r = x - z;
            const double s0 = y - z;
            p = (r * s0 - w) / a(m + 1, m) + a(m, m + 1);
            q = a(m + 1, m + 1) - z - r - s0;
            r = a(m + 2, m + 1);
            const double s = std::fabs(p) + std::fabs(q) + std::fabs(r);
            p /= s;
            q /= s;
            r /= s;
            if (m == l) break;
            const double u = std::fabs(a(m, m - 1)) * (std::fabs(q) + std::fabs(r));
            const double v = std::fabs(p) * (std::fabs(a(m - 1, m - 1)) + std::fabs(z) +
                                             std::fabs(a(m + 1, m + 1)));
            if (u + v == v) break;
          }
          for (int64_t i = m + 2; i <= nn; ++i) {
            a(i, i - 2) = 0.0;
            if (i != m + 2) a(i, i - 3) = 0.0;
          }
          for (int64_t k = m; k <= nn - 1; ++k) {
            if (k != m) {
              p = a(k, k - 1);
              q = a(k + 1, k - 1);
              r = 0.0;
              if (k != nn - 1) r = a(k + 2, k - 1);
              x = std::fabs(p) + std::fabs(q) + std::fabs(r);
              if (x != 0.0) {
                p /= x;
                q /= x;
                r /= x;
              }
            }
            const double s = sgn(std::sqrt(p * p + q * q + r * r), p);
            if (s != 0.0) {
              if (k == m) {
                if (l != m) a(k, k - 1) = -a(k, k - 1);
              } else {
                a(k, k - 1) = -s * x;
              }
              p += s;
              x = p / s;
              y = q / s;
              z = r / s;
              q /= p;
              r /= p;
              for (int64_t j = k; j <= nn; ++j) {
                p = a(k, j) + q * a(k + 1, j);
                if (k != nn - 1) {
                  p += r * a(k + 2, j);
                  a(k + 2, j) -= p * z;
                }
                a(k + 1, j) -= p * y;
                a(k, j) -= p * x;
              }
              const int64_t mmin = nn < k + 3 ? nn : k + 3;
              for (int64_t i = l; i <= mmin; ++i) {
                p = x * a(i, k) + y * a(i, k + 1);
                if (k != nn - 1) {
                  p += z * a(i, k + 2);
                  a(i, k + 2) -= p * r;
                }
                a(i, k + 1) -= p * q;
                a(i, k) -= p;
              }
            }
          }
        }
      }
    } while (l < nn - 1);
  }
  return true;
}

// Eigenvector of the general matrix C for eigenvalue (lr, li) by inverse
// iteration in complex arithmetic; previously found vectors of the same
// cluster are projected out so that a degenerate eigenvalue yields a basis.
void inverse_iteration(int64_t n, const std::vector<double> &C, double lr, double li,
                       const std::vector<std::vector<std::complex<double>>> &cluster,
                       std::vector<std::complex<double>> &x) {
  using cd = std::complex<double>;
  double cn = 0.0;
  for (double v : C) cn = std::max(cn, std::fabs(v));
  const cd lam(lr + 1e-10 * (cn + 1.0), li);
  std::vector<cd> M(n * n);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) M[i + n * j] = cd(C[i + n * j], 0.0) - (i == j ? lam : cd(0.0));
  std::vector<int64_t> piv(n);
  for (int64_t k = 0; k < n; ++k) {
    int64_t p = k;
    double best = std::abs(M[k + n * k]);
    for (int64_t i = k + 1; i < n; ++i)
      if (std::abs(M[i + n * k]) > best) { best = std::abs(M[i + n * k]); p = i; }
    piv[k] = p;
    if (p != k)
      for (int64_t j = 0; j < n; ++j) std::swap(M[k + n * j], M[p + n * j]);
    if (std::abs(M[k + n * k]) == 0.0) M[k + n * k] = cd(1e-300 + 1e-14 * cn, 0.0);
    const cd inv = 1.0 / M[k + n * k];
    for (int64_t i = k + 1; i < n; ++i) M[i + n * k] *= inv;
    for (int64_t j = k + 1; j < n; ++j) {
      const cd f = M[k + n * j];
      if (f == cd(0.0)) continue;
      for (int64_t i = k + 1; i < n; ++i) M[i + n * j] -= M[i + n * k] * f;
    }
  }
  x.assign(n, cd(0.0));
  for (int64_t i = 0; i < n; ++i) x[i] = cd(1.0 + 0.1 * std::sin(1.7 * (double)i + 0.3), 0.0);
  for (int it = 0; it < 3; ++it) {
    for (const auto &y : cluster) {  // x -= y (y^H x)
      cd d(0.0);
      for (int64_t i = 0; i < n; ++i) d += std::conj(y[i]) * x[i];
      for (int64_t i = 0; i < n; ++i) x[i] -= d * y[i];
    }
    for (int64_t k = 0; k < n; ++k) std::swap(x[k], x[piv[k]]);
    for (int64_t k = 0; k < n; ++k)
      for (int64_t i = k + 1; i < n; ++i) x[i] -= M[i + n * k] * x[k];
    for (int64_t k = n - 1; k >= 0; --k) {
      x[k] /= M[k + n * k];
      for (int64_t i = 0; i < k; ++i) x[i] -= M[i + n * k] * x[k];
    }
    double nrm = 0.0;
    for (const auto &v : x) nrm += std::norm(v);
    nrm = std::sqrt(nrm);
    if (!(nrm > 0.0) || !std::isfinite(nrm)) break;
    for (auto &v : x) v /= nrm;
  }
  for (const auto &y : cluster) {
    cd d(0.0);
    for (int64_t i = 0; i < n; ++i) d += std::conj(y[i]) * x[i];
    for (int64_t i = 0; i < n; ++i) x[i] -= d * y[i];
  }
  double nrm = 0.0;
  for (const auto &v : x) nrm += std::norm(v);
  nrm = std::sqrt(nrm);
  if (nrm > 0.0)
    for (auto &v : x) v /= nrm;
  // fix the phase: largest component real and positive
  int64_t im = 0;
  for (int64_t i = 1; i < n; ++i)
    if (std::abs(x[i]) > std::abs(x[im])) im = i;
  if (std::abs(x[im]) > 0.0) {
    const cd ph = std::conj(x[im]) / std::abs(x[im]);
    for (auto &v : x) v *= ph;
  }
}

}  // namespace

bool gen_eig(int64_t n, const double *T, const double *B, std::vector<double> &wr,
             std::vector<double> &wi, std::vector<double> &V) {
  if (n <= 0) { wr.clear(); wi.clear(); V.clear(); return true; }
  // C = B^-1 T
  std::vector<double> lu(B, B + n * n);
  std::vector<int64_t> piv;
  if (!lu_factor(n, lu, piv)) return false;
  std::vector<double> C(T, T + n * n);
  lu_solve(n, lu, piv, C.data(), n);
  for (double v : C)
    if (!std::isfinite(v)) return false;
  std::vector<double> h(C);
  hessenberg(n, h);
  if (!hessenberg_qr(n, h, wr, wi)) return false;
  // eigenvectors: real part (column i) / imaginary part (column i+1) for a pair
  V.assign(n * n, 0.0);
  double cn = 0.0;
  for (double v : C) cn = std::max(cn, std::fabs(v));
  std::vector<std::vector<std::complex<double>>> found;
  std::vector<std::pair<double, double>> found_l;
  for (int64_t i = 0; i < n; ++i) {
    if (wi[i] < 0.0 && i > 0 && wi[i - 1] > 0.0 && wr[i] == wr[i - 1]) continue;  // second of a pair
    std::vector<std::vector<std::complex<double>>> cluster;
    for (size_t f = 0; f < found.size(); ++f)
      if (std::hypot(found_l[f].first - wr[i], found_l[f].second - wi[i]) <= 1e-8 * (cn + 1.0))
        cluster.push_back(found[f]);
    std::vector<std::complex<double>> x;
    inverse_iteration(n, C, wr[i], wi[i], cluster, x);
    found.push_back(x);
    found_l.emplace_back(wr[i], wi[i]);
    for (int64_t r = 0; r < n; ++r) V[r + n * i] = x[r].real();
    if (wi[i] != 0.0 && i + 1 < n)
      for (int64_t r = 0; r < n; ++r) V[r + n * (i + 1)] = x[r].imag();
  }
  return true;
}

}  // namespace vgb
