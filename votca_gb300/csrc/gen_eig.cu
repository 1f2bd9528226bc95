// The harmonic-Ritz problem of the HAM Davidson on the device (FP64), one CTA per problem.
//
// DavidsonSolver::getHarmonicRitz (xtp/src/libxtp/davidsonsolver.cc:241-332) solves the
// generalized eigenproblem T u = theta B u of the projected matrices T = V^T A V and
// B = V^T A A V (Eigen::GeneralizedEigenSolver there), drops the second member of every complex
// conjugate pair, keeps the eigenvectors' real parts (normalised), takes the needed pairs with
// the largest real parts and returns lambda = diag(U^T T U).  Here, with published textbook
// steps and no library code:
//   1. B = P L U (LU with partial pivoting), C = B^-1 T;
//   2. Householder reduction of C to upper Hessenberg form H = Q^T C Q, reflectors kept;
//   3. eigenvalues of H by the Francis double-shift QR iteration with deflation (the classical
//      real-arithmetic algorithm), one warp: every lane runs the scalar recurrence, the row and
//      column updates of each bulge step are split over the lanes;
//   4. the selection of the reference (complex partners, largest real parts first);
//   5. for the selected eigenvalues only: inverse iteration on the Hessenberg matrix in complex
//      arithmetic (Hessenberg LU with partial pivoting, three steps, vectors of eigenvalues
//      closer than 1e-8 (|C| + 1) projected out of each other), back-transformation x = Q z,
//      phase fixed so that the largest component is real and positive, real part normalised.
#include "small_eig.cuh"

#include <algorithm>
#include <memory>
#include <mutex>

namespace vgb {

namespace {

constexpr int kGenThreads = 256;
constexpr int kGenWarps = kGenThreads / 32;
constexpr int kGenJobs = 256;

struct GenEigGroup {
  GenEigJob j[kGenJobs];
  int n;
  int64_t smem_doubles;
};

__device__ inline double sgn_of(double a, double b) { return b >= 0.0 ? fabs(a) : -fabs(a); }

struct cplx {
  double re, im;
};
__device__ inline cplx cmul(cplx a, cplx b) { return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; }
__device__ inline cplx csub(cplx a, cplx b) { return {a.re - b.re, a.im - b.im}; }
__device__ inline double cabs2(cplx a) { return a.re * a.re + a.im * a.im; }
__device__ inline cplx cdiv(cplx a, cplx b) {
  // Smith's division
  if (fabs(b.re) >= fabs(b.im)) {
    const double r = b.im / b.re, d = b.re + r * b.im;
    return {(a.re + r * a.im) / d, (a.im - r * a.re) / d};
  }
  const double r = b.re / b.im, d = b.im + r * b.re;
  return {(a.re * r + a.im) / d, (a.im * r - a.re) / d};
}

__device__ double gsum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < kGenWarps; ++w) t += red[w];
  return t;
}
__device__ double gmax(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = red[0];
  for (int w = 1; w < kGenWarps; ++w) t = fmax(t, red[w]);
  return t;
}
__device__ double wsum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Francis double-shift QR iteration on the upper Hessenberg a (n x n, leading dimension ld),
// eigenvalues only, by one warp.  Returns false when an eigenvalue needs more than 60 steps.
__device__ bool hqr_warp(double *a_, int64_t ld, int64_t n, double *wr, double *wi) {
  const int lane = threadIdx.x & 31;
  auto A = [&](int64_t r, int64_t c) -> double & { return a_[r + ld * c]; };
  double an = 0.0;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = max((int64_t)0, i - 1) + lane; j < n; j += 32) an += fabs(A(i, j));
  const double anorm = wsum(an);
  int64_t nn = n - 1;
  double t = 0.0;
  while (nn >= 0) {
    int its = 0;
    int64_t l;
    do {
      for (l = nn; l >= 1; --l) {
        double s = fabs(A(l - 1, l - 1)) + fabs(A(l, l));
        if (s == 0.0) s = anorm;
        if (fabs(A(l, l - 1)) + s == s) {
          __syncwarp();
          if (lane == 0) A(l, l - 1) = 0.0;
          __syncwarp();
          break;
        }
      }
      double x = A(nn, nn);
      if (l == nn) {  // one root
        if (lane == 0) { wr[nn] = x + t; wi[nn] = 0.0; }
        --nn;
      } else {
        double y = A(nn - 1, nn - 1);
        double w = A(nn, nn - 1) * A(nn - 1, nn);
        if (l == nn - 1) {  // two roots
          const double p = 0.5 * (y - x);
          const double q = p * p + w;
          double z = sqrt(fabs(q));
          x += t;
          if (lane == 0) {
            if (q >= 0.0) {
              z = p + sgn_of(z, p);
              wr[nn - 1] = wr[nn] = x + z;
              if (z != 0.0) wr[nn] = x - w / z;
              wi[nn - 1] = wi[nn] = 0.0;
            } else {
              wr[nn - 1] = wr[nn] = x + p;  // the pair with the positive imaginary part first
              wi[nn - 1] = z;
              wi[nn] = -z;
            }
          }
          nn -= 2;
        } else {  // one double-shift step
          if (its == 60) return false;
          if (its == 10 || its == 20) {  // exceptional shift
            t += x;
            __syncwarp();
            for (int64_t i = lane; i <= nn; i += 32) A(i, i) -= x;
            __syncwarp();
            const double s = fabs(A(nn, nn - 1)) + fabs(A(nn - 1, nn - 2));
            y = x = 0.75 * s;
            w = -0.4375 * s * s;
          }
          ++its;
          int64_t m;
          double p = 0.0, q = 0.0, r = 0.0, z;
          for (m = nn - 2; m >= l; --m) {
            z = A(m, m);
            r = x - z;
            const double s0 = y - z;
            p = (r * s0 - w) / A(m + 1, m) + A(m, m + 1);
            q = A(m + 1, m + 1) - z - r - s0;
            r = A(m + 2, m + 1);
            const double s = fabs(p) + fabs(q) + fabs(r);
            p /= s;
            q /= s;
            r /= s;
            if (m == l) break;
            const double u = fabs(A(m, m - 1)) * (fabs(q) + fabs(r));
            const double v = fabs(p) * (fabs(A(m - 1, m - 1)) + fabs(z) + fabs(A(m + 1, m + 1)));
            if (u + v == v) break;
          }
          __syncwarp();
          for (int64_t i = m + 2 + lane; i <= nn; i += 32) {
            A(i, i - 2) = 0.0;
            if (i != m + 2) A(i, i - 3) = 0.0;
          }
          __syncwarp();
          for (int64_t k = m; k <= nn - 1; ++k) {
            if (k != m) {
              p = A(k, k - 1);
              q = A(k + 1, k - 1);
              r = 0.0;
              if (k != nn - 1) r = A(k + 2, k - 1);
              x = fabs(p) + fabs(q) + fabs(r);
              if (x != 0.0) {
                p /= x;
                q /= x;
                r /= x;
              }
            }
            const double s = sgn_of(sqrt(p * p + q * q + r * r), p);
            if (s != 0.0) {
              __syncwarp();
              if (lane == 0) {
                if (k == m) {
                  if (l != m) A(k, k - 1) = -A(k, k - 1);
                } else {
                  A(k, k - 1) = -s * x;
                }
              }
              __syncwarp();
              p += s;
              x = p / s;
              y = q / s;
              z = r / s;
              q /= p;
              r /= p;
              for (int64_t j = k + lane; j <= nn; j += 32) {
                double pp = A(k, j) + q * A(k + 1, j);
                if (k != nn - 1) {
                  pp += r * A(k + 2, j);
                  A(k + 2, j) -= pp * z;
                }
                A(k + 1, j) -= pp * y;
                A(k, j) -= pp * x;
              }
              __syncwarp();
              const int64_t mmin = nn < k + 3 ? nn : k + 3;
              for (int64_t i = l + lane; i <= mmin; i += 32) {
                double pp = x * A(i, k) + y * A(i, k + 1);
                if (k != nn - 1) {
                  pp += z * A(i, k + 2);
                  A(i, k + 2) -= pp * r;
                }
                A(i, k + 1) -= pp * q;
                A(i, k) -= pp;
              }
              __syncwarp();
            }
          }
        }
      }
    } while (l < nn - 1);
  }
  return true;
}

// one thread: eigenvector of the Hessenberg H (n x n, ld) for the eigenvalue lam by inverse
// iteration (three steps) in complex arithmetic, with the cluster's earlier vectors projected
// out; z (complex, n) returned normalised.  M: 2 n^2 doubles of scratch, lv / pv: n.
__device__ void hess_inverse_iteration(const double *H, int64_t ld, int64_t n, cplx lam, double cn, cplx *M,
                                       cplx *lv, double *pv, const cplx *const *cluster, int ncl, cplx *z) {
  auto Mm = [&](int64_t r, int64_t c) -> cplx & { return M[r + n * c]; };
  for (int64_t c = 0; c < n; ++c)
    for (int64_t r = 0; r < n; ++r) {
      const double h = (r <= c + 1) ? H[r + ld * c] : 0.0;
      Mm(r, c) = (r == c) ? cplx{h - lam.re, -lam.im} : cplx{h, 0.0};
    }
  const double floor_piv = 1e-300 + 1e-14 * cn;
  for (int64_t k = 0; k + 1 < n; ++k) {
    if (cabs2(Mm(k + 1, k)) > cabs2(Mm(k, k))) {  // row interchange
      for (int64_t c = k; c < n; ++c) {
        const cplx tmp = Mm(k, c);
        Mm(k, c) = Mm(k + 1, c);
        Mm(k + 1, c) = tmp;
      }
      pv[k] = 1.0;
    } else {
      pv[k] = 0.0;
    }
    if (cabs2(Mm(k, k)) == 0.0) Mm(k, k) = cplx{floor_piv, 0.0};
    const cplx li = cdiv(Mm(k + 1, k), Mm(k, k));
    lv[k] = li;
    for (int64_t c = k + 1; c < n; ++c) Mm(k + 1, c) = csub(Mm(k + 1, c), cmul(li, Mm(k, c)));
  }
  if (cabs2(Mm(n - 1, n - 1)) == 0.0) Mm(n - 1, n - 1) = cplx{floor_piv, 0.0};
  for (int64_t i = 0; i < n; ++i) z[i] = cplx{1.0 + 0.1 * sin(1.7 * (double)i + 0.3), 0.0};
  auto project = [&]() {
    for (int q = 0; q < ncl; ++q) {  // z -= y (y^H z)
      const cplx *y = cluster[q];
      cplx d{0.0, 0.0};
      for (int64_t i = 0; i < n; ++i) {
        d.re += y[i].re * z[i].re + y[i].im * z[i].im;
        d.im += y[i].re * z[i].im - y[i].im * z[i].re;
      }
      for (int64_t i = 0; i < n; ++i) z[i] = csub(z[i], cmul(d, y[i]));
    }
  };
  auto normalise = [&]() {
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += cabs2(z[i]);
    s = sqrt(s);
    if (s > 0.0 && isfinite(s))
      for (int64_t i = 0; i < n; ++i) { z[i].re /= s; z[i].im /= s; }
    return s;
  };
  for (int it = 0; it < 3; ++it) {
    project();
    for (int64_t k = 0; k + 1 < n; ++k) {  // the row operations of the factorisation
      if (pv[k] != 0.0) {
        const cplx tmp = z[k];
        z[k] = z[k + 1];
        z[k + 1] = tmp;
      }
      z[k + 1] = csub(z[k + 1], cmul(lv[k], z[k]));
    }
    for (int64_t k = n - 1; k >= 0; --k) {  // upper triangular solve
      cplx s = z[k];
      for (int64_t c = k + 1; c < n; ++c) s = csub(s, cmul(Mm(k, c), z[c]));
      z[k] = cdiv(s, Mm(k, k));
    }
    const double s = normalise();
    if (!(s > 0.0) || !isfinite(s)) break;
  }
  project();
  normalise();
}

__global__ void __launch_bounds__(kGenThreads) gen_eig_kernel(const __grid_constant__ GenEigGroup g) {
  const GenEigJob q = g.j[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t m = q.m, nw = q.nw;
  __shared__ double red[32];
  __shared__ int flag, bestidx, nsel;
  __shared__ double bestval, cnorm;
  if (m < 1 || nw < 1 || nw > m || m > kGenEigMaxM) {
    if (tid == 0 && q.info) { q.info[0] = 1; q.info[1] = 0; }
    return;
  }
  extern __shared__ double sm[];
  double *LU = q.work, *C = LU + m * m, *Vh = C + m * m, *piv = Vh + m * m;
  double *wr = piv + m, *wi = wr + m, *sel = wi + m;  // sel: selected eigenvalue indices
  double *vec = sel + m;                              // per selected vector: 2 m^2 + 5 m
  double *Hq = (m * m <= g.smem_doubles) ? sm : vec + nw * (2 * m * m + 5 * m);
  if (tid == 0) flag = 0;
  // ---- load ----
  for (int64_t t = tid; t < m * m; t += kGenThreads) {
    const int64_t r = t % m, c = t / m;
    LU[t] = q.B[r + q.ldt * c];
    C[t] = q.T[r + q.ldt * c];
  }
  double bm = 0.0;
  for (int64_t t = tid; t < m * m; t += kGenThreads) bm = fmax(bm, fabs(q.B[(t % m) + q.ldt * (t / m)]));
  const double tiny = gmax(bm, red) * 1e-300 + 1e-300;
  // ---- 1. B = P L U ----
  for (int64_t k = 0; k < m; ++k) {
    if (tid == 0) {  // pivot: the first largest |LU(i, k)|, i >= k (as the host LU)
      int64_t p = k;
      double best = fabs(LU[k + m * k]);
      for (int64_t i = k + 1; i < m; ++i)
        if (fabs(LU[i + m * k]) > best) { best = fabs(LU[i + m * k]); p = i; }
      bestidx = (int)p;
      bestval = best;
      piv[k] = (double)p;
      if (best <= tiny) flag = 2;
    }
    __syncthreads();
    if (flag) break;
    const int64_t p = bestidx;
    if (p != k)
      for (int64_t c = tid; c < m; c += kGenThreads) {
        const double t = LU[k + m * c];
        LU[k + m * c] = LU[p + m * c];
        LU[p + m * c] = t;
      }
    __syncthreads();
    const double inv = 1.0 / LU[k + m * k];
    for (int64_t i = k + 1 + tid; i < m; i += kGenThreads) LU[i + m * k] *= inv;
    __syncthreads();
    const int64_t nr = m - k - 1;
    for (int64_t t = tid; t < nr * nr; t += kGenThreads) {
      const int64_t i = k + 1 + t % nr, c = k + 1 + t / nr;
      LU[i + m * c] -= LU[i + m * k] * LU[k + m * c];
    }
    __syncthreads();
  }
  if (flag) {
    if (tid == 0 && q.info) { q.info[0] = 2; q.info[1] = 0; }
    return;
  }
  // ---- C = B^-1 T: one column per thread ----
  for (int64_t c = tid; c < m; c += kGenThreads) {
    double *x = C + m * c;
    for (int64_t k = 0; k < m; ++k) {
      const int64_t p = (int64_t)piv[k];
      const double t = x[k];
      x[k] = x[p];
      x[p] = t;
    }
    for (int64_t k = 0; k < m; ++k) {
      const double xk = x[k];
      for (int64_t i = k + 1; i < m; ++i) x[i] -= LU[i + m * k] * xk;
    }
    for (int64_t k = m - 1; k >= 0; --k) {
      x[k] /= LU[k + m * k];
      const double xk = x[k];
      for (int64_t i = 0; i < k; ++i) x[i] -= LU[i + m * k] * xk;
    }
    for (int64_t i = 0; i < m; ++i)
      if (!isfinite(x[i])) flag = 2;
  }
  __syncthreads();
  if (flag) {
    if (tid == 0 && q.info) { q.info[0] = 2; q.info[1] = 0; }
    return;
  }
  double cm = 0.0;
  for (int64_t t = tid; t < m * m; t += kGenThreads) cm = fmax(cm, fabs(C[t]));
  cm = gmax(cm, red);
  if (tid == 0) cnorm = cm;
  // ---- 2. Hessenberg reduction, reflectors kept in Vh (column k: rows k+1..m-1) ----
  for (int64_t t = tid; t < m * m; t += kGenThreads) Vh[t] = 0.0;
  __syncthreads();
  for (int64_t k = 0; k + 2 < m; ++k) {
    double sp = 0.0;
    for (int64_t i = k + 1 + tid; i < m; i += kGenThreads) sp += fabs(C[i + m * k]);
    const double scale = gsum(sp, red);
    if (scale == 0.0) continue;
    double sg = 0.0;
    for (int64_t i = k + 1 + tid; i < m; i += kGenThreads) {
      const double v = C[i + m * k] / scale;
      Vh[i + m * k] = v;
      sg += v * v;
    }
    const double sig = gsum(sg, red);
    const double alpha = -sgn_of(sqrt(sig), Vh[(k + 1) + m * k]);
    __syncthreads();
    if (tid == 0) Vh[(k + 1) + m * k] -= alpha;
    __syncthreads();
    double sv = 0.0;
    for (int64_t i = k + 1 + tid; i < m; i += kGenThreads) sv += Vh[i + m * k] * Vh[i + m * k];
    double vn = gsum(sv, red);
    if (vn == 0.0) {
      for (int64_t i = k + 1 + tid; i < m; i += kGenThreads) Vh[i + m * k] = 0.0;
      __syncthreads();
      continue;
    }
    vn = sqrt(vn);
    for (int64_t i = k + 1 + tid; i < m; i += kGenThreads) Vh[i + m * k] /= vn;
    __syncthreads();
    const double *v = Vh + m * k;
    for (int64_t c = tid; c < m; c += kGenThreads) {  // C <- H C (columns)
      double s = 0.0;
      for (int64_t i = k + 1; i < m; ++i) s += v[i] * C[i + m * c];
      s *= 2.0;
      for (int64_t i = k + 1; i < m; ++i) C[i + m * c] -= s * v[i];
    }
    __syncthreads();
    for (int64_t r = tid; r < m; r += kGenThreads) {  // C <- C H (rows)
      double s = 0.0;
      for (int64_t i = k + 1; i < m; ++i) s += C[r + m * i] * v[i];
      s *= 2.0;
      for (int64_t i = k + 1; i < m; ++i) C[r + m * i] -= s * v[i];
    }
    __syncthreads();
    for (int64_t i = k + 2 + tid; i < m; i += kGenThreads) C[i + m * k] = 0.0;
    __syncthreads();
  }
  // ---- 3. eigenvalues: QR iteration on a copy of H, by warp 0 ----
  for (int64_t t = tid; t < m * m; t += kGenThreads) Hq[t] = C[t];
  __syncthreads();
  if (warp == 0) {
    const bool ok = hqr_warp(Hq, m, m, wr, wi);
    if (!ok && lane == 0) flag = 3;
  }
  __syncthreads();
  if (flag) {
    if (tid == 0 && q.info) { q.info[0] = 3; q.info[1] = 0; }
    return;
  }
  // ---- 4. the reference's selection (davidsonsolver.cc:261-320), thread 0 ----
  if (tid == 0) {
    // complex partners: the second member of each pair is dropped
    int *pf = reinterpret_cast<int *>(Hq);  // first, second, per open pair (Hq is free now)
    int np = 0;
    for (int64_t i = 0; i < m; ++i) {
      if (wi[i] == 0.0) continue;
      bool found = false;
      for (int p = 0; p < np; ++p) {
        if (pf[2 * p + 1] > -1) continue;
        const int64_t f = pf[2 * p];
        if (fabs(wr[f] - wr[i]) < 1e-9 && fabs(wi[f] + wi[i]) < 1e-9) {
          pf[2 * p + 1] = (int)i;
          found = true;
        }
      }
      if (!found) { pf[2 * np] = (int)i; pf[2 * np + 1] = -1; ++np; }
    }
    for (int p = 0; p < np; ++p)
      if (pf[2 * p + 1] < 0) { flag = 4; q.info[1] = pf[2 * p]; }
    if (!flag) {
      // candidates in index order; stable ascending sort by real part, then reversed
      int *cand = pf + 2 * np;
      int nc = 0;
      for (int64_t i = 0; i < m; ++i) {
        bool second = false;
        for (int p = 0; p < np; ++p) second = second || pf[2 * p + 1] == (int)i;
        if (!second) cand[nc++] = (int)i;
      }
      for (int a = 1; a < nc; ++a) {  // insertion sort: stable
        const int x = cand[a];
        int b = a - 1;
        while (b >= 0 && wr[cand[b]] > wr[x]) { cand[b + 1] = cand[b]; --b; }
        cand[b + 1] = x;
      }
      const int ns = (int)min((int64_t)nc, nw);
      for (int c = 0; c < ns; ++c) sel[c] = (double)cand[nc - 1 - c];
      nsel = ns;
    }
  }
  __syncthreads();
  if (flag) {
    if (tid == 0 && q.info) q.info[0] = 4;
    return;
  }
  // ---- 5. eigenvectors of the selected eigenvalues, one thread per cluster ----
  const double cn = cnorm;
  const int ns = nsel;
  // clusters: runs of the selection (ordered by real part) whose neighbours are closer than
  // 1e-8 (|C| + 1); each run is handled by one thread, its vectors one after another
  auto close_to_prev = [&](int c) {
    if (c == 0) return false;
    const int64_t a = (int64_t)sel[c], b = (int64_t)sel[c - 1];
    return hypot(wr[a] - wr[b], wi[a] - wi[b]) <= 1e-8 * (cn + 1.0);
  };
  for (int c0 = tid; c0 < ns; c0 += kGenThreads) {
    if (close_to_prev(c0)) continue;  // not the first of its run
    const cplx *members[64];
    int nmem = 0;
    for (int c = c0; c < ns && (c == c0 || close_to_prev(c)); ++c) {
      const int64_t ic = (int64_t)sel[c];
      double *w = vec + (int64_t)c * (2 * m * m + 5 * m);
      cplx *M = reinterpret_cast<cplx *>(w);
      cplx *lv = reinterpret_cast<cplx *>(w + 2 * m * m);
      double *pv = w + 2 * m * m + 2 * m;
      cplx *z = reinterpret_cast<cplx *>(w + 2 * m * m + 3 * m);  // 2 m doubles
      hess_inverse_iteration(C, m, m, cplx{wr[ic] + 1e-10 * (cn + 1.0), wi[ic]}, cn, M, lv, pv, members,
                             nmem < 64 ? nmem : 64, z);
      if (nmem < 64) members[nmem++] = z;
      // x = Q z (reflectors in reverse order): stored over M, which is free now
      cplx *x = M;
      for (int64_t i = 0; i < m; ++i) x[i] = z[i];
      for (int64_t k = m - 3; k >= 0; --k) {
        const double *v = Vh + m * k;
        cplx d{0.0, 0.0};
        for (int64_t i = k + 1; i < m; ++i) { d.re += v[i] * x[i].re; d.im += v[i] * x[i].im; }
        for (int64_t i = k + 1; i < m; ++i) { x[i].re -= 2.0 * d.re * v[i]; x[i].im -= 2.0 * d.im * v[i]; }
      }
      // normalise, phase: the largest component real and positive; keep the real part
      double nx = 0.0;
      int64_t im = 0;
      for (int64_t i = 0; i < m; ++i) {
        nx += cabs2(x[i]);
        if (cabs2(x[i]) > cabs2(x[im])) im = i;
      }
      nx = sqrt(nx);
      const double ax = sqrt(cabs2(x[im]));
      const cplx ph = ax > 0.0 ? cplx{x[im].re / ax, -x[im].im / ax} : cplx{1.0, 0.0};
      double *u = q.U + q.ldu * c;
      double nu = 0.0;
      for (int64_t i = 0; i < m; ++i) {
        const double re = (nx > 0.0) ? (x[i].re * ph.re - x[i].im * ph.im) / nx : 0.0;
        u[i] = re;
        nu += re * re;
      }
      nu = sqrt(nu);
      if (nu > 0.0)
        for (int64_t i = 0; i < m; ++i) u[i] /= nu;
      // lambda = u^T T u
      double lam = 0.0;
      for (int64_t a = 0; a < m; ++a) {
        double tu = 0.0;
        for (int64_t b = 0; b < m; ++b) tu += q.T[a + q.ldt * b] * u[b];
        lam += u[a] * tu;
      }
      q.lam[c] = lam;
    }
  }
  __syncthreads();
  for (int64_t c = ns + warp; c < nw; c += kGenWarps)  // fewer candidates than wanted: zero columns
    for (int64_t i = lane; i < m; i += 32) {
      q.U[i + q.ldu * c] = 0.0;
      if (i == 0) q.lam[c] = 0.0;
    }
  if (tid == 0 && q.info) { q.info[0] = 0; q.info[1] = ns; }
}

// O = an orthonormal basis of the columns of U (m x r): modified Gram-Schmidt twice, one CTA.
__global__ void __launch_bounds__(kGenThreads) orthonormalise_kernel(const double *U, int64_t ldu, int64_t m,
                                                                    int64_t r, double *O, int64_t ldo) {
  __shared__ double red[32];
  for (int64_t t = threadIdx.x; t < m * r; t += kGenThreads) O[(t % m) + ldo * (t / m)] = U[(t % m) + ldu * (t / m)];
  __syncthreads();
  for (int pass = 0; pass < 2; ++pass)
    for (int64_t j = 0; j < r; ++j) {
      double *oj = O + ldo * j;
      for (int64_t i = 0; i < j; ++i) {
        const double *oi = O + ldo * i;
        double s = 0.0;
        for (int64_t t = threadIdx.x; t < m; t += kGenThreads) s += oi[t] * oj[t];
        const double h = gsum(s, red);
        for (int64_t t = threadIdx.x; t < m; t += kGenThreads) oj[t] -= h * oi[t];
        __syncthreads();
      }
      double s = 0.0;
      for (int64_t t = threadIdx.x; t < m; t += kGenThreads) s += oj[t] * oj[t];
      const double nrm = sqrt(gsum(s, red));
      if (nrm > 0.0)
        for (int64_t t = threadIdx.x; t < m; t += kGenThreads) oj[t] /= nrm;
      __syncthreads();
    }
}

// The symmetric-definite pencil (S, J) of the HAM polish reduced to a standard problem:
// S = L L^T (Cholesky, lower), Mneg = -L^-1 J L^-T.  S: lower triangle read, J: full; both
// m x m with leading dimension ld.  W: 3 m^2 doubles (L, then Y = L^-1 J, then Mneg, each ld m);
// status = 1 when S is not positive definite, else 0.
__global__ void __launch_bounds__(kGenThreads) pencil_reduce_kernel(const double *S, const double *J, int64_t ld,
                                                                   int64_t m, double *W, int *status) {
  __shared__ int bad;
  double *L = W, *Y = W + m * m, *Mn = W + 2 * m * m;
  if (threadIdx.x == 0) bad = 0;
  for (int64_t t = threadIdx.x; t < m * m; t += kGenThreads) {
    const int64_t r = t % m, c = t / m;
    L[t] = r >= c ? S[r + ld * c] : 0.0;
  }
  __syncthreads();
  for (int64_t k = 0; k < m; ++k) {  // right-looking Cholesky
    if (threadIdx.x == 0) {
      const double d = L[k + m * k];
      if (!(d > 0.0)) bad = 1;
      else L[k + m * k] = sqrt(d);
    }
    __syncthreads();
    if (bad) break;
    const double inv = 1.0 / L[k + m * k];
    for (int64_t i = k + 1 + threadIdx.x; i < m; i += kGenThreads) L[i + m * k] *= inv;
    __syncthreads();
    const int64_t nr = m - k - 1;
    for (int64_t t = threadIdx.x; t < nr * nr; t += kGenThreads) {
      const int64_t i = k + 1 + t % nr, c = k + 1 + t / nr;
      if (i >= c) L[i + m * c] -= L[i + m * k] * L[c + m * k];
    }
    __syncthreads();
  }
  if (bad) {
    if (threadIdx.x == 0) *status = 1;
    return;
  }
  for (int64_t c = threadIdx.x; c < m; c += kGenThreads) {  // Y = L^-1 J, one column per thread
    double *y = Y + m * c;
    for (int64_t r = 0; r < m; ++r) {
      double t = J[r + ld * c];
      for (int64_t k = 0; k < r; ++k) t -= L[r + m * k] * y[k];
      y[r] = t / L[r + m * r];
    }
  }
  __syncthreads();
  // M = L^-1 Y^T (M = Y L^-T is symmetric): column r of M from row r of Y; stored negated
  for (int64_t r = threadIdx.x; r < m; r += kGenThreads) {
    double *z = Mn + m * r;
    for (int64_t i = 0; i < m; ++i) {
      double t = Y[r + m * i];
      for (int64_t k = 0; k < i; ++k) t += L[i + m * k] * z[k];  // z holds -M: subtracting becomes adding
      z[i] = -t / L[i + m * i];
    }
  }
  __syncthreads();
  if (threadIdx.x == 0) *status = 0;
}

// After the eigenproblem of Mneg (ascending eigenvalues nu = -mu, eigenvectors Z, ld m): the np
// lowest positive roots omega = 1 / mu = -1 / nu and u = L^-T z.  status = 2 when fewer than np of
// the mu are positive.
__global__ void pencil_finish_kernel(const double *W, int64_t m, const double *nu, const double *Z, int64_t np,
                                     double *U, double *lam, int *status) {
  const double *L = W;
  for (int64_t j = threadIdx.x; j < np; j += blockDim.x) {
    if (!(nu[j] < 0.0)) *status = 2;
    lam[j] = -1.0 / nu[j];
    double *u = U + m * j;
    const double *z = Z + m * j;
    for (int64_t r = m - 1; r >= 0; --r) {  // L^T u = z
      double t = z[r];
      for (int64_t k = r + 1; k < m; ++k) t -= L[k + m * r] * u[k];
      u[r] = t / L[r + m * r];
    }
  }
}

}  // namespace

void pencil_reduce_device(const double *S, const double *J, int64_t ld, int64_t m, double *W, int *status,
                          cudaStream_t s) {
  VGB_REQUIRE(m >= 1 && ld >= m, "pencil_reduce: invalid sizes");
  pencil_reduce_kernel<<<1, kGenThreads, 0, s>>>(S, J, ld, m, W, status);
  VGB_LAUNCH_CHECK();
}

void pencil_finish_device(const double *W, int64_t m, const double *nu, const double *Z, int64_t np, double *U,
                          double *lam, int *status, cudaStream_t s) {
  pencil_finish_kernel<<<1, 128, 0, s>>>(W, m, nu, Z, np, U, lam, status);
  VGB_LAUNCH_CHECK();
}

int64_t gen_eig_work_doubles(int64_t m, int64_t nw) { return 3 * m * m + 5 * m + nw * (2 * m * m + 5 * m) + m * m + 64; }

void gen_eig_device(const GenEigJob *jobs, int64_t njobs, cudaStream_t s) {
  if (njobs <= 0) return;
  int dev = 0;
  VGB_CUDA(cudaGetDevice(&dev));
  int optin = 0;
  VGB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  VGB_CUDA(cudaFuncGetAttributes(&fa, gen_eig_kernel));
  const int dyn_max = optin - (int)fa.sharedSizeBytes;
  static std::mutex mu;
  static int configured[64] = {0};
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && !configured[dev]) {
      VGB_CUDA(cudaFuncSetAttribute(gen_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max));
      configured[dev] = 1;
    }
  }
  const int64_t limit = dyn_max / (int64_t)sizeof(double);
  std::unique_ptr<GenEigGroup> g(new GenEigGroup());
  for (int64_t b = 0; b < njobs; b += kGenJobs) {
    g->n = (int)std::min<int64_t>(kGenJobs, njobs - b);
    int64_t need = 0;
    for (int i = 0; i < g->n; ++i) {
      const GenEigJob &jb = jobs[b + i];
      VGB_REQUIRE(jb.m >= 1 && jb.m <= kGenEigMaxM && jb.nw >= 1 && jb.nw <= jb.m && jb.ldu >= jb.m &&
                      jb.ldt >= jb.m && jb.work != nullptr && jb.info != nullptr,
                  "small generalized eigenproblem: invalid job");
      g->j[i] = jb;
      if (jb.m * jb.m <= limit) need = std::max(need, jb.m * jb.m);
    }
    g->smem_doubles = need;
    gen_eig_kernel<<<g->n, kGenThreads, need * sizeof(double), s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
}

void orthonormalise_device(const double *U, int64_t ldu, int64_t m, int64_t r, double *O, int64_t ldo,
                           cudaStream_t s) {
  VGB_REQUIRE(m >= 1 && r >= 1 && r <= m && ldu >= m && ldo >= m, "orthonormalise: invalid sizes");
  orthonormalise_kernel<<<1, kGenThreads, 0, s>>>(U, ldu, m, r, O, ldo);
  VGB_LAUNCH_CHECK();
}

}  // namespace vgb
