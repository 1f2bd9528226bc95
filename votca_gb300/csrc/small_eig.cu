// Small dense symmetric eigenproblems on the device; the method is described in small_eig.cuh.
#include "small_eig.cuh"

#include <algorithm>
#include <memory>
#include <mutex>

namespace vgb {

namespace {

constexpr int kEigThreads = 256;
constexpr int kEigWarps = kEigThreads / 32;
constexpr int kEigJobs = 256;  // jobs per launch (kernel-parameter space)

struct SymEigGroup {
  SymEigJob j[kEigJobs];
  int n;
  int64_t smem_doubles;  // dynamic shared memory of the launch
};

__host__ __device__ inline int64_t eig_ld(int64_t m) { return (m % 2 == 0) ? m + 1 : m; }
// doubles of the vector part of the shared layout: d, e, tau, v, p (5m), 32 reduction slots,
// then 3m + 2 four-byte words (FP32 diagonal, FP32 squared off-diagonal, FP32 eigenvalues)
// and m + 1 cluster starts
__host__ __device__ inline int64_t eig_vec_doubles(int64_t m) { return 5 * m + 32 + (4 * m + 4) / 2 + 2; }

__device__ double block_sum(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();  // earlier readers of red are done
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  // pairwise in a fixed order (deterministic): three dependent FP64 adds instead of eight
  static_assert(kEigWarps == 8, "block_sum adds eight warp sums");
  return ((red[0] + red[1]) + (red[2] + red[3])) + ((red[4] + red[5]) + (red[6] + red[7]));
}

__device__ double block_max(double v, double *red) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = red[0];
  for (int w = 1; w < kEigWarps; ++w) t = fmax(t, red[w]);
  return t;
}

// number of eigenvalues of the FP32 tridiagonal (d, e2 = e^2) below x
__device__ int sturm_count(const float *d, const float *e2, int64_t m, float x, float pivmin) {
  float q = d[0] - x;
  if (fabsf(q) < pivmin) q = -pivmin;
  int c = q < 0.f;
  for (int64_t i = 1; i < m; ++i) {
    q = d[i] - x - __fdividef(e2[i - 1], q);
    if (fabsf(q) < pivmin) q = -pivmin;
    c += q < 0.f;
  }
  return c;
}

// LU with partial pivoting of the tridiagonal (d - sigma, e): rows i and i+1 swap when the
// subdiagonal entry is larger than the pivot; U has two superdiagonals.  r0 holds 1/U_ii.
__device__ void tri_lu(const double *d, const double *e, int64_t m, double sigma, double tiny,
                       double *r0, double *u1, double *u2, double *l, double *pv) {
  double da = d[0] - sigma, db = m > 1 ? e[0] : 0.0;
  for (int64_t i = 0; i + 1 < m; ++i) {
    const double c = e[i], an = d[i + 1] - sigma, bn = (i + 2 < m) ? e[i + 1] : 0.0;
    if (fabs(da) >= fabs(c)) {
      if (fabs(da) < tiny) da = da < 0.0 ? -tiny : tiny;
      const double r = 1.0 / da;  // one division per row
      const double li = c * r;
      r0[i] = r; l[i] = li; u1[i] = db; u2[i] = 0.0; pv[i] = 0.0;
      da = an - li * db;
      db = bn;
    } else {
      const double r = 1.0 / c;
      const double li = da * r;
      r0[i] = r; l[i] = li; u1[i] = an; u2[i] = bn; pv[i] = 1.0;
      const double nda = db - li * an;
      db = -li * bn;
      da = nda;
    }
  }
  if (fabs(da) < tiny) da = da < 0.0 ? -tiny : tiny;
  r0[m - 1] = 1.0 / da;
}

// z <- (T - sigma)^-1 z with the factors of tri_lu
__device__ void tri_solve(int64_t m, const double *r0, const double *u1, const double *u2,
                          const double *l, const double *pv, double *z, int64_t zs) {
  for (int64_t i = 0; i + 1 < m; ++i) {
    double a = z[i * zs], b = z[(i + 1) * zs];
    if (pv[i] != 0.0) { const double t = a; a = b; b = t; }
    z[i * zs] = a;
    z[(i + 1) * zs] = b - l[i] * a;
  }
  for (int64_t i = m - 1; i >= 0; --i) {
    double s = z[i * zs];
    if (i + 1 < m) s -= u1[i] * z[(i + 1) * zs];
    if (i + 2 < m) s -= u2[i] * z[(i + 2) * zs];
    z[i * zs] = s * r0[i];
  }
}

__device__ double vnorm(const double *z, int64_t m) {
  double s = 0.0;
  for (int64_t i = 0; i < m; ++i) s = fma(z[i], z[i], s);
  return sqrt(s);
}
__device__ void vscale(double *z, int64_t m, double f) {
  for (int64_t i = 0; i < m; ++i) z[i] *= f;
}
// z^T T z for the tridiagonal (d, e)
__device__ double tri_rq(const double *d, const double *e, const double *z, int64_t m) {
  double s = 0.0;
  for (int64_t i = 0; i < m; ++i) {
    double y = d[i] * z[i];
    if (i > 0) y = fma(e[i - 1], z[i - 1], y);
    if (i + 1 < m) y = fma(e[i], z[i + 1], y);
    s = fma(z[i], y, s);
  }
  return s;
}
// a fixed, well-spread positive start vector (an integer hash of (i, j) mapped to [0.5, 1.5))
__device__ void start_vector(double *z, int64_t m, int64_t j) {
  for (int64_t i = 0; i < m; ++i) {
    uint32_t h = (uint32_t)i * 2654435761u ^ ((uint32_t)j * 40503u + 12345u);
    h ^= h >> 15;
    h *= 2246822519u;
    h ^= h >> 13;
    z[i] = 0.5 + (double)(h >> 8) * (1.0 / 16777216.0);
  }
}

__global__ void __launch_bounds__(kEigThreads, 2) sym_eig_kernel(const __grid_constant__ SymEigGroup g) {
  const SymEigJob q = g.j[blockIdx.x];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int64_t m = q.m, nw = q.nw;
  if (m < 1 || nw < 1 || nw > m || m > kSymEigMaxM) {
    if (tid == 0 && q.info) *q.info = 1;
    return;
  }
  extern __shared__ double sm[];
  const int64_t ld = eig_ld(m);
  const int64_t nvec = eig_vec_doubles(m);
  double *d = sm, *e = d + m, *tau = e + m, *vv = tau + m, *pp = vv + m, *red = pp + m;
  float *d32 = reinterpret_cast<float *>(red + 32), *e2 = d32 + m, *lam32 = e2 + m;
  int *cl = reinterpret_cast<int *>(lam32 + m);
  // Shared memory behind the vectors, in this order while it lasts: the lower triangle A, the
  // eigenvectors of the tridiagonal (m per wanted eigenvalue), the LU factors of their inverse
  // iterations (5 m per wanted eigenvalue); the rest in global scratch.  The inverse iteration
  // and the back-transformation are serial chains over m, and each step through global memory
  // waits for an L2 round trip (the vectors are copied to U at the end).
  int64_t off = nvec;
  const bool a_sm = off + ld * m <= g.smem_doubles;
  double *A = a_sm ? sm + off : q.work;
  if (a_sm) off += ld * m;
  const bool z_sm = off + m * nw <= g.smem_doubles;
  double *Z = z_sm ? sm + off : q.U;
  const int64_t ldz = z_sm ? m : q.ldu;
  if (z_sm) off += m * nw;
  const bool lu_sm = z_sm && off + 5 * m * nw <= g.smem_doubles;
  double *scratch = lu_sm ? sm + off : q.work + ld * m;  // 5 m per wanted eigenvalue

  if (tid == 0 && q.clocks) q.clocks[0] = clock64();
  // ---- load the lower triangle ----
  for (int64_t t = tid; t < m * m; t += kEigThreads) {
    const int64_t j = t / m, i = t % m;
    if (i >= j) A[i + ld * j] = q.T[i + q.ldt * j];
  }
  __syncthreads();

  // ---- 1. Householder tridiagonalisation ----
  for (int64_t k = 0; k + 2 < m; ++k) {
    const int64_t k1 = k + 1;
    double s = 0.0;
    for (int64_t i = k + 2 + tid; i < m; i += kEigThreads) s = fma(A[i + ld * k], A[i + ld * k], s);
    const double xn2 = block_sum(s, red);
    const double alpha = A[k1 + ld * k];
    if (xn2 == 0.0) {
      if (tid == 0) { tau[k] = 0.0; e[k] = alpha; d[k] = A[k + ld * k]; }
      __syncthreads();
      continue;
    }
    const double beta = -copysign(sqrt(alpha * alpha + xn2), alpha);
    const double tk = (beta - alpha) / beta;
    const double scal = 1.0 / (alpha - beta);
    for (int64_t i = k1 + tid; i < m; i += kEigThreads) {
      const double vi = (i == k1) ? 1.0 : A[i + ld * k] * scal;
      vv[i] = vi;
      if (i > k1) A[i + ld * k] = vi;
    }
    if (tid == 0) { tau[k] = tk; e[k] = beta; d[k] = A[k + ld * k]; }
    __syncthreads();
    // p = tau A22 v from the lower triangle; four interleaved partial sums per row (a chain of
    // dependent FP64 FMAs is the latency of this step)
    double pv_part = 0.0;
    for (int64_t i = k1 + tid; i < m; i += kEigThreads) {
      double acc[4] = {0.0, 0.0, 0.0, 0.0};
      int64_t j = k1;
      for (; j + 4 <= m; j += 4) {
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int64_t jj = j + u;
          const double a = (jj <= i) ? A[i + ld * jj] : A[jj + ld * i];
          acc[u] = fma(a, vv[jj], acc[u]);
        }
      }
#pragma unroll
      for (int u = 0; u < 3; ++u) {  // at most three left
        const int64_t jj = j + u;
        if (jj < m) {
          const double a = (jj <= i) ? A[i + ld * jj] : A[jj + ld * i];
          acc[u] = fma(a, vv[jj], acc[u]);
        }
      }
      const double p = tk * ((acc[0] + acc[1]) + (acc[2] + acc[3]));
      pp[i] = p;
      pv_part = fma(p, vv[i], pv_part);
    }
    const double K = -0.5 * tk * block_sum(pv_part, red);
    for (int64_t i = k1 + tid; i < m; i += kEigThreads) pp[i] = fma(K, vv[i], pp[i]);  // w
    __syncthreads();
    // A22 -= v w^T + w v^T (lower triangle), one warp per column
    for (int64_t j = k1 + warp; j < m; j += kEigWarps) {
      const double vj = vv[j], wj = pp[j];
      for (int64_t i = j + lane; i < m; i += 32) A[i + ld * j] -= fma(vv[i], wj, pp[i] * vj);
    }
    __syncthreads();
  }
  if (tid == 0) {
    if (m >= 2) {
      d[m - 2] = A[(m - 2) + ld * (m - 2)];
      d[m - 1] = A[(m - 1) + ld * (m - 1)];
      e[m - 2] = A[(m - 1) + ld * (m - 2)];
      tau[m - 2] = 0.0;
    } else {
      d[0] = A[0];
    }
    tau[m - 1] = 0.0;
  }
  __syncthreads();
  if (tid == 0 && q.clocks) q.clocks[1] = clock64();

  // ---- 2. wanted eigenvalues of the tridiagonal: FP32 bisection ----
  double lo = INFINITY, hi = -INFINITY, e2max = 0.0;
  for (int64_t i = tid; i < m; i += kEigThreads) {
    const double r = (i > 0 ? fabs(e[i - 1]) : 0.0) + (i + 1 < m ? fabs(e[i]) : 0.0);
    lo = fmin(lo, d[i] - r);
    hi = fmax(hi, d[i] + r);
    d32[i] = (float)d[i];
    if (i + 1 < m) {
      e2[i] = (float)(e[i] * e[i]);
      e2max = fmax(e2max, e[i] * e[i]);
    }
  }
  lo = -block_max(-lo, red);
  hi = block_max(hi, red);
  e2max = block_max(e2max, red);
  const double nrm = fmax(fmax(fabs(lo), fabs(hi)), 1e-300);
  const float pivmin = (float)(1e-30 * fmax(1.0, e2max));
  for (int64_t j = tid; j < nw; j += kEigThreads) {
    float a = (float)(lo - 1e-6 * nrm) - 1e-30f, b = (float)(hi + 1e-6 * nrm) + 1e-30f;
    for (int it = 0; it < 80; ++it) {
      if (b - a <= 2.4e-7f * fmaxf(fabsf(a), fabsf(b)) + 4.f * pivmin) break;
      const float mid = 0.5f * (a + b);
      if (sturm_count(d32, e2, m, mid, pivmin) > (int)j) b = mid; else a = mid;
    }
    lam32[j] = 0.5f * (a + b);
  }
  __syncthreads();
  // clusters of eigenvalues closer than 1e-5 of the spectral radius (cl: starts, then nw): the
  // FP32 shifts are good to a few 1e-7 of it, so eigenvalues further apart converge separately
  __shared__ int ncl;
  if (tid == 0 && q.clocks) q.clocks[2] = clock64();
  if (tid == 0) {
    int c = 0;
    cl[c++] = 0;
    for (int64_t j = 1; j < nw; ++j)
      if ((double)lam32[j] - (double)lam32[j - 1] > 1e-5 * nrm) cl[c++] = (int)j;
    cl[c] = (int)nw;
    ncl = c;
  }
  __syncthreads();

  // ---- 3. eigenvectors of the tridiagonal by inverse iteration (FP64) ----
  const double tiny = 2.3e-16 * nrm;
  for (int c = tid; c < ncl; c += kEigThreads) {
    const int64_t j0 = cl[c], j1 = cl[c + 1], s = j1 - j0;
    double *w = scratch + 5 * m * j0;  // 5 m per member, contiguous over the cluster
    double *r0 = w, *u1 = w + m, *u2 = w + 2 * m, *l = w + 3 * m, *pv = w + 4 * m;
    for (int64_t jj = j0; jj < j1; ++jj) {
      double *z = Z + ldz * jj;
      start_vector(z, m, jj);
      tri_lu(d, e, m, (double)lam32[jj], tiny, r0, u1, u2, l, pv);
      const int steps = s == 1 ? 2 : 5;
      for (int st = 0; st < steps; ++st) {
        tri_solve(m, r0, u1, u2, l, pv, z, 1);
        for (int64_t kk = j0; kk < jj; ++kk) {  // earlier members of the cluster
          const double *y = Z + ldz * kk;
          double dot = 0.0;
          for (int64_t i = 0; i < m; ++i) dot = fma(y[i], z[i], dot);
          for (int64_t i = 0; i < m; ++i) z[i] = fma(-dot, y[i], z[i]);
        }
        vscale(z, m, 1.0 / vnorm(z, m));
      }
      if (s == 1) {  // Rayleigh quotient iteration: two steps at the FP64 shift
        tri_lu(d, e, m, tri_rq(d, e, z, m), tiny, r0, u1, u2, l, pv);
        for (int st = 0; st < 2; ++st) {
          tri_solve(m, r0, u1, u2, l, pv, z, 1);
          vscale(z, m, 1.0 / vnorm(z, m));
        }
        q.lam[jj] = tri_rq(d, e, z, m);
      }
    }
    if (s > 1) {  // Rayleigh-Ritz on the cluster: cyclic Jacobi on C = Z_c^T T Z_c
      double *C = w, *W = w + s * s, *y = w + 2 * s * s;
      for (int64_t b = 0; b < s; ++b) {
        const double *zb = Z + ldz * (j0 + b);
        for (int64_t i = 0; i < m; ++i) {
          double t = d[i] * zb[i];
          if (i > 0) t = fma(e[i - 1], zb[i - 1], t);
          if (i + 1 < m) t = fma(e[i], zb[i + 1], t);
          y[i] = t;
        }
        for (int64_t a = 0; a < s; ++a) {
          const double *za = Z + ldz * (j0 + a);
          double t = 0.0;
          for (int64_t i = 0; i < m; ++i) t = fma(za[i], y[i], t);
          C[a + s * b] = t;
        }
      }
      for (int64_t b = 0; b < s; ++b)
        for (int64_t a = 0; a < s; ++a) {
          W[a + s * b] = a == b ? 1.0 : 0.0;
          if (a < b) C[a + s * b] = C[b + s * a] = 0.5 * (C[a + s * b] + C[b + s * a]);
        }
      for (int sweep = 0; sweep < 40; ++sweep) {
        double off = 0.0, dg = 0.0;
        for (int64_t b = 0; b < s; ++b)
          for (int64_t a = 0; a < s; ++a) {
            const double v = C[a + s * b] * C[a + s * b];
            if (a == b) dg += v; else off += v;
          }
        if (off <= 1e-34 * dg || off == 0.0) break;
        for (int64_t p = 0; p < s; ++p)
          for (int64_t r = p + 1; r < s; ++r) {
            const double apq = C[p + s * r];
            if (apq == 0.0) continue;
            const double th = (C[r + s * r] - C[p + s * p]) / (2.0 * apq);
            const double t = fabs(th) > 1e150 ? 0.5 / th : copysign(1.0, th) / (fabs(th) + sqrt(th * th + 1.0));
            const double cs = 1.0 / sqrt(t * t + 1.0), sn = t * cs;
            for (int64_t x = 0; x < s; ++x) {  // C J
              const double cp = C[x + s * p], cq = C[x + s * r];
              C[x + s * p] = cs * cp - sn * cq;
              C[x + s * r] = sn * cp + cs * cq;
            }
            for (int64_t x = 0; x < s; ++x) {  // J^T (C J)
              const double cp = C[p + s * x], cq = C[r + s * x];
              C[p + s * x] = cs * cp - sn * cq;
              C[r + s * x] = sn * cp + cs * cq;
            }
            for (int64_t x = 0; x < s; ++x) {
              const double wp = W[x + s * p], wq = W[x + s * r];
              W[x + s * p] = cs * wp - sn * wq;
              W[x + s * r] = sn * wp + cs * wq;
            }
          }
      }
      // ascending order of the Ritz values: selection sort of the columns of W
      for (int64_t a = 0; a < s; ++a) {
        int64_t best = a;
        for (int64_t b = a + 1; b < s; ++b)
          if (C[b + s * b] < C[best + s * best]) best = b;
        if (best != a) {
          const double t = C[a + s * a];
          C[a + s * a] = C[best + s * best];
          C[best + s * best] = t;
          for (int64_t x = 0; x < s; ++x) {
            const double u = W[x + s * a];
            W[x + s * a] = W[x + s * best];
            W[x + s * best] = u;
          }
        }
        q.lam[j0 + a] = C[a + s * a];
      }
      for (int64_t i = 0; i < m; ++i) {  // Z_c <- Z_c W, row by row
        for (int64_t a = 0; a < s; ++a) {
          double t = 0.0;
          for (int64_t b = 0; b < s; ++b) t = fma(Z[i + ldz * (j0 + b)], W[b + s * a], t);
          y[a] = t;
        }
        for (int64_t a = 0; a < s; ++a) Z[i + ldz * (j0 + a)] = y[a];
      }
    }
  }
  __syncthreads();
  if (tid == 0 && q.clocks) q.clocks[3] = clock64();

  // ---- 4. back-transformation U = H_0 H_1 ... H_{m-3} Z ----
  // Up to one vector per warp: each warp applies the reflectors to its vector (a warp reduction
  // per reflector).  More vectors: every reflector is applied to a batch of vectors at once, G
  // threads per vector (all threads busy), each summing every G-th row of the dot product; the
  // G partial sums of a vector are added in a fixed order by each of its threads (no FP64
  // shuffle tree: on GB300's narrow FP64 pipe the five butterfly levels of a warp reduction,
  // repeated for every vector of every warp, cost more than the dot products themselves).
  if (nw <= kEigWarps) {
    for (int64_t j = warp; j < nw; j += kEigWarps) {
      double *z = Z + ldz * j;
      for (int64_t k = m - 3; k >= 0; --k) {
        const double tk = tau[k];
        if (tk == 0.0) continue;
        double s = 0.0;
        for (int64_t i = k + 1 + lane; i < m; i += 32) s = fma(i == k + 1 ? 1.0 : A[i + ld * k], z[i], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
        const double f = tk * s;
        for (int64_t i = k + 1 + lane; i < m; i += 32) z[i] = fma(-f, i == k + 1 ? 1.0 : A[i + ld * k], z[i]);
      }
    }
  } else {
    __shared__ double part[kEigThreads];
    const int G = (int)std::min<int64_t>(32, std::max<int64_t>(1, kEigThreads / nw));
    const int per_batch = kEigThreads / G;
    const int slot = tid / G, sub = tid % G;
    for (int64_t j0 = 0; j0 < nw; j0 += per_batch) {
      const int64_t j = j0 + slot;
      const bool act = slot < per_batch && j < nw;
      double *z = act ? Z + ldz * j : nullptr;
      for (int64_t k = m - 3; k >= 0; --k) {
        const double tk = tau[k];
        if (tk == 0.0) continue;  // uniform over the block
        double s = 0.0;
        if (act)
          for (int64_t i = k + 1 + sub; i < m; i += G) s = fma(i == k + 1 ? 1.0 : A[i + ld * k], z[i], s);
        part[tid] = s;
        __syncthreads();
        if (act) {
          double t = 0.0;
          for (int p = 0; p < G; ++p) t += part[slot * G + p];
          const double f = tk * t;
          for (int64_t i = k + 1 + sub; i < m; i += G) z[i] = fma(-f, i == k + 1 ? 1.0 : A[i + ld * k], z[i]);
        }
        __syncthreads();  // part is written again for the next reflector
      }
    }
  }
  __syncthreads();
  if (z_sm)
    for (int64_t t = tid; t < m * nw; t += kEigThreads) q.U[(t % m) + q.ldu * (t / m)] = Z[t];
  if (tid == 0 && q.clocks) q.clocks[4] = clock64();
  if (tid == 0 && q.info) *q.info = 0;
}

}  // namespace

int64_t sym_eig_work_doubles(int64_t m, int64_t nw) { return eig_ld(m) * m + 5 * m * nw + 64; }

void sym_eig_device(const SymEigJob *jobs, int64_t njobs, cudaStream_t s) {
  if (njobs <= 0) return;
  int dev = 0;
  VGB_CUDA(cudaGetDevice(&dev));
  int optin = 0;
  VGB_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  VGB_CUDA(cudaFuncGetAttributes(&fa, sym_eig_kernel));
  const int dyn_max = optin - (int)fa.sharedSizeBytes;  // the static shared memory counts against the limit
  static std::mutex mu;
  static int configured[64] = {0};
  {
    std::lock_guard<std::mutex> lk(mu);
    if (dev < 64 && !configured[dev]) {
      VGB_CUDA(cudaFuncSetAttribute(sym_eig_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, dyn_max));
      configured[dev] = 1;
    }
  }
  const int64_t limit = dyn_max / (int64_t)sizeof(double);
  std::unique_ptr<SymEigGroup> g(new SymEigGroup());
  for (int64_t b = 0; b < njobs; b += kEigJobs) {
    g->n = (int)std::min<int64_t>(kEigJobs, njobs - b);
    int64_t need = 0;
    for (int i = 0; i < g->n; ++i) {
      const SymEigJob &jb = jobs[b + i];
      VGB_REQUIRE(jb.m >= 1 && jb.m <= kSymEigMaxM && jb.nw >= 1 && jb.nw <= jb.m && jb.ldu >= jb.m &&
                      jb.ldt >= jb.m && jb.work != nullptr,
                  "small symmetric eigenproblem: invalid job");
      g->j[i] = jb;
      // the vectors, then A, the inverse-iteration vectors and their LU factors while they fit
      // (the kernel places them in the same order)
      int64_t job_need = eig_vec_doubles(jb.m);
      if (job_need + eig_ld(jb.m) * jb.m <= limit) job_need += eig_ld(jb.m) * jb.m;
      if (job_need + jb.m * jb.nw <= limit) {
        job_need += jb.m * jb.nw;
        if (job_need + 5 * jb.m * jb.nw <= limit) job_need += 5 * jb.m * jb.nw;
      }
      need = std::max(need, job_need);
    }
    g->smem_doubles = need;
    sym_eig_kernel<<<g->n, kEigThreads, need * sizeof(double), s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
}

}  // namespace vgb
