// Block Davidson on the device.  Every dim-sized vector (search space V, A V,
// Ritz vectors, residuals, corrections) lives in HBM; Gram-Schmidt, the
// projections V^T A V, the Ritz vectors V U, the residuals A V U - q Lambda,
// the residual norms and the DPR/Olsen corrections run as FP64 kernels.  Only
// the projected matrices (<= a few hundred squared) and the norms cross to
// the host, where the small eigenproblem is solved.
//
// Step-by-step correspondence with xtp/src/libxtp/davidsonsolver.cc:
//   checkOptions :44-62, getSizeUpdate :149-170, setupInitialEigenvectors :180-206,
//   getRitz :221-239, getHarmonicRitz :241-332, checkConvergence :347-352,
//   extendProjection :354-378, computeCorrectionVector/dpr/olsen :389-436,
//   gramschmidt :442-478, qr :480-488, restart :490-513, store* :515-555,
// and updateProjection, davidsonsolver.h:239-280.
#include "davidson.cuh"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <numeric>
#include <cstdlib>

#include "small_eig.cuh"

namespace vgb {

namespace {

constexpr int kRedChunks = 64;

unsigned blocks_for(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), 16LL * 152));
}

// partial[c * kRedChunks + b] = sum over chunk b of A[:, c] * B[:, c]
__global__ void coldot_partial_kernel(const double *__restrict__ A, int64_t lda,
                                      const double *__restrict__ B, int64_t ldb, int64_t n,
                                      double *__restrict__ partial) {
  const int64_t c = blockIdx.y;
  const int64_t chunk = ceil_div(n, kRedChunks);
  const int64_t r0 = blockIdx.x * chunk, r1 = min(n, r0 + chunk);
  const double *a = A + c * lda, *b = B + c * ldb;
  double s = 0.0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) s = fma(a[r], b[r], s);
  __shared__ double red[256];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[c * kRedChunks + blockIdx.x] = red[0];
}

__global__ void coldot_final_kernel(const double *__restrict__ partial, int64_t ncols, int take_sqrt,
                                    double *__restrict__ out) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncols;
       c += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int b = 0; b < kRedChunks; ++b) s += partial[c * kRedChunks + b];
    out[c] = take_sqrt ? sqrt(s) : s;
  }
}

__global__ void set_unit_columns_kernel(double *V, int64_t ldv, const int64_t *rows, int64_t count) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < count;
       j += (int64_t)gridDim.x * blockDim.x)
    V[rows[j] + ldv * j] = 1.0;
}

// res[:, j] -= lam[j] * q[:, j]
__global__ void residual_kernel(double *__restrict__ res, const double *__restrict__ q, int64_t n,
                                int64_t ncols, const double *__restrict__ lam) {
  const int64_t total = n * ncols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t j = t / n;
    res[t] -= lam[j] * q[t];
  }
}

// out[:, kk] = -r_j / (D - lambda_j) for the listed roots (DPR, davidsonsolver.cc:416-422);
// with olsen != 0 also dq[:, kk] = -q_j / (D - lambda_j).  clean != 0 zeroes
// non-finite entries (computeCorrectionVector, :411-413).
__global__ void dpr_kernel(double *__restrict__ out, int64_t ldo, const double *__restrict__ res,
                           const double *__restrict__ q, int64_t n, const double *__restrict__ D,
                           const int64_t *__restrict__ cols, const double *__restrict__ lams,
                           int64_t count, int clean, double *__restrict__ dq) {
  const int64_t total = n * count;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, kk = t / n;
    const int64_t j = cols[kk];
    const double den = D[i] - lams[kk];
    double v = -res[j * n + i] / den;
    if (clean && !isfinite(v)) v = 0.0;
    out[kk * ldo + i] = v;
    if (dq) dq[kk * n + i] = -q[j * n + i] / den;
  }
}

// Olsen: delta += (num/denom) q_j, then non-finite -> 0 (davidsonsolver.cc:424-436)
__global__ void olsen_finish_kernel(double *__restrict__ out, int64_t ldo,
                                    const double *__restrict__ q, int64_t n,
                                    const int64_t *__restrict__ cols, const double *__restrict__ num,
                                    const double *__restrict__ den, int64_t count) {
  const int64_t total = n * count;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, kk = t / n;
    const double eps = (-num[kk]) / (-den[kk]);
    double v = out[kk * ldo + i] + eps * q[cols[kk] * n + i];
    if (!isfinite(v)) v = 0.0;
    out[kk * ldo + i] = v;
  }
}

// A[:, c] /= norm[c] where norm[c] > 0 (Eigen's normalize leaves zero columns alone)
__global__ void scale_columns_kernel(double *A, int64_t lda, int64_t n, int64_t ncols,
                                     const double *__restrict__ norm) {
  const int64_t total = n * ncols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, c = t / n;
    const double nv = norm[c];
    if (nv > 0.0) A[c * lda + i] /= nv;
  }
}

__global__ void copy_block_kernel(const double *src, int64_t lds, double *dst, int64_t ldd,
                                  int64_t n, int64_t ncols) {
  const int64_t total = n * ncols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % n, c = t / n;
    dst[c * ldd + i] = src[c * lds + i];
  }
}

// T[c0 + c, r] = T[r, c0 + c] for r < c0, c < nc: the lower block of the projected matrix from
// the columns just computed (updateProjection's bottomLeftCorner = topRightCorner^T)
__global__ void mirror_block_kernel(double *T, int64_t ldt, int64_t c0, int64_t nc) {
  const int64_t total = c0 * nc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % c0, c = t / c0;
    T[(c0 + c) + ldt * r] = T[r + ldt * (c0 + c)];
  }
}

// ---- column-wise classical Gram-Schmidt in one cooperative launch ----
//
// The reference's inner loop (davidsonsolver.cc:453-458 / 468-477) walks the new
// columns one by one: h = Q_{nstart..j-1}^T q_j, q_j -= Q h, normalise, and in
// the second pass checks ||q_j|| against 1e-12 of the column's original norm.
// Each step is a matrix-vector product over dim rows, so as separate launches it
// is launch- and sync-bound.  Here every block owns a contiguous slice of rows;
// one grid barrier after the partial dots and one after the partial norms make
// a column step, and the next column's dots read only the block's own rows, so
// no barrier is needed after the scaling.  The barrier is a bounded spin: if a
// block does not arrive within the limit the kernel records an error and stops.
constexpr int kGsThreads = 256;
constexpr int kGsMaxRange = 1024;

__device__ bool gs_grid_barrier(unsigned *count, volatile unsigned *gen, unsigned nblocks,
                                volatile int *err) {
  __syncthreads();
  __shared__ int failed;
  if (threadIdx.x == 0) {
    failed = 0;
    const unsigned g = *gen;
    __threadfence();
    const unsigned arrived = atomicAdd(count, 1u);
    if (arrived == nblocks - 1) {
      *count = 0;
      __threadfence();
      atomicAdd((unsigned *)gen, 1u);
    } else {
      const uint64_t t0 = clock64();
      while (*gen == g) {
        if (*err) { failed = 1; break; }
        if (clock64() - t0 > (1ull << 32)) {  // ~2 s at 2 GHz
          *err = 2;
          failed = 1;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return failed == 0;
}

__global__ void __launch_bounds__(kGsThreads)
    gs_columns_kernel(double *Q, int64_t n, int64_t nstart, int64_t ncols, int check,
                      const double *__restrict__ norms0, double *partial, double *npartial,
                      unsigned *bar_count, unsigned *bar_gen, int *flag, int *err) {
  const unsigned nb = gridDim.x;
  const int64_t rows_per = ceil_div(n, (int64_t)nb);
  const int64_t r0 = min(n, (int64_t)blockIdx.x * rows_per), r1 = min(n, r0 + rows_per);
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  __shared__ double h[kGsMaxRange];
  __shared__ double red[kGsThreads / 32];
  const double *M = Q + nstart * n;
  for (int64_t j = nstart + 1; j < ncols; ++j) {
    const int64_t range = j - nstart;
    double *qj = Q + j * n;
    double *part = partial + (j & 1) * (int64_t)nb * kGsMaxRange;
    double *npart = npartial + (j & 1) * (int64_t)nb;
    // partial dots of q_j with the previous new columns over this block's rows
    for (int64_t l = warp; l < range; l += kGsThreads / 32) {
      const double *ml = M + l * n;
      double sacc = 0.0;
      for (int64_t i = r0 + lane; i < r1; i += 32) sacc = fma(ml[i], qj[i], sacc);
      for (int o = 16; o > 0; o >>= 1) sacc += __shfl_down_sync(0xffffffffu, sacc, o);
      if (lane == 0) __stcg(part + (int64_t)blockIdx.x * kGsMaxRange + l, sacc);
    }
    if (!gs_grid_barrier(bar_count, bar_gen, nb, err)) return;
    // h = sum over blocks (fixed order: deterministic)
    for (int64_t l = threadIdx.x; l < range; l += kGsThreads) {
      double sacc = 0.0;
      // other blocks wrote these: read through L2 (an L1 line from two columns ago is stale)
      for (unsigned b = 0; b < nb; ++b) sacc += __ldcg(part + (int64_t)b * kGsMaxRange + l);
      h[l] = sacc;
    }
    __syncthreads();
    // q_j -= M h on own rows, partial squared norm
    double nacc = 0.0;
    for (int64_t i = r0 + threadIdx.x; i < r1; i += kGsThreads) {
      double sacc = 0.0;
      for (int64_t l = 0; l < range; ++l) sacc = fma(M[l * n + i], h[l], sacc);
      const double v = qj[i] - sacc;
      qj[i] = v;
      nacc = fma(v, v, nacc);
    }
    for (int o = 16; o > 0; o >>= 1) nacc += __shfl_down_sync(0xffffffffu, nacc, o);
    if (lane == 0) red[warp] = nacc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kGsThreads / 32; ++w) t += red[w];
      __stcg(npart + blockIdx.x, t);
    }
    if (!gs_grid_barrier(bar_count, bar_gen, nb, err)) return;
    __shared__ double nrm;
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (unsigned b = 0; b < nb; ++b) t += __ldcg(npart + b);
      nrm = sqrt(t);
      if (check && blockIdx.x == 0 && !(nrm > 1e-12 * norms0[range])) *flag = 1;
    }
    __syncthreads();
    const double nv = nrm;
    if (nv > 0.0)  // Eigen's normalize leaves a zero column unchanged
      for (int64_t i = r0 + threadIdx.x; i < r1; i += kGsThreads) qj[i] /= nv;
    __syncthreads();  // the next column's dots read rows scaled by other threads of the block
  }
}

}  // namespace

namespace {

struct Ctx {
  cudaStream_t s;
  int64_t n;
  GemmWorkspace ws;
  DeviceBuffer<double> red_partial, scal, gs_part;
  DeviceBuffer<unsigned> gs_bar;
  DeviceBuffer<int> gs_err;

  // out[c] = ||A[:, c]|| (or dot(A[:, c], B[:, c]) when B given), device
  void coldots(const double *A, int64_t lda, const double *B, int64_t ldb, int64_t ncols,
               double *out, bool sqrt_) {
    if (ncols <= 0) return;
    red_partial.resize(ncols * kRedChunks);
    dim3 grid(kRedChunks, (unsigned)ncols);
    coldot_partial_kernel<<<grid, 256, 0, s>>>(A, lda, B ? B : A, B ? ldb : lda, n,
                                               red_partial.get());
    VGB_LAUNCH_CHECK();
    coldot_final_kernel<<<blocks_for(ncols, 128), 128, 0, s>>>(red_partial.get(), ncols,
                                                               sqrt_ ? 1 : 0, out);
    VGB_LAUNCH_CHECK();
  }
  void scale_cols(double *A, int64_t lda, int64_t ncols, const double *norms) {
    if (ncols <= 0) return;
    scale_columns_kernel<<<blocks_for(n * ncols), 256, 0, s>>>(A, lda, n, ncols, norms);
    VGB_LAUNCH_CHECK();
  }
  // C (m x nc, ldc) = alpha * A[:, a0:a0+m]^T B[:, b0:b0+nc] + beta C
  void gemm_tn(const double *A, int64_t lda, int64_t m, const double *B, int64_t ldb, int64_t nc,
               double *C, int64_t ldc, double alpha, double beta, int64_t rows = -1) {
    GemmDesc g;
    g.M = m; g.N = nc; g.K = rows < 0 ? n : rows;
    g.a_colmajor(A, lda, true).b_colmajor(B, ldb, false).c_colmajor(C, ldc);
    g.alpha = alpha; g.beta = beta;
    dgemm(g, s, &ws);
  }
  // C (n x nc) = alpha * A (n x k) B (k x nc) + beta C
  void gemm_nn(const double *A, int64_t lda, int64_t k, const double *B, int64_t ldb, int64_t nc,
               double *C, int64_t ldc, double alpha, double beta) {
    GemmDesc g;
    g.M = n; g.N = nc; g.K = k;
    g.a_colmajor(A, lda, false).b_colmajor(B, ldb, false).c_colmajor(C, ldc);
    g.alpha = alpha; g.beta = beta;
    dgemm(g, s, &ws);
  }
  void copy_cols(const double *src, int64_t lds, double *dst, int64_t ldd, int64_t ncols) {
    if (ncols <= 0) return;
    copy_block_kernel<<<blocks_for(n * ncols), 256, 0, s>>>(src, lds, dst, ldd, n, ncols);
    VGB_LAUNCH_CHECK();
  }
};

// Cholesky QR of a block of nb unit columns: G = W^T W = R^T R (R upper), Rinv = R^-1, one CTA.
// W R^-1 is the Q of the column-wise classical Gram-Schmidt of the block (the QR factorisation
// with a positive diagonal is unique).  ok = 0 when a pivot falls below 1e-10 of G_kk (the block
// is too ill-conditioned for Cholesky QR: the caller runs the column kernel instead); chk: the
// reference's second-pass test, r_kk <= 1e-12 of the column's original norm -> flag = 1.
constexpr int kCholQrMax = 64;
__global__ void __launch_bounds__(256) cholqr_kernel(const double *G, int nb, double *Rinv, const double *norms0,
                                                     int chk, int *ok, int *flag) {
  __shared__ double a[kCholQrMax * kCholQrMax];
  __shared__ int bad;
  const int tid = threadIdx.x;
  for (int t = tid; t < nb * nb; t += blockDim.x) a[t] = G[t];
  if (tid == 0) bad = 0;
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (tid == 0) {
      const double d = a[k + nb * k];
      if (!(d > 1e-10 * G[k + nb * k])) {
        bad = 1;
      } else {
        a[k + nb * k] = sqrt(d);
        if (chk && k > 0 && a[k + nb * k] <= 1e-12 * norms0[k]) *flag = 1;
      }
    }
    __syncthreads();
    if (bad) break;
    const double rkk = a[k + nb * k];
    for (int j = k + 1 + tid; j < nb; j += blockDim.x) a[k + nb * j] /= rkk;
    __syncthreads();
    const int r = nb - k - 1;
    for (int t = tid; t < r * r; t += blockDim.x) {
      const int i = k + 1 + t % r, j = k + 1 + t / r;
      if (i <= j) a[i + nb * j] -= a[k + nb * i] * a[k + nb * j];
    }
    __syncthreads();
  }
  if (bad) {
    if (tid == 0) *ok = 0;
    return;
  }
  for (int j = tid; j < nb; j += blockDim.x) {  // column j of R^-1 by back substitution
    double *x = Rinv + (int64_t)nb * j;
    for (int i = nb - 1; i > j; --i) x[i] = 0.0;
    x[j] = 1.0 / a[j + nb * j];
    for (int i = j - 1; i >= 0; --i) {
      double t = 0.0;
      for (int l = i + 1; l <= j; ++l) t += a[i + nb * l] * x[l];
      x[i] = -t / a[i + nb * i];
    }
  }
  if (tid == 0) *ok = 1;
}

// DavidsonSolver::gramschmidt on columns [nstart, ncols) of Q (ld n).
void gramschmidt(Ctx &x, double *Q, int64_t nstart, int64_t ncols, DeviceBuffer<double> &work,
                 DeviceBuffer<int> &flag) {
  const int64_t n = x.n, nupdate = ncols - nstart;
  if (nupdate <= 0) return;
  work.resize(3 * nupdate + std::max<int64_t>(nstart, 1) * nupdate + ncols + 8);
  double *norms0 = work.get();            // initial norms of the new columns
  double *norms = norms0 + nupdate;       // scratch norms
  double *h = norms + nupdate + 8;        // projection coefficients
  x.coldots(Q + nstart * n, n, nullptr, 0, nupdate, norms0, true);
  VGB_CUDA(cudaMemsetAsync(flag.get(), 0, sizeof(int), x.s));
  bool column_kernel_ran = false;
  for (int pass = 0; pass < 2; ++pass) {
    if (nstart > 0) {
      // Q_new -= Q_old (Q_old^T Q_new); normalise
      x.gemm_tn(Q, n, nstart, Q + nstart * n, n, nupdate, h, nstart, 1.0, 0.0);
      x.gemm_nn(Q, n, nstart, h, nstart, nupdate, Q + nstart * n, n, -1.0, 1.0);
      x.coldots(Q + nstart * n, n, nullptr, 0, nupdate, norms, true);
      x.scale_cols(Q + nstart * n, n, nupdate, norms);
    }
    if (nstart > 0 && nupdate > 1 && nupdate <= kCholQrMax) {
      // the block's columns are unit vectors now: Cholesky QR of the block (two FP64 GEMMs and
      // one small kernel instead of two grid barriers per column)
      x.gs_part.resize(2 * nupdate * nupdate + n * nupdate + 8);
      double *G = x.gs_part.get(), *Ri = G + nupdate * nupdate, *T = Ri + nupdate * nupdate;
      x.gs_err.resize(2);
      x.gemm_tn(Q + nstart * n, n, nupdate, Q + nstart * n, n, nupdate, G, nupdate, 1.0, 0.0);
      cholqr_kernel<<<1, 256, 0, x.s>>>(G, (int)nupdate, Ri, norms0, pass == 1 ? 1 : 0, x.gs_err.get() + 1,
                                        flag.get());
      VGB_LAUNCH_CHECK();
      int ok = 0;
      VGB_CUDA(cudaMemcpyAsync(&ok, x.gs_err.get() + 1, sizeof(int), cudaMemcpyDeviceToHost, x.s));
      VGB_CUDA(cudaStreamSynchronize(x.s));
      if (ok) {
        x.gemm_nn(Q + nstart * n, n, nupdate, Ri, nupdate, nupdate, T, n, 1.0, 0.0);
        x.copy_cols(T, n, Q + nstart * n, n, nupdate);
        continue;
      }
    }
    if (ncols - nstart > 1) {
      VGB_REQUIRE(ncols - nstart <= kGsMaxRange, "Gram-Schmidt: too many new columns in one step");
      int dev = 0, per_sm = 0;
      VGB_CUDA(cudaGetDevice(&dev));
      VGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, gs_columns_kernel, kGsThreads, 0));
      const int64_t want = std::max<int64_t>(1, ceil_div(n, (int64_t)kGsThreads));
      const unsigned nb = (unsigned)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)per_sm * sm_count()));
      x.gs_part.resize(2 * (size_t)nb * kGsMaxRange + 2 * (size_t)nb);
      x.gs_bar.resize(2);
      x.gs_err.resize(1);
      VGB_CUDA(cudaMemsetAsync(x.gs_bar.get(), 0, 2 * sizeof(unsigned), x.s));
      VGB_CUDA(cudaMemsetAsync(x.gs_err.get(), 0, sizeof(int), x.s));
      double *Qp = Q;
      int64_t nn = n, ns = nstart, nc = ncols;
      int chk = pass == 1 ? 1 : 0;
      double *pp = x.gs_part.get(), *np = x.gs_part.get() + 2 * (size_t)nb * kGsMaxRange;
      unsigned *bc = x.gs_bar.get(), *bg = x.gs_bar.get() + 1;
      int *fl = flag.get(), *er = x.gs_err.get();
      void *args[] = {&Qp, &nn, &ns, &nc, &chk, &norms0, &pp, &np, &bc, &bg, &fl, &er};
      VGB_CUDA(cudaLaunchCooperativeKernel((void *)gs_columns_kernel, dim3(nb), dim3(kGsThreads), args, 0, x.s));
      column_kernel_ran = true;
    }
  }
  int hflag[2] = {0, 0};
  VGB_CUDA(cudaMemcpyAsync(&hflag[0], flag.get(), sizeof(int), cudaMemcpyDeviceToHost, x.s));
  if (column_kernel_ran)
    VGB_CUDA(cudaMemcpyAsync(&hflag[1], x.gs_err.get(), sizeof(int), cudaMemcpyDeviceToHost, x.s));
  VGB_CUDA(cudaStreamSynchronize(x.s));
  if (hflag[1]) fail(BSE_ERR_TIMEOUT, "Gram-Schmidt: grid barrier gave up");
  if (hflag[0]) fail(BSE_ERR_NUMERICAL, "Linear dependencies in Gram-Schmidt.");
}

// Products of the Davidson operator, timed with events on the solve's stream.
struct TimedApply {
  DeviceOperator &A;
  cudaStream_t s;
  int64_t n;
  DavidsonOutput &out;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double ms = 0.0;
  TimedApply(DeviceOperator &a, cudaStream_t st, int64_t nn, DavidsonOutput &o) : A(a), s(st), n(nn), out(o) {
    VGB_CUDA(cudaEventCreate(&ev0));
    VGB_CUDA(cudaEventCreate(&ev1));
  }
  ~TimedApply() {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }
  void operator()(const double *X, int64_t k, double *Y, bool fp64 = false) {
    if (k <= 0) return;
    VGB_CUDA(cudaEventRecord(ev0, s));
    if (fp64) A.apply_fp64(X, n, k, Y, n, s); else A.apply(X, n, k, Y, n, s);
    VGB_CUDA(cudaEventRecord(ev1, s));
    VGB_CUDA(cudaEventSynchronize(ev1));
    A.check(s);
    float t = 0.f;
    VGB_CUDA(cudaEventElapsedTime(&t, ev0, ev1));
    ms += t;
    out.matvec_columns += k;
    if (fp64) out.fp64_columns += k;
  }
};

// FP64 polish of a split-precision solve (no counterpart in the reference).  The split
// products agree with FP64 to about 1e-5 of the interaction part, which bounds how far the
// Davidson residuals of the split operator say anything about the FP64 operator.  Here the
// basis restarts from the neigen Ritz vectors q0 with FP64 products A V0; corrections
// (DPR/Olsen of the residuals, as computeCorrectionVector) are added with split products.
// The coupling of a correction t to the FP64 block is taken from the FP64 side,
// t^T (A V0), and a correction enters a Ritz vector with a coefficient of the size of the
// residual over the gap, so the split error reaches the residuals and Rayleigh quotients
// only as that coefficient times 1e-5: they are FP64 quantities for every practical purpose.
// SYMM: Rayleigh-Ritz on V^T A V.  HAM ([[A, B], [-B, -A]] = J S with S = [[A, B], [B, A]]
// symmetric, J = diag(I, -I)): the projected pencil (V^T S V, V^T J V), reduced through the
// Cholesky factor of V^T S V (positive definite for a stable BSE); the lowest positive roots.
// Returns false (nothing changed) when that factor does not exist.
bool fp64_polish(Ctx &x, TimedApply &apply, const double *Dd, const double *q0, int64_t neigen,
                 bool ham, int correction, double tol, int64_t max_iter, double *evecs_dev,
                 DavidsonOutput &out, int verbose) {
  const int64_t n = x.n;
  const int64_t np = std::min(neigen, n);
  const int64_t cap = std::max<int64_t>(np, std::min<int64_t>(n, 9 * np));
  const int64_t half = n / 2;
  cudaStream_t s = x.s;
  DeviceBuffer<double> V(n * cap), AV(n * cap), q(n * np), res(n * np), Ud, lamd, work, cbuf, tmp;
  DeviceBuffer<int64_t> colsd(std::max<int64_t>(np, 64));
  DeviceBuffer<int> flag(1), einfo(2);
  // projected matrices on the device (ld cap): SYMM V^T A V; HAM V^T S V (= V^T J A V) and V^T J V
  DeviceBuffer<double> Td(cap * cap), Jd, Wp, nud, Zd, eigw;
  if (ham) Jd.resize(cap * cap);
  // C (r x c, ldc) = V[:, a0:a0+r]^T J W[:, 0:c], J = diag(I, -I) on the two halves of the rows
  auto projJ = [&](const double *Va, int64_t r, const double *W, int64_t c, double *C, int64_t ldc) {
    x.gemm_tn(Va, n, r, W, n, c, C, ldc, 1.0, 0.0, half);
    x.gemm_tn(Va + half, n, r, W + half, n, c, C, ldc, -1.0, 1.0, half);
  };
  auto to_host = [&](const double *src, int64_t cnt) {
    std::vector<double> h(cnt);
    VGB_CUDA(cudaMemcpyAsync(h.data(), src, cnt * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    return h;
  };
  int64_t m = 0, old = 0;
  auto start_basis = [&](const double *qsrc) {
    x.copy_cols(qsrc, n, V.get(), n, np);
    if (ham) gramschmidt(x, V.get(), 0, np, work, flag);  // harmonic Ritz vectors are not orthogonal
    apply(V.get(), np, AV.get(), true);
    m = np;
    old = 0;
  };
  start_basis(q0);
  std::vector<double> lam(np);
  for (int64_t pit = 0; pit < max_iter; ++pit) {
    out.polish_iterations = pit + 1;
    // ---- projected matrices for the columns [old, m) ----
    if (!ham) {  // lower triangle on the device: coupling from the FP64 side, V_new^T (A V_old)
      const int64_t nv = m - old;
      if (old > 0) x.gemm_tn(V.get() + old * n, n, nv, AV.get(), n, old, Td.get() + old, cap, 1.0, 0.0);
      x.gemm_tn(V.get() + old * n, n, nv, AV.get() + old * n, n, nv, Td.get() + old + cap * old, cap, 1.0, 0.0);
    } else {  // S: lower triangle, coupling from the FP64 side; J: the new columns, mirrored
      const int64_t nv = m - old;
      if (old > 0) projJ(V.get() + old * n, nv, AV.get(), old, Td.get() + old, cap);
      projJ(V.get() + old * n, nv, AV.get() + old * n, nv, Td.get() + old + cap * old, cap);
      projJ(V.get(), m, V.get() + old * n, nv, Jd.get() + cap * old, cap);
      if (old > 0) {
        mirror_block_kernel<<<blocks_for(old * nv), 256, 0, s>>>(Jd.get(), cap, old, nv);
        VGB_LAUNCH_CHECK();
      }
    }
    // ---- Ritz pairs of the projected problem, on the device ----
    Ud.resize(m * np);
    lamd.resize(np);
    if (!ham) {
      eigw.resize(sym_eig_work_doubles(m, np));
      SymEigJob job;
      job.T = Td.get(); job.ldt = cap; job.m = m; job.nw = np;
      job.U = Ud.get(); job.ldu = m; job.lam = lamd.get(); job.work = eigw.get(); job.info = einfo.get();
      sym_eig_device(&job, 1, s);
    } else {
      // S = L L^T, eigenpairs of -L^-1 J L^-T: the np largest positive mu = 1 / omega
      Wp.resize(3 * m * m);
      nud.resize(np);
      Zd.resize(m * np);
      VGB_CUDA(cudaMemsetAsync(einfo.get(), 0, 2 * sizeof(int), s));
      pencil_reduce_device(Td.get(), Jd.get(), cap, m, Wp.get(), einfo.get(), s);
      int st = 0;
      VGB_CUDA(cudaMemcpyAsync(&st, einfo.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
      VGB_CUDA(cudaStreamSynchronize(s));
      if (st != 0) {
        if (pit == 0) return false;
        fail(BSE_ERR_NUMERICAL, "FP64 polish: projected S lost positive definiteness");
      }
      eigw.resize(sym_eig_work_doubles(m, np));
      SymEigJob job;
      job.T = Wp.get() + 2 * m * m; job.ldt = m; job.m = m; job.nw = np;
      job.U = Zd.get(); job.ldu = m; job.lam = nud.get(); job.work = eigw.get(); job.info = einfo.get() + 1;
      sym_eig_device(&job, 1, s);
      pencil_finish_device(Wp.get(), m, nud.get(), Zd.get(), np, Ud.get(), lamd.get(), einfo.get(), s);
      int st2[2] = {0, 0};
      VGB_CUDA(cudaMemcpyAsync(st2, einfo.get(), 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
      VGB_CUDA(cudaStreamSynchronize(s));
      if (st2[1] != 0) fail(BSE_ERR_NUMERICAL, "Small hermitian eigenvalue problem failed.");
      if (st2[0] != 0) {
        if (pit == 0) return false;
        fail(BSE_ERR_NUMERICAL, "FP64 polish: fewer positive roots than requested");
      }
    }
    // ---- Ritz vectors and residuals: q = V U, res = A V U - q lambda (normalised) ----
    x.gemm_nn(V.get(), n, m, Ud.get(), m, np, q.get(), n, 1.0, 0.0);
    x.gemm_nn(AV.get(), n, m, Ud.get(), m, np, res.get(), n, 1.0, 0.0);
    residual_kernel<<<blocks_for(n * np), 256, 0, s>>>(res.get(), q.get(), n, np, lamd.get());
    VGB_LAUNCH_CHECK();
    work.resize(2 * np + 8);
    if (ham) {
      x.coldots(q.get(), n, nullptr, 0, np, work.get(), true);
      x.scale_cols(res.get(), n, np, work.get());
      x.scale_cols(q.get(), n, np, work.get());
    }
    x.coldots(res.get(), n, nullptr, 0, np, work.get() + np, true);
    int einfo_h = 0;
    VGB_CUDA(cudaMemcpyAsync(lam.data(), lamd.get(), np * sizeof(double), cudaMemcpyDeviceToHost, s));
    if (!ham) VGB_CUDA(cudaMemcpyAsync(&einfo_h, einfo.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
    std::vector<double> resn = to_host(work.get() + np, np);
    if (einfo_h != 0) fail(BSE_ERR_NUMERICAL, "Small hermitian eigenvalue problem failed.");
    double maxres = 0.0;
    std::vector<int64_t> upd;
    std::vector<double> upd_lam;
    for (int64_t j = 0; j < np; ++j) {
      maxres = std::max(maxres, resn[j]);
      if (!(resn[j] < tol)) { upd.push_back(j); upd_lam.push_back(lam[j]); }
    }
    out.history_resnorm.push_back(maxres);
    if (verbose)
      fprintf(stderr, "[davidson] fp64 polish %3lld  search space %6lld  max residual %.3e\n",
              (long long)pit, (long long)m, maxres);
    const bool done = upd.empty();
    if (done || pit == max_iter - 1) {
      out.evals.assign(lam.begin(), lam.end());
      out.evals.resize(neigen, 0.0);
      out.info = done ? 0 : 1;
      out.max_residual = maxres;
      if (evecs_dev) x.copy_cols(q.get(), n, evecs_dev, n, np);
      if (!done) {
        for (int64_t j : upd) {
          out.evals[j] = 0.0;
          if (evecs_dev) VGB_CUDA(cudaMemsetAsync(evecs_dev + j * n, 0, n * sizeof(double), s));
        }
      }
      VGB_CUDA(cudaStreamSynchronize(s));
      return true;
    }
    // ---- corrections for the unconverged roots (computeCorrectionVector) ----
    const int64_t nupdate = (int64_t)upd.size();
    if (m + nupdate > cap) {  // restart on the current Ritz vectors with FP64 products
      DeviceBuffer<double> qk(n * np);
      x.copy_cols(q.get(), n, qk.get(), n, np);
      start_basis(qk.get());
      continue;
    }
    colsd.resize(std::max<int64_t>(nupdate, 64));
    tmp.resize(2 * nupdate * n + 2 * nupdate + 8);
    double *lamu = tmp.get();
    double *numd = lamu + nupdate, *dend = numd + nupdate + 4;
    double *dq = dend + nupdate + 4;
    VGB_CUDA(cudaMemcpyAsync(colsd.get(), upd.data(), nupdate * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpyAsync(lamu, upd_lam.data(), nupdate * sizeof(double), cudaMemcpyHostToDevice, s));
    double *Vnew = V.get() + m * n;
    const bool olsen = correction == 1;
    dpr_kernel<<<blocks_for(n * nupdate), 256, 0, s>>>(Vnew, n, res.get(), q.get(), n, Dd, colsd.get(), lamu,
                                                      nupdate, olsen ? 0 : 1, olsen ? dq : nullptr);
    VGB_LAUNCH_CHECK();
    if (olsen) {
      for (int64_t kk = 0; kk < nupdate; ++kk) {
        x.coldots(q.get() + upd[kk] * n, n, Vnew + kk * n, n, 1, numd + kk, false);
        x.coldots(q.get() + upd[kk] * n, n, dq + kk * n, n, 1, dend + kk, false);
      }
      olsen_finish_kernel<<<blocks_for(n * nupdate), 256, 0, s>>>(Vnew, n, q.get(), n, colsd.get(), numd, dend,
                                                                 nupdate);
      VGB_LAUNCH_CHECK();
    }
    work.resize(nupdate + 8);
    x.coldots(Vnew, n, nullptr, 0, nupdate, work.get(), true);
    x.scale_cols(Vnew, n, nupdate, work.get());
    gramschmidt(x, V.get(), m, m + nupdate, work, flag);
    apply(Vnew, nupdate, AV.get() + m * n, false);
    old = m;
    m += nupdate;
  }
  return true;
}

}  // namespace

void davidson_solve(DeviceOperator &A, int64_t neigen, const bse_davidson_options &opt,
                    const double *host_guess, int64_t guess_cols, double *evecs_dev,
                    DavidsonOutput &out, cudaStream_t s) {
  const auto t_start = std::chrono::steady_clock::now();
  // phase timing (verbose >= 2): synchronises at phase boundaries
  const bool phases = opt.verbose >= 2;
  double ph[6] = {0, 0, 0, 0, 0, 0};  // projection, small eig, ritz+residual, correction, GS, restart
  auto tick = std::chrono::steady_clock::now();
  auto mark = [&](int i) {
    if (!phases) return;
    cudaStreamSynchronize(s);
    const auto now = std::chrono::steady_clock::now();
    ph[i] += std::chrono::duration<double>(now - tick).count();
    tick = now;
  };
  const bool ham = opt.matrix_type == 1;
  const bool debug = getenv("VGB_DAVIDSON_DEBUG") != nullptr;
  const int64_t n = A.size();
  VGB_REQUIRE(neigen >= 1 && neigen <= n, "DavidsonSolver: neigen out of range");
  VGB_REQUIRE(opt.correction == 0 || opt.correction == 1, "not a valid Davidson correction method");
  VGB_REQUIRE(opt.update >= 0 && opt.update <= 2, "not a valid Davidson update");
  VGB_REQUIRE(opt.matrix_type == 0 || opt.matrix_type == 1, "not a valid Davidson matrix type");
  const int64_t iter_max = opt.iter_max > 0 ? opt.iter_max : 50;
  const double tol = opt.tolerance;
  int64_t max_space = opt.max_search_space;
  if (max_space < neigen) max_space = neigen * 5;
  if (max_space > n) max_space = n;  // checkOptions
  int64_t size_update;               // getSizeUpdate
  if (opt.update == 0) size_update = neigen;
  else if (opt.update == 1) size_update = neigen < 20 ? (int64_t)(1.5 * (double)neigen) : neigen + 10;
  else size_update = 2 * neigen;
  if (opt.size_update > 0) {
    VGB_REQUIRE(opt.size_update >= neigen, "DavidsonSolver: size_update smaller than neigen");
    size_update = opt.size_update;
  }
  size_update = std::min(size_update, n);
  bool polish = opt.fp64_polish != 0 && A.split_precision();
  A.fp64_products = opt.fp64_polish == 2 ? 1 : 0;

  int64_t restart_size, ncols;
  if (host_guess) {
    VGB_REQUIRE(guess_cols >= neigen, "DavidsonSolver::solve initial_guess has fewer columns than neigen.");
    restart_size = std::min(guess_cols, max_space);
    ncols = guess_cols;
  } else {
    VGB_REQUIRE(opt.initial_size == 0 || opt.initial_size >= neigen,
                "DavidsonSolver: initial search space smaller than neigen");
    restart_size = opt.initial_size > 0 ? opt.initial_size : 2 * neigen;
    ncols = restart_size;
  }
  VGB_REQUIRE(ncols <= n, "DavidsonSolver: initial search space larger than the operator");
  const int64_t cap = std::max(ncols, max_space) + 2 * size_update + restart_size + 2;
  const int64_t capc = std::min(cap, n + 2 * size_update + restart_size + 2);

  Ctx x;
  x.s = s;
  x.n = n;
  DeviceBuffer<double> V(n * capc), AV(n * capc), AAV, D(n), q, res, Ud, tmp, lamd, work, cbuf;
  // the projected matrices stay on the device (ld capc): T = V^T A V and, for HAM, B = V^T A A V
  DeviceBuffer<double> Td(capc * capc), Bd, eigw;
  DeviceBuffer<int64_t> colsd;
  DeviceBuffer<int> flag(1), einfo(2);
  if (ham) {
    AAV.resize(n * capc);
    Bd.resize(capc * capc);
  }
  VGB_CUDA(cudaMemsetAsync(V.get(), 0, n * capc * sizeof(double), s));

  TimedApply apply(A, s, n, out);

  // diagonal of the operator
  A.diagonal(D.get(), s);
  std::vector<double> Dh(n);
  VGB_CUDA(cudaMemcpyAsync(Dh.data(), D.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));

  if (host_guess) {
    VGB_CUDA(cudaMemcpyAsync(V.get(), host_guess, n * guess_cols * sizeof(double),
                             cudaMemcpyHostToDevice, s));
    gramschmidt(x, V.get(), 0, ncols, work, flag);
  } else {
    // setupInitialEigenvectors: unit vectors at the smallest diagonal entries
    // (SYMM) or from the middle of the sorted diagonal (HAM)
    std::vector<int64_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) { return Dh[a] < Dh[b]; });
    const int64_t ind0 = ham ? n / 2 : 0;
    VGB_REQUIRE(ind0 + ncols <= n, "DavidsonSolver: initial guess exceeds the operator size");
    std::vector<int64_t> rows(idx.begin() + ind0, idx.begin() + ind0 + ncols);
    colsd.resize(std::max<int64_t>(ncols, 64));
    VGB_CUDA(cudaMemcpyAsync(colsd.get(), rows.data(), ncols * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    set_unit_columns_kernel<<<blocks_for(ncols), 256, 0, s>>>(V.get(), n, colsd.get(), ncols);
    VGB_LAUNCH_CHECK();
  }

  const int64_t ldT = capc;
  int64_t nav = 0;  // columns of AV
  std::vector<double> lam, U, resn;
  std::vector<char> conv(size_update, 0);
  out.history_resnorm.clear();

  for (int64_t it = 0; it < iter_max; ++it) {
    out.iterations = it;
    // ---- updateProjection ----
    if (phases) { cudaStreamSynchronize(s); tick = std::chrono::steady_clock::now(); }
    {
      const int64_t old = (it == 0) ? 0 : nav, nvec = ncols - old;
      apply(V.get() + old * n, nvec, AV.get() + old * n, false);
      if (!ham) {
        // T[:, old:ncols] = V^T AV_new, T[old:ncols, :old] its transpose, in HBM
        x.gemm_tn(V.get(), n, ncols, AV.get() + old * n, n, nvec, Td.get() + ldT * old, ldT, 1.0, 0.0);
        if (old > 0) {
          mirror_block_kernel<<<blocks_for(old * nvec), 256, 0, s>>>(Td.get(), ldT, old, nvec);
          VGB_LAUNCH_CHECK();
        }
      } else {
        // T[:, old:ncols] = V^T AV_new, T[old:, :old] = V_new^T AV_old (updateProjection, HAM)
        x.gemm_tn(V.get(), n, ncols, AV.get() + old * n, n, nvec, Td.get() + ldT * old, ldT, 1.0, 0.0);
        if (old > 0) x.gemm_tn(V.get() + old * n, n, nvec, AV.get(), n, old, Td.get() + old, ldT, 1.0, 0.0);
        apply(AV.get() + old * n, nvec, AAV.get() + old * n);
        x.gemm_tn(V.get(), n, ncols, AAV.get() + old * n, n, nvec, Bd.get() + ldT * old, ldT, 1.0, 0.0);
        if (old > 0) x.gemm_tn(V.get() + old * n, n, nvec, AAV.get(), n, old, Bd.get() + old, ldT, 1.0, 0.0);
      }
      nav = ncols;
    }
    const int64_t m = ncols;
    const int64_t needed = std::min(m, std::max(restart_size, size_update));
    Ud.resize(m * needed);
    lamd.resize(needed);

    mark(0);
    // ---- getRitzEigenPairs ----
    if (!ham) {
      // Ritz problem on the device (small_eig.cu): U and lambda never leave HBM
      eigw.resize(sym_eig_work_doubles(m, needed));
      SymEigJob job;
      job.T = Td.get(); job.ldt = ldT; job.m = m; job.nw = needed;
      job.U = Ud.get(); job.ldu = m; job.lam = lamd.get(); job.work = eigw.get(); job.info = einfo.get();
      sym_eig_device(&job, 1, s);
    } else {
      // harmonic-Ritz pencil (T, B) on the device (gen_eig.cu)
      eigw.resize(gen_eig_work_doubles(m, needed));
      GenEigJob job;
      job.T = Td.get(); job.B = Bd.get(); job.ldt = ldT; job.m = m; job.nw = needed;
      job.U = Ud.get(); job.ldu = m; job.lam = lamd.get(); job.work = eigw.get(); job.info = einfo.get();
      gen_eig_device(&job, 1, s);
    }
    mark(1);
    // q = V U, res = AV U - q Lambda
    q.resize(n * needed);
    res.resize(n * needed);
    x.gemm_nn(V.get(), n, m, Ud.get(), m, needed, q.get(), n, 1.0, 0.0);
    x.gemm_nn(AV.get(), n, m, Ud.get(), m, needed, res.get(), n, 1.0, 0.0);
    residual_kernel<<<blocks_for(n * needed), 256, 0, s>>>(res.get(), q.get(), n, needed, lamd.get());
    VGB_LAUNCH_CHECK();

    mark(2);
    // ---- checkConvergence ----
    const int64_t nn_check = std::min(needed, size_update);
    work.resize(std::max<int64_t>(needed, 1) + 8);
    x.coldots(res.get(), n, nullptr, 0, nn_check, work.get(), true);
    resn.assign(nn_check, 0.0);
    VGB_CUDA(cudaMemcpyAsync(resn.data(), work.get(), nn_check * sizeof(double), cudaMemcpyDeviceToHost, s));
    // the Ritz values come back with the residual norms (one synchronisation)
    int einfo_h[2] = {0, 0};
    lam.assign(needed, 0.0);
    VGB_CUDA(cudaMemcpyAsync(lam.data(), lamd.get(), needed * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaMemcpyAsync(einfo_h, einfo.get(), (ham ? 2 : 1) * sizeof(int), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    if (!ham && einfo_h[0] != 0) fail(BSE_ERR_NUMERICAL, "Small hermitian eigenvalue problem failed.");
    if (ham && einfo_h[0] == 4)
      fail(BSE_ERR_NUMERICAL, "Eigenvalue:" + std::to_string(einfo_h[1]) + " is complex but has no partner.");
    if (ham && einfo_h[0] != 0) fail(BSE_ERR_NUMERICAL, "Small generalized eigenvalue problem failed.");
    for (int64_t j = 0; j < size_update; ++j) conv[j] = (j < nn_check) ? (resn[j] < tol) : 0;
    bool converged = true;
    double maxres = 0.0;
    for (int64_t j = 0; j < neigen; ++j) {
      if (!conv[j]) converged = false;
      if (j < nn_check) maxres = std::max(maxres, resn[j]);
    }
    out.history_resnorm.push_back(maxres);
    if (opt.verbose)
      fprintf(stderr, "[davidson] iter %4lld  search space %6lld  max residual %.3e\n",
              (long long)it, (long long)ncols, maxres);
    const bool last = it == iter_max - 1;
    out.max_residual = maxres;
    // split-precision residuals that meet the tolerance, or have not halved in three iterations
    // (the floor of the split products), or the last iteration
    const size_t nh = out.history_resnorm.size();
    const bool stalled = nh > 3 && maxres > 0.5 * out.history_resnorm[nh - 4];
    if (polish && (converged || stalled || last)) {
      const auto tp0 = std::chrono::steady_clock::now();
      const int64_t pmax = std::max<int64_t>(iter_max, 20);
      const bool ran = fp64_polish(x, apply, D.get(), q.get(), neigen, ham, opt.correction, tol, pmax, evecs_dev,
                                   out, opt.verbose);
      out.seconds_polish = std::chrono::duration<double>(std::chrono::steady_clock::now() - tp0).count();
      if (ran) {
        out.polished = 1;
        break;
      }
      polish = false;  // the projected S of a HAM problem was not positive definite: carry on as is
    }
    if (converged || last) {
      // storeEigenPairs (+ zeroing of unconverged roots on the last iteration)
      out.evals.assign(lam.begin(), lam.begin() + std::min(neigen, needed));
      out.evals.resize(neigen, 0.0);
      out.info = converged ? 0 : 1;
      if (evecs_dev) {
        const int64_t nc = std::min(neigen, needed);
        x.copy_cols(q.get(), n, evecs_dev, n, nc);
        x.coldots(evecs_dev, n, nullptr, 0, nc, work.get(), true);
        x.scale_cols(evecs_dev, n, nc, work.get());
        if (!converged)
          for (int64_t j = 0; j < neigen; ++j)
            if (j >= nc || !conv[j])
              VGB_CUDA(cudaMemsetAsync(evecs_dev + j * n, 0, n * sizeof(double), s));
      }
      if (!converged)
        for (int64_t j = 0; j < neigen; ++j)
          if (!conv[j]) out.evals[j] = 0.0;
      break;
    }

    // ---- extendProjection ----
    std::vector<int64_t> upd;
    std::vector<double> upd_lam;
    for (int64_t j = 0; j < size_update; ++j)
      if (!conv[j] && j < needed) { upd.push_back(j); upd_lam.push_back(lam[j]); }
    const int64_t nupdate = (int64_t)upd.size();
    VGB_REQUIRE(ncols + nupdate <= capc, "DavidsonSolver: search space capacity exceeded");
    colsd.resize(std::max<int64_t>(nupdate, 64));
    tmp.resize(2 * nupdate * n + 2 * nupdate + 8);
    double *lamu = tmp.get();
    double *numd = lamu + nupdate, *dend = numd + nupdate + 4;
    double *dq = dend + nupdate + 4;
    VGB_CUDA(cudaMemcpyAsync(colsd.get(), upd.data(), nupdate * sizeof(int64_t), cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpyAsync(lamu, upd_lam.data(), nupdate * sizeof(double), cudaMemcpyHostToDevice, s));
    double *Vnew = V.get() + ncols * n;
    const bool olsen = opt.correction == 1;
    dpr_kernel<<<blocks_for(n * nupdate), 256, 0, s>>>(Vnew, n, res.get(), q.get(), n, D.get(),
                                                      colsd.get(), lamu, nupdate, olsen ? 0 : 1,
                                                      olsen ? dq : nullptr);
    VGB_LAUNCH_CHECK();
    if (olsen) {
      // num_k = q_j . delta_k ; den_k = q_j . dpr(q_j)   (signs applied in the finish kernel)
      for (int64_t kk = 0; kk < nupdate; ++kk) {
        x.coldots(q.get() + upd[kk] * n, n, Vnew + kk * n, n, 1, numd + kk, false);
        x.coldots(q.get() + upd[kk] * n, n, dq + kk * n, n, 1, dend + kk, false);
      }
      olsen_finish_kernel<<<blocks_for(n * nupdate), 256, 0, s>>>(Vnew, n, q.get(), n, colsd.get(),
                                                                 numd, dend, nupdate);
      VGB_LAUNCH_CHECK();
    }
    // w.normalized()
    work.resize(nupdate + 8);
    x.coldots(Vnew, n, nullptr, 0, nupdate, work.get(), true);
    x.scale_cols(Vnew, n, nupdate, work.get());
    if (debug) {
      std::vector<double> wn(nupdate);
      VGB_CUDA(cudaMemcpyAsync(wn.data(), work.get(), nupdate * sizeof(double), cudaMemcpyDeviceToHost, s));
      DeviceBuffer<double> G(nupdate * nupdate);
      x.gemm_tn(Vnew, n, nupdate, Vnew, n, nupdate, G.get(), nupdate, 1.0, 0.0);
      std::vector<double> Gh(nupdate * nupdate);
      VGB_CUDA(cudaMemcpyAsync(Gh.data(), G.get(), Gh.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      VGB_CUDA(cudaStreamSynchronize(s));
      fprintf(stderr, "[davidson-debug] corrections: cols");
      for (auto c : upd) fprintf(stderr, " %lld", (long long)c);
      fprintf(stderr, "\n[davidson-debug] norms before normalise:");
      for (auto v : wn) fprintf(stderr, " %.3e", v);
      fprintf(stderr, "\n[davidson-debug] max offdiag overlap of new columns:");
      for (int64_t c = 0; c < nupdate; ++c) {
        double mo = 0; int64_t arg = -1;
        for (int64_t r = 0; r < nupdate; ++r) if (r != c && std::fabs(Gh[r + nupdate * c]) > mo) { mo = std::fabs(Gh[r + nupdate * c]); arg = r; }
        fprintf(stderr, " %lld:%.3f(%lld)", (long long)c, mo, (long long)arg);
      }
      fprintf(stderr, "\n");
    }
    mark(3);
    gramschmidt(x, V.get(), ncols, ncols + nupdate, work, flag);
    ncols += nupdate;
    mark(4);
    if (debug) {
      DeviceBuffer<double> G(ncols * ncols);
      x.gemm_tn(V.get(), n, ncols, V.get(), n, ncols, G.get(), ncols, 1.0, 0.0);
      std::vector<double> Gh(ncols * ncols);
      VGB_CUDA(cudaMemcpyAsync(Gh.data(), G.get(), Gh.size() * sizeof(double), cudaMemcpyDeviceToHost, s));
      VGB_CUDA(cudaStreamSynchronize(s));
      double off = 0.0;
      int64_t worst = -1;
      for (int64_t c = 0; c < ncols; ++c)
        for (int64_t r = 0; r < ncols; ++r) {
          const double d = std::fabs(Gh[r + ncols * c] - (r == c ? 1.0 : 0.0));
          if (d > off) { off = d; worst = r + ncols * c; }
        }
      fprintf(stderr, "[davidson-debug] after GS: ncols %lld  max|V^T V - I| %.3e at (%lld,%lld)\n",
              (long long)ncols, off, (long long)(worst % ncols), (long long)(worst / ncols));
    }

    // ---- restart ----
    if (ncols > max_space) {
      struct M5 { decltype(mark) &m; ~M5() { m(5); } } m5_{mark};
      const int64_t rs = restart_size, nv = nupdate;
      VGB_REQUIRE(rs <= needed, "DavidsonSolver: restart size exceeds the Ritz pairs");
      DeviceBuffer<double> keep(n * nv), avn(n * rs);
      x.copy_cols(V.get() + (ncols - nv) * n, n, keep.get(), n, nv);
      if (!ham) {
        x.copy_cols(q.get(), n, V.get(), n, rs);
        x.gemm_nn(AV.get(), n, nav, Ud.get(), m, rs, avn.get(), n, 1.0, 0.0);
        x.copy_cols(avn.get(), n, AV.get(), n, rs);
      } else {
        // DavidsonSolver::qr of the kept harmonic Ritz coefficients, on the device
        DeviceBuffer<double> Od(m * rs), vn(n * rs);
        orthonormalise_device(Ud.get(), m, m, rs, Od.get(), m, s);
        x.gemm_nn(V.get(), n, nav, Od.get(), m, rs, vn.get(), n, 1.0, 0.0);
        x.gemm_nn(AV.get(), n, nav, Od.get(), m, rs, avn.get(), n, 1.0, 0.0);
        x.copy_cols(vn.get(), n, V.get(), n, rs);
        x.copy_cols(avn.get(), n, AV.get(), n, rs);
        x.gemm_nn(AAV.get(), n, nav, Od.get(), m, rs, avn.get(), n, 1.0, 0.0);
        x.copy_cols(avn.get(), n, AAV.get(), n, rs);
      }
      x.copy_cols(keep.get(), n, V.get() + rs * n, n, nv);
      ncols = rs + nv;
      nav = rs;
      // T = V[:, :rs]^T AV (and B = V^T AAV for HAM)
      x.gemm_tn(V.get(), n, rs, AV.get(), n, rs, Td.get(), ldT, 1.0, 0.0);
      if (ham) x.gemm_tn(V.get(), n, rs, AAV.get(), n, rs, Bd.get(), ldT, 1.0, 0.0);
    }
  }
  VGB_CUDA(cudaStreamSynchronize(s));
  const double matvec_ms = apply.ms;
  if (phases)
    fprintf(stderr,
            "[davidson] phases (s): projection+matvec %.4f (matvec %.4f)  small-eig %.4f  ritz %.4f  "
            "correction %.4f  gram-schmidt %.4f  restart %.4f\n",
            ph[0], matvec_ms * 1e-3, ph[1], ph[2], ph[3], ph[4], ph[5]);
  out.seconds_matvec = matvec_ms * 1e-3;
  out.seconds_total =
      std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
}

}  // namespace vgb
