// Screening that feeds the direct interaction Hd, in FP64 on the GPU.
//
//   rpa_epsilon            RPA::calculate_epsilon_r (xtp/src/libxtp/gwbse/rpa.cc:145-200):
//                          eps = 1 - 2 sum_m M_m^T diag(chi_m) M_m over occupied m, unoccupied c,
//                          chi = (w - dE)/((w - dE)^2 + (wi + eta)^2) - (w + dE)/((w + dE)^2 + (wi - eta)^2)
//                          as one weighted SYRK-shaped GEMM over the (m, c) pairs.
//   cholesky_inverse       eps^-1 = L^-T L^-1 with eps = L L^T: the dense screening W that
//                          bse_op_create_dense_screening folds into the vv block.  It replaces
//                          the host eigen-decomposition of BSE::SetupDirectInteractionOperator
//                          (bse.cc:188-204, eigenvectors rotate Mmn, epsilon_0_inv = 1/lambda):
//                          sum_PQ M^P (eps^-1)_PQ M^Q equals the rotated-diagonal form.
//   mmn_multiply_right     TCMatrix_gwbse::MultiplyRightWithAuxMatrix (threecenter.cc:54-65):
//                          every slice M[m] <- M[m] U.
#include <cmath>
#include <vector>

#include "dgemm.cuh"
#include "host_eig.hpp"

namespace vgb {

namespace {

constexpr int NB = 64;  // Cholesky block

unsigned g1d(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 16LL * 152));
}

// B[(m, c)][P] = M(rpamin+m, lumo+c, P) scaled by -2 chi_{m,c}  (Bw) and unscaled (B)
__global__ void rpa_weights_kernel(const double *raw, int64_t n_occ_chunk, int64_t m0, int64_t n_unocc,
                                   int64_t naux, int64_t nsize, int64_t row0,
                                   const double *energies, int64_t lumo_idx, double wr, double wi,
                                   double eta, double *B, double *Bw, int64_t ldb) {
  const int64_t total = n_occ_chunk * n_unocc * naux;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t c = t % n_unocc;
    const int64_t P = (t / n_unocc) % naux;
    const int64_t mi = t / (n_unocc * naux);
    const double x = raw[(mi * naux + P) * nsize + row0 + c];
    const double dE = energies[lumo_idx + c] - energies[m0 + mi];
    const double dm = wr - dE, dp = wr + dE;
    const double s1 = (wi + eta) * (wi + eta), s2 = (wi - eta) * (wi - eta);
    const double chi = dm / (dm * dm + s1) - dp / (dp * dp + s2);
    const int64_t row = mi * n_unocc + c;
    B[row + ldb * P] = x;
    Bw[row + ldb * P] = -2.0 * chi * x;
  }
}

__global__ void add_identity_kernel(double *A, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    A[i + n * i] += 1.0;
}

// Unblocked Cholesky of the nb x nb diagonal block at A + j (lda), lower triangle;
// the strict upper triangle of the block is zeroed.  One CTA, block in shared memory.
__global__ void potrf_block_kernel(double *A, int64_t lda, int nb, int *info, int64_t j0) {
  __shared__ double a[NB][NB + 1];
  const int t = threadIdx.x;
  for (int e = t; e < nb * nb; e += blockDim.x) a[e % nb][e / nb] = A[(e % nb) + lda * (e / nb)];
  __syncthreads();
  for (int k = 0; k < nb; ++k) {
    if (t == 0) {
      const double d = a[k][k];
      if (!(d > 0.0)) { if (*info == 0) *info = (int)(j0 + k + 1); a[k][k] = 1.0; }
      else a[k][k] = sqrt(d);
    }
    __syncthreads();
    const double dk = a[k][k];
    for (int i = k + 1 + t; i < nb; i += blockDim.x) a[i][k] /= dk;
    __syncthreads();
    for (int e = t; e < (nb - k - 1) * (nb - k - 1); e += blockDim.x) {
      const int i = k + 1 + e % (nb - k - 1), jj = k + 1 + e / (nb - k - 1);
      if (jj <= i) a[i][jj] -= a[i][k] * a[jj][k];
    }
    __syncthreads();
  }
  for (int e = t; e < nb * nb; e += blockDim.x) {
    const int i = e % nb, jj = e / nb;
    A[i + lda * jj] = (jj <= i) ? a[i][jj] : 0.0;
  }
}

// Inverse of the nb x nb lower-triangular block L (lda) into Li (ld nb): column j
// by forward substitution, one thread per column.
__global__ void trtri_block_kernel(const double *L, int64_t lda, int nb, double *Li) {
  __shared__ double l[NB][NB + 1];
  for (int e = threadIdx.x; e < nb * nb; e += blockDim.x) l[e % nb][e / nb] = L[(e % nb) + lda * (e / nb)];
  __syncthreads();
  const int j = threadIdx.x;
  if (j < nb) {
    double x[NB];
    for (int i = 0; i < nb; ++i) {
      double s = (i == j) ? 1.0 : 0.0;
      for (int p = j; p < i; ++p) s -= l[i][p] * x[p];
      x[i] = (i < j) ? 0.0 : s / l[i][i];
    }
    for (int i = 0; i < nb; ++i) Li[i + nb * j] = x[i];
  }
}

__global__ void set_identity_rows_kernel(double *Y, int64_t n, int64_t i0, int64_t nb) {
  // Y[i0:i0+nb, :] = E (identity rows), leaves other rows untouched
  const int64_t total = nb * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % nb, c = t / nb;
    Y[(i0 + r) + n * c] = (i0 + r == c) ? 1.0 : 0.0;
  }
}

}  // namespace

void rpa_epsilon(const bse_mmn_desc &desc, const double *const *slices, const double *energies,
                 int64_t rpatotal, int64_t homo, int64_t rpamin, int64_t rpamax, double wr, double wi,
                 double eta, double *eps_host, cudaStream_t s) {
  const int64_t naux = desc.auxsize;
  const int64_t lumo = homo + 1;
  const int64_t n_occ = lumo - rpamin, n_unocc = rpamax - lumo + 1;
  const int64_t nsize = desc.nmax - desc.nmin + 1;
  VGB_REQUIRE(n_occ >= 1 && n_unocc >= 1, "rpa_epsilon: empty occupied or unoccupied range");
  VGB_REQUIRE(rpatotal == rpamax - rpamin + 1, "rpa_epsilon: energies must cover rpamin..rpamax");
  VGB_REQUIRE(desc.mmin <= rpamin && desc.mmax >= homo, "rpa_epsilon: Mmn m-range misses occupied levels");
  VGB_REQUIRE(nsize >= n_unocc, "rpa_epsilon: Mmn n-range shorter than the unoccupied range");
  DeviceBuffer<double> dE(rpatotal), eps(naux * naux);
  VGB_CUDA(cudaMemcpyAsync(dE.get(), energies, rpatotal * sizeof(double), cudaMemcpyHostToDevice, s));
  // occupied levels in chunks so that the pair matrices stay below ~1 GB
  const int64_t per_m = n_unocc * naux;
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(n_occ, (64LL << 20) / std::max<int64_t>(per_m, 1)));
  DeviceBuffer<double> raw(chunk * naux * nsize), B(chunk * per_m), Bw(chunk * per_m);
  GemmWorkspace ws;
  for (int64_t m0 = 0; m0 < n_occ; m0 += chunk) {
    const int64_t cnt = std::min(chunk, n_occ - m0);
    for (int64_t i = 0; i < cnt; ++i) {
      const double *src = slices[rpamin + m0 + i - desc.mmin];
      VGB_REQUIRE(src != nullptr, "rpa_epsilon: null Mmn slice");
      VGB_CUDA(cudaMemcpyAsync(raw.get() + i * naux * nsize, src, naux * nsize * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    }
    const int64_t rows = cnt * n_unocc;
    // Mmn_[m].bottomRows(n_unocc), as the reference reads it
    rpa_weights_kernel<<<g1d(rows * naux), 256, 0, s>>>(raw.get(), cnt, m0, n_unocc, naux, nsize,
                                                        nsize - n_unocc, dE.get(), lumo - rpamin, wr,
                                                        wi, eta, B.get(), Bw.get(), rows);
    VGB_LAUNCH_CHECK();
    GemmDesc g;  // eps (+)= B^T Bw
    g.M = naux; g.N = naux; g.K = rows;
    g.a_colmajor(B.get(), rows, true).b_colmajor(Bw.get(), rows, false).c_colmajor(eps.get(), naux);
    g.beta = m0 > 0 ? 1.0 : 0.0;
    dgemm(g, s, &ws);
    VGB_CUDA(cudaStreamSynchronize(s));
  }
  add_identity_kernel<<<g1d(naux), 256, 0, s>>>(eps.get(), naux);
  VGB_LAUNCH_CHECK();
  VGB_CUDA(cudaMemcpyAsync(eps_host, eps.get(), naux * naux * sizeof(double), cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
}

void cholesky_inverse(int64_t n, const double *a_host, int64_t lda, double *inv_host, int64_t ldi,
                      cudaStream_t s) {
  VGB_REQUIRE(n >= 1 && lda >= n && ldi >= n, "cholesky_inverse: bad size");
  DeviceBuffer<double> A(n * n), Y(n * n), Li(NB * NB), T(NB * n);
  DeviceBuffer<int> info(1);
  GemmWorkspace ws;
  VGB_CUDA(cudaMemcpy2DAsync(A.get(), n * sizeof(double), a_host, lda * sizeof(double),
                             n * sizeof(double), n, cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaMemsetAsync(info.get(), 0, sizeof(int), s));
  // right-looking blocked Cholesky: A = L L^T (lower)
  for (int64_t j = 0; j < n; j += NB) {
    const int nb = (int)std::min<int64_t>(NB, n - j);
    double *Ajj = A.get() + j + n * j;
    potrf_block_kernel<<<1, 256, 0, s>>>(Ajj, n, nb, info.get(), j);
    VGB_LAUNCH_CHECK();
    const int64_t rest = n - j - nb;
    if (rest > 0) {
      trtri_block_kernel<<<1, NB, 0, s>>>(Ajj, n, nb, Li.get());
      VGB_LAUNCH_CHECK();
      // L21 = A21 L11^-T
      double *A21 = A.get() + (j + nb) + n * j;
      GemmDesc t;
      t.M = rest; t.N = nb; t.K = nb;
      t.a_colmajor(A21, n, false).b_colmajor(Li.get(), nb, true).c_colmajor(T.get(), rest);
      dgemm(t, s, &ws);
      VGB_CUDA(cudaMemcpy2DAsync(A21, n * sizeof(double), T.get(), rest * sizeof(double),
                                 rest * sizeof(double), nb, cudaMemcpyDeviceToDevice, s));
      // A22 -= L21 L21^T
      GemmDesc u;
      u.M = rest; u.N = rest; u.K = nb;
      u.a_colmajor(A21, n, false).b_colmajor(A21, n, true).c_colmajor(A.get() + (j + nb) + n * (j + nb), n);
      u.alpha = -1.0; u.beta = 1.0;
      dgemm(u, s, &ws);
    }
  }
  int hinfo = 0;
  VGB_CUDA(cudaMemcpyAsync(&hinfo, info.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
  if (hinfo != 0)
    fail(BSE_ERR_NUMERICAL, "cholesky_inverse: matrix is not positive definite (pivot " +
                                std::to_string(hinfo) + ")");
  // Y = L^-1 by block forward substitution over block rows: Y_i = L_ii^-1 (E_i - L_i,<i Y_<i)
  // (upper blocks of L were zeroed, so whole block rows can be used)
  VGB_CUDA(cudaMemsetAsync(Y.get(), 0, n * n * sizeof(double), s));
  for (int64_t i = 0; i < n; i += NB) {
    const int nb = (int)std::min<int64_t>(NB, n - i);
    set_identity_rows_kernel<<<g1d(nb * n), 256, 0, s>>>(Y.get(), n, i, nb);
    VGB_LAUNCH_CHECK();
    if (i > 0) {  // Y_i -= L[i, 0:i] Y[0:i, :]
      GemmDesc g;
      g.M = nb; g.N = n; g.K = i;
      g.a_colmajor(A.get() + i, n, false).b_colmajor(Y.get(), n, false).c_colmajor(Y.get() + i, n);
      g.alpha = -1.0; g.beta = 1.0;
      dgemm(g, s, &ws);
    }
    trtri_block_kernel<<<1, NB, 0, s>>>(A.get() + i + n * i, n, nb, Li.get());
    VGB_LAUNCH_CHECK();
    GemmDesc h;  // Y_i = L_ii^-1 Y_i
    h.M = nb; h.N = n; h.K = nb;
    h.a_colmajor(Li.get(), nb, false).b_colmajor(Y.get() + i, n, false).c_colmajor(T.get(), nb);
    dgemm(h, s, &ws);
    VGB_CUDA(cudaMemcpy2DAsync(Y.get() + i, n * sizeof(double), T.get(), nb * sizeof(double),
                               nb * sizeof(double), n, cudaMemcpyDeviceToDevice, s));
  }
  // A^-1 = L^-T L^-1 = Y^T Y
  GemmDesc f;
  f.M = n; f.N = n; f.K = n;
  f.a_colmajor(Y.get(), n, true).b_colmajor(Y.get(), n, false).c_colmajor(A.get(), n);
  dgemm(f, s, &ws);
  VGB_CUDA(cudaMemcpy2DAsync(inv_host, ldi * sizeof(double), A.get(), n * sizeof(double),
                             n * sizeof(double), n, cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
}

void mmn_multiply_right(const bse_mmn_desc &desc, double *const *slices, const double *U_host,
                        int64_t ldu, cudaStream_t s) {
  const int64_t naux = desc.auxsize, nsize = desc.nmax - desc.nmin + 1;
  const int64_t msize = desc.mmax - desc.mmin + 1;
  VGB_REQUIRE(naux >= 1 && nsize >= 1 && msize >= 1 && ldu >= naux, "mmn_multiply_right: bad sizes");
  DeviceBuffer<double> U(naux * naux);
  VGB_CUDA(cudaMemcpy2DAsync(U.get(), naux * sizeof(double), U_host, ldu * sizeof(double),
                             naux * sizeof(double), naux, cudaMemcpyHostToDevice, s));
  const int64_t per = nsize * naux;
  const int64_t chunk = std::max<int64_t>(1, std::min<int64_t>(msize, (64LL << 20) / per));
  DeviceBuffer<double> in(chunk * per), out(chunk * per);
  GemmWorkspace ws;
  for (int64_t m0 = 0; m0 < msize; m0 += chunk) {
    const int64_t cnt = std::min(chunk, msize - m0);
    for (int64_t i = 0; i < cnt; ++i)
      VGB_CUDA(cudaMemcpyAsync(in.get() + i * per, slices[m0 + i], per * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    GemmDesc g;  // out[m] = in[m] U  (each nsize x naux column-major)
    g.M = nsize; g.N = naux; g.K = naux;
    g.a_colmajor(in.get(), nsize, false).b_colmajor(U.get(), naux, false).c_colmajor(out.get(), nsize);
    g.nb1 = cnt; g.a_b1 = per; g.c_b1 = per;
    dgemm(g, s, &ws);
    for (int64_t i = 0; i < cnt; ++i)
      VGB_CUDA(cudaMemcpyAsync(slices[m0 + i], out.get() + i * per, per * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
  }
}

// W = U diag(w) U^T with A = U diag(lambda) U^T and w = 1/lambda for lambda > cutoff, else 0:
// the screening of BSE::SetupDirectInteractionOperator (bse.cc:188-204: eigen-decomposition of
// eps, modes with lambda <= 1e-8 dropped) as one dense matrix.  The symmetric eigenproblem is
// solved on the host (as the reference does), the product U diag(w) U^T on the device.
void positive_inverse(int64_t n, const double *a_host, int64_t lda, double cutoff, double *inv_host,
                      int64_t ldi, cudaStream_t s) {
  VGB_REQUIRE(n >= 1 && lda >= n && ldi >= n, "positive_inverse: bad size");
  std::vector<double> A(n * n);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) A[i + n * j] = a_host[i + lda * j];
  std::vector<double> lam, U;
  if (!sym_eig(n, A.data(), lam, U)) fail(BSE_ERR_NUMERICAL, "positive_inverse: eigenvalue problem failed");
  std::vector<double> UW(n * n);
  for (int64_t j = 0; j < n; ++j) {
    const double w = lam[j] > cutoff ? 1.0 / lam[j] : 0.0;
    for (int64_t i = 0; i < n; ++i) UW[i + n * j] = U[i + n * j] * w;
  }
  DeviceBuffer<double> dU(n * n), dUW(n * n), dW(n * n);
  VGB_CUDA(cudaMemcpyAsync(dU.get(), U.data(), n * n * sizeof(double), cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaMemcpyAsync(dUW.get(), UW.data(), n * n * sizeof(double), cudaMemcpyHostToDevice, s));
  GemmDesc g;  // W = (U diag(w)) U^T
  g.M = n; g.N = n; g.K = n;
  g.A = dUW.get(); g.a_rs = 1; g.a_cs = n;
  g.B = dU.get(); g.b_rs = n; g.b_cs = 1;
  g.C = dW.get(); g.c_rs = 1; g.c_cs = n;
  GemmWorkspace ws;
  dgemm(g, s, &ws);
  VGB_CUDA(cudaMemcpy2DAsync(inv_host, ldi * sizeof(double), dW.get(), n * sizeof(double), n * sizeof(double), n,
                             cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace vgb
