// C ABI of the library (declarations and reference mapping: include/votca_gb300_bse.h).
#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <cstring>
#include <vector>
#include <memory>
#include <string>

#include "bse_ops.cuh"
#include "batch_davidson.cuh"
#include "davidson.cuh"
#include "small_eig.cuh"
#include "tc_engine.cuh"
#include "uks_ops.cuh"

struct bse_handle {
  int kind = 0;  // 0: BSE operator, 1: dense operator, 2: unrestricted (UKS) BSE operator
  std::unique_ptr<vgb::BseOperator> bse;
  std::unique_ptr<vgb::DenseOperator> dense;
  std::unique_ptr<vgb::UksOperator> uks;
  cudaStream_t stream = nullptr;
  vgb::DeviceBuffer<double> dX, dY, dD;
  int64_t size() const { return kind == 0 ? bse->dim : kind == 2 ? uks->dim : dense->n; }
  void matmul(const vgb::Coef &c, const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
              cudaStream_t s) {
    if (kind == 0) bse->matmul(c, X, ldx, k, Y, ldy, s);
    else if (kind == 2) uks->matmul(c, X, ldx, k, Y, ldy, s);
    else dense->matmul(X, ldx, k, Y, ldy, s);
  }
  void diagonal(const vgb::Coef &c, double *D, cudaStream_t s) {
    if (kind == 0) bse->diagonal(c, D, s);
    else if (kind == 2) uks->diagonal(c, D, s);
    else dense->diagonal(D, s);
  }
  void check_errors(cudaStream_t s) {
    if (kind == 0) bse->check_errors(s);
    else if (kind == 2) uks->check_errors(s);
  }
};

namespace {

thread_local std::string g_last_error;

template <typename F>
int guarded(F &&f) {
  try {
    f();
    g_last_error.clear();
    return BSE_OK;
  } catch (const vgb::Error &e) {
    g_last_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_last_error = "host allocation failed";
    return BSE_ERR_OUT_OF_MEMORY;
  } catch (const std::exception &e) {
    g_last_error = e.what();
    return BSE_ERR_ARGUMENT;
  }
}

vgb::Coef coef(int32_t a, int32_t b, int32_t c, int32_t d) {
  vgb::Coef k;
  k.cqp = a; k.cx = b; k.cd = c; k.cd2 = d;
  return k;
}

void require_handle(const bse_handle *h) { VGB_REQUIRE(h != nullptr, "null handle"); }

struct TmpStream {
  cudaStream_t s = nullptr;
  TmpStream() { VGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)); }
  ~TmpStream() { if (s) cudaStreamDestroy(s); }
};

void create_stream(bse_handle *h) {
  VGB_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
}

}  // namespace

namespace {

// P = X + Y, M = X - Y (dim x nr, leading dimensions ldx and dim)
__global__ void plus_minus_kernel(const double *X, const double *Y, int64_t ldx, int64_t dim, int64_t nr,
                                  double *P, double *M) {
  const int64_t total = dim * nr;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % dim, k = t / dim;
    const double x = X[i + ldx * k], y = Y[i + ldx * k];
    P[t] = x + y;
    M[t] = x - y;
  }
}

// The Hellmann-Feynman gradient of sum_k g_k Omega_k into device block buffers (any may be null):
// TDA (Y == nullptr): quadratic forms of the eigenvectors X under H(a); full BSE: X^T dA X +
// Y^T dA Y (weights g) plus 2 X^T dB Y as the quadratic forms of X + Y and X - Y under H(b)
// (weights g/2 and -g/2).  X, Y device, leading dimension ldx.
void eig_gradient_blocks(vgb::BseOperator &op, const vgb::Coef &a, const vgb::Coef *b, const double *X,
                         const double *Y, int64_t ldx, int64_t nr, const double *g, double *gvc, double *gcv,
                         double *gvv, double *gcc, double *gh, double *gw, cudaStream_t s) {
  op.quad_gradient(a, X, ldx, nr, g, gvc, gcv, gvv, gcc, gh, gw, false, s);
  if (!Y) return;
  op.quad_gradient(a, Y, ldx, nr, g, gvc, gcv, gvv, gcc, gh, gw, true, s);
  std::vector<double> half(2 * nr);
  for (int64_t k = 0; k < nr; ++k) {
    half[k] = 0.5 * g[k];
    half[nr + k] = -0.5 * g[k];
  }
  vgb::DeviceBuffer<double> PM(2 * op.dim * nr);
  plus_minus_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(vgb::ceil_div(op.dim * nr, 256), 2432)),
                      256, 0, s>>>(X, Y, ldx, op.dim, nr, PM.get(), PM.get() + op.dim * nr);
  VGB_LAUNCH_CHECK();
  op.quad_gradient(*b, PM.get(), op.dim, 2 * nr, half.data(), gvc, gcv, gvv, gcc, gh, gw, true, s);
}

// Host-pointer gradient: the Mmn-shaped gradient, the Hqp window and the screening (any may be null).
void eig_gradient_host(bse_handle *h, const vgb::Coef &a, const vgb::Coef *b, const double *X, const double *Y,
                       int64_t ldx, int64_t nroots, const double *weights, double *grad_mmn, double *grad_hqp,
                       double *grad_screening) {
  vgb::BseOperator &op = *h->bse;
  VGB_REQUIRE(ldx >= op.dim, "bse_op_eig_gradient: ldx smaller than the operator size");
  cudaStream_t s = h->stream;
  const int64_t vt = op.vt, ct = op.ct, naux = op.naux, dim = op.dim;
  vgb::DeviceBuffer<double> dX(dim * nroots), dY, gMvc, gMcv, gMvv, gMcc, gH, gW;
  VGB_CUDA(cudaMemcpy2DAsync(dX.get(), dim * sizeof(double), X, ldx * sizeof(double), dim * sizeof(double),
                             nroots, cudaMemcpyHostToDevice, s));
  if (Y) {
    dY.resize(dim * nroots);
    VGB_CUDA(cudaMemcpy2DAsync(dY.get(), dim * sizeof(double), Y, ldx * sizeof(double), dim * sizeof(double),
                               nroots, cudaMemcpyHostToDevice, s));
  }
  if (grad_mmn) {
    gMvc.resize(naux * dim);
    gMcv.resize(naux * dim);
    gMvv.resize(naux * vt * vt);
    gMcc.resize(naux * ct * ct);
  }
  const int64_t nh = (vt + ct) * (vt + ct);
  const int64_t nw = op.dense_screening ? naux * naux : naux;
  if (grad_hqp) gH.resize(nh);
  if (grad_screening) gW.resize(nw);
  eig_gradient_blocks(op, a, b, dX.get(), Y ? dY.get() : nullptr, dim, nroots, weights, gMvc.get(), gMcv.get(),
                      gMvv.get(), gMcc.get(), gH.get(), gW.get(), s);
  if (grad_hqp) VGB_CUDA(cudaMemcpy(grad_hqp, gH.get(), nh * sizeof(double), cudaMemcpyDeviceToHost));
  if (grad_screening) VGB_CUDA(cudaMemcpy(grad_screening, gW.get(), nw * sizeof(double), cudaMemcpyDeviceToHost));
  if (grad_mmn) vgb::scatter_mmn_gradient(op, gMvc.get(), gMcv.get(), gMvv.get(), gMcc.get(), grad_mmn, s);
}

}  // namespace

extern "C" {

const char *bse_last_error(void) { return g_last_error.c_str(); }

const char *bse_version(void) { return "votca_gb300 0.1 (sm_103a)"; }

static int create_impl(const bse_mmn_desc *mmn, const double *const *slices, const double *w,
                       bool dense_w, const double *hqp, int64_t ldh, int64_t hqp_size,
                       const bse_options *opt, int32_t precision, bse_handle **out) {
  return guarded([&] {
    VGB_REQUIRE(mmn && slices && w && hqp && opt && out, "bse_op_create: null argument");
    *out = nullptr;
    std::unique_ptr<bse_handle> h(new bse_handle());
    h->kind = 0;
    create_stream(h.get());
    vgb::AllocStreamScope alloc_scope(h->stream);
    h->bse.reset(new vgb::BseOperator());
    try {
      h->bse->stage(*mmn, slices, w, dense_w, hqp, ldh, hqp_size, *opt, precision, h->stream);
    } catch (...) {
      h->bse.reset();  // frees on the handle stream, before it goes away
      cudaStreamSynchronize(h->stream);
      cudaStreamDestroy(h->stream);
      h->stream = nullptr;
      throw;
    }
    *out = h.release();
  });
}

int bse_op_create(const bse_mmn_desc *mmn, const double *const *mmn_slices,
                  const double *epsilon_0_inv, const double *hqp, int64_t ldh,
                  int64_t hqp_size, const bse_options *opt, int32_t precision,
                  bse_handle **out) {
  return create_impl(mmn, mmn_slices, epsilon_0_inv, false, hqp, ldh, hqp_size, opt, precision, out);
}

int bse_op_create_dense_screening(const bse_mmn_desc *mmn, const double *const *mmn_slices,
                                  const double *W, const double *hqp, int64_t ldh,
                                  int64_t hqp_size, const bse_options *opt, int32_t precision,
                                  bse_handle **out) {
  return create_impl(mmn, mmn_slices, W, true, hqp, ldh, hqp_size, opt, precision, out);
}

static int uks_create_impl(const bse_mmn_desc *mmn_alpha, const double *const *mmn_alpha_slices,
                           const bse_mmn_desc *mmn_beta, const double *const *mmn_beta_slices,
                           const double *epsilon_0_inv, bool dense_w, const double *hqp_alpha,
                           int64_t ldh_alpha, int64_t hqp_alpha_size, const double *hqp_beta,
                           int64_t ldh_beta, int64_t hqp_beta_size, const bse_uks_options *opt,
                           int32_t precision, bse_handle **out) {
  return guarded([&] {
    VGB_REQUIRE(mmn_alpha && mmn_alpha_slices && mmn_beta && mmn_beta_slices && epsilon_0_inv && hqp_alpha &&
                    hqp_beta && opt && out,
                "bse_uks_op_create: null argument");
    *out = nullptr;
    std::unique_ptr<bse_handle> h(new bse_handle());
    h->kind = 2;
    create_stream(h.get());
    vgb::AllocStreamScope alloc_scope(h->stream);
    h->uks.reset(new vgb::UksOperator());
    try {
      h->uks->stage(*mmn_alpha, mmn_alpha_slices, *mmn_beta, mmn_beta_slices, epsilon_0_inv, dense_w,
                    hqp_alpha, ldh_alpha, hqp_alpha_size, hqp_beta, ldh_beta, hqp_beta_size, *opt, precision,
                    h->stream);
    } catch (...) {
      h->uks.reset();
      cudaStreamSynchronize(h->stream);
      cudaStreamDestroy(h->stream);
      h->stream = nullptr;
      throw;
    }
    *out = h.release();
  });
}

int bse_uks_op_create(const bse_mmn_desc *mmn_alpha, const double *const *mmn_alpha_slices,
                      const bse_mmn_desc *mmn_beta, const double *const *mmn_beta_slices,
                      const double *epsilon_0_inv, const double *hqp_alpha, int64_t ldh_alpha,
                      int64_t hqp_alpha_size, const double *hqp_beta, int64_t ldh_beta,
                      int64_t hqp_beta_size, const bse_uks_options *opt, int32_t precision,
                      bse_handle **out) {
  return uks_create_impl(mmn_alpha, mmn_alpha_slices, mmn_beta, mmn_beta_slices, epsilon_0_inv, false, hqp_alpha,
                         ldh_alpha, hqp_alpha_size, hqp_beta, ldh_beta, hqp_beta_size, opt, precision, out);
}

int bse_uks_op_create_dense_screening(const bse_mmn_desc *mmn_alpha, const double *const *mmn_alpha_slices,
                                      const bse_mmn_desc *mmn_beta, const double *const *mmn_beta_slices,
                                      const double *W, const double *hqp_alpha, int64_t ldh_alpha,
                                      int64_t hqp_alpha_size, const double *hqp_beta, int64_t ldh_beta,
                                      int64_t hqp_beta_size, const bse_uks_options *opt, int32_t precision,
                                      bse_handle **out) {
  return uks_create_impl(mmn_alpha, mmn_alpha_slices, mmn_beta, mmn_beta_slices, W, true, hqp_alpha, ldh_alpha,
                         hqp_alpha_size, hqp_beta, ldh_beta, hqp_beta_size, opt, precision, out);
}

int bse_dense_op_create(const double *a, const double *b, int64_t n, int64_t lda,
                        bse_handle **out) {
  return guarded([&] {
    VGB_REQUIRE(out != nullptr, "bse_dense_op_create: null out");
    *out = nullptr;
    std::unique_ptr<bse_handle> h(new bse_handle());
    h->kind = 1;
    create_stream(h.get());
    vgb::AllocStreamScope alloc_scope(h->stream);
    h->dense.reset(new vgb::DenseOperator());
    try {
      h->dense->stage(a, b, n, lda, h->stream);
    } catch (...) {
      h->dense.reset();
      cudaStreamSynchronize(h->stream);
      cudaStreamDestroy(h->stream);
      h->stream = nullptr;
      throw;
    }
    *out = h.release();
  });
}

int bse_op_destroy(bse_handle *h) {
  return guarded([&] {
    if (!h) return;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cudaStream_t s = h->stream;
    {
      vgb::AllocStreamScope alloc_scope(s);
      delete h;
    }
    if (s) {
      cudaStreamSynchronize(s);
      cudaStreamDestroy(s);
    }
    vgb::trim_pool();
  });
}

int bse_op_size(const bse_handle *h, int64_t *size) {
  return guarded([&] {
    require_handle(h);
    VGB_REQUIRE(size != nullptr, "bse_op_size: null out");
    *size = h->size();
  });
}

int bse_op_matmul_device(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd, int32_t cd2,
                         const double *dX, int64_t ldx, int64_t k, double *dY, int64_t ldy,
                         void *stream) {
  return guarded([&] {
    require_handle(h);
    h->matmul(coef(cqp, cx, cd, cd2), dX, ldx, k, dY, ldy, (cudaStream_t)stream);
  });
}

int bse_op_matmul_device_noalloc(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd,
                                 int32_t cd2, const double *dX, int64_t ldx, int64_t k,
                                 double *dY, int64_t ldy, void *stream) {
  return guarded([&] {
    require_handle(h);
    VGB_REQUIRE(h->kind == 0, "bse_op_matmul_device_noalloc: not a BSE operator");
    vgb::matmul_noalloc(*h->bse, coef(cqp, cx, cd, cd2), dX, ldx, k, dY, ldy, (cudaStream_t)stream);
  });
}

int bse_op_matmul(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd, int32_t cd2,
                  const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy) {
  return guarded([&] {
    require_handle(h);
    vgb::AllocStreamScope alloc_scope(h->stream);
    const int64_t n = h->size();
    VGB_REQUIRE(X && Y, "bse_op_matmul: null matrix");
    VGB_REQUIRE(ldx >= n && ldy >= n && k >= 0, "bse_op_matmul: bad leading dimension or k");
    if (k == 0) return;
    h->dX.resize(n * k);
    h->dY.resize(n * k);
    cudaStream_t s = h->stream;
    VGB_CUDA(cudaMemcpy2DAsync(h->dX.get(), n * sizeof(double), X, ldx * sizeof(double),
                               n * sizeof(double), k, cudaMemcpyHostToDevice, s));
    h->matmul(coef(cqp, cx, cd, cd2), h->dX.get(), n, k, h->dY.get(), n, s);
    VGB_CUDA(cudaMemcpy2DAsync(Y, ldy * sizeof(double), h->dY.get(), n * sizeof(double),
                               n * sizeof(double), k, cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    h->check_errors(s);
  });
}

int bse_op_diagonal_device(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd, int32_t cd2,
                           double *dD, void *stream) {
  return guarded([&] {
    require_handle(h);
    h->diagonal(coef(cqp, cx, cd, cd2), dD, (cudaStream_t)stream);
  });
}

int bse_op_diagonal(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd, int32_t cd2, double *D) {
  return guarded([&] {
    require_handle(h);
    vgb::AllocStreamScope alloc_scope(h->stream);
    VGB_REQUIRE(D != nullptr, "bse_op_diagonal: null output");
    const int64_t n = h->size();
    h->dD.resize(n);
    cudaStream_t s = h->stream;
    h->diagonal(coef(cqp, cx, cd, cd2), h->dD.get(), s);
    VGB_CUDA(cudaMemcpyAsync(D, h->dD.get(), n * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
  });
}

int bse_ham_matmul(bse_handle *h, const int32_t a_coef[4], const int32_t b_coef[4],
                   const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy) {
  return guarded([&] {
    require_handle(h);
    vgb::AllocStreamScope alloc_scope(h->stream);
    const int64_t n = 2 * h->size();
    VGB_REQUIRE(X && Y, "bse_ham_matmul: null matrix");
    VGB_REQUIRE(ldx >= n && ldy >= n && k >= 0, "bse_ham_matmul: bad leading dimension or k");
    if (k == 0) return;
    h->dX.resize(n * k);
    h->dY.resize(n * k);
    cudaStream_t s = h->stream;
    VGB_CUDA(cudaMemcpy2DAsync(h->dX.get(), n * sizeof(double), X, ldx * sizeof(double),
                               n * sizeof(double), k, cudaMemcpyHostToDevice, s));
    if (h->kind == 0 || h->kind == 2) {
      VGB_REQUIRE(a_coef && b_coef, "bse_ham_matmul: null coefficients");
      const vgb::Coef a = coef(a_coef[0], a_coef[1], a_coef[2], a_coef[3]);
      const vgb::Coef b = coef(b_coef[0], b_coef[1], b_coef[2], b_coef[3]);
      if (h->kind == 0) h->bse->ham_matmul(a, b, h->dX.get(), n, k, h->dY.get(), n, s);
      else h->uks->ham_matmul(a, b, h->dX.get(), n, k, h->dY.get(), n, s);
    } else {
      h->dense->ham_matmul(h->dX.get(), n, k, h->dY.get(), n, s);
    }
    VGB_CUDA(cudaMemcpy2DAsync(Y, ldy * sizeof(double), h->dY.get(), n * sizeof(double),
                               n * sizeof(double), k, cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    h->check_errors(s);
  });
}

int bse_davidson_solve(bse_handle *h, const int32_t a_coef[4], const int32_t b_coef[4],
                       const bse_davidson_options *opt, int64_t neigen, const double *guess,
                       int64_t guess_cols, double *evals, double *evecs, int64_t ldv,
                       bse_davidson_result *result) {
  return guarded([&] {
    require_handle(h);
    vgb::AllocStreamScope alloc_scope(h->stream);
    VGB_REQUIRE(opt != nullptr, "bse_davidson_solve: null options");
    const bool ham = opt->matrix_type == 1;
    std::unique_ptr<vgb::DeviceOperator> op;
    if (h->kind == 0 || h->kind == 2) {
      VGB_REQUIRE(a_coef != nullptr, "bse_davidson_solve: null operator coefficients");
      vgb::Coef a = coef(a_coef[0], a_coef[1], a_coef[2], a_coef[3]);
      vgb::Coef b;
      if (ham) {
        VGB_REQUIRE(b_coef != nullptr, "bse_davidson_solve: HAM needs B coefficients");
        b = coef(b_coef[0], b_coef[1], b_coef[2], b_coef[3]);
      }
      if (h->kind == 0) {
        if (ham) op.reset(new vgb::BseHamApply(h->bse.get(), a, b));
        else op.reset(new vgb::BseApply(h->bse.get(), a));
      } else {
        if (ham) op.reset(new vgb::UksHamApply(h->uks.get(), a, b));
        else op.reset(new vgb::UksApply(h->uks.get(), a));
      }
    } else {
      VGB_REQUIRE(!ham || h->dense->has_b, "bse_davidson_solve: HAM needs a B block");
      op.reset(new vgb::DenseApply(h->dense.get(), ham));
    }
    const int64_t n = op->size();
    VGB_REQUIRE(evecs == nullptr || ldv >= n, "bse_davidson_solve: ldv smaller than the operator size");
    vgb::DeviceBuffer<double> devecs;
    if (evecs) devecs.resize(n * neigen);
    vgb::DavidsonOutput o;
    vgb::davidson_solve(*op, neigen, *opt, guess, guess_cols, evecs ? devecs.get() : nullptr, o,
                        h->stream);
    if (evals) std::memcpy(evals, o.evals.data(), neigen * sizeof(double));
    if (evecs) {
      VGB_CUDA(cudaMemcpy2DAsync(evecs, ldv * sizeof(double), devecs.get(), n * sizeof(double),
                                 n * sizeof(double), neigen, cudaMemcpyDeviceToHost, h->stream));
      VGB_CUDA(cudaStreamSynchronize(h->stream));
    }
    if (result) {
      result->iterations = o.iterations;
      result->info = o.info;
      result->polished = o.polished;
      result->matvec_columns = o.matvec_columns;
      result->seconds_matvec = o.seconds_matvec;
      result->seconds_total = o.seconds_total;
      result->max_residual = o.max_residual;
      result->fp64_columns = o.fp64_columns;
      result->polish_iterations = o.polish_iterations;
      result->seconds_polish = o.seconds_polish;
    }
  });
}

int bse_op_eig_gradient(bse_handle *h, int32_t cqp, int32_t cx, int32_t cd, int32_t cd2,
                        const double *X, int64_t ldx, int64_t nroots, const double *weights,
                        double *grad_mmn, double *grad_hqp, double *grad_screening) {
  return guarded([&] {
    require_handle(h);
    vgb::AllocStreamScope alloc_scope(h->stream);
    VGB_REQUIRE(h->kind == 0, "bse_op_eig_gradient: not a BSE operator");
    VGB_REQUIRE(X && weights && nroots >= 1, "bse_op_eig_gradient: null eigenvectors or weights");
    eig_gradient_host(h, coef(cqp, cx, cd, cd2), nullptr, X, nullptr, ldx, nroots, weights, grad_mmn, grad_hqp,
                      grad_screening);
  });
}

int bse_op_eig_gradient_full(bse_handle *h, const int32_t a_coef[4], const int32_t b_coef[4], const double *X,
                             const double *Y, int64_t ldx, int64_t nroots, const double *weights,
                             double *grad_mmn, double *grad_hqp, double *grad_screening) {
  return guarded([&] {
    require_handle(h);
    vgb::AllocStreamScope alloc_scope(h->stream);
    VGB_REQUIRE(h->kind == 0, "bse_op_eig_gradient_full: not a BSE operator");
    VGB_REQUIRE(a_coef && b_coef && X && Y && weights && nroots >= 1,
                "bse_op_eig_gradient_full: null argument");
    const vgb::Coef a = coef(a_coef[0], a_coef[1], a_coef[2], a_coef[3]);
    const vgb::Coef b = coef(b_coef[0], b_coef[1], b_coef[2], b_coef[3]);
    eig_gradient_host(h, a, &b, X, Y, ldx, nroots, weights, grad_mmn, grad_hqp, grad_screening);
  });
}

int bse_op_eig_gradient_device(bse_handle *h, const int32_t a_coef[4], const int32_t b_coef[4],
                               const double *dX, const double *dY, int64_t ldx, int64_t nroots,
                               const double *weights, double *d_grad_vc, double *d_grad_cv, double *d_grad_vv,
                               double *d_grad_cc, double *d_grad_hqp, double *d_grad_screening, void *stream) {
  return guarded([&] {
    require_handle(h);
    VGB_REQUIRE(h->kind == 0, "bse_op_eig_gradient_device: not a BSE operator");
    VGB_REQUIRE(a_coef && dX && weights && nroots >= 1, "bse_op_eig_gradient_device: null argument");
    VGB_REQUIRE(!dY || b_coef, "bse_op_eig_gradient_device: full BSE needs the B coefficients");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    vgb::AllocStreamScope alloc_scope(s);
    vgb::BseOperator &op = *h->bse;
    VGB_REQUIRE(ldx >= op.dim, "bse_op_eig_gradient_device: ldx smaller than the operator size");
    const vgb::Coef a = coef(a_coef[0], a_coef[1], a_coef[2], a_coef[3]);
    vgb::Coef b;
    if (dY) b = coef(b_coef[0], b_coef[1], b_coef[2], b_coef[3]);
    eig_gradient_blocks(op, a, dY ? &b : nullptr, dX, dY, ldx, nroots, weights, d_grad_vc, d_grad_cv, d_grad_vv,
                        d_grad_cc, d_grad_hqp, d_grad_screening, s);
  });
}

int bse_rpa_epsilon(const bse_mmn_desc *mmn, const double *const *mmn_slices,
                    const double *rpa_energies, int64_t rpatotal, int64_t homo, int64_t rpamin,
                    int64_t rpamax, double freq_re, double freq_im, double *epsilon) {
  return guarded([&] {
    VGB_REQUIRE(mmn && mmn_slices && rpa_energies && epsilon, "bse_rpa_epsilon: null argument");
    TmpStream ts;
    vgb::rpa_epsilon(*mmn, mmn_slices, rpa_energies, rpatotal, homo, rpamin, rpamax, freq_re, freq_im,
                     1e-4, epsilon, ts.s);
  });
}

int bse_cholesky_inverse(int64_t n, const double *A, int64_t lda, double *Ainv, int64_t ldi) {
  return guarded([&] {
    VGB_REQUIRE(A && Ainv, "bse_cholesky_inverse: null matrix");
    TmpStream ts;
    vgb::cholesky_inverse(n, A, lda, Ainv, ldi, ts.s);
  });
}

int bse_positive_inverse(int64_t n, const double *A, int64_t lda, double cutoff, double *W, int64_t ldw) {
  return guarded([&] {
    VGB_REQUIRE(A && W, "bse_positive_inverse: null matrix");
    TmpStream ts;
    vgb::positive_inverse(n, A, lda, cutoff, W, ldw, ts.s);
  });
}

int bse_mmn_multiply_right(const bse_mmn_desc *mmn, double *const *mmn_slices, const double *U,
                           int64_t ldu) {
  return guarded([&] {
    VGB_REQUIRE(mmn && mmn_slices && U, "bse_mmn_multiply_right: null argument");
    TmpStream ts;
    vgb::mmn_multiply_right(*mmn, mmn_slices, U, ldu, ts.s);
  });
}

int bse_mmn_fill_3c_mo(const bse_mmn_desc *mmn, double *const *mmn_slices, const double *ao3c, int64_t nbf,
                       const double *mo_coefficients, int64_t ldc, int64_t nmo) {
  return guarded([&] {
    VGB_REQUIRE(mmn && mmn_slices && ao3c && mo_coefficients, "bse_mmn_fill_3c_mo: null argument");
    TmpStream ts;
    vgb::fill_3c_mo(*mmn, mmn_slices, ao3c, nbf, mo_coefficients, ldc, nmo, ts.s);
  });
}

int bse_aux_pseudo_inv_sqrt(int64_t n, const double *V, int64_t ldv, double etol, double *out, int64_t ldo,
                            int64_t *removed) {
  return guarded([&] {
    VGB_REQUIRE(n >= 1 && V && out && ldv >= n && ldo >= n, "bse_aux_pseudo_inv_sqrt: bad arguments");
    TmpStream ts;
    vgb::aux_pseudo_inv_sqrt(n, V, ldv, etol, out, ldo, removed, ts.s);
  });
}

int bse_aux_pseudo_inv_sqrt_gwbse(int64_t n, const double *S, int64_t lds, const double *V, int64_t ldv,
                                  double etol, double *out, int64_t ldo, int64_t *removed) {
  return guarded([&] {
    VGB_REQUIRE(n >= 1 && S && V && out && lds >= n && ldv >= n && ldo >= n,
                "bse_aux_pseudo_inv_sqrt_gwbse: bad arguments");
    TmpStream ts;
    vgb::aux_pseudo_inv_sqrt_gwbse(n, S, lds, V, ldv, etol, out, ldo, removed, ts.s);
  });
}

int bse_transition_dipoles(const double *ao_dipoles, int64_t nbf, const double *mo_coefficients, int64_t ldc,
                           int64_t nmo, int64_t vmin, int64_t vtotal, int64_t cmin, int64_t ctotal,
                           const double *X, const double *Y, int64_t ldx, int64_t nstates, double prefactor,
                           int32_t accumulate, double *dipoles) {
  return guarded([&] {
    VGB_REQUIRE(ao_dipoles && mo_coefficients && X && dipoles, "bse_transition_dipoles: null argument");
    TmpStream ts;
    vgb::transition_dipoles(ao_dipoles, nbf, mo_coefficients, ldc, nmo, vmin, vtotal, cmin, ctotal, X, Y, ldx,
                            nstates, prefactor, accumulate != 0, dipoles, ts.s);
  });
}

int bse_davidson_solve_batch(bse_handle *const *handles, int64_t nhandles, const int32_t a_coef[4],
                             const int32_t b_coef[4], const bse_davidson_options *opt,
                             int64_t neigen, double *evals, int32_t *infos, int64_t *iterations,
                             int32_t nthreads) {
  return guarded([&] {
    VGB_REQUIRE(handles && opt && evals && nhandles >= 0, "bse_davidson_solve_batch: null argument");
    for (int64_t i = 0; i < nhandles; ++i) require_handle(handles[i]);
    if (nhandles == 0) return;
    if (nthreads <= 0) {
      // lockstep: every step one grouped launch over all molecules
      VGB_REQUIRE(a_coef != nullptr, "bse_davidson_solve_batch: null operator coefficients");
      std::vector<vgb::BseOperator *> ops;
      for (int64_t i = 0; i < nhandles; ++i) {
        VGB_REQUIRE(handles[i]->kind == 0, "bse_davidson_solve_batch: lockstep mode needs BSE operators");
        if (handles[i]->stream) VGB_CUDA(cudaStreamSynchronize(handles[i]->stream));
        ops.push_back(handles[i]->bse.get());
      }
      TmpStream ts;
      vgb::davidson_solve_batch(ops, coef(a_coef[0], a_coef[1], a_coef[2], a_coef[3]), neigen, *opt,
                                evals, infos, iterations, ts.s);
      return;
    }
    int dev = 0;
    VGB_CUDA(cudaGetDevice(&dev));
    const int nt = (int)std::max<int64_t>(1, std::min<int64_t>(nthreads > 0 ? nthreads : 8, nhandles));
    std::atomic<int64_t> next(0);
    std::mutex mu;
    int first_code = 0;
    int64_t first_index = nhandles;  // the lowest failing molecule is reported
    std::string first_msg;
    auto worker = [&] {
      cudaSetDevice(dev);
      for (;;) {
        const int64_t i = next.fetch_add(1);
        if (i >= nhandles) break;
        bse_davidson_result r;
        const int rc = bse_davidson_solve(handles[i], a_coef, b_coef, opt, neigen, nullptr, 0,
                                          evals + i * neigen, nullptr, 0, &r);
        if (rc != BSE_OK) {
          std::lock_guard<std::mutex> lock(mu);
          if (i < first_index) {
            first_index = i;
            first_code = rc;
            first_msg = "molecule " + std::to_string(i) + ": " + bse_last_error();
          }
          continue;
        }
        if (infos) infos[i] = r.info;
        if (iterations) iterations[i] = r.iterations;
      }
    };
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto &t : pool) t.join();
    if (first_code != 0) vgb::fail(first_code, first_msg);
  });
}

int bse_op_profile(bse_handle *h, int32_t enable) {
  return guarded([&] {
    require_handle(h);
    VGB_REQUIRE(h->kind == 0, "bse_op_profile: not a BSE operator");
    h->bse->timer.enable(enable != 0);
  });
}

int bse_op_profile_read(bse_handle *h, double *stage_ms, int64_t *stage_calls, int32_t nstages) {
  return guarded([&] {
    require_handle(h);
    VGB_REQUIRE(h->kind == 0, "bse_op_profile_read: not a BSE operator");
    h->bse->timer.read(stage_ms, stage_calls, nstages);
  });
}

int bse_probe_fp64_tflops(double *tflops) {
  return guarded([&] {
    VGB_REQUIRE(tflops != nullptr, "bse_probe_fp64_tflops: null out");
    *tflops = vgb::probe_fp64_tflops();
  });
}

int bse_small_sym_eig(int64_t njobs, const int64_t *m, const int64_t *nw, const double *T, double *evals,
                      double *evecs, int64_t *phase_cycles) {
  return guarded([&] {
    VGB_REQUIRE(njobs >= 0 && (njobs == 0 || (m && nw && T && evals && evecs)), "bse_small_sym_eig: null argument");
    int64_t nt = 0, nl = 0, nu = 0, wmax = 0;
    for (int64_t i = 0; i < njobs; ++i) {
      VGB_REQUIRE(m[i] >= 1 && m[i] <= vgb::kSymEigMaxM && nw[i] >= 1 && nw[i] <= m[i],
                  "bse_small_sym_eig: sizes out of range");
      nt += m[i] * m[i];
      nl += nw[i];
      nu += m[i] * nw[i];
      wmax += vgb::sym_eig_work_doubles(m[i], nw[i]);
    }
    if (njobs == 0) return;
    cudaStream_t s = nullptr;
    vgb::DeviceBuffer<double> dT(nt), dl(nl), dU(nu), dw(wmax);
    vgb::DeviceBuffer<int> dinfo(njobs);
    vgb::DeviceBuffer<long long> dclk(phase_cycles ? 5 * njobs : 0);
    VGB_CUDA(cudaMemcpyAsync(dT.get(), T, nt * sizeof(double), cudaMemcpyHostToDevice, s));
    std::vector<vgb::SymEigJob> jobs(njobs);
    int64_t ot = 0, ol = 0, ou = 0, ow = 0;
    for (int64_t i = 0; i < njobs; ++i) {
      vgb::SymEigJob &j = jobs[i];
      j.T = dT.get() + ot; j.ldt = m[i]; j.m = m[i]; j.nw = nw[i];
      j.U = dU.get() + ou; j.ldu = m[i]; j.lam = dl.get() + ol; j.work = dw.get() + ow; j.info = dinfo.get() + i;
      if (phase_cycles) j.clocks = dclk.get() + 5 * i;
      ot += m[i] * m[i]; ol += nw[i]; ou += m[i] * nw[i]; ow += vgb::sym_eig_work_doubles(m[i], nw[i]);
    }
    vgb::sym_eig_device(jobs.data(), njobs, s);
    std::vector<int> info(njobs);
    VGB_CUDA(cudaMemcpyAsync(evals, dl.get(), nl * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaMemcpyAsync(evecs, dU.get(), nu * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaMemcpyAsync(info.data(), dinfo.get(), njobs * sizeof(int), cudaMemcpyDeviceToHost, s));
    std::vector<long long> clk(phase_cycles ? 5 * njobs : 0);
    if (phase_cycles)
      VGB_CUDA(cudaMemcpyAsync(clk.data(), dclk.get(), clk.size() * sizeof(long long), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    for (int64_t i = 0; i < njobs; ++i)
      if (info[i] != 0) vgb::fail(BSE_ERR_NUMERICAL, "Small hermitian eigenvalue problem failed.");
    if (phase_cycles)
      for (int64_t i = 0; i < njobs; ++i)
        for (int p = 0; p < 4; ++p) phase_cycles[4 * i + p] = clk[5 * i + p + 1] - clk[5 * i + p];
  });
}

int bse_autotune_report(char *buf, int64_t cap, int64_t *needed) {
  return guarded([&] {
    const std::string r = vgb::autotune_report();
    if (needed) *needed = (int64_t)r.size() + 1;
    if (buf && cap > 0) {
      const size_t n = std::min<size_t>((size_t)cap - 1, r.size());
      memcpy(buf, r.data(), n);
      buf[n] = 0;
    }
  });
}

int bse_small_gen_eig(int64_t m, int64_t nw, const double *T, const double *B, double *evals, double *evecs,
                      int64_t *selected) {
  return guarded([&] {
    VGB_REQUIRE(T && B && evals && evecs, "bse_small_gen_eig: null argument");
    VGB_REQUIRE(m >= 1 && m <= vgb::kGenEigMaxM && nw >= 1 && nw <= m, "bse_small_gen_eig: sizes out of range");
    cudaStream_t s = nullptr;
    vgb::DeviceBuffer<double> dT(m * m), dB(m * m), dl(nw), dU(m * nw), dw(vgb::gen_eig_work_doubles(m, nw));
    vgb::DeviceBuffer<int> dinfo(2);
    VGB_CUDA(cudaMemcpyAsync(dT.get(), T, m * m * sizeof(double), cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpyAsync(dB.get(), B, m * m * sizeof(double), cudaMemcpyHostToDevice, s));
    vgb::GenEigJob j;
    j.T = dT.get(); j.B = dB.get(); j.ldt = m; j.m = m; j.nw = nw;
    j.U = dU.get(); j.ldu = m; j.lam = dl.get(); j.work = dw.get(); j.info = dinfo.get();
    vgb::gen_eig_device(&j, 1, s);
    int info[2] = {0, 0};
    VGB_CUDA(cudaMemcpyAsync(evals, dl.get(), nw * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaMemcpyAsync(evecs, dU.get(), m * nw * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaMemcpyAsync(info, dinfo.get(), 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
    if (info[0] == 4)
      vgb::fail(BSE_ERR_NUMERICAL, "Eigenvalue:" + std::to_string(info[1]) + " is complex but has no partner.");
    if (info[0] != 0) vgb::fail(BSE_ERR_NUMERICAL, "Small generalized eigenvalue problem failed.");
    if (selected) *selected = info[1];
  });
}

}  // extern "C"
