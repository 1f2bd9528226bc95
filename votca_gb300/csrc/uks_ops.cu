// Unrestricted BSE operator: two spin channels plus the cross-spin products
// (xtp/src/libxtp/gwbse/bse_operator_uks.cc).
#include <algorithm>
#include <vector>

#include "uks_ops.cuh"

namespace vgb {

namespace {

// A spin channel without occupied (homo = vmin - 1) or without virtual (homo = cmax) levels in
// the BSE window carries an empty block: setup_block's size vtotal * ctotal is 0
// (bse_operator_uks.cc:25-35), and the operator is the other channel's alone.
bool channel_empty(const bse_uks_options &o, int64_t homo) {
  return homo - o.vmin + 1 == 0 || o.cmax - homo == 0;
}

bse_options channel_options(const bse_uks_options &o, int64_t homo) {
  bse_options r;
  r.homo = homo;
  r.rpamin = o.rpamin;
  r.qpmin = o.qpmin;
  r.vmin = o.vmin;
  r.cmax = o.cmax;
  return r;
}

// M(m, n, P) of a TCMatrix_gwbse given as host slices (slice m: column-major nsize x naux)
struct HostMmn {
  const bse_mmn_desc &d;
  const double *const *slices;
  double operator()(int64_t m, int64_t n, int64_t P) const {
    return slices[m - d.mmin][P * (d.nmax - d.nmin + 1) + (n - d.nmin)];
  }
};

// F[P][r][c] = (w ? w_P : 1) M(m0 + (mrow ? r : c), n0 + (mrow ? c : r), P): the factor blocks
// of the cross-spin Hd2 product, built on the host and uploaded once.
void stage_factor(const HostMmn &M, const double *w, int64_t naux, int64_t rows, int64_t cols,
                  int64_t m_first, int64_t n_first, bool m_is_row, DeviceBuffer<double> &out,
                  cudaStream_t s) {
  std::vector<double> h(naux * rows * cols);
  for (int64_t P = 0; P < naux; ++P) {
    const double wp = w ? w[P] : 1.0;
    for (int64_t r = 0; r < rows; ++r)
      for (int64_t c = 0; c < cols; ++c) {
        const int64_t m = m_first + (m_is_row ? r : c), n = n_first + (m_is_row ? c : r);
        h[(P * rows + r) * cols + c] = wp * M(m, n, P);
      }
  }
  out.resize(h.size());
  VGB_CUDA(cudaMemcpyAsync(out.get(), h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void UksOperator::stage(const bse_mmn_desc &desc_a, const double *const *slices_a,
                        const bse_mmn_desc &desc_b, const double *const *slices_b, const double *w,
                        bool dense_w, const double *hqp_a, int64_t ldh_a, int64_t size_a,
                        const double *hqp_b, int64_t ldh_b, int64_t size_b, const bse_uks_options &opt,
                        int prec, cudaStream_t s) {
  // BSE_OPERATOR_UKS::configure / setup_block, bse_operator_uks.cc:25-43
  VGB_REQUIRE(desc_a.auxsize == desc_b.auxsize, "bse_uks_op_create: alpha and beta Naux differ");
  VGB_REQUIRE(slices_a && slices_b && w && hqp_a && hqp_b, "bse_uks_op_create: null input");
  precision = prec;
  const bool ea = channel_empty(opt, opt.homo_alpha), eb = channel_empty(opt, opt.homo_beta);
  VGB_REQUIRE(!(ea && eb), "bse_uks_op_create: both spin channels have an empty BSE window");
  for (BseOperator *ch : {&alpha, &beta}) {
    const bool empty = ch == &alpha ? ea : eb;
    const int64_t homo = ch == &alpha ? opt.homo_alpha : opt.homo_beta;
    if (!empty) continue;
    ch->vt = homo - opt.vmin + 1;
    ch->ct = opt.cmax - homo;
    ch->naux = desc_a.auxsize;
    ch->dim = 0;
    ch->precision = prec;
  }
  if (!ea)
    alpha.stage(desc_a, slices_a, w, dense_w, hqp_a, ldh_a, size_a, channel_options(opt, opt.homo_alpha), prec, s);
  if (!eb)
    beta.stage(desc_b, slices_b, w, dense_w, hqp_b, ldh_b, size_b, channel_options(opt, opt.homo_beta), prec, s);
  dim = alpha.dim + beta.dim;
  // the cross-spin Hd2 blocks read each channel's Mmn over the other channel's ranges
  for (const bse_mmn_desc *d : {&desc_a, &desc_b}) {
    VGB_REQUIRE(opt.vmin >= d->mmin && opt.cmax <= d->mmax && opt.vmin >= d->nmin && opt.cmax <= d->nmax,
                "bse_uks_op_create: BSE window outside an Mmn range");
  }
  if (ea || eb) return;  // no cross-spin blocks
  const int64_t naux = alpha.naux;
  const HostMmn Ma{desc_a, slices_a}, Mb{desc_b, slices_b};
  const int64_t ca0 = opt.homo_alpha + 1, cb0 = opt.homo_beta + 1;
  // Xab[P][v1][c2] = M_b(vmin + v1, cb0 + c2), Yab[P][v2][c1] = w M_a(ca0 + c1, vmin + v2)
  const double *wd = dense_w ? nullptr : w;
  stage_factor(Mb, nullptr, naux, alpha.vt, beta.ct, opt.vmin, cb0, true, Xab, s);
  stage_factor(Ma, wd, naux, beta.vt, alpha.ct, ca0, opt.vmin, false, Yab, s);
  stage_factor(Ma, nullptr, naux, beta.vt, alpha.ct, opt.vmin, ca0, true, Xba, s);
  stage_factor(Mb, wd, naux, alpha.vt, beta.ct, cb0, opt.vmin, false, Yba, s);
  if (dense_w) {
    // Y(rc, Q) = sum_P Y(rc, P) W(P, Q): the screened factors carry the dense W
    DeviceBuffer<double> dW(naux * naux);
    VGB_CUDA(cudaMemcpyAsync(dW.get(), w, naux * naux * sizeof(double), cudaMemcpyHostToDevice, s));
    for (DeviceBuffer<double> *Y : {&Yab, &Yba}) {
      const int64_t rc = (int64_t)Y->count / naux;
      DeviceBuffer<double> tmp(rc * naux);
      GemmDesc g;
      g.M = rc; g.N = naux; g.K = naux;
      g.A = Y->get(); g.a_rs = 1; g.a_cs = rc;
      g.B = dW.get(); g.b_rs = 1; g.b_cs = naux;
      g.C = tmp.get(); g.c_rs = 1; g.c_cs = rc;
      dgemm(g, s, &ws_);
      VGB_CUDA(cudaMemcpyAsync(Y->get(), tmp.get(), rc * naux * sizeof(double), cudaMemcpyDeviceToDevice, s));
      VGB_CUDA(cudaStreamSynchronize(s));
    }
  }
}

// Yout += alpha sum_P Mcv_out[P][I1] (sum_I2 Bvc_in[P][I2] Xin[I2]):
// add_direct_cross_tda_block (bse_operator_uks.cc:179-218) with w folded into Mcv_out.
void UksOperator::cross_tda(const BseOperator &out, const BseOperator &in, double alpha_,
                            const double *Xin, int64_t ldx, int64_t k, double *Yout, int64_t ldy,
                            cudaStream_t s) {
  const int64_t naux = in.naux;
  Z_.resize(naux * k);
  GemmDesc g;  // Z (naux x k) = Bvc_in^T X_in
  g.M = naux; g.N = k; g.K = in.dim;
  g.A = in.Bvc.get(); g.a_rs = in.dim; g.a_cs = 1;
  g.B = Xin; g.b_rs = 1; g.b_cs = ldx;
  g.C = Z_.get(); g.c_rs = 1; g.c_cs = naux;
  dgemm(g, s, &ws_);
  GemmDesc h;  // Y_out += alpha Mcv_out Z
  h.M = out.dim; h.N = k; h.K = naux;
  h.A = out.Mcv.get(); h.a_rs = 1; h.a_cs = out.dim;
  h.B = Z_.get(); h.b_rs = 1; h.b_cs = naux;
  h.C = Yout; h.c_rs = 1; h.c_cs = ldy;
  h.alpha = alpha_; h.beta = 1.0;
  dgemm(h, s, &ws_);
}

// Yout(v1, c1) += alpha sum_{P, v2} Yf[P][v2][c1] sum_c2 Xf[P][v1][c2] Xin(v2, c2):
// add_direct2_block with Mout and Min of different spins (bse_operator_uks.cc:139-177).
void UksOperator::cross_hd2(const BseOperator &out, const BseOperator &in, const double *Xf,
                            const double *Yf, double alpha_, const double *Xin, int64_t ldx, int64_t k,
                            double *Yout, int64_t ldy, cudaStream_t s) {
  const int64_t naux = in.naux, vo = out.vt, co = out.ct, vi = in.vt, ci = in.ct;
  const int64_t per_vec = vo * naux * vi;
  const int64_t jchunk =
      std::max<int64_t>(1, std::min<int64_t>(k, u_budget_bytes_ / (per_vec * (int64_t)sizeof(double))));
  U_.resize(jchunk * per_vec);
  for (int64_t j0 = 0; j0 < k; j0 += jchunk) {
    const int64_t kc = std::min(jchunk, k - j0);
    GemmDesc a;  // U[j][v1][P][v2] = sum_c2 X_j(v2, c2) Xf_P(v1, c2)
    a.M = vi; a.N = vo; a.K = ci;
    a.A = Xin + j0 * ldx; a.a_rs = ci; a.a_cs = 1;
    a.B = Xf; a.b_rs = 1; a.b_cs = ci;
    a.C = U_.get(); a.c_rs = 1; a.c_cs = naux * vi;
    a.nb1 = kc; a.nb2 = naux;
    a.a_b1 = ldx; a.a_b2 = 0;
    a.b_b1 = 0; a.b_b2 = vo * ci;
    a.c_b1 = per_vec; a.c_b2 = vi;
    dgemm(a, s, &ws_);
    GemmDesc b;  // Y_j(c1, v1) += alpha sum_{P,v2} Yf(c1, (P,v2)) U_j((P,v2), v1)
    b.M = co; b.N = vo; b.K = naux * vi;
    b.A = Yf; b.a_rs = 1; b.a_cs = co;
    b.B = U_.get(); b.b_rs = 1; b.b_cs = naux * vi; b.b_b1 = per_vec;
    b.C = Yout + j0 * ldy; b.c_rs = 1; b.c_cs = co; b.c_b1 = ldy;
    b.nb1 = kc; b.alpha = alpha_; b.beta = 1.0;
    dgemm(b, s, &ws_);
  }
}

void UksOperator::matmul(const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y,
                         int64_t ldy, cudaStream_t s) {
  // BSE_OPERATOR_UKS::matmul, bse_operator_uks.cc:220-270
  VGB_REQUIRE(!(c.cd != 0 && c.cd2 != 0), "Hamiltonian cannot contain Hd and Hd2 at the same time");
  VGB_REQUIRE(ldx >= dim && ldy >= dim, "uks matmul: leading dimension too small");
  if (k == 0) return;
  const int64_t da = alpha.dim;
  if (alpha.dim > 0) alpha.matmul(c, X, ldx, k, Y, ldy, s);
  if (beta.dim > 0) beta.matmul(c, X + da, ldx, k, Y + da, ldy, s);
  if (alpha.dim == 0 || beta.dim == 0) return;  // an empty channel couples to nothing
  if (c.cd != 0) {
    cross_tda(alpha, beta, -(double)c.cd, X + da, ldx, k, Y, ldy, s);
    cross_tda(beta, alpha, -(double)c.cd, X, ldx, k, Y + da, ldy, s);
  }
  if (c.cd2 != 0) {
    cross_hd2(alpha, beta, Xab.get(), Yab.get(), -(double)c.cd2, X + da, ldx, k, Y, ldy, s);
    cross_hd2(beta, alpha, Xba.get(), Yba.get(), -(double)c.cd2, X, ldx, k, Y + da, ldy, s);
  }
}

void UksOperator::diagonal(const Coef &c, double *D, cudaStream_t s) {
  if (alpha.dim > 0) alpha.diagonal(c, D, s);
  if (beta.dim > 0) beta.diagonal(c, D + alpha.dim, s);
}

void UksOperator::ham_matmul(const Coef &a, const Coef &b, const double *X, int64_t ldx, int64_t k,
                             double *Y, int64_t ldy, cudaStream_t s) {
  VGB_REQUIRE(ldx >= 2 * dim && ldy >= 2 * dim, "uks ham_matmul: leading dimension too small");
  if (k == 0) return;
  // view X (2 dim x k) as dim x 2k (columns M1_0, M2_0, M1_1, ...)
  const double *Xr = X;
  if (ldx != 2 * dim) {
    hamX_.resize(2 * dim * k);
    copy_cols(X, ldx, 2 * dim, k, hamX_.get(), 2 * dim, s);
    Xr = hamX_.get();
  }
  hamA_.resize(2 * dim * k);
  hamB_.resize(2 * dim * k);
  matmul(a, Xr, dim, 2 * k, hamA_.get(), dim, s);
  matmul(b, Xr, dim, 2 * k, hamB_.get(), dim, s);
  ham_combine(hamA_.get(), hamB_.get(), dim, k, Y, ldy, s);
}

void UksOperator::check_errors(cudaStream_t s) {
  if (alpha.dim > 0) alpha.check_errors(s);
  if (beta.dim > 0) beta.check_errors(s);
}

}  // namespace vgb
