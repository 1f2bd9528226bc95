// Device-resident unrestricted (UKS) BSE operator.
//
// BSE_OPERATOR_UKS<cqp, cx, cd, cd2> (xtp/src/libxtp/gwbse/bse_operator_uks.cc) acts on
// [x_alpha; x_beta] (alpha pairs first, pair index v * ctotal + c within a spin block):
//   y_s  = (cqp Hqp_s + cx Hx_ss - cd Hd_ss - cd2 Hd2_ss) x_s               (same spin)
//        - cd  sum_P w_P t^s_P (t^s'_P . x_s')                              (cross, TDA)
//        - cd2 sum_P w_P M^s(c1, v2, P) M^s'(v1, c2, P) x_s'(v2, c2)        (cross, B block)
// with t^s_P(v, c) = M^s(c, v, P) for the output spin and M^s'(v, c, P) for the input spin
// (add_direct_cross_tda_block, :179-218; add_direct2_block with mixed spins, :139-177).
// The same-spin blocks are two BseOperator instances (one per spin channel, each with its own
// HOMO); the cross-spin products reuse their staged Bvc / Mcv blocks (TDA form) or four
// extra FP64 blocks staged here (B-block form).  The cross-spin products run in FP64 in both
// precision modes.
#pragma once

#include "bse_ops.cuh"

namespace vgb {

class UksOperator {
 public:
  BseOperator alpha, beta;
  int64_t dim = 0;  // alpha.dim + beta.dim
  int precision = BSE_PRECISION_FP64;
  // cross-spin Hd2 factors, [P][row][col] with col fastest:
  //   Xab[P][v1 < vt_a][c2 < ct_b] = M_b(vmin + v1, homo_b + 1 + c2, P)
  //   Yab[P][v2 < vt_b][c1 < ct_a] = w_P M_a(homo_a + 1 + c1, vmin + v2, P)
  //   Xba, Yba: the same with the spins exchanged
  DeviceBuffer<double> Xab, Yab, Xba, Yba;

  // Stage both spin channels from host data (see bse_uks_op_create).  w: the diagonal screening
  // (naux), or with dense_w a symmetric naux x naux W (column-major) folded into the screened
  // factors: sum_PQ M^P W_PQ M^Q in every direct term.
  void stage(const bse_mmn_desc &desc_a, const double *const *slices_a, const bse_mmn_desc &desc_b,
             const double *const *slices_b, const double *w, bool dense_w, const double *hqp_a,
             int64_t ldh_a, int64_t size_a, const double *hqp_b, int64_t ldh_b, int64_t size_b,
             const bse_uks_options &opt, int prec, cudaStream_t s);

  // Y = H(coef) X on device, X and Y dim x k (ldx, ldy >= dim).
  void matmul(const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
              cudaStream_t s);
  // same-spin diagonals only, as the reference's diagonal() (:283-352)
  void diagonal(const Coef &c, double *D, cudaStream_t s);
  // [[A, B], [-B, -A]] X, X and Y (2 dim) x k
  void ham_matmul(const Coef &a, const Coef &b, const double *X, int64_t ldx, int64_t k, double *Y,
                  int64_t ldy, cudaStream_t s);
  void check_errors(cudaStream_t s);

 private:
  DeviceBuffer<double> Z_, U_, hamA_, hamB_, hamX_;
  GemmWorkspace ws_;
  int64_t u_budget_bytes_ = 2LL << 30;
  void cross_tda(const BseOperator &out, const BseOperator &in, double alpha, const double *Xin,
                 int64_t ldx, int64_t k, double *Yout, int64_t ldy, cudaStream_t s);
  void cross_hd2(const BseOperator &out, const BseOperator &in, const double *Xf, const double *Yf,
                 double alpha, const double *Xin, int64_t ldx, int64_t k, double *Yout, int64_t ldy,
                 cudaStream_t s);
};

struct UksApply : DeviceOperator {
  UksOperator *op;
  Coef coef;
  UksApply(UksOperator *o, Coef c) : op(o), coef(c) {}
  int64_t size() const override { return op->dim; }
  void apply(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
             cudaStream_t s) override {
    op->matmul(coef, X, ldx, k, Y, ldy, s);
  }
  void diagonal(double *D, cudaStream_t s) override { op->diagonal(coef, D, s); }
  void check(cudaStream_t s) override { op->check_errors(s); }
  bool split_precision() const override { return op->precision == BSE_PRECISION_MIXED; }
  void apply_fp64(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                  cudaStream_t s) override {
    ForceFp64 g(&op->alpha, &op->beta, fp64_products);
    op->matmul(coef, X, ldx, k, Y, ldy, s);
  }
};

struct UksHamApply : DeviceOperator {
  UksOperator *op;
  Coef a, b;
  UksHamApply(UksOperator *o, Coef a_, Coef b_) : op(o), a(a_), b(b_) {}
  int64_t size() const override { return 2 * op->dim; }
  void apply(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
             cudaStream_t s) override {
    op->ham_matmul(a, b, X, ldx, k, Y, ldy, s);
  }
  void diagonal(double *D, cudaStream_t s) override {
    // HamiltonianOperator::get_diagonal: [D_A; -D_A] (bseoperator_btda.h:81-87)
    op->diagonal(a, D, s);
    ham_diag(D, op->dim, D, s);
  }
  void check(cudaStream_t s) override { op->check_errors(s); }
  bool split_precision() const override { return op->precision == BSE_PRECISION_MIXED; }
  void apply_fp64(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                  cudaStream_t s) override {
    ForceFp64 g(&op->alpha, &op->beta, fp64_products);
    op->ham_matmul(a, b, X, ldx, k, Y, ldy, s);
  }
};

}  // namespace vgb
