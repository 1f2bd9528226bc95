// Device-resident BSE operator: staged Mmn blocks + the matrix-free product.
//
// The reference (xtp/src/libxtp/gwbse/bse_operator.cc:39-119) builds every
// row of Hd explicitly for each (c1, v1) pair and rebuilds every c x c block of
// Hx for each v1 <= v2 pair, re-copying Mmn slices to the GPU for every row.
// Here the blocks are staged into HBM once (at handle creation) in layouts
// chosen for the contractions, and the product is factorised over the
// auxiliary index:
//   Hx  X : Z = Bvc^T X (Naux x k),   Y += cx Bvc Z
//   Hd  X : S_{jP} = Mcc_P X_j (c x v),   Y_j -= cd sum_{P,v} S_{jP} G_P
//   Hd2 X : U_{jP} = X_j^T Bvc_P (v x v), Y_j -= cd2 sum_{P,v} Mcv_P U_{jP}
//   Hqp X : (e_c - e_v) X, or the two small GEMMs with off-diagonal Hqp
// with the screening (diagonal w or dense W) folded into G and Mcv at staging.
#pragma once

#include <memory>
#include <vector>

#include "common.cuh"
#include "dgemm.cuh"

namespace vgb {

struct Coef {
  int cqp = 0, cx = 0, cd = 0, cd2 = 0;
};

// Per-stage device timing with CUDA events on the launch stream (off by default).
enum Stage {
  STAGE_HQP = 0,
  STAGE_HX = 1,
  STAGE_HD_A = 2,   // FP64 Hd: S = Mcc X (c-contraction)
  STAGE_HD_B = 3,   // FP64 Hd: Y -= S G (v,P-contraction)
  STAGE_HD2_A = 4,
  STAGE_HD2_B = 5,
  STAGE_TC_HD = 6,  // tensor-core Hd
  STAGE_TC_HX = 7,
  STAGE_TC_HD2 = 8,
  STAGE_TC_SPLIT = 9,
  STAGE_TC_HD_B = 10,  // tensor-core Hd stage 2 (+ partial reduction)
  STAGE_TC_HD2_B = 11,
  STAGE_COUNT = 12
};

class StageTimer {
 public:
  ~StageTimer();
  void enable(bool on);
  bool on() const { return on_; }
  void begin(int stage, cudaStream_t s);
  void end(int stage, cudaStream_t s);
  // accumulated milliseconds and call counts since enable(true)
  void read(double *ms, int64_t *calls, int n);

 private:
  struct Rec { cudaEvent_t a, b; int stage; };
  bool on_ = false;
  std::vector<Rec> pending_;
  std::vector<cudaEvent_t> pool_;
  double ms_[STAGE_COUNT] = {0};
  int64_t calls_[STAGE_COUNT] = {0};
  cudaEvent_t get_();
  void drain_();
};

// Linear operator on device vectors (what the Davidson driver needs).
struct DeviceOperator {
  virtual ~DeviceOperator() = default;
  virtual int64_t size() const = 0;
  // Y = Op X; X, Y device, column-major, size x k.
  virtual void apply(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                     cudaStream_t s) = 0;
  virtual void diagonal(double *D, cudaStream_t s) = 0;
  // raise if an asynchronous device-side failure was recorded (synchronises)
  virtual void check(cudaStream_t) {}
  // true when apply() runs split-precision (tensor-core) products; apply_fp64 is then the
  // same operator with FP64-accurate products (the Davidson polish): Ozaki slice products where
  // the operator has a tensor-core engine and fp64_products == 0, else FP64 DGEMM
  virtual bool split_precision() const { return false; }
  int fp64_products = 0;
  virtual void apply_fp64(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                          cudaStream_t s) {
    apply(X, ldx, k, Y, ldy, s);
  }
};

class MixedEngine;  // tensor-core contractions (tc_engine.cu)

class BseOperator {
 public:
  int64_t vt = 0, ct = 0, naux = 0, dim = 0;
  int precision = BSE_PRECISION_FP64;
  bool hqp_diagonal = true;
  // set while a split-precision operator must run its FP64-accurate path (FP64 blocks are always
  // staged): Ozaki slice products on the tensor cores (fp64_products 0) or FP64 DGEMM (1)
  bool force_fp64 = false;
  int fp64_products = 0;

  // FP64 staged blocks (layouts documented in bse_ops.cu)
  DeviceBuffer<double> Bvc, Mcc, Gvv, Mcv, dcc, dvv, Hcc, Hvv;
  // unscreened vv block [P][v1][v], unscreened cv block [P][v][c1] = M(c1, v, P) (the Hd2
  // adjoint), and the screening (naux, or naux x naux when dense)
  DeviceBuffer<double> Mvv, Mcv0, Wscr;
  bool dense_screening = false;
  // index window of the staged blocks inside the caller's Mmn
  int64_t m_v0 = 0, m_c0 = 0, n_v0 = 0, n_c0 = 0, msize = 0, nsize = 0;
  // scratch
  DeviceBuffer<double> S, Z, Xc, Ttmp;
  // diagonal of the last coefficient set a batched solve used (the operator is immutable)
  DeviceBuffer<double> diag_cache;
  Coef diag_coef;
  bool diag_valid = false;
  GemmWorkspace ws;
  int64_t s_budget_bytes = 4LL << 30;
  std::unique_ptr<MixedEngine> mixed;
  StageTimer timer;

  BseOperator();
  ~BseOperator();

  // Stage from host data (see bse_op_create).  W: diagonal (naux) when dense_w == false,
  // else naux x naux column-major.
  void stage(const bse_mmn_desc &desc, const double *const *slices, const double *w, bool dense_w,
             const double *hqp, int64_t ldh, int64_t hqp_size, const bse_options &opt,
             int prec, cudaStream_t s);

  // Y = H(coef) X on device (ldx/ldy >= dim).
  void matmul(const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
              cudaStream_t s);
  void diagonal(const Coef &c, double *D, cudaStream_t s);
  void check_errors(cudaStream_t s);
  void stage_unscreened_vv(const bse_mmn_desc &desc, const double *const *slices,
                           const bse_options &opt, cudaStream_t s);
  // Gradient of sum_i g_i u_i^T H(c) u_i (adjoint.cu) for any coefficient set, accumulated into
  // device buffers (zeroed first unless accumulate): gMvc [P][v][c] (Bvc layout), gMcv [P][v][c1]
  // (the cv block, Mcv0 layout), gMvv [P][v1][v], gMcc [P][c][c1], gH the Hqp window
  // ((vt+ct)^2), gW the screening (naux, or naux^2 when dense).  Any output may be null.
  void quad_gradient(const Coef &c, const double *U, int64_t ldu, int64_t nr, const double *g_host,
                     double *gMvc, double *gMcv, double *gMvv, double *gMcc, double *gH, double *gW,
                     bool accumulate, cudaStream_t s);
  // [[A, B], [-B, -A]] X, X and Y (2 dim) x k
  void ham_matmul(const Coef &a, const Coef &b, const double *X, int64_t ldx, int64_t k, double *Y,
                  int64_t ldy, cudaStream_t s);

  // FP64 stage entry points (also used by the mixed engine for checks)
  void apply_hqp(double cqp, const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                 bool accumulate, cudaStream_t s);
  void apply_hx_fp64(double cx, const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                     bool accumulate, cudaStream_t s);
  void apply_hd_fp64(double alpha, const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                     bool accumulate, cudaStream_t s);
  void apply_hd2_fp64(double alpha, const double *X, int64_t ldx, int64_t k, double *Y,
                      int64_t ldy, bool accumulate, cudaStream_t s);

 private:
  DeviceBuffer<double> hamA_, hamB_, hamX_;
};

// [[A, B], [-B, -A]] assembly helpers: Y[:dim] = TA_top + TB_bot, Y[dim:] = -TA_bot - TB_top
// for products TA = A [M1_0, M2_0, M1_1, ...], TB = B [...]; D2 = [D; -D]; column copy.
void ham_combine(const double *TA, const double *TB, int64_t dim, int64_t k, double *Y, int64_t ldy,
                 cudaStream_t s);
void ham_diag(const double *D, int64_t dim, double *D2, cudaStream_t s);
void copy_cols(const double *X, int64_t ldx, int64_t rows, int64_t k, double *Y, int64_t ldy,
               cudaStream_t s);

// The Mmn-shaped gradient (the caller's slice layout, msize x naux x nsize, host memory) from the
// block gradients of BseOperator::eig_gradient: scattered on the device, copied in chunks.
void scatter_mmn_gradient(const BseOperator &op, const double *gMvc, const double *gMcv,
                          const double *gMvv, const double *gMcc, double *host_out, cudaStream_t s);

// One molecule's share of a grouped product: Y = H(c) X on its own operator.
struct GroupedItem {
  BseOperator *op = nullptr;
  const double *X = nullptr;
  int64_t ldx = 0, k = 0;
  double *Y = nullptr;
  int64_t ldy = 0;
  bool dense = false;  // use the operator's dense form (MixedEngine::build_dense_grouped)
  const double *diag = nullptr;  // with dense: the operator's full diagonal (device, FP64)
};
// Scratch shared by the operators of a grouped product (the Hd intermediates); kept by
// the caller across products so that it is allocated once.
struct GroupScratch {
  DeviceBuffer<uint16_t> hi, lo;
  int64_t elems = 0;
};
// Products of many operators with one coefficient set, stage by stage: every
// tensor-core stage of all mixed-precision operators runs as grouped launches
// (FP64 operators fall back to one product each).  Hd2 is not supported here.
void matmul_grouped(const Coef &c, const std::vector<GroupedItem> &items, cudaStream_t s,
                    GroupScratch *scratch = nullptr);
// Diagonals of many operators (same arithmetic as BseOperator::diagonal) in one launch per 192.
void diagonal_grouped(const Coef &c, const std::vector<BseOperator *> &ops,
                      const std::vector<double *> &D, cudaStream_t s);

// Runs the operators' FP64-accurate path for its lifetime (split-precision handles keep FP64
// blocks); mode: BseOperator::fp64_products.
struct ForceFp64 {
  BseOperator *a, *b;
  bool sa, sb;
  int ma, mb;
  explicit ForceFp64(BseOperator *x, BseOperator *y = nullptr, int mode = 1)
      : a(x), b(y), sa(x->force_fp64), sb(y ? y->force_fp64 : false), ma(x->fp64_products),
        mb(y ? y->fp64_products : 0) {
    a->force_fp64 = true;
    a->fp64_products = mode;
    if (b) {
      b->force_fp64 = true;
      b->fp64_products = mode;
    }
  }
  ~ForceFp64() {
    a->force_fp64 = sa;
    a->fp64_products = ma;
    if (b) {
      b->force_fp64 = sb;
      b->fp64_products = mb;
    }
  }
};

struct BseApply : DeviceOperator {
  BseOperator *op;
  Coef coef;
  BseApply(BseOperator *o, Coef c) : op(o), coef(c) {}
  int64_t size() const override { return op->dim; }
  void apply(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
             cudaStream_t s) override {
    op->matmul(coef, X, ldx, k, Y, ldy, s);
  }
  void diagonal(double *D, cudaStream_t s) override { op->diagonal(coef, D, s); }
  void check(cudaStream_t s) override { op->check_errors(s); }
  bool split_precision() const override { return op->precision == BSE_PRECISION_MIXED && op->mixed; }
  void apply_fp64(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                  cudaStream_t s) override {
    ForceFp64 g(op, nullptr, fp64_products);
    op->matmul(coef, X, ldx, k, Y, ldy, s);
  }
};

struct BseHamApply : DeviceOperator {
  BseOperator *op;
  Coef a, b;
  BseHamApply(BseOperator *o, Coef a_, Coef b_) : op(o), a(a_), b(b_) {}
  int64_t size() const override { return 2 * op->dim; }
  void apply(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
             cudaStream_t s) override {
    op->ham_matmul(a, b, X, ldx, k, Y, ldy, s);
  }
  void diagonal(double *D, cudaStream_t s) override;
  void check(cudaStream_t s) override { op->check_errors(s); }
  bool split_precision() const override { return op->precision == BSE_PRECISION_MIXED && op->mixed; }
  void apply_fp64(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                  cudaStream_t s) override {
    ForceFp64 g(op, nullptr, fp64_products);
    op->ham_matmul(a, b, X, ldx, k, Y, ldy, s);
  }
};

// Dense FP64 symmetric operator(s): A, optionally B for [[A, B], [-B, -A]].
class DenseOperator {
 public:
  int64_t n = 0;
  bool has_b = false;
  DeviceBuffer<double> A, B, tmpA, tmpB, Xr;
  GemmWorkspace ws;
  void stage(const double *a, const double *b, int64_t n_, int64_t lda, cudaStream_t s);
  void matmul(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy, cudaStream_t s);
  void diagonal(double *D, cudaStream_t s);
  void ham_matmul(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy, cudaStream_t s);
};

struct DenseApply : DeviceOperator {
  DenseOperator *op;
  bool ham;
  DenseApply(DenseOperator *o, bool h) : op(o), ham(h) {}
  int64_t size() const override { return ham ? 2 * op->n : op->n; }
  void apply(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
             cudaStream_t s) override {
    if (ham) op->ham_matmul(X, ldx, k, Y, ldy, s); else op->matmul(X, ldx, k, Y, ldy, s);
  }
  void diagonal(double *D, cudaStream_t s) override;
};

// Combine kernel for the HamiltonianOperator reshaping trick
// (bseoperator_btda.h:136-148): TA = A [M1_0, M2_0, M1_1, ...], TB likewise.
void ham_combine(const double *TA, const double *TB, int64_t dim, int64_t k, double *Y,
                 int64_t ldy, cudaStream_t s);
// D2 = [D; -D]
void ham_diag(const double *D, int64_t dim, double *D2, cudaStream_t s);

// FP64 product with every temporary in a static device array (noalloc.cu).
void matmul_noalloc(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k,
                    double *Y, int64_t ldy, cudaStream_t s);

}  // namespace vgb
