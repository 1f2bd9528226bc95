// Mixed-precision (tensor-core) contractions of the BSE product.
#pragma once

#include <string>

#include "bse_ops.cuh"
#include "tc_gemm.cuh"

namespace vgb {

// The launch shapes chosen by the autotuner so far, with the candidates' times (JSON).
std::string autotune_report();

class MixedEngine {
 public:
  MixedEngine();
  ~MixedEngine();
  // Build the split (hi/lo) operand copies from the FP64 staged blocks (split_operands false:
  // only the sizes, for operators whose products all run as slice products).
  void stage(BseOperator &op, cudaStream_t s, bool split_operands = true);
  // Y (+)= cx Hx X - cd Hd X - cd2 Hd2 X with tensor-core split products.
  void apply(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y,
             int64_t ldy, bool accumulate, cudaStream_t s);
  // Y (+)= cx Hx X - cd Hd X - cd2 Hd2 X with Ozaki slice products on the tensor cores
  // (slice_f64): every operand cut into 7-bit digit planes with power-of-two scales per run of
  // at most 1024 K elements, each pair of digit planes accumulated exactly in FP32 over one run,
  // the runs and pairs summed in FP64, the intermediates kept in FP64 and sliced again.  With
  // five digits the result agrees with the FP64 product to about 1e-11 of its scale.
  void apply_sliced(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y,
                    int64_t ldy, bool accumulate, cudaStream_t s);
  // FP64-accurate GEMM of FP64 operands on the tensor cores (the slice products of
  // apply_sliced): C(i, n) = sum_q A(i, q) B(n, q) for i < M, n < N, q < K, elements read through
  // the split maps (row i of A at am, row n of B at bm, column q), result through the FP64
  // epilogue e (AXPBY_F64).  mcc_as_b: B is the operator's cc block [(P, c1)][c] (its digit planes
  // are built once and kept; bm is then ignored).
  void gemm_sliced(BseOperator &op, const double *A, const SplitMap &am, int64_t M, const double *B,
                   const SplitMap &bm, int64_t N, int64_t K, bool mcc_as_b, const TcEpilogue &e, cudaStream_t s);
  // The same for many operators at once (GroupedItem.op->mixed engines), one grouped
  // launch per stage and tile shape; accumulate: Y already holds the Hqp term.
  static void apply_grouped(const Coef &c, const std::vector<GroupedItem> &items, bool accumulate,
                            cudaStream_t s, GroupScratch *scratch);
  // Dense form for small TDA operators: the off-diagonal part of cx Hx - cd Hd, built once with
  // two tensor-core GEMMs over the aux index into FP64, symmetrised, kept as bf16 hi/lo rows; a
  // product is one GEMM plus the operator's exact FP64 diagonal (Hqp included) applied beside
  // it (GroupedItem::diag), so the large diagonal is never rounded to bf16.  Needs a diagonal
  // Hqp and Naux <= 1024 (one FP32 chain per element).
  static void build_dense_grouped(const std::vector<BseOperator *> &ops, const Coef &c, cudaStream_t s);
  bool dense_ready(const Coef &c) const;
  // Y (+)= (off-diagonal part of cx Hx - cd Hd) X for every item; accumulate: Y holds diag X.
  static void apply_dense_grouped(const Coef &c, const std::vector<GroupedItem> &items, bool accumulate,
                                  cudaStream_t s);
  // Allocate, ahead of a series of grouped products of at most kmax columns, every
  // per-operator buffer they use (one pool growth instead of one per buffer).
  static void prepare_grouped(const std::vector<BseOperator *> &ops, int64_t kmax, cudaStream_t s);
  // Synchronise and raise if a kernel reported a bounded-wait timeout.
  void check(cudaStream_t s);

 private:
  struct Impl;
  Impl *impl_ = nullptr;
};

}  // namespace vgb
