// Mixed-precision (tensor-core) contractions of the BSE product.
#pragma once

#include "bse_ops.cuh"

namespace vgb {

class MixedEngine {
 public:
  MixedEngine();
  ~MixedEngine();
  // Build the split (hi/lo) operand copies from the FP64 staged blocks.
  void stage(BseOperator &op, cudaStream_t s);
  // Y (+)= cx Hx X - cd Hd X - cd2 Hd2 X with tensor-core split products.
  void apply(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y,
             int64_t ldy, bool accumulate, cudaStream_t s);
  // The same for many operators at once (GroupedItem.op->mixed engines), one grouped
  // launch per stage and tile shape; accumulate: Y already holds the Hqp term.
  static void apply_grouped(const Coef &c, const std::vector<GroupedItem> &items, bool accumulate,
                            cudaStream_t s, GroupScratch *scratch);
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
