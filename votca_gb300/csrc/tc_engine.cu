// Mixed-precision engine (placeholder until the tcgen05 kernels land).
#include "tc_engine.cuh"

namespace vgb {

struct MixedEngine::Impl {};

MixedEngine::MixedEngine() : impl_(new Impl()) {}
MixedEngine::~MixedEngine() { delete impl_; }

void MixedEngine::stage(BseOperator &, cudaStream_t) {
  fail(BSE_ERR_UNSUPPORTED, "mixed precision is not available in this build");
}

void MixedEngine::apply(BseOperator &, const Coef &, const double *, int64_t, int64_t, double *,
                        int64_t, bool, cudaStream_t) {
  fail(BSE_ERR_UNSUPPORTED, "mixed precision is not available in this build");
}

}  // namespace vgb
