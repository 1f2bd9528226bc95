// Strided, two-level-batched FP64 GEMM on CUDA cores with deterministic split-K.
//
// GB300 runs FP64 at ~1.2 TFLOP/s (2 DFMA/clk/SM), so every FP64 contraction
// of this library is DFMA-bound long before it is bandwidth-bound: the kernel
// needs only enough register blocking (4x4 per thread) and resident warps to
// keep the DFMA pipe busy, and arbitrary element strides cost nothing that
// matters.  This lets one kernel serve all FP64 contractions (the Hd/Hd2/Hx
// stages and the Davidson projections) by describing the operands with
// strides instead of materialising transposes.
#pragma once

#include "common.cuh"

namespace vgb {

struct GemmDesc {
  int64_t M = 0, N = 0, K = 0;
  // A(i, l) = A[i * a_rs + l * a_cs]
  const double *A = nullptr;
  int64_t a_rs = 1, a_cs = 0;
  // B(l, n) = B[l * b_rs + n * b_cs]
  const double *B = nullptr;
  int64_t b_rs = 1, b_cs = 0;
  // C(i, n) = C[i * c_rs + n * c_cs]
  double *C = nullptr;
  int64_t c_rs = 1, c_cs = 0;
  double alpha = 1.0, beta = 0.0;
  // batch b = b1 * nb2 + b2 adds b1 * x_b1 + b2 * x_b2 to each base pointer
  int64_t nb1 = 1, nb2 = 1;
  int64_t a_b1 = 0, a_b2 = 0, b_b1 = 0, b_b2 = 0, c_b1 = 0, c_b2 = 0;

  // column-major helpers: op(A) = A (M x K, ld) or A^T (A stored K x M, ld)
  GemmDesc &a_colmajor(const double *p, int64_t ld, bool trans) {
    A = p;
    if (!trans) { a_rs = 1; a_cs = ld; } else { a_rs = ld; a_cs = 1; }
    return *this;
  }
  GemmDesc &b_colmajor(const double *p, int64_t ld, bool trans) {
    B = p;
    if (!trans) { b_rs = 1; b_cs = ld; } else { b_rs = ld; b_cs = 1; }
    return *this;
  }
  GemmDesc &c_colmajor(double *p, int64_t ld) {
    C = p; c_rs = 1; c_cs = ld;
    return *this;
  }
};

// Scratch owned by the caller (split-K partials).  Grows on demand.
struct GemmWorkspace {
  DeviceBuffer<double> partial;
};

// Launch.  splitk = 0 picks a split so that the grid covers the GPU.
void dgemm(const GemmDesc &d, cudaStream_t stream, GemmWorkspace *ws, int splitk = 0);

// Same kernels with caller-owned split-K scratch of ws_count doubles: the K
// split is reduced until its partials fit (no split when ws is null).  Never
// allocates.
void dgemm_prealloc(const GemmDesc &d, cudaStream_t stream, double *ws, int64_t ws_count);

}  // namespace vgb
