// BF16x3 split-product GEMM on the 5th-generation tensor cores (tcgen05, sm_103a).
//
//   D[M x N] (+)= sum_K A[M x K] B[N x K]^T,  A = A_hi + A_lo, B = B_hi + B_lo
//   computed as A_hi B_hi + A_hi B_lo + A_lo B_hi with FP32 accumulation in TMEM.
//
// Operands are K-major bf16 matrices (rows x K, K contiguous, K padded to a
// multiple of 64 with zeros) loaded by TMA with the 128-byte swizzle into a
// shared-memory ring; one elected thread issues tcgen05.mma, four epilogue
// warps drain the (double-buffered) TMEM accumulator with tcgen05.ld and write
// the tile through a generic index map.  The kernel is persistent: one CTA per
// SM walks the tile list, so the epilogue of tile t overlaps the MMAs of t+1.
#pragma once

#include <cuda.h>

#include <vector>

#include "common.cuh"

namespace vgb {

// A K-major bf16 hi/lo operand pair: rows x K (row stride ld elements).
struct TcMat {
  const uint16_t *hi = nullptr, *lo = nullptr;
  int64_t rows = 0, K = 0, ld = 0;
  CUtensorMap map_hi, map_lo;
  int box_rows = 0;
  int bk = 64;
};

// Build the TMA descriptors of an operand; box_rows = tile rows (128 for A, BN for B);
// bk = K elements per pipeline stage (64: 128-byte swizzle, 32: 64-byte swizzle).
TcMat make_tc_mat(const uint16_t *hi, const uint16_t *lo, int64_t rows, int64_t K, int64_t ld,
                  int box_rows, int bk = 64);

// Output index map of the epilogue.  Element (i, n) of batch b, K-split s goes to
//   (i / rd) * ro1 + (i % rd) * ro2 + (n / cd) * co1 + (n % cd) * co2 + b * bo + s * so
// and is written only when i < M, n < N, (i % rd) < rlim, (n % cd) < clim.
struct TcEpilogue {
  // PAIR_F32 (slice mode with kacc only): the FP64 sum as an unevaluated pair of floats
  // (hi, lo), stored as a float2 at out_f32 + 2 * offset
  enum Kind { SPLIT_BF16 = 0, STORE_F32 = 1, AXPBY_F64 = 2, PAIR_F32 = 3 };
  int kind = AXPBY_F64;
  int64_t rd = 1, ro1 = 0, ro2 = 0, rlim = 1;
  int64_t cd = 1, co1 = 0, co2 = 0, clim = 1;
  int64_t bo = 0, so = 0;
  uint16_t *out_hi = nullptr, *out_lo = nullptr;
  float *out_f32 = nullptr;
  double *out_f64 = nullptr;
  double alpha = 1.0, beta = 0.0;
};

struct TcShape {
  int64_t M = 0, N = 0, K = 0;  // K: multiple of 64
  int64_t nbatch = 1;
  int64_t a_batch_rows = 0, b_batch_rows = 0;  // row offset of A / B per batch
  int ksplit = 1;                              // K split into ksplit ranges (STORE_F32 partials)
  int products = 3;                            // 3 (BF16x3) or 4 (adds A_lo B_lo)
  // with ksplit > 1 and BN <= 64: one CTA runs all splits of a tile and sums them in FP64
  // registers (in split order) before the epilogue map; no partials, no reduction launch
  bool kacc = false;
  // kacc: the splits of a tile shared out to kgroups CTAs (kgroups divides the split count);
  // group g writes its FP64 sum through the epilogue map at offset g * epi.so (beta = 0), and
  // reduce_f64_groups adds the groups
  int kgroups = 1;
  // slice mode (nslices > 0, nbatch 1, K box 64, BN <= 64): the operands hold nslices bf16 digit
  // planes stacked by rows (digit t of operand row r is row t * plane + r, see slice_f64); the
  // product is the sum of A plane a times B plane b over all a + b < nslices, one bf16 MMA per K
  // step.  Every K split covers one digit pair on one run of at most `chain` K elements (the run
  // of one digit scale), its FP32 accumulator is exact, and the splits are summed on the CTA.
  // A pipeline stage holds A plane a and B planes 0 .. nslices - 1 - a of one K block, whose
  // products go to separate accumulators (one A load for up to nslices pairs).  kgroups must
  // divide the number of runs.
  int nslices = 0;
  int64_t a_plane = 0, b_plane = 0;
  int64_t chain = 1024;
};

// Launch the persistent GEMM; bn in {32, 64, 128, 256}.  err: device int set
// non-zero if a bounded wait inside the kernel gives up.  Returns the number of
// K splits actually used (partials written for STORE_F32).
int tc_gemm(const TcMat &A, const TcMat &B, const TcShape &shape, const TcEpilogue &epi, int bn,
             int *err, cudaStream_t s);

// One GEMM of a group: operands, shape and epilogue as for tc_gemm.
struct TcProblem {
  TcMat A, B;
  TcShape shape;
  TcEpilogue epi;
};

// Several independent GEMMs with the same tile (bn, K box) in as few launches as
// possible: each launch walks the concatenated tile lists of up to 32 problems,
// whose tensor maps and parameters travel in the kernel parameter space.
// ksplit_out[i] (optional) receives problem i's K splits, as tc_gemm returns.
// group_max: problems per launch (at most 32); nstreams > 1: the launches spread over that many
// auxiliary streams (forked from and joined back into s), so that their tails overlap.
void tc_gemm_grouped(const std::vector<const TcProblem *> &probs, int bn, int *err, cudaStream_t s,
                     int *ksplit_out = nullptr, int group_max = 32, int nstreams = 1);

// FP64 -> bf16 hi/lo split into a row-major padded operand out[r * ldo + c] for
// r < rows, c < cols; the source element (r, c) is
//   x[(r / rdiv) * rs1 + (r % rdiv) * rs2 + c * cs]
// and rows with (r % rdiv) >= rlim are skipped (left as they are: zero padding).
struct SplitMap {
  int64_t rdiv = 1, rs1 = 0, rs2 = 0, cs = 1, rlim = 1;
};
void split_f64_to_bf16(const double *x, int64_t rows, int64_t cols, const SplitMap &m, uint16_t *hi,
                       uint16_t *lo, int64_t ldo, cudaStream_t s);

// Ozaki slices (Ozaki, Ogita, Oishi, Rump, Numer. Algorithms 59 (2012) 95-118; on tensor cores:
// Mukunoki, Ozaki, Ogita, Imamura, ISC 2020) of the FP64 matrix x (element (r, c) through the map
// as above): for every row and every run of `chunk` columns (c / chunk equal) a power of two
// sigma >= max |x| over the run, and nslices (<= 7) digits d_t = the t-th balanced base-2^7
// digit of x / sigma rounded to 7 nslices bits (|d_1| <= 128, |d_t| <= 64 after), stored as the bf16 value
// d_t sigma 2^(-7 t) at out[(t - 1) * plane + r * ldo + c].  The bf16 values are exact, and the
// product of two digits is an integer times sigma_a sigma_b 2^(-7 (s + t)) below 2^14 of it, so
// a sum of at most 1024 such products for one slice pair and one output element, with the
// same sigmas, is exact in FP32.  Rows with (r % rdiv) >= rlim and columns >= cols are left
// as they are (zero padding).
void slice_f64(const double *x, int64_t rows, int64_t cols, const SplitMap &m, int nslices, int64_t chunk,
               uint16_t *out, int64_t ldo, int64_t plane, cudaStream_t s);
// The same for a matrix held as float pairs (hi, lo) (element value hi + lo; PAIR_F32 output);
// the map addresses float2 elements.
void slice_pairs(const float *x2, int64_t rows, int64_t cols, const SplitMap &m, int nslices, int64_t chunk,
                 uint16_t *out, int64_t ldo, int64_t plane, cudaStream_t s);

// Y = epi(sum over g < ngroups of part[g * M * N + n * M + i]) for the M x N partials of a
// kgroups product (column-major per group), summed in FP64 in group order; epi: AXPBY_F64.
void reduce_f64_groups(const double *part, int64_t M, int64_t N, int ngroups, const TcEpilogue &epi,
                       cudaStream_t s);

// Many independent splits / reductions in one launch per 96 jobs (one grid row per job).
struct SplitJob {
  const double *x = nullptr;
  int64_t rows = 0, cols = 0;
  SplitMap map;
  uint16_t *hi = nullptr, *lo = nullptr;
  int64_t ldo = 0;
};
void split_grouped(const std::vector<SplitJob> &jobs, cudaStream_t s);

// Sum ksplit FP32 partial tiles (each M x N, element (i, n) at p[s * M * N + i * N + n])
// and apply an epilogue map (SPLIT_BF16 or AXPBY_F64) with nbatch = 1.
void reduce_partials(const float *partial, int64_t M, int64_t N, int ksplit, const TcEpilogue &epi,
                     cudaStream_t s);
struct ReduceJob {
  const float *part = nullptr;
  int64_t M = 0, N = 0;
  int ksplit = 0;
  TcEpilogue epi;
};
void reduce_grouped(const std::vector<ReduceJob> &jobs, cudaStream_t s);

}  // namespace vgb
