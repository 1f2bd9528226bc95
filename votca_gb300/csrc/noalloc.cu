// Allocation-free entry point of the FP64 BSE product.
//
// Some callers cannot call cudaMalloc at the point where they need a product:
// code that runs while another component owns all device memory through its
// own pool (an application that reserved the HBM up front and forbids further
// runtime allocations), or code that must not take the implicit device-wide
// synchronisation that cudaMalloc/cudaFree can trigger in the middle of a
// pipelined solve.  bse_op_matmul_device_noalloc serves them: it computes the
// same product as bse_op_matmul_device in FP64 but takes every temporary (the
// aux-contracted intermediates and the split-K partial sums) from one static
// device array declared in this file, and calls no cudaMalloc, cudaFree or
// allocating library routine.
//
// The array costs kNoAllocScratchBytes of HBM on every GPU that loads the
// library, until the process exits.  Its device address is looked up once per
// device, on the first call made while that device is current; make that first
// call before any stream capture.  All calls share the array and it keeps the
// last call's contents: every region is fully written before it is read, so
// nothing has to start at zero, but two calls that overlap on the GPU (on
// different streams, or from different threads) race on it.
#include <mutex>

#include "bse_ops.cuh"

namespace vgb {

namespace {

constexpr int64_t kNoAllocScratchDoubles = 8LL << 20;  // 64 MiB
constexpr int64_t kNoAllocPartialDoubles = 1LL << 20;  // split-K partials: first 8 MiB
constexpr int kMaxDevices = 64;

std::mutex g_noalloc_mu;
double *g_noalloc_ptr[kMaxDevices] = {nullptr};

}  // namespace

static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

namespace {

// Device address of the static scratch for the current device (looked up once per device).
double *noalloc_scratch() {
  int dev = 0;
  VGB_CUDA(cudaGetDevice(&dev));
  VGB_REQUIRE(dev >= 0 && dev < kMaxDevices, "no-alloc product: device index out of range");
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || p == nullptr)
      fail(BSE_ERR_CUDA, std::string("cudaGetSymbolAddress of the no-alloc scratch failed: ") +
                             cudaGetErrorString(e));
    g_noalloc_ptr[dev] = (double *)p;
  }
  return g_noalloc_ptr[dev];
}

__global__ void na_hqp_diag_kernel(double cqp, const double *__restrict__ Hcc,
                                   const double *__restrict__ Hvv, int64_t vt, int64_t ct,
                                   const double *__restrict__ X, int64_t ldx, int64_t k,
                                   double *__restrict__ Y, int64_t ldy) {
  const int64_t dim = vt * ct, total = dim * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t I = t % dim, j = t / dim;
    const int64_t v = I / ct, c = I % ct;
    Y[I + ldy * j] = cqp * (Hcc[c + ct * c] - Hvv[v + vt * v]) * X[I + ldx * j];
  }
}

__global__ void na_zero_kernel(double *Y, int64_t ldy, int64_t rows, int64_t k) {
  const int64_t total = rows * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    Y[(t % rows) + ldy * (t / rows)] = 0.0;
}

unsigned na_grid(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 16LL * 152));
}

}  // namespace

// Y = H(c) X in FP64 using only the static scratch (see the file comment).
void matmul_noalloc(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k,
                    double *Y, int64_t ldy, cudaStream_t s) {
  VGB_REQUIRE(ldx >= op.dim && ldy >= op.dim, "no-alloc product: leading dimension too small");
  VGB_REQUIRE(k >= 0, "no-alloc product: negative column count");
  VGB_REQUIRE(!(c.cd != 0 && c.cd2 != 0), "Hamiltonian cannot contain Hd and Hd2 at the same time");
  if (k == 0) return;
  const int64_t vt = op.vt, ct = op.ct, naux = op.naux, dim = op.dim;
  const int64_t region = kNoAllocScratchDoubles - kNoAllocPartialDoubles;
  // size checks before anything is launched
  if (c.cx != 0 && naux * k > region)
    fail(BSE_ERR_ARGUMENT, "no-alloc product: Naux*k = " + std::to_string(naux * k) +
                               " doubles exceeds the static scratch (" + std::to_string(region) +
                               " doubles); split the columns into smaller calls");
  int64_t per_vec = 0;
  if (c.cd != 0) per_vec = naux * dim;
  if (c.cd2 != 0) per_vec = vt * naux * vt;
  if (per_vec > region)
    fail(BSE_ERR_ARGUMENT, "no-alloc product: one column needs " + std::to_string(per_vec) +
                               " scratch doubles, the static scratch holds " +
                               std::to_string(region) + " (maximum Naux*v*c for Hd, Naux*v*v for Hd2)");
  double *scratch = noalloc_scratch();
  double *part = scratch;
  double *T = scratch + kNoAllocPartialDoubles;

  bool acc = false;
  if (c.cqp != 0) {
    if (op.hqp_diagonal) {
      na_hqp_diag_kernel<<<na_grid(dim * k), 256, 0, s>>>(c.cqp, op.Hcc.get(), op.Hvv.get(), vt, ct,
                                                           X, ldx, k, Y, ldy);
      VGB_LAUNCH_CHECK();
    } else {
      GemmDesc g;
      g.M = ct; g.N = vt; g.K = ct;
      g.A = op.Hcc.get(); g.a_rs = ct; g.a_cs = 1;
      g.B = X; g.b_rs = 1; g.b_cs = ct; g.b_b1 = ldx;
      g.C = Y; g.c_rs = 1; g.c_cs = ct; g.c_b1 = ldy;
      g.nb1 = k; g.alpha = c.cqp; g.beta = 0.0;
      dgemm_prealloc(g, s, part, kNoAllocPartialDoubles);
      GemmDesc h;
      h.M = ct; h.N = vt; h.K = vt;
      h.A = X; h.a_rs = 1; h.a_cs = ct; h.a_b1 = ldx;
      h.B = op.Hvv.get(); h.b_rs = 1; h.b_cs = vt;
      h.C = Y; h.c_rs = 1; h.c_cs = ct; h.c_b1 = ldy;
      h.nb1 = k; h.alpha = -c.cqp; h.beta = 1.0;
      dgemm_prealloc(h, s, part, kNoAllocPartialDoubles);
    }
    acc = true;
  }
  if (c.cx != 0) {
    double *Z = T;
    GemmDesc g;  // Z (naux x k) = Bvc^T X
    g.M = naux; g.N = k; g.K = dim;
    g.A = op.Bvc.get(); g.a_rs = dim; g.a_cs = 1;
    g.B = X; g.b_rs = 1; g.b_cs = ldx;
    g.C = Z; g.c_rs = 1; g.c_cs = naux;
    dgemm_prealloc(g, s, part, kNoAllocPartialDoubles);
    GemmDesc h;  // Y (+)= cx Bvc Z
    h.M = dim; h.N = k; h.K = naux;
    h.A = op.Bvc.get(); h.a_rs = 1; h.a_cs = dim;
    h.B = Z; h.b_rs = 1; h.b_cs = naux;
    h.C = Y; h.c_rs = 1; h.c_cs = ldy;
    h.alpha = c.cx; h.beta = acc ? 1.0 : 0.0;
    dgemm_prealloc(h, s, part, kNoAllocPartialDoubles);
    acc = true;
  }
  if (c.cd != 0 || c.cd2 != 0) {
    const int64_t jchunk = std::max<int64_t>(1, std::min<int64_t>(k, region / per_vec));
    for (int64_t j0 = 0; j0 < k; j0 += jchunk) {
      const int64_t kc = std::min(jchunk, k - j0);
      if (c.cd != 0) {
        GemmDesc a;  // S[j][P](c1, v) = sum_c Mcc_P(c1, c) X_j(c, v)
        a.M = ct; a.N = vt; a.K = ct;
        a.A = op.Mcc.get(); a.a_rs = 1; a.a_cs = ct;
        a.B = X + j0 * ldx; a.b_rs = 1; a.b_cs = ct;
        a.C = T; a.c_rs = 1; a.c_cs = ct;
        a.nb1 = kc; a.nb2 = naux;
        a.a_b1 = 0; a.a_b2 = ct * ct;
        a.b_b1 = ldx; a.b_b2 = 0;
        a.c_b1 = per_vec; a.c_b2 = dim;
        dgemm_prealloc(a, s, part, kNoAllocPartialDoubles);
        GemmDesc b;  // Y_j(c1, v1) (+)= -cd sum_{P,v} S[j](c1, (P,v)) Gvv((P,v), v1)
        b.M = ct; b.N = vt; b.K = naux * vt;
        b.A = T; b.a_rs = 1; b.a_cs = ct; b.a_b1 = per_vec;
        b.B = op.Gvv.get(); b.b_rs = 1; b.b_cs = naux * vt;
        b.C = Y + j0 * ldy; b.c_rs = 1; b.c_cs = ct; b.c_b1 = ldy;
        b.nb1 = kc; b.alpha = -(double)c.cd; b.beta = acc ? 1.0 : 0.0;
        dgemm_prealloc(b, s, part, kNoAllocPartialDoubles);
      } else {
        GemmDesc a;  // U[j][v1][P][v] = sum_c X_j(c, v) Bvc_P(c, v1)
        a.M = vt; a.N = vt; a.K = ct;
        a.A = X + j0 * ldx; a.a_rs = ct; a.a_cs = 1;
        a.B = op.Bvc.get(); a.b_rs = 1; a.b_cs = ct;
        a.C = T; a.c_rs = 1; a.c_cs = naux * vt;
        a.nb1 = kc; a.nb2 = naux;
        a.a_b1 = ldx; a.a_b2 = 0;
        a.b_b1 = 0; a.b_b2 = dim;
        a.c_b1 = per_vec; a.c_b2 = vt;
        dgemm_prealloc(a, s, part, kNoAllocPartialDoubles);
        GemmDesc b;  // Y_j(c1, v1) (+)= -cd2 sum_{P,v} Mcv(c1, (P,v)) U_j((P,v), v1)
        b.M = ct; b.N = vt; b.K = naux * vt;
        b.A = op.Mcv.get(); b.a_rs = 1; b.a_cs = ct;
        b.B = T; b.b_rs = 1; b.b_cs = naux * vt; b.b_b1 = per_vec;
        b.C = Y + j0 * ldy; b.c_rs = 1; b.c_cs = ct; b.c_b1 = ldy;
        b.nb1 = kc; b.alpha = -(double)c.cd2; b.beta = acc ? 1.0 : 0.0;
        dgemm_prealloc(b, s, part, kNoAllocPartialDoubles);
      }
    }
    acc = true;
  }
  if (!acc) {
    na_zero_kernel<<<na_grid(dim * k), 256, 0, s>>>(Y, ldy, dim, k);
    VGB_LAUNCH_CHECK();
  }
}

}  // namespace vgb
