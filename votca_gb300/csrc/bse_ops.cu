// BSE operator: staging of the Mmn blocks and the factorised FP64 product.
//
// Device layouts (P = auxiliary index, v/v1 occupied, c/c1 virtual, all
// BSE-window-local; I(v, c) = ct*v + c as in vc2index.h:42-44):
//   Bvc[P*dim + v*ct + c]            = M(v, c, P)             (Hx, Hd2 stage 1)
//   Mcc[P*ct*ct + c*ct + c1]         = M(c1, c, P)            (Hd stage 1)
//   Gvv[v1*naux*vt + P*vt + v]       = sum_Q W_PQ M(v1, v, Q) (Hd stage 2; W = diag(w) or dense)
//   Mcv[P*dim + v*ct + c1]           = sum_Q W_PQ M(c1, v, Q) (Hd2 stage 2)
//   dcc[P*ct + c] = M(c, c, P),  dvv[P*vt + v] = Gvv(v, P, v) (diagonal)
//   Hcc[c + ct*c1] = Hqp(vt+c, vt+c1),  Hvv[v + vt*v1] = Hqp(v, v1)
// M(m, n, P) is element (n, P) of the reference's slice Mmn_[m]
// (TCMatrix_gwbse, threecenter.h:70-142).
#include <algorithm>
#include <cstring>

#include "bse_ops.cuh"
#include "tc_engine.cuh"

namespace vgb {

namespace {

struct ScatterArgs {
  const double *raw;  // chunk: [mi][P][n] with n over the full nsize rows
  int64_t m_first;    // window index of the first slice in the chunk
  int64_t m_count;
  int64_t nsize, naux, vt, ct, dim;
  int64_t n_v0, n_c0;  // row index (in slice) of the first occupied / virtual BSE level
  const double *w;     // diagonal screening or nullptr (dense W applied later)
  double *Bvc, *Mcc, *Gvv, *Mcv, *Mcv0, *dcc;
};

__global__ void scatter_kernel(const ScatterArgs a) {
  const int64_t nwin = a.vt + a.ct;
  const int64_t total = a.m_count * a.naux * nwin;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t nl = t % nwin;
    const int64_t P = (t / nwin) % a.naux;
    const int64_t mi = t / (nwin * a.naux);
    const int64_t ml = a.m_first + mi;
    const int64_t row = nl < a.vt ? a.n_v0 + nl : a.n_c0 + (nl - a.vt);
    const double val = a.raw[(mi * a.naux + P) * a.nsize + row];
    const double wp = a.w ? a.w[P] : 1.0;
    if (ml < a.vt) {
      const int64_t v1 = ml;
      if (nl < a.vt) {
        const int64_t v = nl;
        a.Gvv[(v1 * a.naux + P) * a.vt + v] = wp * val;
      } else {
        const int64_t c = nl - a.vt;
        a.Bvc[P * a.dim + v1 * a.ct + c] = val;
      }
    } else {
      const int64_t c1 = ml - a.vt;
      if (nl < a.vt) {
        const int64_t v = nl;
        a.Mcv[P * a.dim + v * a.ct + c1] = wp * val;
        a.Mcv0[P * a.dim + v * a.ct + c1] = val;
      } else {
        const int64_t c = nl - a.vt;
        a.Mcc[(P * a.ct + c) * a.ct + c1] = val;
        if (c == c1) a.dcc[P * a.ct + c] = val;
      }
    }
  }
}

__global__ void dvv_from_gvv_kernel(const double *Gvv, int64_t naux, int64_t vt, double *dvv) {
  const int64_t total = naux * vt;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t v = t % vt, P = t / vt;
    dvv[P * vt + v] = Gvv[(v * naux + P) * vt + v];
  }
}

__global__ void hqp_diag_kernel(double cqp, const double *__restrict__ Hcc,
                                const double *__restrict__ Hvv, int64_t vt, int64_t ct,
                                const double *__restrict__ X, int64_t ldx, int64_t k,
                                double *__restrict__ Y, int64_t ldy, int accumulate) {
  const int64_t dim = vt * ct, total = dim * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t I = t % dim, j = t / dim;
    const int64_t v = I / ct, c = I % ct;
    const double e = Hcc[c + ct * c] - Hvv[v + vt * v];
    const double val = cqp * e * X[I + ldx * j];
    double *y = Y + I + ldy * j;
    *y = accumulate ? *y + val : val;
  }
}

struct HqpJob {
  double cqp;
  const double *Hcc, *Hvv;
  const double *diag;  // if set: Y = diag o X (the full diagonal), Hcc/Hvv unused
  int64_t vt, ct;
  const double *X;
  int64_t ldx, k;
  double *Y;
  int64_t ldy;
  int accumulate;
};
constexpr int kHqpJobsMax = 128;
struct HqpGroup {
  HqpJob j[kHqpJobsMax];
  int n;
};
static_assert(sizeof(HqpGroup) <= 32000, "Hqp job list too large");

__global__ void hqp_diag_group_kernel(const __grid_constant__ HqpGroup g) {
  const HqpJob q = g.j[blockIdx.y];
  const int64_t dim = q.vt * q.ct, total = dim * q.k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t I = t % dim, j = t / dim;
    const int64_t v = I / q.ct, c = I % q.ct;
    const double e = q.diag ? q.diag[I] : q.cqp * (q.Hcc[c + q.ct * c] - q.Hvv[v + q.vt * v]);
    const double val = e * q.X[I + q.ldx * j];
    double *y = q.Y + I + q.ldy * j;
    *y = q.accumulate ? *y + val : val;
  }
}

__global__ void zero_cols_kernel(double *Y, int64_t ldy, int64_t rows, int64_t k) {
  const int64_t total = rows * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    Y[(t % rows) + ldy * (t / rows)] = 0.0;
}

struct DiagArgs {
  double cqp, cx, cd, cd2;
  int64_t vt, ct, naux, dim;
  const double *Bvc, *Mcv, *dcc, *dvv, *Hcc, *Hvv;
  double *D;
};

// sum_P x[P * sx] * y[P * sy] with four independent FMA chains (the FP64 pipe of GB300 has a long
// latency: one chain per thread leaves it idle), combined in a fixed order
__device__ __forceinline__ double strided_dot(const double *x, int64_t sx, const double *y, int64_t sy,
                                              int64_t n) {
  double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
  int64_t P = 0;
  for (; P + 4 <= n; P += 4) {
    s0 = fma(x[P * sx], y[P * sy], s0);
    s1 = fma(x[(P + 1) * sx], y[(P + 1) * sy], s1);
    s2 = fma(x[(P + 2) * sx], y[(P + 2) * sy], s2);
    s3 = fma(x[(P + 3) * sx], y[(P + 3) * sy], s3);
  }
  for (; P < n; ++P) s0 = fma(x[P * sx], y[P * sy], s0);
  return (s0 + s1) + (s2 + s3);
}

// BSE_OPERATOR::diagonal (bse_operator.cc:133-175), one thread per pair.
__device__ __forceinline__ void diagonal_range(const DiagArgs &a, int64_t I0, int64_t step) {
  for (int64_t I = I0; I < a.dim; I += step) {
    const int64_t v = I / a.ct, c = I % a.ct;
    double entry = 0.0;
    if (a.cx != 0.0) entry += a.cx * strided_dot(a.Bvc + I, a.dim, a.Bvc + I, a.dim, a.naux);
    if (a.cqp != 0.0) entry += a.cqp * (a.Hcc[c + a.ct * c] - a.Hvv[v + a.vt * v]);
    if (a.cd != 0.0) entry -= a.cd * strided_dot(a.dcc + c, a.ct, a.dvv + v, a.vt, a.naux);
    if (a.cd2 != 0.0) entry -= a.cd2 * strided_dot(a.Mcv + I, a.dim, a.Bvc + I, a.dim, a.naux);
    a.D[I] = entry;
  }
}

// One operator: 32 pairs per 256-thread block, the aux sum of each pair split over the block's 8
// warps (P = w, w + 8, ...; lanes run over consecutive pairs, so every load is a coalesced 256-byte
// row segment) and the 8 partial sums added in a fixed order: enough independent FMA chains per
// SM to keep the FP64 pipe and the memory system busy.
constexpr int kDiagSlices = 8;
__global__ void __launch_bounds__(32 * kDiagSlices) diagonal_kernel(const DiagArgs a) {
  __shared__ double part[kDiagSlices][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int64_t I0 = blockIdx.x * 32LL; I0 < a.dim; I0 += (int64_t)gridDim.x * 32) {
    const int64_t I = I0 + lane;
    double sx0 = 0.0, sx1 = 0.0, sd0 = 0.0, sd1 = 0.0, s20 = 0.0, s21 = 0.0;
    if (I < a.dim) {
      const int64_t v = I / a.ct, c = I % a.ct;
      int64_t P = w;
      for (; P + kDiagSlices < a.naux; P += 2 * kDiagSlices) {
        const int64_t P1 = P + kDiagSlices;
        if (a.cx != 0.0 || a.cd2 != 0.0) {
          const double b0 = a.Bvc[P * a.dim + I], b1 = a.Bvc[P1 * a.dim + I];
          sx0 = fma(b0, b0, sx0);
          sx1 = fma(b1, b1, sx1);
          if (a.cd2 != 0.0) {
            s20 = fma(a.Mcv[P * a.dim + I], b0, s20);
            s21 = fma(a.Mcv[P1 * a.dim + I], b1, s21);
          }
        }
        if (a.cd != 0.0) {
          sd0 = fma(a.dcc[P * a.ct + c], a.dvv[P * a.vt + v], sd0);
          sd1 = fma(a.dcc[P1 * a.ct + c], a.dvv[P1 * a.vt + v], sd1);
        }
      }
      for (; P < a.naux; P += kDiagSlices) {
        if (a.cx != 0.0 || a.cd2 != 0.0) {
          const double b0 = a.Bvc[P * a.dim + I];
          sx0 = fma(b0, b0, sx0);
          if (a.cd2 != 0.0) s20 = fma(a.Mcv[P * a.dim + I], b0, s20);
        }
        if (a.cd != 0.0) sd0 = fma(a.dcc[P * a.ct + c], a.dvv[P * a.vt + v], sd0);
      }
    }
    part[w][lane] = a.cx * (sx0 + sx1) - a.cd * (sd0 + sd1) - a.cd2 * (s20 + s21);
    __syncthreads();
    if (w == 0 && I < a.dim) {
      double entry = 0.0;
#pragma unroll
      for (int q = 0; q < kDiagSlices; ++q) entry += part[q][lane];
      const int64_t v = I / a.ct, c = I % a.ct;
      if (a.cqp != 0.0) entry += a.cqp * (a.Hcc[c + a.ct * c] - a.Hvv[v + a.vt * v]);
      a.D[I] = entry;
    }
    __syncthreads();
  }
}

constexpr int kDiagJobsMax = 192;
struct DiagGroup {
  DiagArgs j[kDiagJobsMax];
  int n;
};
static_assert(sizeof(DiagGroup) <= 32000, "diagonal job list too large");

__global__ void diagonal_group_kernel(const __grid_constant__ DiagGroup g) {
  const DiagArgs a = g.j[blockIdx.y];
  diagonal_range(a, blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

__global__ void ham_combine_kernel(const double *__restrict__ TA, const double *__restrict__ TB,
                                   int64_t dim, int64_t k, double *__restrict__ Y, int64_t ldy) {
  const int64_t total = dim * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t q = t % dim, j = t / dim;
    const double a_top = TA[(2 * j) * dim + q], a_bot = TA[(2 * j + 1) * dim + q];
    const double b_top = TB[(2 * j) * dim + q], b_bot = TB[(2 * j + 1) * dim + q];
    Y[q + ldy * j] = a_top + b_bot;
    Y[dim + q + ldy * j] = -a_bot - b_top;
  }
}

__global__ void ham_diag_kernel(const double *D, int64_t dim, double *D2) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < dim;
       t += (int64_t)gridDim.x * blockDim.x) {
    D2[t] = D[t];
    D2[dim + t] = -D[t];
  }
}

__global__ void copy_cols_kernel(const double *X, int64_t ldx, int64_t rows, int64_t k, double *Y,
                                 int64_t ldy) {
  const int64_t total = rows * k;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    Y[(t % rows) + ldy * (t / rows)] = X[(t % rows) + ldx * (t / rows)];
}

unsigned grid_for(int64_t n, int threads = 256) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, threads), 16LL * 152));
}

}  // namespace

void ham_combine(const double *TA, const double *TB, int64_t dim, int64_t k, double *Y,
                 int64_t ldy, cudaStream_t s) {
  ham_combine_kernel<<<grid_for(dim * k), 256, 0, s>>>(TA, TB, dim, k, Y, ldy);
  VGB_LAUNCH_CHECK();
}

void ham_diag(const double *D, int64_t dim, double *D2, cudaStream_t s) {
  ham_diag_kernel<<<grid_for(dim), 256, 0, s>>>(D, dim, D2);
  VGB_LAUNCH_CHECK();
}

void copy_cols(const double *X, int64_t ldx, int64_t rows, int64_t k, double *Y, int64_t ldy,
               cudaStream_t s) {
  copy_cols_kernel<<<grid_for(rows * k), 256, 0, s>>>(X, ldx, rows, k, Y, ldy);
  VGB_LAUNCH_CHECK();
}

// ---------------- stage timer ----------------

StageTimer::~StageTimer() {
  for (auto &r : pending_) { cudaEventDestroy(r.a); cudaEventDestroy(r.b); }
  for (auto e : pool_) cudaEventDestroy(e);
}

cudaEvent_t StageTimer::get_() {
  if (!pool_.empty()) { cudaEvent_t e = pool_.back(); pool_.pop_back(); return e; }
  cudaEvent_t e;
  VGB_CUDA(cudaEventCreate(&e));
  return e;
}

void StageTimer::drain_() {
  for (auto &r : pending_) {
    VGB_CUDA(cudaEventSynchronize(r.b));
    float ms = 0.f;
    VGB_CUDA(cudaEventElapsedTime(&ms, r.a, r.b));
    ms_[r.stage] += ms;
    calls_[r.stage] += 1;
    pool_.push_back(r.a);
    pool_.push_back(r.b);
  }
  pending_.clear();
}

void StageTimer::enable(bool on) {
  drain_();
  on_ = on;
  for (int i = 0; i < STAGE_COUNT; ++i) { ms_[i] = 0.0; calls_[i] = 0; }
}

void StageTimer::begin(int stage, cudaStream_t s) {
  if (!on_) return;
  Rec r{get_(), get_(), stage};
  VGB_CUDA(cudaEventRecord(r.a, s));
  pending_.push_back(r);
}

void StageTimer::end(int stage, cudaStream_t s) {
  if (!on_) return;
  for (auto it = pending_.rbegin(); it != pending_.rend(); ++it)
    if (it->stage == stage) { VGB_CUDA(cudaEventRecord(it->b, s)); break; }
  if (pending_.size() > 4096) drain_();
}

void StageTimer::read(double *ms, int64_t *calls, int n) {
  drain_();
  for (int i = 0; i < n && i < STAGE_COUNT; ++i) {
    if (ms) ms[i] = ms_[i];
    if (calls) calls[i] = calls_[i];
  }
}

// Mvv[(P*vt + v1)*vt + v] = M(v1, v, P): the vv block before screening (for gradients).
void BseOperator::stage_unscreened_vv(const bse_mmn_desc &desc, const double *const *slices,
                                      const bse_options &opt, cudaStream_t s) {
  msize = desc.mmax - desc.mmin + 1;
  nsize = desc.nmax - desc.nmin + 1;
  m_v0 = opt.vmin - desc.mmin;
  m_c0 = opt.homo + 1 - desc.mmin;
  n_v0 = opt.vmin - desc.nmin;
  n_c0 = opt.homo + 1 - desc.nmin;
  std::vector<double> h(naux * vt * vt);
  for (int64_t v1 = 0; v1 < vt; ++v1) {
    const double *src = slices[m_v0 + v1];
    for (int64_t P = 0; P < naux; ++P)
      for (int64_t v = 0; v < vt; ++v) h[(P * vt + v1) * vt + v] = src[P * nsize + n_v0 + v];
  }
  Mvv.resize(naux * vt * vt);
  VGB_CUDA(cudaMemcpyAsync(Mvv.get(), h.data(), h.size() * sizeof(double), cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaStreamSynchronize(s));
}

BseOperator::BseOperator() = default;
BseOperator::~BseOperator() = default;

void BseOperator::stage(const bse_mmn_desc &desc, const double *const *slices, const double *w,
                        bool dense_w, const double *hqp, int64_t ldh, int64_t hqp_size,
                        const bse_options &opt, int prec, cudaStream_t s) {
  // BSE_OPERATOR::configure, bse_operator.cc:28-37
  const int64_t bse_vmax = opt.homo;
  const int64_t bse_cmin = opt.homo + 1;
  vt = bse_vmax - opt.vmin + 1;
  ct = opt.cmax - bse_cmin + 1;
  naux = desc.auxsize;
  dim = vt * ct;
  precision = prec;
  VGB_REQUIRE(vt >= 1 && ct >= 1, "bse_op_create: empty BSE window (homo/vmin/cmax)");
  VGB_REQUIRE(naux >= 1, "bse_op_create: auxsize must be positive");
  VGB_REQUIRE(slices != nullptr && w != nullptr && hqp != nullptr, "bse_op_create: null input");
  VGB_REQUIRE(prec == BSE_PRECISION_FP64 || prec == BSE_PRECISION_MIXED || prec == BSE_PRECISION_SLICED,
              "bse_op_create: unknown precision");
  const int64_t msize = desc.mmax - desc.mmin + 1, nsize = desc.nmax - desc.nmin + 1;
  VGB_REQUIRE(opt.vmin >= desc.mmin && opt.cmax <= desc.mmax,
              "bse_op_create: BSE window outside the Mmn m-range");
  VGB_REQUIRE(opt.vmin >= desc.nmin && opt.cmax <= desc.nmax,
              "bse_op_create: BSE window outside the Mmn n-range");
  VGB_REQUIRE(hqp_size >= vt + ct && ldh >= hqp_size, "bse_op_create: Hqp smaller than the BSE window");
  (void)msize;

  Bvc.resize(naux * dim);
  Mcc.resize(naux * ct * ct);
  Gvv.resize(vt * naux * vt);
  Mcv.resize(naux * dim);
  Mcv0.resize(naux * dim);
  dcc.resize(naux * ct);
  dvv.resize(naux * vt);
  Hcc.resize(ct * ct);
  Hvv.resize(vt * vt);

  DeviceBuffer<double> dw;
  if (!dense_w) {
    dw.resize(naux);
    VGB_CUDA(cudaMemcpyAsync(dw.get(), w, naux * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  // slices of the window, uploaded in chunks of <= 256 MB
  const int64_t slice_elems = nsize * naux;
  const int64_t nwin = vt + ct;
  int64_t chunk = std::max<int64_t>(1, (256LL << 20) / (slice_elems * (int64_t)sizeof(double)));
  chunk = std::min(chunk, nwin);
  DeviceBuffer<double> raw(chunk * slice_elems);
  for (int64_t m0 = 0; m0 < nwin; m0 += chunk) {
    const int64_t cnt = std::min(chunk, nwin - m0);
    for (int64_t i = 0; i < cnt; ++i) {
      const int64_t ml = m0 + i;
      const int64_t abs_m = ml < vt ? opt.vmin + ml : bse_cmin + (ml - vt);
      const double *src = slices[abs_m - desc.mmin];
      VGB_REQUIRE(src != nullptr, "bse_op_create: null Mmn slice");
      VGB_CUDA(cudaMemcpyAsync(raw.get() + i * slice_elems, src, slice_elems * sizeof(double),
                               cudaMemcpyHostToDevice, s));
    }
    ScatterArgs a;
    a.raw = raw.get();
    a.m_first = m0;
    a.m_count = cnt;
    a.nsize = nsize;
    a.naux = naux;
    a.vt = vt;
    a.ct = ct;
    a.dim = dim;
    a.n_v0 = opt.vmin - desc.nmin;
    a.n_c0 = bse_cmin - desc.nmin;
    a.w = dense_w ? nullptr : dw.get();
    a.Bvc = Bvc.get();
    a.Mcc = Mcc.get();
    a.Gvv = Gvv.get();
    a.Mcv = Mcv.get();
    a.Mcv0 = Mcv0.get();
    a.dcc = dcc.get();
    scatter_kernel<<<grid_for(cnt * naux * nwin), 256, 0, s>>>(a);
    VGB_LAUNCH_CHECK();
    VGB_CUDA(cudaStreamSynchronize(s));  // raw is reused by the next chunk
  }

  if (dense_w) {
    // fold the dense screening into the vv and cv blocks: X(., Q) = sum_P X(., P) W(P, Q)
    DeviceBuffer<double> dW(naux * naux), tmp(std::max(vt * naux * vt, naux * dim));
    VGB_CUDA(cudaMemcpyAsync(dW.get(), w, naux * naux * sizeof(double), cudaMemcpyHostToDevice, s));
    {
      GemmDesc g;
      g.M = vt; g.N = naux; g.K = naux;
      g.A = Gvv.get(); g.a_rs = 1; g.a_cs = vt;
      g.B = dW.get(); g.b_rs = 1; g.b_cs = naux;
      g.C = tmp.get(); g.c_rs = 1; g.c_cs = vt;
      g.nb1 = vt; g.a_b1 = naux * vt; g.c_b1 = naux * vt;
      dgemm(g, s, &ws);
      VGB_CUDA(cudaMemcpyAsync(Gvv.get(), tmp.get(), vt * naux * vt * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    }
    {
      GemmDesc g;
      g.M = dim; g.N = naux; g.K = naux;
      g.A = Mcv.get(); g.a_rs = 1; g.a_cs = dim;
      g.B = dW.get(); g.b_rs = 1; g.b_cs = naux;
      g.C = tmp.get(); g.c_rs = 1; g.c_cs = dim;
      dgemm(g, s, &ws);
      VGB_CUDA(cudaMemcpyAsync(Mcv.get(), tmp.get(), naux * dim * sizeof(double),
                               cudaMemcpyDeviceToDevice, s));
    }
    VGB_CUDA(cudaStreamSynchronize(s));
  }
  dvv_from_gvv_kernel<<<grid_for(naux * vt), 256, 0, s>>>(Gvv.get(), naux, vt, dvv.get());
  VGB_LAUNCH_CHECK();
  VGB_CUDA(cudaStreamSynchronize(s));
  stage_unscreened_vv(desc, slices, opt, s);
  dense_screening = dense_w;
  Wscr.resize(dense_w ? naux * naux : naux);
  VGB_CUDA(cudaMemcpyAsync(Wscr.get(), w, (dense_w ? naux * naux : naux) * sizeof(double),
                           cudaMemcpyHostToDevice, s));

  // Hqp window (BSE_OPERATOR::Hqp_row, bse_operator.cc:121-131)
  std::vector<double> hcc(ct * ct), hvv(vt * vt);
  hqp_diagonal = true;
  for (int64_t c1 = 0; c1 < ct; ++c1)
    for (int64_t c = 0; c < ct; ++c) {
      hcc[c + ct * c1] = hqp[(vt + c) + (vt + c1) * ldh];
      if (c != c1 && hcc[c + ct * c1] != 0.0) hqp_diagonal = false;
    }
  for (int64_t v1 = 0; v1 < vt; ++v1)
    for (int64_t v = 0; v < vt; ++v) {
      hvv[v + vt * v1] = hqp[v + v1 * ldh];
      if (v != v1 && hvv[v + vt * v1] != 0.0) hqp_diagonal = false;
    }
  // off-diagonal v-c couplings of Hqp are never read by the reference (Hqp_row)
  VGB_CUDA(cudaMemcpyAsync(Hcc.get(), hcc.data(), ct * ct * sizeof(double), cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaMemcpyAsync(Hvv.get(), hvv.data(), vt * vt * sizeof(double), cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaStreamSynchronize(s));

  if (precision == BSE_PRECISION_MIXED || precision == BSE_PRECISION_SLICED) {
    mixed.reset(new MixedEngine());
    mixed->stage(*this, s, precision == BSE_PRECISION_MIXED);
  }
}

void BseOperator::apply_hqp(double cqp, const double *X, int64_t ldx, int64_t k, double *Y,
                            int64_t ldy, bool accumulate, cudaStream_t s) {
  timer.begin(STAGE_HQP, s);
  struct End { StageTimer &t; cudaStream_t s; ~End() { t.end(STAGE_HQP, s); } } end_{timer, s};
  if (hqp_diagonal) {
    hqp_diag_kernel<<<grid_for(dim * k), 256, 0, s>>>(cqp, Hcc.get(), Hvv.get(), vt, ct, X, ldx, k,
                                                      Y, ldy, accumulate ? 1 : 0);
    VGB_LAUNCH_CHECK();
    return;
  }
  // Y_j(c1, v1) (+)= cqp * sum_c Hcc(c, c1) X_j(c, v1) - cqp * sum_v X_j(c1, v) Hvv(v, v1)
  GemmDesc g;
  g.M = ct; g.N = vt; g.K = ct;
  g.A = Hcc.get(); g.a_rs = ct; g.a_cs = 1;
  g.B = X; g.b_rs = 1; g.b_cs = ct; g.b_b1 = ldx;
  g.C = Y; g.c_rs = 1; g.c_cs = ct; g.c_b1 = ldy;
  g.nb1 = k; g.alpha = cqp; g.beta = accumulate ? 1.0 : 0.0;
  dgemm(g, s, &ws);
  GemmDesc h;
  h.M = ct; h.N = vt; h.K = vt;
  h.A = X; h.a_rs = 1; h.a_cs = ct; h.a_b1 = ldx;
  h.B = Hvv.get(); h.b_rs = 1; h.b_cs = vt;
  h.C = Y; h.c_rs = 1; h.c_cs = ct; h.c_b1 = ldy;
  h.nb1 = k; h.alpha = -cqp; h.beta = 1.0;
  dgemm(h, s, &ws);
}

void BseOperator::apply_hx_fp64(double cx, const double *X, int64_t ldx, int64_t k, double *Y,
                                int64_t ldy, bool accumulate, cudaStream_t s) {
  Z.resize(naux * k);
  timer.begin(STAGE_HX, s);
  GemmDesc g;  // Z (naux x k) = Bvc^T X
  g.M = naux; g.N = k; g.K = dim;
  g.A = Bvc.get(); g.a_rs = dim; g.a_cs = 1;
  g.B = X; g.b_rs = 1; g.b_cs = ldx;
  g.C = Z.get(); g.c_rs = 1; g.c_cs = naux;
  dgemm(g, s, &ws);
  GemmDesc h;  // Y (+)= cx Bvc Z
  h.M = dim; h.N = k; h.K = naux;
  h.A = Bvc.get(); h.a_rs = 1; h.a_cs = dim;
  h.B = Z.get(); h.b_rs = 1; h.b_cs = naux;
  h.C = Y; h.c_rs = 1; h.c_cs = ldy;
  h.alpha = cx; h.beta = accumulate ? 1.0 : 0.0;
  dgemm(h, s, &ws);
  timer.end(STAGE_HX, s);
}

void BseOperator::apply_hd_fp64(double alpha, const double *X, int64_t ldx, int64_t k, double *Y,
                                int64_t ldy, bool accumulate, cudaStream_t s) {
  const int64_t per_vec = naux * dim;
  const int64_t jchunk =
      std::max<int64_t>(1, std::min<int64_t>(k, s_budget_bytes / (per_vec * (int64_t)sizeof(double))));
  S.resize(jchunk * per_vec);
  for (int64_t j0 = 0; j0 < k; j0 += jchunk) {
    const int64_t kc = std::min(jchunk, k - j0);
    GemmDesc a;  // S[j][P](c1, v) = sum_c Mcc_P(c1, c) X_j(c, v)
    a.M = ct; a.N = vt; a.K = ct;
    a.A = Mcc.get(); a.a_rs = 1; a.a_cs = ct;
    a.B = X + j0 * ldx; a.b_rs = 1; a.b_cs = ct;
    a.C = S.get(); a.c_rs = 1; a.c_cs = ct;
    a.nb1 = kc; a.nb2 = naux;
    a.a_b1 = 0; a.a_b2 = ct * ct;
    a.b_b1 = ldx; a.b_b2 = 0;
    a.c_b1 = per_vec; a.c_b2 = dim;
    timer.begin(STAGE_HD_A, s);
    dgemm(a, s, &ws);
    timer.end(STAGE_HD_A, s);
    GemmDesc b;  // Y_j(c1, v1) (+)= alpha sum_{P,v} S[j](c1, (P,v)) Gvv((P,v), v1)
    b.M = ct; b.N = vt; b.K = naux * vt;
    b.A = S.get(); b.a_rs = 1; b.a_cs = ct; b.a_b1 = per_vec;
    b.B = Gvv.get(); b.b_rs = 1; b.b_cs = naux * vt;
    b.C = Y + j0 * ldy; b.c_rs = 1; b.c_cs = ct; b.c_b1 = ldy;
    b.nb1 = kc; b.alpha = alpha; b.beta = accumulate ? 1.0 : 0.0;
    timer.begin(STAGE_HD_B, s);
    dgemm(b, s, &ws);
    timer.end(STAGE_HD_B, s);
  }
}

void BseOperator::apply_hd2_fp64(double alpha, const double *X, int64_t ldx, int64_t k, double *Y,
                                 int64_t ldy, bool accumulate, cudaStream_t s) {
  const int64_t per_vec = vt * naux * vt;
  const int64_t jchunk =
      std::max<int64_t>(1, std::min<int64_t>(k, s_budget_bytes / (per_vec * (int64_t)sizeof(double))));
  Ttmp.resize(jchunk * per_vec);
  for (int64_t j0 = 0; j0 < k; j0 += jchunk) {
    const int64_t kc = std::min(jchunk, k - j0);
    GemmDesc a;  // U[j][v1][P][v] = sum_c X_j(c, v) Bvc_P(c, v1)
    a.M = vt; a.N = vt; a.K = ct;
    a.A = X + j0 * ldx; a.a_rs = ct; a.a_cs = 1;
    a.B = Bvc.get(); a.b_rs = 1; a.b_cs = ct;
    a.C = Ttmp.get(); a.c_rs = 1; a.c_cs = naux * vt;
    a.nb1 = kc; a.nb2 = naux;
    a.a_b1 = ldx; a.a_b2 = 0;
    a.b_b1 = 0; a.b_b2 = dim;
    a.c_b1 = per_vec; a.c_b2 = vt;
    timer.begin(STAGE_HD2_A, s);
    dgemm(a, s, &ws);
    timer.end(STAGE_HD2_A, s);
    GemmDesc b;  // Y_j(c1, v1) (+)= alpha sum_{P,v} Mcv(c1, (P,v)) U_j((P,v), v1)
    b.M = ct; b.N = vt; b.K = naux * vt;
    b.A = Mcv.get(); b.a_rs = 1; b.a_cs = ct;
    b.B = Ttmp.get(); b.b_rs = 1; b.b_cs = naux * vt; b.b_b1 = per_vec;
    b.C = Y + j0 * ldy; b.c_rs = 1; b.c_cs = ct; b.c_b1 = ldy;
    b.nb1 = kc; b.alpha = alpha; b.beta = accumulate ? 1.0 : 0.0;
    timer.begin(STAGE_HD2_B, s);
    dgemm(b, s, &ws);
    timer.end(STAGE_HD2_B, s);
  }
}

void BseOperator::matmul(const Coef &c, const double *X, int64_t ldx, int64_t k, double *Y,
                         int64_t ldy, cudaStream_t s) {
  VGB_REQUIRE(ldx >= dim && ldy >= dim, "matmul: leading dimension smaller than the operator size");
  VGB_REQUIRE(k >= 0, "matmul: negative column count");
  if (k == 0) return;
  VGB_REQUIRE(!(c.cd != 0 && c.cd2 != 0), "Hamiltonian cannot contain Hd and Hd2 at the same time");
  bool acc = false;
  if (c.cqp != 0) { apply_hqp(c.cqp, X, ldx, k, Y, ldy, acc, s); acc = true; }
  if (mixed && (precision == BSE_PRECISION_SLICED ||
                (precision == BSE_PRECISION_MIXED && force_fp64 && fp64_products == 0))) {
    mixed->apply_sliced(*this, c, X, ldx, k, Y, ldy, acc, s);
    return;
  }
  if (precision == BSE_PRECISION_MIXED && mixed && !force_fp64) {
    mixed->apply(*this, c, X, ldx, k, Y, ldy, acc, s);
    return;
  }
  if (c.cx != 0) { apply_hx_fp64(c.cx, X, ldx, k, Y, ldy, acc, s); acc = true; }
  if (c.cd != 0) { apply_hd_fp64(-(double)c.cd, X, ldx, k, Y, ldy, acc, s); acc = true; }
  if (c.cd2 != 0) { apply_hd2_fp64(-(double)c.cd2, X, ldx, k, Y, ldy, acc, s); acc = true; }
  if (!acc) {
    zero_cols_kernel<<<grid_for(dim * k), 256, 0, s>>>(Y, ldy, dim, k);
    VGB_LAUNCH_CHECK();
  }
}

void matmul_grouped(const Coef &c, const std::vector<GroupedItem> &items, cudaStream_t s,
                    GroupScratch *scratch) {
  VGB_REQUIRE(c.cd2 == 0, "grouped products: Hd2 is not grouped");
  std::vector<GroupedItem> mixed_items, dense_items;
  std::vector<HqpJob> hq;
  for (const GroupedItem &it : items) {
    BseOperator &op = *it.op;
    VGB_REQUIRE(it.ldx >= op.dim && it.ldy >= op.dim, "matmul: leading dimension smaller than the operator size");
    if (it.k <= 0) continue;
    if (it.dense) {
      VGB_REQUIRE(op.mixed && op.mixed->dense_ready(c) && it.diag, "grouped products: dense form not built");
      HqpJob j;  // the exact diagonal, then the off-diagonal dense part accumulates
      j.cqp = 1; j.Hcc = nullptr; j.Hvv = nullptr; j.diag = it.diag; j.vt = op.vt; j.ct = op.ct;
      j.X = it.X; j.ldx = it.ldx; j.k = it.k; j.Y = it.Y; j.ldy = it.ldy; j.accumulate = 0;
      hq.push_back(j);
      dense_items.push_back(it);
      continue;
    }
    if (op.precision != BSE_PRECISION_MIXED || !op.mixed) {  // FP64 operators: one product each
      op.matmul(c, it.X, it.ldx, it.k, it.Y, it.ldy, s);
      continue;
    }
    if (c.cqp != 0) {
      if (op.hqp_diagonal) {
        HqpJob j;
        j.cqp = c.cqp; j.Hcc = op.Hcc.get(); j.Hvv = op.Hvv.get(); j.diag = nullptr; j.vt = op.vt; j.ct = op.ct;
        j.X = it.X; j.ldx = it.ldx; j.k = it.k; j.Y = it.Y; j.ldy = it.ldy; j.accumulate = 0;
        hq.push_back(j);
      } else {
        op.apply_hqp(c.cqp, it.X, it.ldx, it.k, it.Y, it.ldy, false, s);
      }
    }
    mixed_items.push_back(it);
  }
  std::unique_ptr<HqpGroup> g(new HqpGroup());
  for (size_t i = 0; i < hq.size();) {
    g->n = 0;
    int64_t mx = 0;
    for (; i < hq.size() && g->n < kHqpJobsMax; ++i) {
      g->j[g->n++] = hq[i];
      mx = std::max(mx, hq[i].vt * hq[i].ct * hq[i].k);
    }
    const unsigned bx = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(mx, 256), 64));
    hqp_diag_group_kernel<<<dim3(bx, (unsigned)g->n), 256, 0, s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
  MixedEngine::apply_grouped(c, mixed_items, c.cqp != 0, s, scratch);
  MixedEngine::apply_dense_grouped(c, dense_items, true, s);
}

void BseOperator::check_errors(cudaStream_t s) {
  if (mixed) mixed->check(s);
}

void BseOperator::diagonal(const Coef &c, double *D, cudaStream_t s) {
  VGB_REQUIRE(!(c.cd != 0 && c.cd2 != 0), "Hamiltonian cannot contain Hd and Hd2 at the same time");
  DiagArgs a;
  a.cqp = c.cqp; a.cx = c.cx; a.cd = c.cd; a.cd2 = c.cd2;
  a.vt = vt; a.ct = ct; a.naux = naux; a.dim = dim;
  a.Bvc = Bvc.get(); a.Mcv = Mcv.get(); a.dcc = dcc.get(); a.dvv = dvv.get();
  a.Hcc = Hcc.get(); a.Hvv = Hvv.get(); a.D = D;
  diagonal_kernel<<<(unsigned)std::min<int64_t>(ceil_div(dim, 32), 64LL * sm_count()), 32 * kDiagSlices, 0, s>>>(a);
  VGB_LAUNCH_CHECK();
}

void diagonal_grouped(const Coef &c, const std::vector<BseOperator *> &ops,
                      const std::vector<double *> &D, cudaStream_t s) {
  VGB_REQUIRE(!(c.cd != 0 && c.cd2 != 0), "Hamiltonian cannot contain Hd and Hd2 at the same time");
  VGB_REQUIRE(ops.size() == D.size(), "diagonal_grouped: one output per operator");
  std::unique_ptr<DiagGroup> g(new DiagGroup());
  for (size_t i = 0; i < ops.size();) {
    g->n = 0;
    int64_t mx = 1;
    for (; i < ops.size() && g->n < kDiagJobsMax; ++i) {
      const BseOperator &op = *ops[i];
      DiagArgs &a = g->j[g->n++];
      a.cqp = c.cqp; a.cx = c.cx; a.cd = c.cd; a.cd2 = c.cd2;
      a.vt = op.vt; a.ct = op.ct; a.naux = op.naux; a.dim = op.dim;
      a.Bvc = op.Bvc.get(); a.Mcv = op.Mcv.get(); a.dcc = op.dcc.get(); a.dvv = op.dvv.get();
      a.Hcc = op.Hcc.get(); a.Hvv = op.Hvv.get(); a.D = D[i];
      mx = std::max(mx, op.dim);
    }
    diagonal_group_kernel<<<dim3((unsigned)ceil_div(mx, 128), (unsigned)g->n), 128, 0, s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
}

void BseOperator::ham_matmul(const Coef &a, const Coef &b, const double *X, int64_t ldx, int64_t k,
                             double *Y, int64_t ldy, cudaStream_t s) {
  VGB_REQUIRE(ldx >= 2 * dim && ldy >= 2 * dim, "ham_matmul: leading dimension too small");
  if (k == 0) return;
  // view X (2dim x k) as dim x 2k (columns M1_0, M2_0, M1_1, ...): needs ldx == 2 dim
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

void BseHamApply::diagonal(double *D, cudaStream_t s) {
  // HamiltonianOperator::get_diagonal: [D_A; -D_A] (bseoperator_btda.h:81-87)
  op->diagonal(a, D, s);
  ham_diag(D, op->dim, D, s);
}

// ---------------- dense operator ----------------

void DenseOperator::stage(const double *a, const double *b, int64_t n_, int64_t lda,
                          cudaStream_t s) {
  VGB_REQUIRE(n_ >= 1 && lda >= n_ && a != nullptr, "bse_dense_op_create: bad arguments");
  n = n_;
  has_b = b != nullptr;
  A.resize(n * n);
  VGB_CUDA(cudaMemcpy2DAsync(A.get(), n * sizeof(double), a, lda * sizeof(double),
                             n * sizeof(double), n, cudaMemcpyHostToDevice, s));
  if (has_b) {
    B.resize(n * n);
    VGB_CUDA(cudaMemcpy2DAsync(B.get(), n * sizeof(double), b, lda * sizeof(double),
                               n * sizeof(double), n, cudaMemcpyHostToDevice, s));
  }
  VGB_CUDA(cudaStreamSynchronize(s));
}

void DenseOperator::matmul(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                           cudaStream_t s) {
  if (k == 0) return;
  GemmDesc g;
  g.M = n; g.N = k; g.K = n;
  g.a_colmajor(A.get(), n, false).b_colmajor(X, ldx, false).c_colmajor(Y, ldy);
  dgemm(g, s, &ws);
}

__global__ void dense_diag_kernel(const double *A, int64_t n, double *D) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    D[t] = A[t + n * t];
}

void DenseOperator::diagonal(double *D, cudaStream_t s) {
  dense_diag_kernel<<<grid_for(n), 256, 0, s>>>(A.get(), n, D);
  VGB_LAUNCH_CHECK();
}

void DenseOperator::ham_matmul(const double *X, int64_t ldx, int64_t k, double *Y, int64_t ldy,
                               cudaStream_t s) {
  VGB_REQUIRE(has_b, "dense operator has no B block");
  if (k == 0) return;
  const double *Xv = X;
  if (ldx != 2 * n) {
    Xr.resize(2 * n * k);
    copy_cols(X, ldx, 2 * n, k, Xr.get(), 2 * n, s);
    Xv = Xr.get();
  }
  tmpA.resize(2 * n * k);
  tmpB.resize(2 * n * k);
  GemmDesc g;
  g.M = n; g.N = 2 * k; g.K = n;
  g.a_colmajor(A.get(), n, false).b_colmajor(Xv, n, false).c_colmajor(tmpA.get(), n);
  dgemm(g, s, &ws);
  g.a_colmajor(B.get(), n, false).c_colmajor(tmpB.get(), n);
  dgemm(g, s, &ws);
  ham_combine(tmpA.get(), tmpB.get(), n, k, Y, ldy, s);
}

void DenseApply::diagonal(double *D, cudaStream_t s) {
  op->diagonal(D, s);
  if (ham) ham_diag(D, op->n, D, s);
}

}  // namespace vgb
