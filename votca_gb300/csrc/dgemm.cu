// FP64 strided batched GEMM (see dgemm.cuh for the design note).
#include "dgemm.cuh"

#include <mutex>

namespace vgb {

namespace {

constexpr int TM = 64;
constexpr int TN = 64;
constexpr int TK = 16;
constexpr int THREADS = 256;

struct Grid {
  int64_t mt, nt, nbatch, splits, kchunk;
};

__global__ void __launch_bounds__(THREADS)
    dgemm_kernel(const GemmDesc d, const Grid g, double *__restrict__ partial, int a_icontig,
                 int b_lcontig) {
  __shared__ double As[TK][TM + 1];
  __shared__ double Bs[TK][TN + 1];

  // flat block index -> (split, batch, n-tile, m-tile)
  int64_t bid = blockIdx.x;
  const int64_t mtile = bid % g.mt;
  bid /= g.mt;
  const int64_t ntile = bid % g.nt;
  bid /= g.nt;
  const int64_t s = bid % g.splits;
  const int64_t batch = bid / g.splits;
  const int64_t b1 = batch / d.nb2, b2 = batch % d.nb2;

  const double *__restrict__ A = d.A + b1 * d.a_b1 + b2 * d.a_b2;
  const double *__restrict__ B = d.B + b1 * d.b_b1 + b2 * d.b_b2;

  const int64_t m0 = mtile * TM, n0 = ntile * TN;
  const int64_t kbeg = s * g.kchunk;
  const int64_t kend = min(d.K, kbeg + g.kchunk);

  const int tid = threadIdx.x;
  const int tx = tid & 15, ty = tid >> 4;
  double acc[4][4];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;

  for (int64_t k0 = kbeg; k0 < kend; k0 += TK) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int e = tid + THREADS * r;
      int i, l;
      if (a_icontig) { i = e & (TM - 1); l = e >> 6; } else { l = e & (TK - 1); i = e >> 4; }
      const int64_t gi = m0 + i, gl = k0 + l;
      As[l][i] = (gi < d.M && gl < kend) ? A[gi * d.a_rs + gl * d.a_cs] : 0.0;
      int n;
      if (b_lcontig) { l = e & (TK - 1); n = e >> 4; } else { n = e & (TN - 1); l = e >> 6; }
      const int64_t gn = n0 + n, gl2 = k0 + l;
      Bs[l][n] = (gn < d.N && gl2 < kend) ? B[gl2 * d.b_rs + gn * d.b_cs] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int l = 0; l < TK; ++l) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[l][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[l][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }

  if (g.splits == 1) {
    double *__restrict__ C = d.C + b1 * d.c_b1 + b2 * d.c_b2;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t gi = m0 + ty + 16 * i;
      if (gi >= d.M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t gn = n0 + tx + 16 * j;
        if (gn >= d.N) continue;
        double *c = C + gi * d.c_rs + gn * d.c_cs;
        const double v = d.alpha * acc[i][j];
        *c = (d.beta == 0.0) ? v : fma(d.beta, *c, v);
      }
    }
  } else {
    double *__restrict__ P = partial + (batch * g.splits + s) * d.M * d.N;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const int64_t gi = m0 + ty + 16 * i;
      if (gi >= d.M) continue;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        const int64_t gn = n0 + tx + 16 * j;
        if (gn >= d.N) continue;
        P[gi + gn * d.M] = acc[i][j];
      }
    }
  }
}

// C = alpha * sum_s partial[s] + beta * C, in a fixed order (deterministic).
__global__ void splitk_reduce_kernel(const GemmDesc d, const Grid g,
                                     const double *__restrict__ partial) {
  const int64_t mn = d.M * d.N;
  const int64_t total = mn * g.nbatch;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t batch = t / mn, e = t % mn;
    const int64_t i = e % d.M, n = e / d.M;
    const double *p = partial + batch * g.splits * mn + e;
    double acc = 0.0;
    for (int64_t s = 0; s < g.splits; ++s) acc += p[s * mn];
    const int64_t b1 = batch / d.nb2, b2 = batch % d.nb2;
    double *c = d.C + b1 * d.c_b1 + b2 * d.c_b2 + i * d.c_rs + n * d.c_cs;
    const double v = d.alpha * acc;
    *c = (d.beta == 0.0) ? v : fma(d.beta, *c, v);
  }
}

__global__ void scale_kernel(const GemmDesc d, int64_t nbatch) {
  const int64_t mn = d.M * d.N, total = mn * nbatch;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t batch = t / mn, e = t % mn;
    const int64_t i = e % d.M, n = e / d.M;
    const int64_t b1 = batch / d.nb2, b2 = batch % d.nb2;
    double *c = d.C + b1 * d.c_b1 + b2 * d.c_b2 + i * d.c_rs + n * d.c_cs;
    *c = (d.beta == 0.0) ? 0.0 : d.beta * *c;
  }
}

}  // namespace

cudaStream_t &alloc_stream() {
  static thread_local cudaStream_t s = nullptr;
  return s;
}

namespace {
// Freed blocks stay in the device's default pool instead of being returned to
// the driver at every synchronisation (the Davidson loop synchronises once per
// iteration); bse_op_destroy trims the pool.
void keep_pool_blocks() {
  static std::once_flag once;
  std::call_once(once, [] {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t thr = UINT64_MAX;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
  });
}
}  // namespace

void *device_alloc(size_t bytes, cudaStream_t &used) {
  void *p = nullptr;
  used = alloc_stream();
  if (used) {
    keep_pool_blocks();
    VGB_CUDA(cudaMallocAsync(&p, bytes, used));
  } else {
    VGB_CUDA(cudaMalloc(&p, bytes));
  }
  return p;
}

// A stream-ordered block is freed on the stream of the running call, which is
// ordered after every use in this call; uses in earlier calls on other streams
// are complete by the handle's contract.  Outside a stream scope the free waits
// for the device first, as cudaFree does.
void device_free(void *p, cudaStream_t used) {
  if (!used) {
    cudaFree(p);
  } else if (cudaStream_t cur = alloc_stream()) {
    cudaFreeAsync(p, cur);
  } else {
    cudaDeviceSynchronize();  // nothing is in flight: any stream may take the free
    cudaFreeAsync(p, 0);
  }
}

void trim_pool() {
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess)
    cudaMemPoolTrimTo(pool, 0);
}

int sm_count() {
  static const int n = [] {
    int dev = 0, v = 0;
    VGB_CUDA(cudaGetDevice(&dev));
    VGB_CUDA(cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev));
    return v;
  }();
  return n;
}

void dgemm(const GemmDesc &d, cudaStream_t stream, GemmWorkspace *ws, int splitk) {
  VGB_REQUIRE(d.M >= 0 && d.N >= 0 && d.K >= 0, "dgemm: negative size");
  const int64_t nbatch = d.nb1 * d.nb2;
  if (d.M == 0 || d.N == 0 || nbatch == 0) return;
  if (d.K == 0) {  // C = beta * C
    const int64_t total = d.M * d.N * nbatch;
    scale_kernel<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 65535), 256, 0, stream>>>(d, nbatch);
    VGB_LAUNCH_CHECK();
    return;
  }
  Grid g;
  g.mt = ceil_div(d.M, TM);
  g.nt = ceil_div(d.N, TN);
  g.nbatch = nbatch;
  const int64_t tiles = g.mt * g.nt * nbatch;
  int64_t splits = splitk;
  if (splits <= 0) {
    const int64_t target = 3LL * sm_count();
    splits = 1;
    if (tiles < target && d.K > 4 * TK) {
      splits = std::min<int64_t>(ceil_div(target, tiles), ceil_div(d.K, 8 * TK));
      splits = std::max<int64_t>(1, std::min<int64_t>(splits, 256));
    }
  }
  g.kchunk = ceil_div(ceil_div(d.K, splits), TK) * TK;
  g.splits = ceil_div(d.K, g.kchunk);
  double *partial = nullptr;
  if (g.splits > 1) {
    VGB_REQUIRE(ws != nullptr, "dgemm: split-K needs a workspace");
    ws->partial.resize((size_t)(nbatch * g.splits * d.M * d.N));
    partial = ws->partial.get();
  }
  const int64_t blocks = tiles * g.splits;
  VGB_REQUIRE(blocks < (1LL << 31), "dgemm: grid too large");
  const int a_icontig = (d.a_rs == 1) ? 1 : 0;
  const int b_lcontig = (d.b_rs == 1) ? 1 : 0;
  dgemm_kernel<<<(unsigned)blocks, THREADS, 0, stream>>>(d, g, partial, a_icontig, b_lcontig);
  VGB_LAUNCH_CHECK();
  if (g.splits > 1) {
    const int64_t total = d.M * d.N * nbatch;
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 8 * sm_count()), 256, 0,
                           stream>>>(d, g, partial);
    VGB_LAUNCH_CHECK();
  }
}

void dgemm_prealloc(const GemmDesc &d, cudaStream_t stream, double *ws, int64_t ws_count) {
  VGB_REQUIRE(d.M >= 0 && d.N >= 0 && d.K >= 0, "dgemm: negative size");
  const int64_t nbatch = d.nb1 * d.nb2;
  if (d.M == 0 || d.N == 0 || nbatch == 0) return;
  if (d.K == 0) {
    const int64_t total = d.M * d.N * nbatch;
    scale_kernel<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 65535), 256, 0, stream>>>(d, nbatch);
    VGB_LAUNCH_CHECK();
    return;
  }
  Grid g;
  g.mt = ceil_div(d.M, TM);
  g.nt = ceil_div(d.N, TN);
  g.nbatch = nbatch;
  const int64_t tiles = g.mt * g.nt * nbatch;
  int64_t splits = 1;
  const int64_t target = 3LL * sm_count();
  if (ws && tiles < target && d.K > 4 * TK) {
    splits = std::min<int64_t>(ceil_div(target, tiles), ceil_div(d.K, 8 * TK));
    splits = std::max<int64_t>(1, std::min<int64_t>(splits, 256));
    const int64_t fit = ws_count / std::max<int64_t>(1, nbatch * d.M * d.N);
    splits = std::max<int64_t>(1, std::min(splits, fit));
  }
  g.kchunk = ceil_div(ceil_div(d.K, splits), TK) * TK;
  g.splits = ceil_div(d.K, g.kchunk);
  const int64_t blocks = tiles * g.splits;
  VGB_REQUIRE(blocks < (1LL << 31), "dgemm: grid too large");
  dgemm_kernel<<<(unsigned)blocks, THREADS, 0, stream>>>(d, g, g.splits > 1 ? ws : nullptr,
                                                          (d.a_rs == 1) ? 1 : 0, (d.b_rs == 1) ? 1 : 0);
  VGB_LAUNCH_CHECK();
  if (g.splits > 1) {
    const int64_t total = d.M * d.N * nbatch;
    splitk_reduce_kernel<<<(unsigned)std::min<int64_t>(ceil_div(total, 256), 8 * sm_count()), 256, 0,
                           stream>>>(d, g, ws);
    VGB_LAUNCH_CHECK();
  }
}

}  // namespace vgb
