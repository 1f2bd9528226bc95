// Lockstep Davidson over many independent molecules.
//
// Every molecule runs the DavidsonSolver iteration of davidson.cu (SYMM
// matrices, DPR correction, SAFE/MIN/MAX update, restart; davidsonsolver.cc
// :149-555) with its own search space, but all molecules advance together: each
// step of an iteration is one grouped launch over the molecules that are still
// iterating.  The operator products go through matmul_grouped (tensor-core
// stages grouped across molecules), the FP64 projections, Ritz vectors,
// corrections and Gram-Schmidt through the grouped kernels below, and the small
// eigenproblems of all molecules in one launch of the device eigensolver
// (small_eig.cu) on projected matrices that never leave HBM.  Per iteration the
// host synchronises twice (residual norms and Ritz values; the Gram-Schmidt
// flags ride with them), whatever the number of molecules.
#include "batch_davidson.cuh"

#include <algorithm>
#include <functional>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <exception>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <unistd.h>

#include <cooperative_groups.h>

#include "small_eig.cuh"
#include "tc_engine.cuh"

namespace vgb {

namespace {

namespace cg = cooperative_groups;

constexpr int kThreads = 256;
constexpr int kJobs = 320;       // jobs per grouped launch: a 256-molecule step in one launch
                                 // (the job list travels in the 32 KB kernel-parameter space)
constexpr int kTnRows = 512;     // rows per block of a transposed product
constexpr int kTile = 32;        // rows per shared-memory tile
constexpr int kTileLd = kTile + 1;
constexpr int kTnCols = 160;     // m + p columns per transposed-product job
constexpr int kTnOut = 8;        // outputs per thread: m * p <= 8 * 256
constexpr int kNnSmem = 48 * 1024;
// Dense form up to dim 16384 (1 GB of bf16 hi/lo per molecule), smallest molecules first, while
// the dense forms of the batch stay within 32 GB.  A dense product costs 6 d^2 flops per column
// against 6 Naux v c^2 for the factorised Hd alone (v < Naux in practice) and reads 4 d^2 bytes.
// Its FP32 chains over K = dim are kept at 256 terms (the dense chain bound of the engine): with
// 1024-term chains some residuals of the 256-molecule set stalled above 1e-7 from dim ~5000.
constexpr int64_t kDenseMaxDim = 16384;
constexpr int64_t kDenseBudgetBytes = 32LL << 30;

template <class Job>
struct Group {
  Job j[kJobs];
  int n;
};

// ---- C (m x p) = A^T B over row chunks: partial sums per chunk (fixed order) ----
struct TnJob {
  const double *A, *B;
  int64_t lda, ldb, n, m, p;
  double *part;  // [chunk][m * p]
};
__global__ void __launch_bounds__(kThreads, 4) tn_partial_kernel(const __grid_constant__ Group<TnJob> g) {
  const TnJob q = g.j[blockIdx.y];
  const int64_t r0 = (int64_t)blockIdx.x * kTnRows;
  if (r0 >= q.n) return;
  const int64_t r1 = min(q.n, r0 + kTnRows);
  __shared__ double sm[kTileLd * kTnCols];
  const int cols = (int)(q.m + q.p);
  const int64_t mp = q.m * q.p;
  // Fewer outputs than threads (m p <= 128): the rows of a tile are split over S lanes of one
  // warp per output, so that every warp of the block issues FP64 FMAs (GB300 has about 2 FP64
  // FMA lanes per clock and SM: a block whose outputs fit in two warps would use half of them).
  int S = 1;
  while (S < 32 && mp * 2 * S <= kThreads) S *= 2;
  const int sub = threadIdx.x & (S - 1);
  const int64_t os = threadIdx.x / S;  // the output of this thread when S > 1
  double acc[kTnOut];
#pragma unroll
  for (int k = 0; k < kTnOut; ++k) acc[k] = 0.0;
  for (int64_t rt = r0; rt < r1; rt += kTile) {
    const int rows = (int)min((int64_t)kTile, r1 - rt);
    for (int e = threadIdx.x; e < kTile * cols; e += kThreads) {
      const int col = e / kTile, r = e % kTile;
      double v = 0.0;
      if (r < rows) v = col < q.m ? q.A[rt + r + col * q.lda] : q.B[rt + r + (col - q.m) * q.ldb];
      sm[col * kTileLd + r] = v;
    }
    __syncthreads();
    if (S > 1) {
      if (os < mp) {
        const double *a = sm + (os % q.m) * kTileLd, *b = sm + (q.m + os / q.m) * kTileLd;
        double s = acc[0];
        for (int r = sub; r < rows; r += S) s = fma(a[r], b[r], s);
        acc[0] = s;
      }
    } else {
#pragma unroll
      for (int k = 0; k < kTnOut; ++k) {
        const int64_t o = threadIdx.x + (int64_t)k * kThreads;
        if (o < mp) {
          const double *a = sm + (o % q.m) * kTileLd, *b = sm + (q.m + o / q.m) * kTileLd;
          double s = acc[k];
          for (int r = 0; r < rows; ++r) s = fma(a[r], b[r], s);
          acc[k] = s;
        }
      }
    }
    __syncthreads();
  }
  if (S > 1) {  // the S lanes of an output are consecutive lanes of one warp (S divides 32)
    double v = acc[0];
    for (int off = S / 2; off > 0; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    if (sub == 0 && os < mp) q.part[blockIdx.x * mp + os] = v;
    return;
  }
#pragma unroll
  for (int k = 0; k < kTnOut; ++k) {
    const int64_t o = threadIdx.x + (int64_t)k * kThreads;
    if (o < mp) q.part[blockIdx.x * mp + o] = acc[k];
  }
}
struct TnReduceJob {
  const double *part;
  int64_t chunks, m, p;
  double *C;
  int64_t ldc;
};
__global__ void tn_reduce_kernel(const __grid_constant__ Group<TnReduceJob> g) {
  const TnReduceJob q = g.j[blockIdx.y];
  const int64_t mp = q.m * q.p;
  for (int64_t o = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; o < mp;
       o += (int64_t)gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int64_t c = 0; c < q.chunks; ++c) s += q.part[c * mp + o];
    q.C[(o % q.m) + (o / q.m) * q.ldc] = s;
  }
}

// ---- C (n x PC) = alpha A (n x m) U (m x PC) + beta C (jobs with exactly PC columns) ----
struct NnJob {
  const double *A, *U;  // U: m x p, leading dimension ldu
  int64_t lda, ldu, n, m, p;
  double *C;
  int64_t ldc;
  double alpha, beta;
};
template <int PC>
__global__ void __launch_bounds__(kThreads) nn_kernel(const __grid_constant__ Group<NnJob> g) {
  const NnJob q = g.j[blockIdx.y];
  __shared__ double us[kNnSmem / sizeof(double)];
  for (int64_t e = threadIdx.x; e < q.m * q.p; e += kThreads)
    us[e] = q.U[(e % q.m) + (e / q.m) * q.ldu];
  __syncthreads();
  for (int64_t r = blockIdx.x * (int64_t)kThreads + threadIdx.x; r < q.n;
       r += (int64_t)gridDim.x * kThreads) {
    double acc[PC];
#pragma unroll
    for (int j = 0; j < PC; ++j) acc[j] = 0.0;
    for (int64_t l = 0; l < q.m; ++l) {
      const double a = q.A[r + l * q.lda];
#pragma unroll
      for (int j = 0; j < PC; ++j) acc[j] = fma(a, us[l + q.m * j], acc[j]);
    }
#pragma unroll
    for (int j = 0; j < PC; ++j) {
      double *c = q.C + r + j * q.ldc;
      *c = q.beta == 0.0 ? q.alpha * acc[j] : fma(q.beta, *c, q.alpha * acc[j]);
    }
  }
}

// ---- column norms (or dots with B) over n rows, one block per column ----
struct NormJob {
  const double *A, *B;  // B null: norms
  int64_t lda, ldb, n, p;
  double *out;
  double *inv = nullptr;  // norms only: also 1 / norm where norm > 0, else 0
};
__global__ void norm_kernel(const __grid_constant__ Group<NormJob> g) {
  const NormJob q = g.j[blockIdx.y];
  const int64_t c = blockIdx.x;
  if (c >= q.p) return;
  const double *a = q.A + c * q.lda, *b = q.B ? q.B + c * q.ldb : a;
  double s = 0.0;
  for (int64_t r = threadIdx.x; r < q.n; r += kThreads) s = fma(a[r], b[r], s);
  __shared__ double red[kThreads];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = kThreads / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double r = q.B ? red[0] : sqrt(red[0]);
    q.out[c] = r;
    // the FP64 division runs once per column here instead of once per element of a scaling
    if (q.inv) q.inv[c] = r > 0.0 ? 1.0 / r : 0.0;
  }
}

// ---- elementwise column work ----
struct ColJob {
  int kind;  // 0: A *= 1 / norm (v holds the reciprocal norms, 0 for a zero column);
             // 1: A -= lam * B (residual); 2: copy B -> A;
             // 3: DPR A[:, kk] = -B[:, cols[kk]] / (D - lam[kk]), non-finite -> 0
  double *A;
  const double *B, *D, *v;  // v: norms or lambdas
  const double *cols;       // DPR: root index of each new column (exact small integers)
  int64_t lda, ldb, n, p;
};
__global__ void col_kernel(const __grid_constant__ Group<ColJob> g) {
  const ColJob q = g.j[blockIdx.y];
  const int64_t total = q.n * q.p;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % q.n, j = t / q.n;
    double *a = q.A + i + j * q.lda;
    if (q.kind == 0) {
      const double iv = q.v[j];
      if (iv > 0.0) *a *= iv;  // Eigen's normalize leaves a zero column unchanged
    } else if (q.kind == 1) {
      *a -= q.v[j] * q.B[i + j * q.ldb];
    } else if (q.kind == 2) {
      *a = q.B[i + j * q.ldb];
    } else {
      double v = -q.B[i + (int64_t)q.cols[j] * q.ldb] / (q.D[i] - q.v[j]);
      if (!isfinite(v)) v = 0.0;
      *a = v;
    }
  }
}

// ---- column-wise Gram-Schmidt of Q[:, nstart:ncols] within the block (the column loops of
// DavidsonSolver::gramschmidt, davidsonsolver.cc:453-458 and 468-477) ----
struct GsJob {
  double *Q;
  int64_t n, nstart, ncols;
  const double *norms0;  // initial norms of the new columns
  int check;
  int *flag;
};
// A cluster of kGsCluster CTAs per molecule, each owning a contiguous range of rows: the dots
// and the norm of every column are summed over the cluster through distributed shared memory
// (each CTA publishes its partial sums in a double-buffered slot; one cluster barrier per
// reduction; the partials are added in rank order, so every CTA gets the same, deterministic
// value).  With one CTA per molecule the FP64 work of the largest molecules ran on one SM (at
// about 2 FP64 FMAs per clock) while the others idled.  Rows are unrolled by 4: a pass over
// the rows of a column is a few dependent loads per thread.
constexpr int kGsCluster = 4;
constexpr int kGsThreads = 128;
__global__ void __cluster_dims__(kGsCluster, 1, 1) __launch_bounds__(kGsThreads, 8)
    gs_kernel(const __grid_constant__ Group<GsJob> g) {
  cg::cluster_group cluster = cg::this_cluster();
  const unsigned rank = cluster.block_rank();
  const GsJob q = g.j[blockIdx.x / kGsCluster];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  constexpr int kMaxRange = 256;
  constexpr int kReg = 8;  // dots accumulated per pass over the rows
  __shared__ double h[kMaxRange];
  __shared__ double red[kGsThreads / 32][kReg];
  __shared__ double part[2][kReg];  // this CTA's published partial sums
  __shared__ double nrm;
  const int64_t per = (q.n + kGsCluster - 1) / kGsCluster;
  const int64_t r0 = min(q.n, (int64_t)rank * per), r1 = min(q.n, r0 + per);
  const double *M = q.Q + q.nstart * q.n;
  int buf = 0;
  for (int64_t j = q.nstart + 1; j < q.ncols; ++j) {
    const int64_t range = j - q.nstart;
    double *qj = q.Q + j * q.n;
    // h = M[:, :range]^T q_j: every thread sums its rows for kReg columns at once (the
    // loads are independent, so they overlap), then one reduction per kReg columns
    for (int64_t l0 = 0; l0 < range; l0 += kReg) {
      const int lc = (int)min((int64_t)kReg, range - l0);
      double acc[kReg];
#pragma unroll
      for (int l = 0; l < kReg; ++l) acc[l] = 0.0;
#pragma unroll 4
      for (int64_t i = r0 + threadIdx.x; i < r1; i += kGsThreads) {
        const double x = qj[i];
#pragma unroll
        for (int l = 0; l < kReg; ++l)
          if (l < lc) acc[l] = fma(M[(l0 + l) * q.n + i], x, acc[l]);
      }
#pragma unroll
      for (int l = 0; l < kReg; ++l) {
        double v = acc[l];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][l] = v;
      }
      __syncthreads();
      if (threadIdx.x < lc) {
        double t = 0.0;
        for (int w = 0; w < kGsThreads / 32; ++w) t += red[w][threadIdx.x];
        part[buf][threadIdx.x] = t;
      }
      cluster.sync();  // every CTA's partials of this reduction are published
      if (threadIdx.x < lc) {
        double t = 0.0;
        for (unsigned r = 0; r < kGsCluster; ++r) t += cluster.map_shared_rank(&part[buf][0], r)[threadIdx.x];
        h[l0 + threadIdx.x] = t;
      }
      buf ^= 1;  // the next barrier orders these reads before the slot is written again
      __syncthreads();
    }
    double nacc = 0.0;
#pragma unroll 4
    for (int64_t i = r0 + threadIdx.x; i < r1; i += kGsThreads) {
      double s = 0.0;
      for (int64_t l = 0; l < range; ++l) s = fma(M[l * q.n + i], h[l], s);
      const double v = qj[i] - s;
      qj[i] = v;
      nacc = fma(v, v, nacc);
    }
    for (int o = 16; o > 0; o >>= 1) nacc += __shfl_down_sync(0xffffffffu, nacc, o);
    if (lane == 0) red[warp][0] = nacc;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (int w = 0; w < kGsThreads / 32; ++w) t += red[w][0];
      part[buf][0] = t;
    }
    cluster.sync();
    if (threadIdx.x == 0) {
      double t = 0.0;
      for (unsigned r = 0; r < kGsCluster; ++r) t += cluster.map_shared_rank(&part[buf][0], r)[0];
      const double nv = sqrt(t);
      if (rank == 0 && q.check && !(nv > 1e-12 * q.norms0[range])) *q.flag = 1;
      nrm = nv > 0.0 ? 1.0 / nv : 0.0;  // one FP64 division per column, not one per row
    }
    buf ^= 1;
    __syncthreads();
    const double iv = nrm;
    if (iv > 0.0) {  // Eigen's normalize leaves a zero column unchanged
#pragma unroll 4
      for (int64_t i = r0 + threadIdx.x; i < r1; i += kGsThreads) qj[i] *= iv;
    }
    __syncthreads();
  }
  cluster.sync();  // no CTA leaves while another may still read its partial sums
}

// ---- unit vectors V[rows[j], j] = 1 ----
struct UnitJob {
  double *V;
  int64_t ldv;
  const double *rows;  // exact small integers
  int64_t count;
};
__global__ void unit_kernel(const __grid_constant__ Group<UnitJob> g) {
  const UnitJob q = g.j[blockIdx.y];
  for (int64_t j = threadIdx.x; j < q.count; j += blockDim.x) q.V[(int64_t)q.rows[j] + q.ldv * j] = 1.0;
}

static_assert(sizeof(Group<TnJob>) <= 32000 && sizeof(Group<TnReduceJob>) <= 32000 &&
                  sizeof(Group<NnJob>) <= 32000 && sizeof(Group<NormJob>) <= 32000 &&
                  sizeof(Group<ColJob>) <= 32000 && sizeof(Group<GsJob>) <= 32000 &&
                  sizeof(Group<UnitJob>) <= 32000,
              "grouped job lists must fit the kernel-parameter space");

// T[c0 + c, r] = T[r, c0 + c] for r < c0, c < nc (the lower block of the projected matrix)
struct MirrorJob {
  double *T;
  int64_t ldt, c0, nc;
};
__global__ void mirror_kernel(const __grid_constant__ Group<MirrorJob> g) {
  const MirrorJob q = g.j[blockIdx.y];
  const int64_t total = q.c0 * q.nc;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % q.c0, c = t / q.c0;
    q.T[(q.c0 + c) + q.ldt * r] = q.T[r + q.ldt * (q.c0 + c)];
  }
}

template <class Job, class Kernel>
void launch_jobs(const std::vector<Job> &jobs, Kernel kernel, unsigned bx, bool grid_x_is_job,
                 cudaStream_t s, int threads = kThreads) {
  std::unique_ptr<Group<Job>> g(new Group<Job>());
  for (size_t i = 0; i < jobs.size();) {
    g->n = 0;
    for (; i < jobs.size() && g->n < kJobs; ++i) g->j[g->n++] = jobs[i];
    // grid_x_is_job: bx consecutive CTAs (a cluster) per job along x
    const dim3 grid = grid_x_is_job ? dim3((unsigned)g->n * bx) : dim3(bx, (unsigned)g->n);
    kernel<<<grid, threads, 0, s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
}

unsigned rows_blocks(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kThreads), 16)); }

struct Mol {
  BseOperator *op = nullptr;
  bool dense = false;  // products through the operator's dense form
  int64_t n = 0, size_update = 0, restart_size = 0, max_space = 0, capc = 0, needmax = 0;
  int64_t ncols = 0, nav = 0, m = 0, needed = 0, nupdate = 0, chunks = 0;
  bool done = false;
  int info = 1;
  int64_t iterations = 0;
  std::vector<double> lam, evals;
  std::vector<int64_t> upd;
  std::vector<double> upd_lam;
  // device (views into the pool)
  double *V, *AV, *D, *q, *res, *Ud, *lamd, *cbuf, *norms0, *norms, *inorms, *h, *part, *Td, *eigw;
  int *flag, *einfo;
  // packed host transfer offsets (doubles): off_in = [U (capc x needmax) | lambdas (needmax) |
  // correction columns (capc) | their lambdas (capc)] in din/hin; off_out in hout (diagonal);
  // off_pack = this step's block in dpack/hpack (every molecule's result of a step is packed
  // back to back and copied to the host in one transfer)
  int64_t off_in = 0, off_out = 0, off_pack = 0;
  int64_t dpr_in() const { return off_in + capc * needmax + needmax; }
};

// Grouped A^T B for every (mol, A, B, m, p, C) request; splits wide requests over m.
struct TnReq {
  Mol *mol;
  const double *A, *B;
  int64_t m, p;
  double *C;
  int64_t ldc;
};
void run_tn(const std::vector<TnReq> &reqs, cudaStream_t s) {
  std::vector<TnJob> jobs;
  std::vector<TnReduceJob> red;
  for (const TnReq &r : reqs) {
    if (r.m <= 0 || r.p <= 0) continue;
    VGB_REQUIRE(r.p <= kTnCols / 2, "batched Davidson: too many new columns per step");
    const int64_t mcap = std::max<int64_t>(1, std::min<int64_t>(kTnCols - r.p, (kTnOut * kThreads) / r.p));
    // the molecule's partial scratch holds chunks * capc^2 doubles: one m-range at a time fits
    // because m0-ranges write disjoint parts of it (offset m0 * p)
    for (int64_t m0 = 0; m0 < r.m; m0 += mcap) {
      const int64_t mm = std::min(mcap, r.m - m0);
      TnJob j;
      j.A = r.A + m0 * r.mol->n; j.lda = r.mol->n;
      j.B = r.B; j.ldb = r.mol->n;
      j.n = r.mol->n; j.m = mm; j.p = r.p;
      j.part = r.mol->part + r.mol->chunks * m0 * r.p;
      jobs.push_back(j);
      TnReduceJob t;
      t.part = j.part; t.chunks = r.mol->chunks; t.m = mm; t.p = r.p;
      t.C = r.C + m0; t.ldc = r.ldc;
      red.push_back(t);
    }
  }
  int64_t maxchunks = 1;
  for (const TnJob &j : jobs) maxchunks = std::max(maxchunks, ceil_div(j.n, (int64_t)kTnRows));
  launch_jobs(jobs, tn_partial_kernel, (unsigned)maxchunks, false, s);
  launch_jobs(red, tn_reduce_kernel, 4, false, s);
}

void run_nn(const std::vector<NnJob> &jobs, cudaStream_t s) {
  // U's columns in exact power-of-two blocks (16, 8, 4, 2, 1): every FMA slot of a
  // thread works on a present column (the FP64 issue rate limits these products)
  std::vector<NnJob> bucket[5];  // 1, 2, 4, 8, 16 columns
  int64_t mx = 1;
  for (const NnJob &j : jobs) {
    if (j.n <= 0 || j.p <= 0) continue;
    VGB_REQUIRE(j.m * 16 * (int64_t)sizeof(double) <= kNnSmem, "batched Davidson: search space too large");
    int64_t c0 = 0;
    while (c0 < j.p) {
      const int64_t left = j.p - c0;
      int b = 4;
      while ((1LL << b) > left) --b;
      NnJob t = j;
      t.U = j.U + c0 * j.ldu;
      t.C = j.C + c0 * j.ldc;
      t.p = 1LL << b;
      bucket[b].push_back(t);
      c0 += t.p;
    }
    mx = std::max(mx, j.n);
  }
  launch_jobs(bucket[0], nn_kernel<1>, rows_blocks(mx), false, s);
  launch_jobs(bucket[1], nn_kernel<2>, rows_blocks(mx), false, s);
  launch_jobs(bucket[2], nn_kernel<4>, rows_blocks(mx), false, s);
  launch_jobs(bucket[3], nn_kernel<8>, rows_blocks(mx), false, s);
  launch_jobs(bucket[4], nn_kernel<16>, rows_blocks(mx), false, s);
}

void run_norms(const std::vector<NormJob> &jobs, cudaStream_t s) {
  int64_t mx = 1;
  for (const NormJob &j : jobs) mx = std::max(mx, j.p);
  launch_jobs(jobs, norm_kernel, (unsigned)mx, false, s);
}

void run_cols(const std::vector<ColJob> &jobs, cudaStream_t s) {
  int64_t mx = 1;
  for (const ColJob &j : jobs) mx = std::max(mx, j.n * j.p);
  launch_jobs(jobs, col_kernel, rows_blocks(mx), false, s);
}

// Parallel loop over molecules on host threads: a pool of workers kept for the process (starting
// 16 threads per Davidson step cost about as much as the small eigenproblems they solve).  One
// loop runs at a time; the calling thread takes part.
class HostPool {
 public:
  static HostPool &get() {
    // never destroyed: the workers stay parked until the process exits (no join at exit, and
    // none attempted in a forked child, where the threads do not exist)
    static HostPool *pool = new HostPool();
    return *pool;
  }
  void run(size_t count, const std::function<void(size_t)> &f) {
    std::lock_guard<std::mutex> one(run_mu_);
    // a forked child has no workers (threads do not survive fork): run serially there
    if (workers_.empty() || count <= 1 || getpid() != pid_) {
      for (size_t i = 0; i < count; ++i) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lock(mu_);
      f_ = &f;
      count_ = count;
      next_.store(0);
      first_ = nullptr;
      busy_ = workers_.size();
      ++generation_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lock(mu_);
    done_cv_.wait(lock, [&] { return busy_ == 0; });
    f_ = nullptr;
    if (first_) std::rethrow_exception(first_);
  }

 private:
  HostPool() : pid_(getpid()) {
    const unsigned n = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    for (unsigned t = 1; t < n; ++t) workers_.emplace_back([this] { loop(); });
  }
  void work() {
    for (;;) {
      const size_t i = next_.fetch_add(1);
      if (i >= count_) break;
      try {
        (*f_)(i);
      } catch (...) {
        std::lock_guard<std::mutex> lock(err_mu_);
        if (!first_) first_ = std::current_exception();
      }
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lock(mu_);
        cv_.wait(lock, [&] { return generation_ != seen; });
        seen = generation_;
      }
      work();
      {
        std::lock_guard<std::mutex> lock(mu_);
        if (--busy_ == 0) done_cv_.notify_one();
      }
    }
  }
  std::vector<std::thread> workers_;
  std::mutex run_mu_, mu_, err_mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t)> *f_ = nullptr;
  size_t count_ = 0, busy_ = 0;
  std::atomic<size_t> next_{0};
  uint64_t generation_ = 0;
  std::exception_ptr first_;
  pid_t pid_;
};

template <class F>
void host_parallel(size_t count, F f) {
  const std::function<void(size_t)> fn = f;
  HostPool::get().run(count, fn);
}

// Page-locked staging of the packed transfers, kept per host thread across solves
// (allocating page-locked memory costs milliseconds).
double *pinned_scratch(size_t doubles) {
  struct Buf {
    double *p = nullptr;
    size_t cap = 0;
    ~Buf() { if (p) cudaFreeHost(p); }
  };
  static thread_local Buf buf;
  if (buf.cap < doubles) {
    if (buf.p) cudaFreeHost(buf.p);
    buf.p = nullptr;
    buf.cap = 0;
    VGB_CUDA(cudaMallocHost(&buf.p, doubles * sizeof(double)));
    buf.cap = doubles;
  }
  return buf.p;
}

}  // namespace

void davidson_solve_batch(const std::vector<BseOperator *> &ops, const Coef &coef, int64_t neigen,
                          const bse_davidson_options &opt, double *evals, int32_t *infos,
                          int64_t *iterations, cudaStream_t s) {
  VGB_REQUIRE(opt.matrix_type == 0, "batched Davidson: SYMM matrices only");
  VGB_REQUIRE(opt.correction == 0, "batched Davidson: DPR correction only");
  VGB_REQUIRE(opt.update >= 0 && opt.update <= 2, "not a valid Davidson update");
  const size_t nm = ops.size();
  if (nm == 0) return;
  const int64_t iter_max = opt.iter_max > 0 ? opt.iter_max : 50;
  const double tol = opt.tolerance;
  std::vector<Mol> mols(nm);
  int64_t pool_doubles = 0, in_doubles = 0, out_doubles = 0, pack_doubles = 0;
  for (size_t b = 0; b < nm; ++b) {
    Mol &M = mols[b];
    M.op = ops[b];
    M.n = M.op->dim;
    if (!(neigen >= 1 && neigen <= M.n))
      fail(BSE_ERR_ARGUMENT, "molecule " + std::to_string(b) + ": DavidsonSolver: neigen out of range");
    int64_t max_space = opt.max_search_space;
    if (max_space < neigen) max_space = neigen * 5;
    if (max_space > M.n) max_space = M.n;
    M.max_space = max_space;
    if (opt.update == 0) M.size_update = neigen;
    else if (opt.update == 1) M.size_update = neigen < 20 ? (int64_t)(1.5 * (double)neigen) : neigen + 10;
    else M.size_update = 2 * neigen;
    if (opt.size_update > 0) {
      VGB_REQUIRE(opt.size_update >= neigen, "DavidsonSolver: size_update smaller than neigen");
      M.size_update = opt.size_update;
    }
    M.size_update = std::min(M.size_update, M.n);
    VGB_REQUIRE(opt.initial_size == 0 || opt.initial_size >= neigen,
                "DavidsonSolver: initial search space smaller than neigen");
    M.restart_size = opt.initial_size > 0 ? opt.initial_size : 2 * neigen;
    M.ncols = M.restart_size;
    VGB_REQUIRE(M.ncols <= M.n, "DavidsonSolver: initial search space larger than the operator");
    const int64_t cap = std::max(M.ncols, max_space) + 2 * M.size_update + M.restart_size + 2;
    M.capc = std::min(cap, M.n + 2 * M.size_update + M.restart_size + 2);
    M.needmax = std::min(M.capc, std::max(M.restart_size, M.size_update));
    M.chunks = ceil_div(M.n, (int64_t)kTnRows);
    M.evals.assign(neigen, 0.0);
    pool_doubles += 2 * M.n * M.capc + 2 * M.n * M.needmax + 4 * M.capc + M.capc * M.capc +
                    M.chunks * M.capc * M.capc + 64;
    // projected matrix, Ritz coefficients and values, eigensolver scratch (device)
    pool_doubles += M.capc * M.capc + M.capc * M.needmax + M.needmax + sym_eig_work_doubles(M.capc, M.needmax) + 64;
    M.off_in = in_doubles;
    in_doubles += M.capc * M.needmax + M.needmax + 2 * M.capc + 8;  // U, lambdas, update lists
    M.off_out = out_doubles;
    out_doubles += M.n + 8;                                           // diagonal
    pack_doubles += M.capc * M.capc + 2 * M.needmax + 8;              // T blocks, or norms + Ritz values
  }
  AllocStreamScope scope(s);
  DeviceBuffer<double> pool(pool_doubles);
  DeviceBuffer<double> din(in_doubles), dpack(pack_doubles);
  double *hbuf = pinned_scratch((size_t)(in_doubles + out_doubles + pack_doubles));
  double *hin = hbuf, *hout = hbuf + in_doubles, *hpack = hout + out_doubles;
  VGB_CUDA(cudaMemsetAsync(pool.get(), 0, pool_doubles * sizeof(double), s));
  {
    double *p = pool.get();
    for (Mol &M : mols) {
      auto take = [&](int64_t cnt) { double *r = p; p += cnt; return r; };
      M.V = take(M.n * M.capc);
      M.AV = take(M.n * M.capc);
      M.q = take(M.n * M.needmax);
      M.res = take(M.n * M.needmax);
      M.norms0 = take(M.capc);
      M.norms = take(M.capc);
      M.inorms = take(M.capc);
      M.h = take(M.capc + M.capc * M.capc);
      M.part = take(M.chunks * M.capc * M.capc);
      p += 64;
      M.Td = take(M.capc * M.capc);
      M.Ud = take(M.capc * M.needmax);
      M.lamd = take(M.needmax);
      M.eigw = take(sym_eig_work_doubles(M.capc, M.needmax));
      p += 64;
    }
  }
  {
    // small split-precision TDA operators: the dense form (one GEMM per product)
    const char *env = getenv("VGB_BATCH_DENSE");
    const bool allow_dense = !(env && atoi(env) == 0);
    const char *envmax = getenv("VGB_BATCH_DENSE_MAX");
    const int64_t dense_max = envmax ? atoll(envmax) : kDenseMaxDim;
    std::vector<BseOperator *> dense;
    for (BseOperator *op : ops)
      if (allow_dense && coef.cd2 == 0 && op->precision == BSE_PRECISION_MIXED && op->mixed &&
          op->hqp_diagonal && op->dim <= dense_max && ceil_div(op->naux, 64) * 64 <= 1024 &&
          std::find(dense.begin(), dense.end(), op) == dense.end())
        dense.push_back(op);
    std::stable_sort(dense.begin(), dense.end(),
                     [](const BseOperator *a, const BseOperator *b) { return a->dim < b->dim; });
    int64_t dense_bytes = 0;
    size_t nd = 0;
    for (; nd < dense.size(); ++nd) {
      dense_bytes += 4 * dense[nd]->dim * ceil_div(dense[nd]->dim, 64) * 64;
      if (dense_bytes > kDenseBudgetBytes) break;
    }
    dense.resize(nd);
    MixedEngine::build_dense_grouped(dense, coef, s);
    for (BseOperator *op : dense)
      for (Mol &M : mols)
        if (M.op == op) M.dense = true;
    int64_t kmax = 1;
    for (const Mol &M : mols) kmax = std::max(kmax, std::max(M.ncols, M.size_update));
    MixedEngine::prepare_grouped(ops, kmax, s);
  }
  GroupScratch arena;  // Hd intermediates of the grouped products, shared by all molecules
  DeviceBuffer<int> flags(2 * nm);  // Gram-Schmidt linear dependence, then eigensolver status
  VGB_CUDA(cudaMemsetAsync(flags.get(), 0, 2 * nm * sizeof(int), s));
  for (size_t b = 0; b < nm; ++b) {
    mols[b].flag = flags.get() + b;
    mols[b].einfo = flags.get() + nm + b;
  }
  // packs the given blocks back to back: off_pack and the device block of each molecule
  auto pack = [&](const std::vector<Mol *> &ms, const std::function<int64_t(const Mol &)> &size) {
    int64_t off = 0;
    for (Mol *M : ms) {
      M->off_pack = off;
      M->cbuf = dpack.get() + off;
      off += size(*M);
    }
    return off;
  };

  // ---- diagonal and unit-vector guesses (setupInitialEigenvectors) ----
  {
    // kept on the operator: a later solve with the same coefficients reads it again
    std::vector<BseOperator *> dops;
    std::vector<double *> dd;
    for (Mol &M : mols) {
      BseOperator &op = *M.op;
      const bool same = op.diag_valid && op.diag_coef.cqp == coef.cqp && op.diag_coef.cx == coef.cx &&
                        op.diag_coef.cd == coef.cd && op.diag_coef.cd2 == coef.cd2;
      if (!same && std::find(dops.begin(), dops.end(), &op) == dops.end()) {
        op.diag_valid = false;
        op.diag_cache.resize(op.dim);
        dops.push_back(&op);
        dd.push_back(op.diag_cache.get());
      }
    }
    diagonal_grouped(coef, dops, dd, s);
    for (BseOperator *op : dops) {
      op->diag_coef = coef;
      op->diag_valid = true;
    }
    for (Mol &M : mols) M.D = M.op->diag_cache.get();
  }
  for (Mol &M : mols)
    VGB_CUDA(cudaMemcpyAsync(hout + M.off_out, M.D, M.n * sizeof(double), cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
  {
    std::vector<UnitJob> uj;
    host_parallel(mols.size(), [&](size_t b) {
      Mol &M = mols[b];
      std::vector<int64_t> idx(M.n);
      std::iota(idx.begin(), idx.end(), 0);
      const double *Dh = hout + M.off_out;
      // the first ncols of a stable argsort of the diagonal (ties by index)
      std::partial_sort(idx.begin(), idx.begin() + M.ncols, idx.end(), [&](int64_t a, int64_t c) {
        return Dh[a] < Dh[c] || (Dh[a] == Dh[c] && a < c);
      });
      // stage the row list in the H2D buffer (as doubles holding exact small integers)
      double *dst = hin + M.off_in;
      for (int64_t j = 0; j < M.ncols; ++j) dst[j] = (double)idx[j];
    });
    VGB_CUDA(cudaMemcpyAsync(din.get(), hin, in_doubles * sizeof(double), cudaMemcpyHostToDevice, s));
    for (Mol &M : mols) {
      UnitJob u;
      u.V = M.V; u.ldv = M.n; u.rows = din.get() + M.off_in; u.count = M.ncols;
      uj.push_back(u);
    }
    launch_jobs(uj, unit_kernel, 1, false, s);
  }

  // phase timing (verbose >= 2): synchronises at phase boundaries
  const bool phases = opt.verbose >= 2;
  double ph[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // matvec, projection, small eig, ritz, host, dpr, gs, restart
  auto tick = std::chrono::steady_clock::now();
  auto mark = [&](int i) {
    if (!phases) return;
    VGB_CUDA(cudaStreamSynchronize(s));
    const auto now = std::chrono::steady_clock::now();
    ph[i] += std::chrono::duration<double>(now - tick).count();
    tick = now;
  };
  mark(4);
  for (int64_t it = 0; it < iter_max; ++it) {
    std::vector<Mol *> act;
    for (Mol &M : mols)
      if (!M.done) act.push_back(&M);
    if (act.empty()) break;
    // ---- updateProjection: AV[:, old:ncols] = A V[:, old:ncols]; T[:, old:] = V^T AV_new ----
    {
      std::vector<GroupedItem> items;
      std::vector<TnReq> tn;
      std::vector<MirrorJob> mj;
      for (Mol *M : act) {
        M->iterations = it;
        const int64_t old = (it == 0) ? 0 : M->nav, nvec = M->ncols - old;
        GroupedItem gi;
        gi.op = M->op; gi.X = M->V + old * M->n; gi.ldx = M->n; gi.k = nvec;
        gi.Y = M->AV + old * M->n; gi.ldy = M->n; gi.dense = M->dense; gi.diag = M->D;
        items.push_back(gi);
        // T[:, old:ncols] = V^T AV_new straight into the device projected matrix
        tn.push_back({M, M->V, M->AV + old * M->n, M->ncols, nvec, M->Td + M->capc * old, M->capc});
        if (old > 0) mj.push_back({M->Td, M->capc, old, nvec});
        M->nav = M->ncols;
      }
      matmul_grouped(coef, items, s, &arena);
      mark(0);
      run_tn(tn, s);
      int64_t mx = 1;
      for (const MirrorJob &j : mj) mx = std::max(mx, j.c0 * j.nc);
      launch_jobs(mj, mirror_kernel, rows_blocks(mx), false, s);
    }
    mark(1);
    // ---- getRitzEigenPairs: every molecule's Ritz problem in one device launch ----
    {
      std::vector<SymEigJob> ej;
      for (Mol *M : act) {
        const int64_t m = M->ncols;
        M->m = m;
        M->needed = std::min(m, std::max(M->restart_size, M->size_update));
        SymEigJob j;
        j.T = M->Td; j.ldt = M->capc; j.m = m; j.nw = M->needed;
        j.U = M->Ud; j.ldu = m; j.lam = M->lamd; j.work = M->eigw; j.info = M->einfo;
        ej.push_back(j);
      }
      sym_eig_device(ej.data(), (int64_t)ej.size(), s);
    }
    mark(2);
    // ---- Ritz vectors q = V U, residuals res = AV U - q Lambda, their norms ----
    {
      std::vector<NnJob> nn;
      std::vector<ColJob> cj;
      std::vector<NormJob> nj;
      std::vector<ColJob> lc;
      const int64_t packed =
          pack(act, [](const Mol &M) { return std::min(M.needed, M.size_update) + M.needed; });
      for (Mol *M : act) {
        // only the first min(needed, size_update) pairs enter the convergence check and the
        // corrections; the Ritz vectors a restart keeps are formed there
        const int64_t pr = std::min(M->needed, M->size_update);
        nn.push_back({M->V, M->Ud, M->n, M->m, M->n, M->m, pr, M->q, M->n, 1.0, 0.0});
        nn.push_back({M->AV, M->Ud, M->n, M->m, M->n, M->m, pr, M->res, M->n, 1.0, 0.0});
        ColJob c;
        c.kind = 1; c.A = M->res; c.B = M->q; c.D = nullptr; c.v = M->lamd; c.cols = nullptr;
        c.lda = M->n; c.ldb = M->n; c.n = M->n; c.p = pr;
        cj.push_back(c);
        NormJob w;
        w.A = M->res; w.B = nullptr; w.lda = M->n; w.ldb = M->n; w.n = M->n;
        w.p = std::min(M->needed, M->size_update); w.out = M->cbuf;
        nj.push_back(w);
        ColJob l;  // the Ritz values travel behind the norms
        l.kind = 2; l.A = M->cbuf + pr; l.B = M->lamd; l.D = nullptr; l.v = nullptr; l.cols = nullptr;
        l.lda = M->needed; l.ldb = M->needed; l.n = M->needed; l.p = 1;
        lc.push_back(l);
      }
      run_nn(nn, s);
      run_cols(cj, s);
      run_norms(nj, s);
      run_cols(lc, s);
      VGB_CUDA(cudaMemcpyAsync(hpack, dpack.get(), packed * sizeof(double), cudaMemcpyDeviceToHost, s));
      std::vector<int> hflags(2 * nm);
      VGB_CUDA(cudaMemcpyAsync(hflags.data(), flags.get(), 2 * nm * sizeof(int), cudaMemcpyDeviceToHost, s));
      VGB_CUDA(cudaStreamSynchronize(s));
      act.front()->op->check_errors(s);  // grouped tensor-core stages report into the first engine
      for (size_t b = 0; b < nm; ++b) {
        if (hflags[b]) fail(BSE_ERR_NUMERICAL, "molecule " + std::to_string(b) + ": Linear dependencies in Gram-Schmidt.");
        if (hflags[nm + b]) fail(BSE_ERR_NUMERICAL, "molecule " + std::to_string(b) + ": Small hermitian eigenvalue problem failed.");
      }
      for (Mol *M : act) {
        const int64_t pr = std::min(M->needed, M->size_update);
        M->lam.assign(hpack + M->off_pack + pr, hpack + M->off_pack + pr + M->needed);
      }
    }
    mark(3);
    // ---- checkConvergence / storeEigenPairs / extendProjection (host) ----
    const bool last = it == iter_max - 1;
    std::vector<Mol *> ext;
    for (Mol *M : act) {
      const int64_t nn_check = std::min(M->needed, M->size_update);
      const double *resn = hpack + M->off_pack;
      std::vector<char> conv(M->size_update, 0);
      for (int64_t j = 0; j < M->size_update; ++j) conv[j] = (j < nn_check) ? (resn[j] < tol) : 0;
      bool converged = true;
      for (int64_t j = 0; j < neigen; ++j)
        if (!conv[j]) converged = false;
      if (converged || last) {
        for (int64_t j = 0; j < neigen; ++j) M->evals[j] = j < M->needed ? M->lam[j] : 0.0;
        M->info = converged ? 0 : 1;
        if (!converged)
          for (int64_t j = 0; j < neigen; ++j)
            if (!conv[j]) M->evals[j] = 0.0;
        M->done = true;
        continue;
      }
      M->upd.clear();
      M->upd_lam.clear();
      for (int64_t j = 0; j < M->size_update; ++j)
        if (!conv[j] && j < M->needed) { M->upd.push_back(j); M->upd_lam.push_back(M->lam[j]); }
      M->nupdate = (int64_t)M->upd.size();
      VGB_REQUIRE(M->ncols + M->nupdate <= M->capc, "DavidsonSolver: search space capacity exceeded");
      double *dst = hin + M->dpr_in();  // [cols as doubles | lambdas]
      for (int64_t k = 0; k < M->nupdate; ++k) {
        dst[k] = (double)M->upd[k];
        dst[M->capc + k] = M->upd_lam[k];
      }
      ext.push_back(M);
    }
    mark(4);
    if (ext.empty()) continue;
    VGB_CUDA(cudaMemcpyAsync(din.get(), hin, in_doubles * sizeof(double), cudaMemcpyHostToDevice, s));
    // ---- DPR corrections, normalised ----
    {
      std::vector<ColJob> cj;
      std::vector<NormJob> nj;
      std::vector<ColJob> sc;
      for (Mol *M : ext) {
        ColJob c;
        c.kind = 3; c.A = M->V + M->ncols * M->n; c.B = M->res; c.D = M->D;
        c.v = din.get() + M->dpr_in() + M->capc; c.cols = din.get() + M->dpr_in();
        c.lda = M->n; c.ldb = M->n; c.n = M->n; c.p = M->nupdate;
        cj.push_back(c);
        NormJob w;
        w.A = c.A; w.B = nullptr; w.lda = M->n; w.ldb = M->n; w.n = M->n; w.p = M->nupdate; w.out = M->norms;
        w.inv = M->inorms;
        nj.push_back(w);
        ColJob z;
        z.kind = 0; z.A = c.A; z.B = nullptr; z.D = nullptr; z.v = M->inorms; z.cols = nullptr;
        z.lda = M->n; z.ldb = M->n; z.n = M->n; z.p = M->nupdate;
        sc.push_back(z);
      }
      run_cols(cj, s);
      run_norms(nj, s);
      run_cols(sc, s);
    }
    mark(5);
    // ---- gramschmidt on the new columns (two passes) ----
    {
      std::vector<NormJob> n0;
      for (Mol *M : ext) {
        NormJob w;
        w.A = M->V + M->ncols * M->n; w.B = nullptr; w.lda = M->n; w.ldb = M->n; w.n = M->n;
        w.p = M->nupdate; w.out = M->norms0;
        n0.push_back(w);
      }
      run_norms(n0, s);
      for (int pass = 0; pass < 2; ++pass) {
        std::vector<TnReq> tn;
        std::vector<NnJob> nn;
        std::vector<NormJob> nj;
        std::vector<ColJob> sc;
        std::vector<GsJob> gs;
        for (Mol *M : ext) {
          double *Vn = M->V + M->ncols * M->n;
          tn.push_back({M, M->V, Vn, M->ncols, M->nupdate, M->h, M->ncols});
          nn.push_back({M->V, M->h, M->n, M->ncols, M->n, M->ncols, M->nupdate, Vn, M->n, -1.0, 1.0});
          NormJob w;
          w.A = Vn; w.B = nullptr; w.lda = M->n; w.ldb = M->n; w.n = M->n; w.p = M->nupdate; w.out = M->norms;
          w.inv = M->inorms;
          nj.push_back(w);
          ColJob z;
          z.kind = 0; z.A = Vn; z.B = nullptr; z.D = nullptr; z.v = M->inorms; z.cols = nullptr;
          z.lda = M->n; z.ldb = M->n; z.n = M->n; z.p = M->nupdate;
          sc.push_back(z);
          if (M->nupdate > 1) {
            VGB_REQUIRE(M->nupdate <= 256, "batched Davidson: too many new columns");
            GsJob gj;
            gj.Q = M->V; gj.n = M->n; gj.nstart = M->ncols; gj.ncols = M->ncols + M->nupdate;
            gj.norms0 = M->norms0; gj.check = pass == 1 ? 1 : 0; gj.flag = M->flag;
            gs.push_back(gj);
          }
        }
        run_tn(tn, s);
        run_nn(nn, s);
        run_norms(nj, s);
        run_cols(sc, s);
        launch_jobs(gs, gs_kernel, kGsCluster, true, s, kGsThreads);
      }
      for (Mol *M : ext) M->ncols += M->nupdate;
    }
    mark(6);
    // ---- restart (SYMM): V[:, :rs] = q, AV[:, :rs] = AV U, keep the new columns ----
    std::vector<Mol *> rst;
    for (Mol *M : ext)
      if (M->ncols > M->max_space) rst.push_back(M);
    if (!rst.empty()) {
      std::vector<ColJob> keep, back, cq;
      std::vector<NnJob> nn, qn;
      std::vector<ColJob> cav;
      for (Mol *M : rst) {
        const int64_t rs = M->restart_size, nv = M->nupdate;
        VGB_REQUIRE(rs <= M->needed, "DavidsonSolver: restart size exceeds the Ritz pairs");
        // the kept Ritz vectors q = V[:, :m] U[:, :rs] (V's first m columns are unchanged)
        qn.push_back({M->V, M->Ud, M->n, M->m, M->n, M->m, rs, M->q, M->n, 1.0, 0.0});
        // scratch: res holds the kept columns (nv <= needmax), q is copied into V
        VGB_REQUIRE(nv <= M->needmax, "batched Davidson: restart scratch too small");
        ColJob k;
        k.kind = 2; k.A = M->res; k.B = M->V + (M->ncols - nv) * M->n; k.D = nullptr; k.v = nullptr;
        k.cols = nullptr; k.lda = M->n; k.ldb = M->n; k.n = M->n; k.p = nv;
        keep.push_back(k);
        ColJob c;
        c.kind = 2; c.A = M->V; c.B = M->q; c.D = nullptr; c.v = nullptr; c.cols = nullptr;
        c.lda = M->n; c.ldb = M->n; c.n = M->n; c.p = rs;
        cq.push_back(c);
        // AV U[:, :rs] into q (free after the copy above), then into AV
        nn.push_back({M->AV, M->Ud, M->n, M->m, M->n, M->nav, rs, M->q, M->n, 1.0, 0.0});
        ColJob a;
        a.kind = 2; a.A = M->AV; a.B = M->q; a.D = nullptr; a.v = nullptr; a.cols = nullptr;
        a.lda = M->n; a.ldb = M->n; a.n = M->n; a.p = rs;
        cav.push_back(a);
        ColJob bk;
        bk.kind = 2; bk.A = M->V + rs * M->n; bk.B = M->res; bk.D = nullptr; bk.v = nullptr;
        bk.cols = nullptr; bk.lda = M->n; bk.ldb = M->n; bk.n = M->n; bk.p = nv;
        back.push_back(bk);
      }
      run_nn(qn, s);
      run_cols(keep, s);
      run_cols(cq, s);
      run_nn(nn, s);
      run_cols(cav, s);
      run_cols(back, s);
      std::vector<TnReq> tn;  // T = V[:, :rs]^T AV[:, :rs], in the device projected matrix
      for (Mol *M : rst) tn.push_back({M, M->V, M->AV, M->restart_size, M->restart_size, M->Td, M->capc});
      run_tn(tn, s);
      for (Mol *M : rst) {
        M->ncols = M->restart_size + M->nupdate;
        M->nav = M->restart_size;
      }
    }
    mark(7);
  }
  VGB_CUDA(cudaStreamSynchronize(s));
  if (phases)
    fprintf(stderr,
            "[davidson-batch] %zu molecules, phases (s): matvec %.4f  projection %.4f  small-eig %.4f  "
            "ritz %.4f  host %.4f  dpr %.4f  gram-schmidt %.4f  restart %.4f\n",
            nm, ph[0], ph[1], ph[2], ph[3], ph[4], ph[5], ph[6], ph[7]);
  for (size_t b = 0; b < nm; ++b) {
    std::copy(mols[b].evals.begin(), mols[b].evals.end(), evals + b * neigen);
    if (infos) infos[b] = mols[b].info;
    if (iterations) iterations[b] = mols[b].iterations;
  }
}

}  // namespace vgb
