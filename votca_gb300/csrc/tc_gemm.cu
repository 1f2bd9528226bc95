// tcgen05 BF16x3 GEMM (see tc_gemm.cuh).
#include "tc_gemm.cuh"

#include <cuda_bf16.h>

#include <map>
#include <memory>
#include <mutex>

namespace vgb {

namespace {

constexpr int BM = 128;
constexpr int kEpiWarps = 8;   // two warps per TMEM lane quarter, each drains half the columns
constexpr int kThreads = 64 + 32 * kEpiWarps;  // warp 0: TMA, warp 1: MMA + TMEM owner, rest: epilogue
constexpr unsigned long long kWaitNs = 2000000000ull;  // bounded waits: 2 s
constexpr int kSmemRing = 196608;                     // bytes of operand ring per CTA

// BK = bf16 elements of K per stage row: 64 -> 128-byte rows (SWIZZLE_128B),
// 32 -> 64-byte rows (SWIZZLE_64B, half the stage size, twice the stages).
// SLICE: the slice-mode kernel (Ozaki digit planes).  A unit is one A plane a and up to UNIT
// B planes b0 .. b0 + nb - 1 (pairs of one digit level or less): a stage holds the unit's planes
// of one K block, and one MMA of width nb * BN multiplies the A plane by the stacked B planes
// into nb adjacent accumulators (A is read once per K step for nb pairs).
constexpr int kMaxDigits = 5;
template <int BN, int BK, bool SLICE = false>
struct Cfg {
  static constexpr int A_BYTES = BM * BK * 2;            // one of hi / lo (one plane)
  static constexpr int B_BYTES = BN * BK * 2;
  static constexpr int UNIT = 256 / BN < kMaxDigits ? 256 / BN : kMaxDigits;  // B planes per unit
  static constexpr int STAGE_BYTES = SLICE ? A_BYTES + UNIT * B_BYTES : 2 * A_BYTES + 2 * B_BYTES;
  static constexpr int STAGES = kSmemRing / STAGE_BYTES > 8 ? 8 : kSmemRing / STAGE_BYTES;
  // accumulator buffers in TMEM: four for the narrow tiles (short K splits: the epilogue of a
  // split may lag the MMAs of the next three), two for the wide ones; slice mode: two unit
  // buffers of 256 columns
  static constexpr int NBUF = SLICE ? 2 : (BN <= 64 ? 4 : 2);
  static constexpr int BUFW = SLICE ? 256 : BN;  // TMEM columns per buffer
  static constexpr int TMEM_COLS = NBUF * BUFW < 32 ? 32 : NBUF * BUFW;
  static constexpr int SMEM = STAGES * STAGE_BYTES + 1024 /*align*/ + 256 /*barriers*/;
  static constexpr uint32_t SBO = BK == 64 ? 1024 : 512;     // 8 rows of one swizzle atom
  static constexpr uint64_t LAYOUT = BK == 64 ? 2 : 4;       // SWIZZLE_128B / SWIZZLE_64B
};

struct KParams {
  int64_t M, N, K;
  int products;  // 3: hi.hi + hi.lo + lo.hi;  4: + lo.lo;  1: slice mode (hi maps only)
  int64_t nbatch, a_brows, b_brows;
  int ksplit, kc_per;
  int kacc;  // 1: one CTA runs K splits of a tile and sums them in FP64 registers
  int spg;   // kacc: consecutive splits per work item (ksplit / spg groups per tile)
  // slice mode: digit planes per operand, K runs, runs per split group; the splits of a group are
  // (a, q, b) for A plane a, run q, B plane b < nsl - a (pairs up to digit level nsl - 1)
  int nsl, cpr, rpg;
  int64_t a_plane, b_plane;  // slice mode: operand rows between consecutive digit planes
  int64_t mt, nt, ntiles;
  TcEpilogue epi;
  int *err;
};

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: gives up after kWaitNs or when another role aborted.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          int *err, int code) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = now_ns();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 0) {
      if (*abort_flag) return false;
      if (now_ns() - t0 > kWaitNs) {
        *abort_flag = 1;
        atomicExch(err, code);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap *map, uint64_t *bar,
                                            int x, int y) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, "
      "%3}], [%4];" ::"r"(dst),
      "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Swizzled K-major shared-memory matrix descriptor (8-row core groups sbo bytes apart).
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t sbo, uint64_t layout) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr & 0x3FFFF) >> 4);
  d |= (uint64_t)(16 >> 4) << 16;  // leading byte offset (unused for swizzled K-major)
  d |= (uint64_t)(sbo >> 4) << 32; // stride byte offset
  d |= (uint64_t)1 << 46;          // descriptor version (tcgen05)
  d |= layout << 61;               // swizzle mode
  return d;
}
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, "
      "%12, %13, %14, %15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, "
      "%30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
        "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
        "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
        "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

struct TileCoord {
  int64_t m, n, s, b;
};
__device__ __forceinline__ TileCoord decode(const KParams &p, int64_t t) {
  TileCoord c;
  if (p.kacc) {  // the K splits of a (tile, group) item are consecutive jobs of one CTA
    const int64_t u = t % p.spg;
    t /= p.spg;
    const int64_t groups = p.ksplit / p.spg;
    c.s = (t % groups) * p.spg + u;
    t /= groups;
    c.m = t % p.mt;
    t /= p.mt;
    c.n = t % p.nt;
    c.b = t / p.nt;
    return c;
  }
  c.m = t % p.mt;
  t /= p.mt;
  c.n = t % p.nt;
  t /= p.nt;
  c.s = t % p.ksplit;
  c.b = t / p.ksplit;
  return c;
}

// v - float(hi) is exact in FP32 (hi is v rounded to 8 significant bits), so
// the split costs no FP64 work in the epilogue.
__device__ __forceinline__ void epi_store(const TcEpilogue &e, int64_t off, float v) {
  if (e.kind == TcEpilogue::SPLIT_BF16) {
    const __nv_bfloat16 h = __float2bfloat16_rn(v);
    const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
    e.out_hi[off] = __bfloat16_as_ushort(h);
    e.out_lo[off] = __bfloat16_as_ushort(l);
  } else if (e.kind == TcEpilogue::STORE_F32) {
    e.out_f32[off] = v;
  } else {
    double *y = e.out_f64 + off;
    const double r = e.alpha * (double)v;
    *y = (e.beta == 0.0) ? r : fma(e.beta, *y, r);
  }
}

// The K splits' FP32 sums of a tile are added as an unevaluated pair of floats (Knuth's TwoSum,
// error-free; about 48 significant bits) in kh[j] + kl[j]: no FP64 instruction per split (the
// FP64 pipe of GB300 runs at 2 operations per clock and SM).  In slice mode every split sum is
// exact, so the result is the exact sum of the splits to that precision.
__device__ __forceinline__ void pair_add(float (&kh)[32], float (&kl)[32], const uint32_t (&r)[32], bool first) {
  if (first) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      kh[j] = __uint_as_float(r[j]);
      kl[j] = 0.f;
    }
    return;
  }
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    const float x = __uint_as_float(r[j]), hi = kh[j];
    const float sum = hi + x;
    const float bb = sum - hi;
    kl[j] += (hi - (sum - bb)) + (x - bb);
    kh[j] = sum;
  }
}

// Writes a thread's 32 float-pair sums (columns n0 ..) of row base rbase through the epilogue map.
__device__ __forceinline__ void pair_write(const float (&kh)[32], const float (&kl)[32], const TcEpilogue &e,
                                           int64_t N, int64_t n0,
                                           int64_t rbase) {
  int64_t n = n0, nq = n / e.cd, nr = n % e.cd;
#pragma unroll
  for (int j = 0; j < 32; ++j) {
    if (n < N && nr < e.clim) {
      const int64_t off = rbase + nq * e.co1 + nr * e.co2;
      const float hi = kh[j], lo = kl[j];
      if (e.kind == TcEpilogue::PAIR_F32) {
        reinterpret_cast<float2 *>(e.out_f32)[off] = make_float2(hi, lo);
      } else {
        const double val = (double)hi + (double)lo;
        if (e.kind == TcEpilogue::AXPBY_F64) {
          double *y = e.out_f64 + off;
          const double rv = e.alpha * val;
          *y = (e.beta == 0.0) ? rv : fma(e.beta, *y, rv);
        } else {
          epi_store(e, off, (float)val);
        }
      }
    }
    ++n;
    if (++nr == e.cd) { nr = 0; ++nq; }
  }
}

// Work items of the persistent kernel: an item is one tile job, or, for a problem with in-CTA K
// accumulation (kacc), the ksplit consecutive jobs of one output tile; items are strided over
// the CTAs and a CTA runs the jobs of its item in order.
__host__ __device__ __forceinline__ int64_t item_count(const KParams &p) {
  return p.kacc ? p.ntiles / p.spg : p.ntiles;
}
__device__ __forceinline__ int64_t item_len(const KParams &p) { return p.kacc ? p.spg : 1; }

// K blocks [kb, ke) of split s.
struct KRange {
  int kb, ke;
};
template <int BK>
__device__ __forceinline__ KRange k_range(const KParams &p, int64_t s) {
  KRange r;
  const int kchunks = (int)(p.K / BK);
  r.kb = (int)s * p.kc_per;
  r.ke = min(kchunks, r.kb + p.kc_per);
  return r;
}

// Problem sources of the persistent kernel: one problem, or a group of up to
// kGroupMax problems (same tile shape) whose item lists are concatenated.  Both
// live in the kernel parameter space, so every tensor map is a __grid_constant__.
struct SingleSrc {
  CUtensorMap maps[4];  // A hi, A lo, B hi, B lo
  KParams p;
  __device__ __forceinline__ int64_t total() const { return item_count(p); }
  __device__ __forceinline__ int locate(int64_t t, int64_t &local, int &) const {
    local = t;
    return 0;
  }
  __device__ __forceinline__ const KParams &params(int) const { return p; }
  __device__ __forceinline__ const CUtensorMap *map(int, int w) const { return &maps[w]; }
  __device__ __forceinline__ int *err() const { return p.err; }
};

constexpr int kGroupMax = 32;
struct GroupSrc {
  CUtensorMap maps[4 * kGroupMax];
  KParams p[kGroupMax];
  int64_t begin[kGroupMax + 1];  // first global item of each problem; begin[n] = total
  int n;
  int *err_ptr;
  __device__ __forceinline__ int64_t total() const { return begin[n]; }
  // t grows along a CTA's walk, so the problem index only moves forward from the hint
  __device__ __forceinline__ int locate(int64_t t, int64_t &local, int &hint) const {
    while (hint + 1 < n && begin[hint + 1] <= t) ++hint;
    local = t - begin[hint];
    return hint;
  }
  __device__ __forceinline__ const KParams &params(int i) const { return p[i]; }
  __device__ __forceinline__ const CUtensorMap *map(int i, int w) const { return &maps[4 * i + w]; }
  __device__ __forceinline__ int *err() const { return err_ptr; }
};
static_assert(sizeof(GroupSrc) <= 32000, "grouped GEMM parameters exceed the kernel parameter space");

template <int BN, int BK, class Src, bool SLICE = false>
__global__ void __launch_bounds__(kThreads, 1) tc_gemm_kernel(const __grid_constant__ Src src) {
  using C = Cfg<BN, BK, SLICE>;
  extern __shared__ uint8_t smem_raw[];
  uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
  uint64_t *full = (uint64_t *)(smem + C::STAGES * C::STAGE_BYTES);
  uint64_t *empty = full + C::STAGES;
  uint64_t *accf = empty + C::STAGES;
  uint64_t *acce = accf + C::NBUF;
  uint32_t *tmem_slot = (uint32_t *)(acce + C::NBUF);
  volatile int *abort_flag = (volatile int *)(tmem_slot + 1);

  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (threadIdx.x == 0) {
    for (int i = 0; i < C::STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    for (int i = 0; i < C::NBUF; ++i) {
      mbar_init(&accf[i], 1);
      mbar_init(&acce[i], kEpiWarps);  // one arrive per epilogue warp
    }
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"((uint32_t)C::TMEM_COLS));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  fence_before();
  __syncthreads();
  fence_after();
  const uint32_t tmem_base = *tmem_slot;
  int *const err = src.err();
  const int64_t nitems = src.total();  // item R: jobs li * len + u, u < len (see item_len)

  if (warp == 0) {
    if (lane == 0) {
      // ---------------- TMA producer ----------------
      int stage = 0;
      uint32_t phase = 0;
      int hint = 0;
      for (int64_t R = blockIdx.x; R < nitems; R += gridDim.x) {
        int64_t li;
        const int pi = src.locate(R, li, hint);
        const KParams p = src.params(pi);  // registers: no reloads behind the stores
        const int64_t len = item_len(p);
        const CUtensorMap *mAhi = src.map(pi, 0), *mAlo = src.map(pi, 1);
        const CUtensorMap *mBhi = src.map(pi, 2), *mBlo = src.map(pi, 3);
        // the jobs of an item share the tile; only the K split advances (decode once per item)
        TileCoord tc = decode(p, li * len);
        const int ya = (int)(tc.b * p.a_brows + tc.m * BM);
        const int yb = (int)(tc.b * p.b_brows + tc.n * BN);
        if constexpr (SLICE) {
          // the item's split group g: runs [q0, q0 + rpg); units (a, run, b0) in order, each K
          // block of a unit one stage with A plane a and B planes b0 .. b0 + nb - 1
          const int kchunks = (int)(p.K / BK);
          const int q0 = (int)(tc.s / p.spg) * p.rpg;
          for (int a = 0; a < p.nsl; ++a)
            for (int qr = q0; qr < q0 + p.rpg; ++qr)
              for (int b0 = 0; b0 < p.nsl - a; b0 += C::UNIT) {
                const int nb = min(C::UNIT, p.nsl - a - b0);
                const int kb = qr * p.kc_per, ke = min(kchunks, kb + p.kc_per);
                for (int kc = kb; kc < ke; ++kc) {
                  if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err, 1)) goto producer_done;
                  uint8_t *st = smem + stage * C::STAGE_BYTES;
                  mbar_expect_tx(&full[stage], (uint32_t)(C::A_BYTES + nb * C::B_BYTES));
                  tma_load_2d(smem_u32(st), mAhi, &full[stage], kc * BK, ya + a * (int)p.a_plane);
                  for (int b = 0; b < nb; ++b)
                    tma_load_2d(smem_u32(st + C::A_BYTES + b * C::B_BYTES), mBhi, &full[stage], kc * BK,
                                yb + (b0 + b) * (int)p.b_plane);
                  if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
                }
              }
        } else {
          for (int64_t u = 0; u < len; ++u, ++tc.s) {
            const KRange kr = k_range<BK>(p, tc.s);
            for (int kc = kr.kb; kc < kr.ke; ++kc) {
              if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err, 1)) goto producer_done;
              uint8_t *st = smem + stage * C::STAGE_BYTES;
              mbar_expect_tx(&full[stage], (uint32_t)C::STAGE_BYTES);
              tma_load_2d(smem_u32(st), mAhi, &full[stage], kc * BK, ya);
              tma_load_2d(smem_u32(st + C::A_BYTES), mAlo, &full[stage], kc * BK, ya);
              tma_load_2d(smem_u32(st + 2 * C::A_BYTES), mBhi, &full[stage], kc * BK, yb);
              tma_load_2d(smem_u32(st + 2 * C::A_BYTES + C::B_BYTES), mBlo, &full[stage], kc * BK, yb);
              if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
            }
          }
        }
      }
      // drain: wait until the MMA warp has consumed every stage issued (bounded)
      for (int i = 0; i < C::STAGES; ++i) {
        if (!mbar_wait(&empty[stage], phase ^ 1, abort_flag, err, 5)) break;
        if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
      }
    producer_done:;
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // ---------------- MMA issuer ----------------
      constexpr uint32_t idesc = (1u << 4)                   // D: FP32
                                 | (1u << 7) | (1u << 10)     // A, B: BF16
                                 | ((uint32_t)(BN >> 3) << 17) // N
                                 | ((uint32_t)(BM >> 4) << 24); // M
      int stage = 0;
      uint32_t phase = 0;
      int buf = 0;
      uint32_t aphase = 0;
      int hint = 0;
      for (int64_t R = blockIdx.x; R < nitems; R += gridDim.x) {
        int64_t li;
        const KParams p = src.params(src.locate(R, li, hint));
        const int64_t len = item_len(p);
        // the jobs of an item share the tile; only the K split advances (decode once per item)
        TileCoord tc = decode(p, li * len);
        if constexpr (SLICE) {
          // units (a, run, b0) in the producer's order: one accumulator buffer per unit, nb
          // adjacent accumulators of BN columns filled by one MMA of width nb * BN per K step
          const int kchunks = (int)(p.K / BK);
          const int q0 = (int)(tc.s / p.spg) * p.rpg;
          for (int a = 0; a < p.nsl; ++a)
            for (int qr = q0; qr < q0 + p.rpg; ++qr)
              for (int b0 = 0; b0 < p.nsl - a; b0 += C::UNIT) {
                const int nb = min(C::UNIT, p.nsl - a - b0);
                const int kb = qr * p.kc_per, ke = min(kchunks, kb + p.kc_per);
                const uint32_t idesc_u = (idesc & ~(0x3Fu << 17)) | ((uint32_t)((nb * BN) >> 3) << 17);
                if (!mbar_wait(&acce[buf], aphase ^ 1, abort_flag, err, 2)) goto mma_done;
                fence_after();
                const uint32_t dtu = tmem_base + (uint32_t)(buf * C::BUFW);
                for (int kc = kb; kc < ke; ++kc) {
                  if (!mbar_wait(&full[stage], phase, abort_flag, err, 3)) goto mma_done;
                  fence_after();
                  const uint32_t st = smem_u32(smem + stage * C::STAGE_BYTES);
                  // descriptors are linear in the address (bits 0-13 hold addr >> 4): + 2 per
                  // 16-element K step; the B planes of the unit are one stacked operand
                  const uint64_t da = sdesc(st, C::SBO, C::LAYOUT);
                  const uint64_t db = sdesc(st + C::A_BYTES, C::SBO, C::LAYOUT);
                  mma_bf16(dtu, da, db, idesc_u, kc > kb ? 1u : 0u);
#pragma unroll
                  for (int kk = 1; kk < BK / 16; ++kk) mma_bf16(dtu, da + 2 * kk, db + 2 * kk, idesc_u, 1u);
                  mma_commit(&empty[stage]);
                  if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
                }
                mma_commit(&accf[buf]);
                if (++buf == C::NBUF) { buf = 0; aphase ^= 1; }
              }
          continue;
        }
        for (int64_t u = 0; u < len; ++u, ++tc.s) {
          const KRange kr = k_range<BK>(p, tc.s);
          const int kb = kr.kb, ke = kr.ke;
          if (!mbar_wait(&acce[buf], aphase ^ 1, abort_flag, err, 2)) goto mma_done;
          fence_after();
          const uint32_t d_tmem = tmem_base + (uint32_t)(buf * BN);
          for (int kc = kb; kc < ke; ++kc) {
            if (!mbar_wait(&full[stage], phase, abort_flag, err, 3)) goto mma_done;
            fence_after();
            const uint32_t st = smem_u32(smem + stage * C::STAGE_BYTES);
            // descriptors are linear in the address: + 2 per 16 bf16 (32 bytes) along K
            const uint64_t dah0 = sdesc(st, C::SBO, C::LAYOUT);
            const uint64_t dal0 = dah0 + (C::A_BYTES >> 4);
            const uint64_t dbh0 = dah0 + ((2 * C::A_BYTES) >> 4);
            const uint64_t dbl0 = dbh0 + (C::B_BYTES >> 4);
#pragma unroll
            for (int kk = 0; kk < BK / 16; ++kk) {
              const uint32_t acc0 = (kc > kb || kk > 0) ? 1u : 0u;
              const uint64_t dah = dah0 + 2 * kk, dal = dal0 + 2 * kk;
              const uint64_t dbh = dbh0 + 2 * kk, dbl = dbl0 + 2 * kk;
              mma_bf16(d_tmem, dah, dbh, idesc, acc0);
              mma_bf16(d_tmem, dah, dbl, idesc, 1u);
              mma_bf16(d_tmem, dal, dbh, idesc, 1u);
              if (p.products == 4) mma_bf16(d_tmem, dal, dbl, idesc, 1u);
            }
            mma_commit(&empty[stage]);  // frees the smem stage when these MMAs complete
            if (++stage == C::STAGES) { stage = 0; phase ^= 1; }
          }
          mma_commit(&accf[buf]);  // accumulator ready for the epilogue
          if (++buf == C::NBUF) { buf = 0; aphase ^= 1; }
        }
      }
    mma_done:;
    }
  } else {
    // ---------------- epilogue warps ----------------
    // A warp may only read the TMEM lane quarter 32 * (warp % 4); the two warps
    // of each quarter split the tile's columns.
    const int q = warp % 4;
    const int half = (warp - 2) / 4;
    constexpr int COLS = BN >= 64 ? BN / 2 : BN;
    const int cbeg = (BN >= 64 || half == 0) ? half * COLS : BN;
    const int cend = (BN >= 64 || half == 0) ? cbeg + COLS : BN;
    // float-pair sums over the K splits of a tile (kacc; BN <= 64: at most 32 columns per thread)
    constexpr int KACC = BN <= 64 ? 32 : 1;
    float kh[KACC], kl[KACC];
    int buf = 0;
    uint32_t aphase = 0;
    int hint = 0;
    for (int64_t R = blockIdx.x; R < nitems; R += gridDim.x) {
      int64_t li;
      // a register copy: the stores below cannot alias it, so nothing is reloaded per element
      const KParams p = src.params(src.locate(R, li, hint));
      const TcEpilogue &e = p.epi;
      const int64_t len = item_len(p);
      // the jobs of an item share the tile and the split group: row terms once per item
      TileCoord tc = decode(p, li * len);
      const int64_t i = tc.m * BM + q * 32 + lane;
      const bool row_ok = i < p.M && (i % e.rd) < e.rlim;
      // partial offset: the K split (F32 partials) or the split group (kacc groups)
      const int64_t rbase = (i / e.rd) * e.ro1 + (i % e.rd) * e.ro2 + tc.b * e.bo +
                            (p.kacc ? (tc.s / p.spg) * e.so : tc.s * e.so);
      if constexpr (SLICE) {
        // the units of the item in the MMA's order; each buffer holds nb adjacent accumulators
        const int q0 = (int)(tc.s / p.spg) * p.rpg;
        bool first = true;
        for (int a = 0; a < p.nsl; ++a)
          for (int qr = q0; qr < q0 + p.rpg; ++qr)
            for (int b0 = 0; b0 < p.nsl - a; b0 += C::UNIT) {
              const int nb = min(C::UNIT, p.nsl - a - b0);
              if (!mbar_wait(&accf[buf], aphase, abort_flag, err, 4)) goto epi_done;
              fence_after();
              if (cbeg < cend) {
                for (int j = 0; j < nb; ++j) {
                  uint32_t r[32];
                  tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * C::BUFW + j * BN + cbeg), r);
                  pair_add(kh, kl, r, first);
                  first = false;
                }
              }
              fence_before();
              __syncwarp();
              if (lane == 0) mbar_arrive(&acce[buf]);
              if (++buf == C::NBUF) { buf = 0; aphase ^= 1; }
            }
        if (row_ok && cbeg < cend) pair_write(kh, kl, e, p.N, tc.n * BN + cbeg, rbase);
        continue;
      }
      for (int64_t u = 0; u < len; ++u, ++tc.s) {
      if (!mbar_wait(&accf[buf], aphase, abort_flag, err, 4)) goto epi_done;
      fence_after();
      if constexpr (BN <= 64) {
        if (p.kacc) {
          // this thread's 32 columns (cbeg == cend for the idle half of a BN = 32 tile)
          if (cbeg < cend) {
            uint32_t r[32];
            tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * C::BUFW + cbeg), r);
            const int64_t sg = u;  // position inside the split group (an item is one group)
            pair_add(kh, kl, r, sg == 0);
            if (row_ok && sg == p.spg - 1) pair_write(kh, kl, e, p.N, tc.n * BN + cbeg, rbase);  // split order
          }
          fence_before();
          __syncwarp();
          if (lane == 0) mbar_arrive(&acce[buf]);
          if (++buf == C::NBUF) { buf = 0; aphase ^= 1; }
          continue;
        }
      }
#pragma unroll 1
      for (int c0 = cbeg; c0 < cend; c0 += 32) {
        uint32_t r[32];
        tmem_ld32(tmem_base + ((uint32_t)(q * 32) << 16) + (uint32_t)(buf * C::BUFW + c0), r);
        if (!row_ok) continue;
        const int64_t n0 = tc.n * BN + c0;
        const int64_t nq0 = n0 / e.cd, nr0 = n0 % e.cd;
        if (nr0 + 32 <= e.cd && n0 + 32 <= p.N && nr0 + 32 <= e.clim) {
          // fast path: the 32 columns are one arithmetic run of offsets
          const int64_t base = rbase + nq0 * e.co1 + nr0 * e.co2;
          const int64_t st = e.co2;
          if (e.kind == TcEpilogue::SPLIT_BF16) {
            uint16_t *oh = e.out_hi + base, *ol = e.out_lo + base;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const float v = __uint_as_float(r[j]);
              const __nv_bfloat16 h = __float2bfloat16_rn(v);
              const __nv_bfloat16 l = __float2bfloat16_rn(v - __bfloat162float(h));
              oh[j * st] = __bfloat16_as_ushort(h);
              ol[j * st] = __bfloat16_as_ushort(l);
            }
          } else if (e.kind == TcEpilogue::STORE_F32) {
            float *o = e.out_f32 + base;
#pragma unroll
            for (int j = 0; j < 32; ++j) o[j * st] = __uint_as_float(r[j]);
          } else {
            double *o = e.out_f64 + base;
            const double al = e.alpha, be = e.beta;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
              const double rv = al * (double)__uint_as_float(r[j]);
              o[j * st] = (be == 0.0) ? rv : fma(be, o[j * st], rv);
            }
          }
        } else {
          int64_t n = n0, nq = nq0, nr = nr0;
#pragma unroll
          for (int j = 0; j < 32; ++j) {
            if (n < p.N && nr < e.clim)
              epi_store(e, rbase + nq * e.co1 + nr * e.co2, __uint_as_float(r[j]));
            ++n;
            if (++nr == e.cd) { nr = 0; ++nq; }
          }
        }
      }
      fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&acce[buf]);
      if (++buf == C::NBUF) { buf = 0; aphase ^= 1; }
      }
    }
  epi_done:;
  }
  fence_before();
  __syncthreads();
  if (warp == 1) {
    fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem_base),
                 "r"((uint32_t)C::TMEM_COLS));
  }
}

// ---------------- helpers ----------------

__device__ __forceinline__ void split_range(const double *__restrict__ x, int64_t rows, int64_t cols,
                                            const SplitMap &m, uint16_t *__restrict__ hi,
                                            uint16_t *__restrict__ lo, int64_t ldo, int64_t t0,
                                            int64_t step) {
  const int64_t total = rows * cols;
  for (int64_t t = t0; t < total; t += step) {
    const int64_t r = t / cols, c = t % cols;
    const int64_t rq = r / m.rdiv, rr = r % m.rdiv;
    if (rr >= m.rlim) continue;
    const double v = x[rq * m.rs1 + rr * m.rs2 + c * m.cs];
    const __nv_bfloat16 h = __double2bfloat16(v);
    const __nv_bfloat16 l = __double2bfloat16(v - (double)__bfloat162float(h));
    hi[r * ldo + c] = __bfloat16_as_ushort(h);
    lo[r * ldo + c] = __bfloat16_as_ushort(l);
  }
}

__global__ void split_kernel(const double *__restrict__ x, int64_t rows, int64_t cols,
                             const SplitMap m, uint16_t *__restrict__ hi, uint16_t *__restrict__ lo,
                             int64_t ldo) {
  split_range(x, rows, cols, m, hi, lo, ldo, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
              (int64_t)gridDim.x * blockDim.x);
}

constexpr int kJobsMax = 96;  // jobs per grouped elementwise launch (parameter space)
struct SplitGroup {
  SplitJob j[kJobsMax];
  int n;
};
struct ReduceGroup {
  ReduceJob j[kJobsMax];
  int n;
};
static_assert(sizeof(SplitGroup) <= 32000 && sizeof(ReduceGroup) <= 32000, "grouped job lists too large");

__global__ void split_group_kernel(const __grid_constant__ SplitGroup g) {
  const SplitJob q = g.j[blockIdx.y];
  split_range(q.x, q.rows, q.cols, q.map, q.hi, q.lo, q.ldo,
              blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

__device__ __forceinline__ void reduce_range(const float *__restrict__ part, int64_t M, int64_t N,
                                             int ksplit, const TcEpilogue &e, int64_t t0, int64_t step) {
  const int64_t total = M * N;
  for (int64_t t = t0; t < total; t += step) {
    const int64_t i = t / N, n = t % N;
    if ((i % e.rd) >= e.rlim || (n % e.cd) >= e.clim) continue;
    double acc = 0.0;
    // the same summation order as a plain loop; the unroll lets the independent loads of
    // eight partials be in flight together (the loop is latency-bound otherwise)
#pragma unroll 8
    for (int s = 0; s < ksplit; ++s) acc += (double)part[s * total + t];
    // the partial sums are added in FP64; the final value enters the epilogue
    // as FP64 for AXPBY (no extra rounding) and as FP32 for the bf16 split
    const int64_t off = (i / e.rd) * e.ro1 + (i % e.rd) * e.ro2 + (n / e.cd) * e.co1 + (n % e.cd) * e.co2;
    if (e.kind == TcEpilogue::AXPBY_F64) {
      double *y = e.out_f64 + off;
      const double r = e.alpha * acc;
      *y = (e.beta == 0.0) ? r : fma(e.beta, *y, r);
    } else {
      epi_store(e, off, (float)acc);
    }
  }
}

__global__ void reduce_partials_kernel(const float *__restrict__ part, int64_t M, int64_t N,
                                       int ksplit, const TcEpilogue e) {
  reduce_range(part, M, N, ksplit, e, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
               (int64_t)gridDim.x * blockDim.x);
}

// One warp per (row, run of chunk columns): the run's maximum, then its digits, all in integer
// arithmetic on the FP64 bit patterns (the FP64 pipe of GB300 is slow; these are INT32/INT64
// operations): the run scale is 2^e with e the frexp exponent of the largest |x|, an element is
// m = round(x 2^(B - e)) with B = 7 nsl (|m| <= 2^B, a 64-bit integer from its mantissa), and the
// digits are its balanced base-2^7 digits, d_t = round(r / 2^(B - 7t)), r -= d_t 2^(B - 7t).
__device__ __forceinline__ long long fixed_point(unsigned long long bits, int e, int B) {
  const int ef = (int)((bits >> 52) & 0x7FF);
  if (ef == 0) return 0;  // zero or subnormal: below 2^-1022, far under the run scale
  const long long mant = (long long)((bits & 0xFFFFFFFFFFFFFull) | 0x10000000000000ull);
  // value = mant 2^(ef - 1075), m = mant 2^(ef - 1075 + B - e): a right shift by sh >= 53 - B
  const int sh = 1075 + e - ef - B;
  long long m = 0;
  if (sh < 63) m = (mant + (1LL << (sh - 1))) >> sh;
  return (bits >> 63) ? -m : m;
}

// The same fixed point for a float given by its bits.
__device__ __forceinline__ long long fixed_point_f32(unsigned bits, int e, int B) {
  const int ef = (int)((bits >> 23) & 0xFF);
  if (ef == 0) return 0;
  const long long mant = (long long)((bits & 0x7FFFFFu) | 0x800000u);
  // value = mant 2^(ef - 150), m = mant 2^(ef - 150 + B - e)
  const int sh = 150 + e - ef - B;
  long long m;
  if (sh <= 0) m = mant << (-sh);  // |value| < 2^(e + 1): at most 2^(B + 1)
  else m = sh < 40 ? (mant + (1LL << (sh - 1))) >> sh : 0;
  return (bits >> 31) ? -m : m;
}

// Input element access of the slicer: FP64 values, or float pairs (hi, lo) with value hi + lo.
struct F64In {
  const unsigned long long *p;
  __device__ __forceinline__ unsigned long long abs_bits(int64_t i) const {
    return __ldg(p + i) & 0x7FFFFFFFFFFFFFFFull;
  }
  // frexp exponent of a maximum (abs_bits): mx < 2^e; subnormal maxima as 2^-1022
  __device__ __forceinline__ static int exponent(unsigned long long mx) {
    return mx == 0 ? 0 : max((int)(mx >> 52), 1) - 1022;
  }
  __device__ __forceinline__ long long fixed(int64_t i, int e, int B) const {
    return fixed_point(__ldg(p + i), e, B);
  }
  // four consecutive elements (32-byte aligned): raw words, |x| bits, fixed point of a word
  __device__ __forceinline__ void load4(int64_t i, unsigned long long (&w)[4]) const {
    const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2 *>(p + i));
    const ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2 *>(p + i) + 1);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
  }
  __device__ __forceinline__ static unsigned long long abs_word(unsigned long long w) {
    return w & 0x7FFFFFFFFFFFFFFFull;
  }
  __device__ __forceinline__ static long long fixed_word(unsigned long long w, int e, int B) {
    return fixed_point(w, e, B);
  }
};
struct PairIn {
  const unsigned long long *p;  // float2 elements
  __device__ __forceinline__ unsigned long long abs_bits(int64_t i) const {
    return (unsigned long long)((unsigned)__ldg(p + i) & 0x7FFFFFFFu);  // |hi|; hi holds the sum
  }
  __device__ __forceinline__ static int exponent(unsigned long long mx) {
    return mx == 0 ? 0 : max((int)(mx >> 23), 1) - 126;
  }
  __device__ __forceinline__ long long fixed(int64_t i, int e, int B) const {
    return fixed_word(__ldg(p + i), e, B);
  }
  __device__ __forceinline__ void load4(int64_t i, unsigned long long (&w)[4]) const {
    const ulonglong2 a = __ldg(reinterpret_cast<const ulonglong2 *>(p + i));
    const ulonglong2 b = __ldg(reinterpret_cast<const ulonglong2 *>(p + i) + 1);
    w[0] = a.x; w[1] = a.y; w[2] = b.x; w[3] = b.y;
  }
  __device__ __forceinline__ static unsigned long long abs_word(unsigned long long w) {
    return (unsigned long long)((unsigned)w & 0x7FFFFFFFu);
  }
  __device__ __forceinline__ static long long fixed_word(unsigned long long v, int e, int B) {
    // little-endian float2: hi in the low word
    return fixed_point_f32((unsigned)v, e, B) + fixed_point_f32((unsigned)(v >> 32), e, B);
  }
};

// The bf16 bits of digit d (|d| <= 128) of a run with scale exponent e at digit position t >= 1:
// d 2^(e - 7 t), exact; scales below the FP32 normal range flush to 0.
__device__ __forceinline__ uint16_t digit_bits(long long d, int e, int t) {
  const int pe = e - 7 * t + 127;
  float v = 0.f;
  if (pe >= 1 && pe <= 254) v = (float)(int)d * __int_as_float(pe << 23);
  return __bfloat16_as_ushort(__float2bfloat16_rn(v));
}

// The digits of one element (fixed point rem of B = 7 nsl bits) into d[0 .. nsl).
__device__ __forceinline__ void digits(long long rem, int nsl, long long (&d)[kMaxDigits]) {
#pragma unroll
  for (int sl = 0; sl < kMaxDigits; ++sl) {
    const int shift = 7 * (nsl - 1 - sl);  // digit sl + 1 has weight 2^(B - 7 (sl + 1))
    long long v = sl < nsl ? rem : 0;      // the last digit: the remaining |rem| <= 64
    if (shift > 0) {
      v = (rem + (1LL << (shift - 1))) >> shift;  // round half up (arithmetic shift: floor)
      rem -= v << shift;
    }
    d[sl] = v;
  }
}

// VEC = 4: a lane handles 4 consecutive columns (one 32-byte load, one 8-byte store per plane);
// needs unit column stride, runs and row bases aligned to 4 elements.
// NSL > 0: the digit count as a compile-time constant (constant shifts); 0: nsl at run time.
template <class In, int VEC, int NSL>
__global__ void slice_kernel(const In in, int64_t rows, int64_t cols, const SplitMap m, int nsl_rt, int64_t chunk,
                             uint16_t *__restrict__ out, int64_t ldo, int64_t plane) {
  const int nsl = NSL > 0 ? NSL : nsl_rt;
  const int lane = threadIdx.x & 31;
  const int64_t nchunks = (cols + chunk - 1) / chunk;
  const int64_t units = rows * nchunks;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < units; u += nwarps) {
    const int64_t r = u / nchunks, q = u % nchunks;
    const int64_t rq = r / m.rdiv, rr = r % m.rdiv;
    if (rr >= m.rlim) continue;  // uniform over the warp
    const int64_t base = rq * m.rs1 + rr * m.rs2;
    const int64_t c0 = q * chunk, c1 = min(cols, c0 + chunk);
    unsigned long long mx = 0;  // largest |x| as a bit pattern (ordered like the values)
    if constexpr (VEC == 4) {
      for (int64_t c = c0 + 4 * lane; c < c1; c += 128) {
        if (c + 4 <= c1) {
          unsigned long long w[4];
          in.load4(base + c, w);
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const unsigned long long a = In::abs_word(w[v]);
            mx = a > mx ? a : mx;
          }
        } else {
          for (int64_t cc = c; cc < c1; ++cc) {
            const unsigned long long a = In::abs_word(__ldg(in.p + base + cc));
            mx = a > mx ? a : mx;
          }
        }
      }
    } else {
      for (int64_t c = c0 + lane; c < c1; c += 32) {
        const unsigned long long a = in.abs_bits(base + c * m.cs);
        mx = a > mx ? a : mx;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = y > mx ? y : mx;
    }
    const int e = In::exponent(mx);
    uint16_t *orow = out + r * ldo;
    if constexpr (VEC == 4) {
      for (int64_t c = c0 + 4 * lane; c < c1; c += 128) {
        const int nv = (int)min((int64_t)4, c1 - c);
        unsigned long long w[4] = {0, 0, 0, 0};
        if (nv == 4) {
          in.load4(base + c, w);
        } else {
#pragma unroll
          for (int v = 0; v < 4; ++v)
            if (v < nv) w[v] = __ldg(in.p + base + c + v);
        }
        long long d[4][kMaxDigits];
#pragma unroll
        for (int v = 0; v < 4; ++v) digits((v < nv && mx != 0) ? In::fixed_word(w[v], e, 7 * nsl) : 0, nsl, d[v]);
#pragma unroll
        for (int sl = 0; sl < kMaxDigits; ++sl) {
          if (sl >= nsl) break;
          uint16_t *o = orow + sl * plane + c;
          if (nv == 4) {
            const unsigned long long bits = (unsigned long long)digit_bits(d[0][sl], e, sl + 1) |
                                            ((unsigned long long)digit_bits(d[1][sl], e, sl + 1) << 16) |
                                            ((unsigned long long)digit_bits(d[2][sl], e, sl + 1) << 32) |
                                            ((unsigned long long)digit_bits(d[3][sl], e, sl + 1) << 48);
            *reinterpret_cast<unsigned long long *>(o) = bits;
          } else {
#pragma unroll
            for (int v = 0; v < 4; ++v)
              if (v < nv) o[v] = digit_bits(d[v][sl], e, sl + 1);
          }
        }
      }
    } else {
      for (int64_t c = c0 + lane; c < c1; c += 32) {
        long long d[kMaxDigits];
        digits(mx == 0 ? 0 : in.fixed(base + c * m.cs, e, 7 * nsl), nsl, d);
#pragma unroll
        for (int sl = 0; sl < kMaxDigits; ++sl) {
          if (sl >= nsl) break;
          orow[sl * plane + c] = digit_bits(d[sl], e, sl + 1);
        }
      }
    }
  }
}

// Single pass of the same slicing for runs of at most 1024 columns and NSL digits: a lane
// holds its (up to) 8 groups of 4 consecutive elements of the run in registers, so every load
// of the run is in flight at once and the input is read from memory once (the two-pass kernel
// above re-reads the run for its digits and keeps one load per lane in flight).  The digits and
// their bf16 bits are those of slice_kernel, element for element.
constexpr int kRunGroups = 8;  // 8 groups x 4 elements x 32 lanes = 1024 columns per run
template <class In, int NSL>
__global__ void __launch_bounds__(256) slice_run_kernel(const In in, int64_t rows, int64_t cols, const SplitMap m,
                                                        int64_t chunk, uint16_t *__restrict__ out, int64_t ldo,
                                                        int64_t plane) {
  const int lane = threadIdx.x & 31;
  const int64_t nchunks = (cols + chunk - 1) / chunk;
  const int64_t units = rows * nchunks;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < units; u += nwarps) {
    const int64_t r = u / nchunks, q = u % nchunks;
    const int64_t rq = r / m.rdiv, rr = r % m.rdiv;
    if (rr >= m.rlim) continue;  // uniform over the warp
    const int64_t base = rq * m.rs1 + rr * m.rs2;
    const int64_t c0 = q * chunk, c1 = min(cols, c0 + chunk);
    unsigned long long w[kRunGroups][4];
    unsigned long long mx = 0;
#pragma unroll
    for (int g = 0; g < kRunGroups; ++g) {
      const int64_t c = c0 + 128 * g + 4 * lane;
#pragma unroll
      for (int v = 0; v < 4; ++v) w[g][v] = 0;
      if (c + 4 <= c1) {
        in.load4(base + c, w[g]);
      } else if (c < c1) {
#pragma unroll
        for (int v = 0; v < 3; ++v)
          if (c + v < c1) w[g][v] = __ldg(in.p + base + c + v);
      }
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const unsigned long long a = In::abs_word(w[g][v]);
        mx = a > mx ? a : mx;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      const unsigned long long y = __shfl_xor_sync(0xffffffffu, mx, o);
      mx = y > mx ? y : mx;
    }
    const int e = In::exponent(mx);
    uint16_t *orow = out + r * ldo;
#pragma unroll
    for (int g = 0; g < kRunGroups; ++g) {
      const int64_t c = c0 + 128 * g + 4 * lane;
      if (c >= c1) continue;
      unsigned long long packed[NSL];
#pragma unroll
      for (int sl = 0; sl < NSL; ++sl) packed[sl] = 0;
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        // zero-filled words past the run's end slice to zero digits and are not stored
        long long rem = mx != 0 ? In::fixed_word(w[g][v], e, 7 * NSL) : 0;
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl) {
          const int shift = 7 * (NSL - 1 - sl);
          long long d = rem;
          if (shift > 0) {
            d = (rem + (1LL << (shift - 1))) >> shift;  // round half up, as digits()
            rem -= d << shift;
          }
          packed[sl] |= (unsigned long long)digit_bits(d, e, sl + 1) << (16 * v);
        }
      }
      if (c + 4 <= c1) {
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl)
          *reinterpret_cast<unsigned long long *>(orow + sl * plane + c) = packed[sl];
      } else {
        const int nv = (int)(c1 - c);
#pragma unroll
        for (int sl = 0; sl < NSL; ++sl)
#pragma unroll
          for (int v = 0; v < 3; ++v)
            if (v < nv) orow[sl * plane + c + v] = (uint16_t)(packed[sl] >> (16 * v));
      }
    }
  }
}

__global__ void reduce_f64_kernel(const double *__restrict__ part, int64_t M, int64_t N, int G,
                                  const TcEpilogue e) {
  const int64_t total = M * N;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t % M, n = t / M;
    if ((i % e.rd) >= e.rlim || (n % e.cd) >= e.clim) continue;
    double acc = 0.0;
    for (int g = 0; g < G; ++g) acc += part[g * total + t];
    double *y = e.out_f64 + (i / e.rd) * e.ro1 + (i % e.rd) * e.ro2 + (n / e.cd) * e.co1 + (n % e.cd) * e.co2;
    const double r = e.alpha * acc;
    *y = (e.beta == 0.0) ? r : fma(e.beta, *y, r);
  }
}

__global__ void reduce_group_kernel(const __grid_constant__ ReduceGroup g) {
  const ReduceJob q = g.j[blockIdx.y];
  reduce_range(q.part, q.M, q.N, q.ksplit, q.epi, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
               (int64_t)gridDim.x * blockDim.x);
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    VGB_CUDA(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q));
    if (q != cudaDriverEntryPointSuccess || !p) fail(BSE_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
    fn = (EncodeTiledFn)p;
  });
  return fn;
}

void encode(CUtensorMap *m, const uint16_t *base, int64_t rows, int64_t K, int64_t ld, int box_rows,
            int bk) {
  VGB_REQUIRE(((uintptr_t)base & 15) == 0, "tc operand base must be 16-byte aligned");
  VGB_REQUIRE(bk == 32 || bk == 64, "tc operand: K box must be 32 or 64");
  VGB_REQUIRE(K % bk == 0 && (ld * 2) % 16 == 0 && ld >= K, "tc operand K/ld not padded");
  cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)(ld * 2)};
  cuuint32_t box[2] = {(cuuint32_t)bk, (cuuint32_t)box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, (void *)base, dims, strides, box,
                           estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           bk == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B,
                           CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) fail(BSE_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
}

template <int BN, int BK, class Src, bool SLICE = false>
void launch_src(const Src &src, int64_t ntiles, cudaStream_t s) {
  using C = Cfg<BN, BK, SLICE>;
  static std::once_flag attr;
  std::call_once(attr, [] {
    VGB_CUDA(cudaFuncSetAttribute(tc_gemm_kernel<BN, BK, Src, SLICE>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM));
  });
  const int64_t grid = std::min<int64_t>(ntiles, sm_count());
  tc_gemm_kernel<BN, BK, Src, SLICE><<<(unsigned)grid, kThreads, C::SMEM, s>>>(src);
  VGB_LAUNCH_CHECK();
}

template <class Src>
void launch_any(int bn, int bk, const Src &src, int64_t ntiles, cudaStream_t s) {
  if (bk == 64) {
    switch (bn) {
      case 32: launch_src<32, 64>(src, ntiles, s); break;
      case 64: launch_src<64, 64>(src, ntiles, s); break;
      case 128: launch_src<128, 64>(src, ntiles, s); break;
      default: launch_src<256, 64>(src, ntiles, s); break;
    }
  } else {
    switch (bn) {
      case 32: launch_src<32, 32>(src, ntiles, s); break;
      case 64: launch_src<64, 32>(src, ntiles, s); break;
      case 128: launch_src<128, 32>(src, ntiles, s); break;
      default: launch_src<256, 32>(src, ntiles, s); break;
    }
  }
}

unsigned grid_1d(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 16LL * 152));
}

}  // namespace

TcMat make_tc_mat(const uint16_t *hi, const uint16_t *lo, int64_t rows, int64_t K, int64_t ld,
                  int box_rows, int bk) {
  TcMat m;
  m.hi = hi;
  m.lo = lo;
  m.rows = rows;
  m.K = K;
  m.ld = ld;
  m.box_rows = box_rows;
  m.bk = bk;
  encode(&m.map_hi, hi, rows, K, ld, box_rows, bk);
  encode(&m.map_lo, lo, rows, K, ld, box_rows, bk);
  return m;
}

namespace {

// Validated kernel parameters of one problem (tiles == 0 when there is nothing to do).
KParams make_params(const TcMat &A, const TcMat &B, const TcShape &sh, const TcEpilogue &epi, int bn,
                    int *err) {
  VGB_REQUIRE(bn == 32 || bn == 64 || bn == 128 || bn == 256, "tc_gemm: unsupported tile N");
  VGB_REQUIRE(A.box_rows == BM && B.box_rows == bn, "tc_gemm: operand boxes do not match the tile");
  VGB_REQUIRE(A.bk == B.bk, "tc_gemm: operands staged with different K boxes");
  const int BK = A.bk;
  VGB_REQUIRE(sh.K % BK == 0 && A.K >= sh.K && B.K >= sh.K, "tc_gemm: K not padded");
  int64_t a_extra = 0, b_extra = 0;  // slice mode: rows of the highest digit plane addressed
  if (sh.nslices > 0) {
    VGB_REQUIRE(sh.nslices <= kMaxDigits && sh.chain >= BK && sh.chain % BK == 0 && sh.nbatch == 1 &&
                    BK == 64 && bn <= 64,
                "tc_gemm: bad slice-mode shape");
    VGB_REQUIRE(sh.a_plane >= sh.M && sh.b_plane >= sh.N, "tc_gemm: slice planes smaller than the problem");
    VGB_REQUIRE((int64_t)sh.nslices * std::max(sh.a_plane, sh.b_plane) < (1LL << 31), "tc_gemm: planes too large");
    a_extra = (sh.nslices - 1) * sh.a_plane;
    b_extra = (sh.nslices - 1) * sh.b_plane;
  }
  VGB_REQUIRE(epi.rd >= 1 && epi.cd >= 1, "tc_gemm: bad epilogue map");
  KParams p;
  p.ntiles = 0;
  p.ksplit = 0;
  if (sh.M <= 0 || sh.N <= 0 || sh.nbatch <= 0) return p;
  // rows addressed by the last batch must exist in the operands (TMA fills beyond with zeros,
  // but row coordinates must stay within the int32 range of the descriptor)
  VGB_REQUIRE((sh.nbatch - 1) * sh.a_batch_rows + a_extra + sh.M <= A.rows + BM, "tc_gemm: A rows");
  VGB_REQUIRE((sh.nbatch - 1) * sh.b_batch_rows + b_extra + sh.N <= B.rows + bn, "tc_gemm: B rows");
  VGB_REQUIRE(A.rows < (1LL << 31) && B.rows < (1LL << 31), "tc_gemm: too many rows");
  p.M = sh.M; p.N = sh.N; p.K = sh.K;
  p.products = sh.nslices > 0 ? 1 : (sh.products == 4 ? 4 : 3);
  p.nsl = sh.nslices > 0 ? sh.nslices : 0;
  p.a_plane = sh.a_plane;
  p.b_plane = sh.b_plane;
  p.nbatch = sh.nbatch;
  p.a_brows = sh.a_batch_rows;
  p.b_brows = sh.b_batch_rows;
  const int kchunks = (int)(sh.K / BK);
  VGB_REQUIRE(kchunks >= 1, "tc_gemm: K must be positive");
  const int npairs = p.nsl * (p.nsl + 1) / 2;
  int groups = 1;
  if (p.nsl) {  // every split: one digit pair on one run of at most chain K elements
    p.kc_per = (int)std::min<int64_t>(kchunks, sh.chain / BK);
    p.cpr = (int)ceil_div(kchunks, p.kc_per);
    p.ksplit = npairs * p.cpr;
    p.kacc = 1;
    groups = std::max(1, sh.kgroups);
    VGB_REQUIRE(p.cpr % groups == 0, "tc_gemm: split groups must divide the K runs");
    p.rpg = p.cpr / groups;
  } else {
    int ks = std::max(1, std::min(sh.ksplit, kchunks));
    p.kc_per = (int)ceil_div(kchunks, ks);
    p.ksplit = (int)ceil_div(kchunks, p.kc_per);
    p.cpr = p.ksplit;
    p.rpg = 0;
    p.kacc = (sh.kacc && p.ksplit > 1) ? 1 : 0;
    groups = p.kacc ? std::max(1, sh.kgroups) : 1;
    VGB_REQUIRE(p.ksplit % groups == 0, "tc_gemm: split groups must divide the K splits");
  }
  VGB_REQUIRE(groups == 1 || (epi.kind == TcEpilogue::AXPBY_F64 && epi.beta == 0.0),
              "tc_gemm: split groups write FP64 partials");
  p.spg = p.ksplit / groups;
  VGB_REQUIRE(!p.kacc || (bn <= 64 && epi.kind != TcEpilogue::STORE_F32),
              "tc_gemm: in-CTA K accumulation needs BN <= 64 and a final (split or FP64) epilogue");
  VGB_REQUIRE(epi.kind != TcEpilogue::PAIR_F32 || (p.kacc && p.nsl > 0 && (int64_t)bn <= 64),
              "tc_gemm: float-pair output needs slice mode with in-CTA K accumulation");
  VGB_REQUIRE(p.ksplit == 1 || p.kacc || epi.kind == TcEpilogue::STORE_F32,
              "tc_gemm: K split needs F32 partials or in-CTA accumulation");
  p.mt = ceil_div(sh.M, BM);
  p.nt = ceil_div(sh.N, bn);
  p.ntiles = p.mt * p.nt * p.ksplit * sh.nbatch;
  p.epi = epi;
  p.err = err;
  return p;
}

}  // namespace

int tc_gemm(const TcMat &A, const TcMat &B, const TcShape &sh, const TcEpilogue &epi, int bn,
            int *err, cudaStream_t s) {
  const KParams p = make_params(A, B, sh, epi, bn, err);
  if (p.ntiles == 0) return 0;
  SingleSrc src;
  src.maps[0] = A.map_hi;
  src.maps[1] = A.map_lo;
  src.maps[2] = B.map_hi;
  src.maps[3] = B.map_lo;
  src.p = p;
  if (p.nsl) {  // slice mode (validated: K box 64, BN <= 64)
    if (bn == 32) launch_src<32, 64, SingleSrc, true>(src, item_count(p), s);
    else launch_src<64, 64, SingleSrc, true>(src, item_count(p), s);
  } else {
    launch_any(bn, A.bk, src, item_count(p), s);
  }
  return p.ksplit;
}

namespace {

// Non-blocking auxiliary streams per device (created once, kept for the process): the launches
// of one grouped product spread over them so that the tail of one launch overlaps the start of
// the next.
std::vector<cudaStream_t> aux_streams(int n) {
  static std::mutex mu;
  static std::map<int, std::vector<cudaStream_t>> pool;
  int dev = 0;
  VGB_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  auto &v = pool[dev];
  while ((int)v.size() < n) {
    cudaStream_t st;
    VGB_CUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    v.push_back(st);
  }
  return std::vector<cudaStream_t>(v.begin(), v.begin() + n);
}

}  // namespace

void tc_gemm_grouped(const std::vector<const TcProblem *> &probs, int bn, int *err, cudaStream_t s,
                     int *ksplit_out, int group_max, int nstreams) {
  std::unique_ptr<GroupSrc> src(new GroupSrc());
  const int gmax = std::max(1, std::min(group_max, kGroupMax));
  // more than one launch and several streams: launch l on stream l % nstreams, ordered after the
  // work already on s, and s waits for all of them at the end
  std::vector<cudaStream_t> sts;
  cudaEvent_t fork = nullptr;
  if (nstreams > 1 && (int64_t)probs.size() > gmax) {
    sts = aux_streams(std::min(nstreams, 8));
    VGB_CUDA(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    VGB_CUDA(cudaEventRecord(fork, s));
    for (cudaStream_t st : sts) VGB_CUDA(cudaStreamWaitEvent(st, fork, 0));
  }
  int launches = 0;
  int bk = 0;
  size_t i = 0;
  while (i < probs.size()) {
    src->n = 0;
    src->err_ptr = err;
    int64_t total = 0;
    for (; i < probs.size() && src->n < gmax; ++i) {
      const TcProblem &q = *probs[i];
      VGB_REQUIRE(q.shape.nslices == 0, "tc_gemm_grouped: slice mode runs through tc_gemm");
      const KParams p = make_params(q.A, q.B, q.shape, q.epi, bn, err);
      if (ksplit_out) ksplit_out[i] = p.ksplit;
      if (p.ntiles == 0) continue;
      VGB_REQUIRE(bk == 0 || bk == q.A.bk, "tc_gemm_grouped: problems with different K boxes");
      bk = q.A.bk;
      const int g = src->n++;
      src->maps[4 * g + 0] = q.A.map_hi;
      src->maps[4 * g + 1] = q.A.map_lo;
      src->maps[4 * g + 2] = q.B.map_hi;
      src->maps[4 * g + 3] = q.B.map_lo;
      src->p[g] = p;
      src->begin[g] = total;
      total += item_count(p);
    }
    if (src->n == 0) continue;
    src->begin[src->n] = total;
    launch_any(bn, bk, *src, total, sts.empty() ? s : sts[launches % sts.size()]);
    ++launches;
  }
  if (!sts.empty()) {
    for (cudaStream_t st : sts) {
      cudaEvent_t join;
      VGB_CUDA(cudaEventCreateWithFlags(&join, cudaEventDisableTiming));
      VGB_CUDA(cudaEventRecord(join, st));
      VGB_CUDA(cudaStreamWaitEvent(s, join, 0));
      VGB_CUDA(cudaEventDestroy(join));
    }
    VGB_CUDA(cudaEventDestroy(fork));
  }
}

void split_f64_to_bf16(const double *x, int64_t rows, int64_t cols, const SplitMap &m, uint16_t *hi,
                       uint16_t *lo, int64_t ldo, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  VGB_REQUIRE(m.rdiv >= 1, "split: bad row map");
  split_kernel<<<grid_1d(rows * cols), 256, 0, s>>>(x, rows, cols, m, hi, lo, ldo);
  VGB_LAUNCH_CHECK();
}

namespace {
// blocks per job of a grouped elementwise launch: about 4 waves of 256-thread blocks in total
unsigned group_blocks(int64_t max_elems, int njobs) {
  const int64_t want = ceil_div(max_elems, 256);
  const int64_t cap = std::max<int64_t>(1, (4LL * 8 * sm_count()) / std::max(1, njobs));
  return (unsigned)std::max<int64_t>(1, std::min(want, std::max<int64_t>(cap, 4)));
}
}  // namespace

void split_grouped(const std::vector<SplitJob> &jobs, cudaStream_t s) {
  std::unique_ptr<SplitGroup> g(new SplitGroup());
  size_t i = 0;
  while (i < jobs.size()) {
    g->n = 0;
    int64_t mx = 0;
    for (; i < jobs.size() && g->n < kJobsMax; ++i) {
      if (jobs[i].rows <= 0 || jobs[i].cols <= 0) continue;
      VGB_REQUIRE(jobs[i].map.rdiv >= 1, "split: bad row map");
      g->j[g->n++] = jobs[i];
      mx = std::max(mx, jobs[i].rows * jobs[i].cols);
    }
    if (g->n == 0) continue;
    split_group_kernel<<<dim3(group_blocks(mx, g->n), (unsigned)g->n), 256, 0, s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
}

void reduce_grouped(const std::vector<ReduceJob> &jobs, cudaStream_t s) {
  std::unique_ptr<ReduceGroup> g(new ReduceGroup());
  size_t i = 0;
  while (i < jobs.size()) {
    g->n = 0;
    int64_t mx = 0;
    for (; i < jobs.size() && g->n < kJobsMax; ++i) {
      if (jobs[i].M <= 0 || jobs[i].N <= 0 || jobs[i].ksplit <= 0) continue;
      g->j[g->n++] = jobs[i];
      mx = std::max(mx, jobs[i].M * jobs[i].N);
    }
    if (g->n == 0) continue;
    reduce_group_kernel<<<dim3(group_blocks(mx, g->n), (unsigned)g->n), 256, 0, s>>>(*g);
    VGB_LAUNCH_CHECK();
  }
}

void slice_f64(const double *x, int64_t rows, int64_t cols, const SplitMap &m, int nslices, int64_t chunk,
               uint16_t *out, int64_t ldo, int64_t plane, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  VGB_REQUIRE(m.rdiv >= 1 && nslices >= 1 && nslices <= kMaxDigits && chunk >= 1 && chunk <= 1024 &&
                  ldo >= cols && plane >= rows * ldo,
              "slice: bad map or sizes");
  const int64_t warps = rows * ceil_div(cols, chunk);
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(warps, 8), 64LL * sm_count()));
  const F64In in{reinterpret_cast<const unsigned long long *>(x)};
  if (m.cs == 1 && chunk % 4 == 0 && m.rs1 % 4 == 0 && m.rs2 % 4 == 0 && ldo % 4 == 0 && plane % 4 == 0 &&
      ((uintptr_t)x & 31) == 0 && ((uintptr_t)out & 7) == 0) {
    if (nslices == 5) slice_run_kernel<F64In, 5><<<blocks, 256, 0, s>>>(in, rows, cols, m, chunk, out, ldo, plane);
    else slice_kernel<F64In, 4, 0><<<blocks, 256, 0, s>>>(in, rows, cols, m, nslices, chunk, out, ldo, plane);
  } else {
    slice_kernel<F64In, 1, 0><<<blocks, 256, 0, s>>>(in, rows, cols, m, nslices, chunk, out, ldo, plane);
  }
  VGB_LAUNCH_CHECK();
}

void slice_pairs(const float *x2, int64_t rows, int64_t cols, const SplitMap &m, int nslices, int64_t chunk,
                 uint16_t *out, int64_t ldo, int64_t plane, cudaStream_t s) {
  if (rows <= 0 || cols <= 0) return;
  VGB_REQUIRE(((uintptr_t)x2 & 7) == 0 && m.rdiv >= 1 && nslices >= 1 && nslices <= kMaxDigits && chunk >= 1 &&
                  chunk <= 1024 && ldo >= cols && plane >= rows * ldo,
              "slice: bad map or sizes");
  const int64_t warps = rows * ceil_div(cols, chunk);
  const unsigned blocks = (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(warps, 8), 64LL * sm_count()));
  const PairIn in{reinterpret_cast<const unsigned long long *>(x2)};
  if (m.cs == 1 && chunk % 4 == 0 && m.rs1 % 4 == 0 && m.rs2 % 4 == 0 && ldo % 4 == 0 && plane % 4 == 0 &&
      ((uintptr_t)x2 & 31) == 0 && ((uintptr_t)out & 7) == 0) {
    if (nslices == 5) slice_run_kernel<PairIn, 5><<<blocks, 256, 0, s>>>(in, rows, cols, m, chunk, out, ldo, plane);
    else slice_kernel<PairIn, 4, 0><<<blocks, 256, 0, s>>>(in, rows, cols, m, nslices, chunk, out, ldo, plane);
  } else {
    slice_kernel<PairIn, 1, 0><<<blocks, 256, 0, s>>>(in, rows, cols, m, nslices, chunk, out, ldo, plane);
  }
  VGB_LAUNCH_CHECK();
}

void reduce_f64_groups(const double *part, int64_t M, int64_t N, int ngroups, const TcEpilogue &epi,
                       cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  VGB_REQUIRE(epi.kind == TcEpilogue::AXPBY_F64 && ngroups >= 1 && epi.rd >= 1 && epi.cd >= 1,
              "reduce_f64_groups: bad epilogue");
  reduce_f64_kernel<<<grid_1d(M * N), 256, 0, s>>>(part, M, N, ngroups, epi);
  VGB_LAUNCH_CHECK();
}

void reduce_partials(const float *partial, int64_t M, int64_t N, int ksplit, const TcEpilogue &epi,
                     cudaStream_t s) {
  reduce_partials_kernel<<<grid_1d(M * N), 256, 0, s>>>(partial, M, N, ksplit, epi);
  VGB_LAUNCH_CHECK();
}

}  // namespace vgb
