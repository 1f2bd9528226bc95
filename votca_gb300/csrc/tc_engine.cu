// Mixed-precision engine of the BSE product: every contraction over the
// auxiliary index (Hx, Hd, Hd2) as BF16x3 split products on tcgen05 tensor
// cores with FP32 accumulation; the operator's FP64 input X is split into
// bf16 hi/lo once per call and the results are accumulated into the FP64
// output.  Hqp is applied in FP64 by the caller.
//
// Padded layouts (Kc = ct rounded up to 64, Kg = naux*vt rounded up to 64,
// Kn = naux rounded up to 64, pair index I' = v*Kc + c, dimP = vt*Kc):
//   Xs   [(j, v)][Kc]          X split                        (A of Hd/Hd2 stage 1, B of Hx 1)
//   Mcc2 [(P, c1)][Kc]         M(c1, c, P)                    (B of Hd stage 1, batched over P)
//   G2   [v1][Kg]              G(v1, P, v) (screened vv)      (B of Hd stage 2)
//   Bvc2 [P][dimP] == [(P, v1)][Kc]  M(v, c, P)               (A of Hx 1, B of Hd2 stage 1)
//   BvcT [I'][Kn]              M(v, c, P)                     (A of Hx 2)
//   McvT [c1][Kg]              screened M(c1, v, P)           (A of Hd2 stage 2)
//   S    [(j, c1)][Kg]         sum_c M(c1,c,P) X_j(v,c)       (Hd intermediate)
//   U    [(j, v1)][Kg]         sum_c X_j(v,c) M(v1,c,P)       (Hd2 intermediate)
//   Zs   [j][Kn]               sum_I M(I,P) X_j(I)            (Hx intermediate)
#include <algorithm>
#include "tc_engine.cuh"

#include <cstdlib>
#include <array>
#include <map>
#include <string>
#include <tuple>
#include <mutex>

#include "tc_gemm.cuh"

#include <cuda_bf16.h>

namespace vgb {

namespace {

int64_t pad64(int64_t x) { return ceil_div(x, 64) * 64; }

struct SplitBuf {
  DeviceBuffer<uint16_t> hi, lo;
  int64_t rows = 0, ld = 0;
  // (re)allocate rows x ld zero-filled
  void ensure(int64_t r, int64_t l, cudaStream_t s) {
    if (r * l > (int64_t)hi.count || !hi.get()) {
      hi.resize(r * l);
      lo.resize(r * l);
      VGB_CUDA(cudaMemsetAsync(hi.get(), 0, r * l * sizeof(uint16_t), s));
      VGB_CUDA(cudaMemsetAsync(lo.get(), 0, r * l * sizeof(uint16_t), s));
    }
    rows = r;
    ld = l;
  }
};

int g_slices = 5;  // Ozaki digits per operand (7 bits each; pairs up to the 5th digit level)
int g_autotune = 1;  // VGB_TC_AUTOTUNE=0: grouped dense products with the fixed shape (K box 64, 32 per launch)
int g_bk256 = 32;  // K box of the BN = 256 tiles (4-stage ring); 64 gives a 2-stage ring
int bk_for(int bn) { return bn == 256 ? g_bk256 : 64; }

int pick_bn(int64_t N) {
  if (N > 128) return 256;
  if (N > 64) return 128;
  if (N > 32) return 64;
  return 32;
}

// K splits: enough to cover the SMs about twice, and enough that no FP32
// accumulation chain in TMEM is longer than max_chain (the partial sums are
// reduced in FP64).
int64_t g_max_chain = 1024;
constexpr int64_t kGroupArenaElems = 1LL << 30;  // shared Hd intermediates of a group: 4 GB (hi + lo)
int g_products = 3;
int g_kacc = 1;                   // in-CTA K accumulation for N <= 64 stages with enough tiles
int64_t g_s_budget = 10LL << 30;  // bytes of Hd/Hd2 intermediate per vector chunk
int64_t g_dense_chain = 256;      // chain bound of the dense-form products (K = dim)
int pick_ksplit(int64_t tiles, int64_t K, int64_t chain = 0) {
  const int64_t target = 2LL * sm_count();
  int64_t ks = 1;
  if (tiles < target) ks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(target, tiles), K / 64 / 4));
  ks = std::max<int64_t>(ks, ceil_div(K, chain > 0 ? chain : g_max_chain));
  return (int)std::min<int64_t>(ks, std::max<int64_t>(1, K / 64));
}
void read_tuning() {
  static std::once_flag once;
  std::call_once(once, [] {
    if (const char *e = getenv("VGB_TC_MAX_CHAIN")) g_max_chain = std::max(64LL, atoll(e));
    if (const char *e = getenv("VGB_TC_PRODUCTS")) g_products = atoi(e) == 4 ? 4 : 3;
    if (const char *e = getenv("VGB_TC_BK256")) g_bk256 = atoi(e) == 64 ? 64 : 32;
    if (const char *e = getenv("VGB_TC_KACC")) g_kacc = atoi(e) != 0;
    if (const char *e = getenv("VGB_TC_S_BUDGET_GB")) g_s_budget = std::max(1LL, atoll(e)) << 30;
    if (const char *e = getenv("VGB_TC_DENSE_CHAIN")) g_dense_chain = std::max(64LL, atoll(e));
    if (const char *e = getenv("VGB_TC_SLICES")) g_slices = std::max(2, std::min(5, atoi(e)));
    if (const char *e = getenv("VGB_TC_AUTOTUNE")) g_autotune = atoi(e) != 0;
  });
}

// Ozaki slice planes: nsl planes of rows x ld bf16 (plane t at t * rows * ld), zero-filled when
// (re)allocated; a buffer keeps one ld, so its K padding stays zero.
struct Planes {
  DeviceBuffer<uint16_t> b;
  int64_t rows = 0, ld = 0;
  int nsl = 0;
  void ensure(int64_t r, int64_t l, int n, cudaStream_t s) {
    const int64_t need = r * l * n;
    if (need > (int64_t)b.count || !b.get() || l != ld) {
      b.resize(need);
      VGB_CUDA(cudaMemsetAsync(b.get(), 0, need * sizeof(uint16_t), s));
    }
    rows = r;
    ld = l;
    nsl = n;
  }
  uint16_t *get() { return b.get(); }
  int64_t plane() const { return rows * ld; }
};

// The largest multiple of 64 that divides K and is at most 1024: the run of one digit scale
// and the longest exact FP32 chain of a slice pair.
int64_t slice_chain(int64_t K) {
  for (int64_t c = std::min<int64_t>(K, 1024) / 64 * 64; c >= 64; c -= 64)
    if (K % c == 0) return c;
  return 64;
}

}  // namespace

struct MixedEngine::Impl {
  int64_t vt = 0, ct = 0, naux = 0, dim = 0;
  int64_t Kc = 0, Kg = 0, Kn = 0, dimP = 0;
  SplitBuf Mcc2, G2, Bvc2, BvcT, McvT;
  // Ozaki slice planes of the FP64-equivalent products (apply_sliced), built on first use
  Planes pMcc, pG2, pBvc2, pBvcT, pMcvT, pX, pZ, pT, pA, pB;
  DeviceBuffer<double> fZ, fT, gpart;
  SplitBuf Xs, S, U, Zs;
  DeviceBuffer<float> part;
  DeviceBuffer<int> err;
  // dense form (small operators in batches): H(coef) as bf16 hi/lo rows [I][Kd], Kd = pad64(dim)
  SplitBuf Hdense, Xd;  // Xd [j][Kd]: its own buffer, the K padding of Xs must stay zero
  int64_t Kd = 0;
  bool dense_ready = false;
  Coef dense_coef;
  // operand descriptors of the grouped products, encoded once per (buffer, shape)
  // (the key holds every value the descriptors encode, so a hit is exact even when an
  // address is reused by a later allocation)
  std::map<std::tuple<const void *, const void *, int64_t, int64_t, int, int>, TcMat> maps;
  const TcMat &mat(const uint16_t *hi, const uint16_t *lo, int64_t rows, int64_t K, int box_rows, int bk) {
    const auto key = std::make_tuple((const void *)hi, (const void *)lo, rows, K, box_rows, bk);
    auto it = maps.find(key);
    if (it == maps.end()) it = maps.emplace(key, make_tc_mat(hi, lo, rows, K, K, box_rows, bk)).first;
    return it->second;
  }
};

MixedEngine::MixedEngine() : impl_(new Impl()) {}
MixedEngine::~MixedEngine() { delete impl_; }

void MixedEngine::stage(BseOperator &op, cudaStream_t s, bool split_operands) {
  Impl &m = *impl_;
  m.vt = op.vt;
  m.ct = op.ct;
  m.naux = op.naux;
  m.dim = op.dim;
  m.Kc = pad64(op.ct);
  m.Kg = pad64(op.naux * op.vt);
  m.Kn = pad64(op.naux);
  m.dimP = op.vt * m.Kc;
  const int64_t vt = m.vt, ct = m.ct, naux = m.naux, dim = m.dim;
  m.err.resize(1);
  VGB_CUDA(cudaMemsetAsync(m.err.get(), 0, sizeof(int), s));
  if (!split_operands) {  // slice-product operators build their planes on first use
    VGB_CUDA(cudaStreamSynchronize(s));
    return;
  }
  {  // Mcc2[(P, c1)][c] = Mcc[P*ct*ct + c*ct + c1]
    m.Mcc2.ensure(naux * ct, m.Kc, s);
    SplitMap sm;
    sm.rdiv = ct; sm.rs1 = ct * ct; sm.rs2 = 1; sm.cs = ct; sm.rlim = ct;
    split_f64_to_bf16(op.Mcc.get(), naux * ct, ct, sm, m.Mcc2.hi.get(), m.Mcc2.lo.get(), m.Kc, s);
  }
  {  // G2[v1][(P, v)] = Gvv[v1*naux*vt + P*vt + v]
    m.G2.ensure(vt, m.Kg, s);
    SplitMap sm;
    sm.rdiv = vt; sm.rs1 = 0; sm.rs2 = naux * vt; sm.cs = 1; sm.rlim = vt;
    split_f64_to_bf16(op.Gvv.get(), vt, naux * vt, sm, m.G2.hi.get(), m.G2.lo.get(), m.Kg, s);
  }
  {  // Bvc2[(P, v)][c] = Bvc[P*dim + v*ct + c]
    m.Bvc2.ensure(naux * vt, m.Kc, s);
    SplitMap sm;
    sm.rdiv = vt; sm.rs1 = dim; sm.rs2 = ct; sm.cs = 1; sm.rlim = vt;
    split_f64_to_bf16(op.Bvc.get(), naux * vt, ct, sm, m.Bvc2.hi.get(), m.Bvc2.lo.get(), m.Kc, s);
  }
  {  // BvcT[(v, c')][P] = Bvc[P*dim + v*ct + c'] for c' < ct
    m.BvcT.ensure(m.dimP, m.Kn, s);
    SplitMap sm;
    sm.rdiv = m.Kc; sm.rs1 = ct; sm.rs2 = 1; sm.cs = dim; sm.rlim = ct;
    split_f64_to_bf16(op.Bvc.get(), m.dimP, naux, sm, m.BvcT.hi.get(), m.BvcT.lo.get(), m.Kn, s);
  }
  {  // McvT[c1][(P, v)] = Mcv[(P*vt + v)*ct + c1]
    m.McvT.ensure(ct, m.Kg, s);
    SplitMap sm;
    sm.rdiv = ct; sm.rs1 = 0; sm.rs2 = 1; sm.cs = ct; sm.rlim = ct;
    split_f64_to_bf16(op.Mcv.get(), ct, naux * vt, sm, m.McvT.hi.get(), m.McvT.lo.get(), m.Kg, s);
  }
  VGB_CUDA(cudaStreamSynchronize(s));
}

void MixedEngine::check(cudaStream_t s) {
  int h = 0;
  VGB_CUDA(cudaMemcpyAsync(&h, impl_->err.get(), sizeof(int), cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
  if (h != 0) {
    VGB_CUDA(cudaMemsetAsync(impl_->err.get(), 0, sizeof(int), s));
    fail(BSE_ERR_TIMEOUT, "tensor-core GEMM: a bounded pipeline wait gave up (code " +
                              std::to_string(h) + ")");
  }
}

void MixedEngine::apply(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k,
                        double *Y, int64_t ldy, bool accumulate, cudaStream_t s) {
  Impl &m = *impl_;
  read_tuning();
  const int64_t vt = m.vt, ct = m.ct, naux = m.naux;
  int *err = m.err.get();
  bool acc = accumulate;
  // X -> Xs[(j, v)][c]
  op.timer.begin(STAGE_TC_SPLIT, s);
  m.Xs.ensure(k * vt, m.Kc, s);
  {
    SplitMap sm;
    sm.rdiv = vt; sm.rs1 = ldx; sm.rs2 = ct; sm.cs = 1; sm.rlim = vt;
    split_f64_to_bf16(X, k * vt, ct, sm, m.Xs.hi.get(), m.Xs.lo.get(), m.Kc, s);
  }
  op.timer.end(STAGE_TC_SPLIT, s);

  if (c.cx != 0) {
    op.timer.begin(STAGE_TC_HX, s);
    // Z[P][j] = sum_I' Bvc2[P][I'] Xs[j][I']
    const int bn = pick_bn(k);
    TcMat A = make_tc_mat(m.Bvc2.hi.get(), m.Bvc2.lo.get(), naux, m.dimP, m.dimP, 128, bk_for(bn));
    TcMat B = make_tc_mat(m.Xs.hi.get(), m.Xs.lo.get(), k, m.dimP, m.dimP, bn, bk_for(bn));
    TcShape sh;
    sh.M = naux; sh.N = k; sh.K = m.dimP; sh.products = g_products;
    sh.ksplit = pick_ksplit(ceil_div(naux, 128) * ceil_div(k, bn), m.dimP);
    m.part.resize((size_t)sh.ksplit * naux * k);
    // partials column-major [split][j][P]: the epilogue lanes (rows P) store contiguously
    TcEpilogue e;
    e.kind = TcEpilogue::STORE_F32;
    e.rd = naux; e.ro2 = 1; e.rlim = naux;
    e.cd = k; e.co2 = naux; e.clim = k;
    e.so = naux * k;
    e.out_f32 = m.part.get();
    const int ks = tc_gemm(A, B, sh, e, bn, err, s);
    m.Zs.ensure(k, m.Kn, s);
    // reduced as the transposed (j x P) problem, so that reads and writes run along P
    TcEpilogue r;
    r.kind = TcEpilogue::SPLIT_BF16;
    r.rd = k; r.ro2 = m.Kn; r.rlim = k;
    r.cd = naux; r.co2 = 1; r.clim = naux;
    r.out_hi = m.Zs.hi.get(); r.out_lo = m.Zs.lo.get();
    reduce_partials(m.part.get(), k, naux, ks, r, s);
    // Y(I, j) (+)= cx sum_P BvcT[I'][P] Zs[j][P]
    TcMat A2 = make_tc_mat(m.BvcT.hi.get(), m.BvcT.lo.get(), m.dimP, m.Kn, m.Kn, 128, bk_for(bn));
    TcMat B2 = make_tc_mat(m.Zs.hi.get(), m.Zs.lo.get(), k, m.Kn, m.Kn, bn, bk_for(bn));
    TcShape sh2;
    sh2.M = m.dimP; sh2.N = k; sh2.K = m.Kn; sh2.products = g_products;
    sh2.ksplit = 1;
    TcEpilogue e2;
    e2.kind = TcEpilogue::AXPBY_F64;
    e2.rd = m.Kc; e2.ro1 = ct; e2.ro2 = 1; e2.rlim = ct;
    e2.cd = k; e2.co2 = ldy; e2.clim = k;
    e2.out_f64 = Y; e2.alpha = c.cx; e2.beta = acc ? 1.0 : 0.0;
    tc_gemm(A2, B2, sh2, e2, bn, err, s);
    acc = true;
    op.timer.end(STAGE_TC_HX, s);
  }

  if (c.cd != 0 || c.cd2 != 0) {
    const bool hd = c.cd != 0;
    const double alpha = hd ? -(double)c.cd : -(double)c.cd2;
    op.timer.begin(hd ? STAGE_TC_HD : STAGE_TC_HD2, s);
    // vectors per chunk so that the intermediate stays within the budget
    const int64_t per_vec = (hd ? ct : vt) * m.Kg * 4;
    int64_t jmax = std::max<int64_t>(1, std::min<int64_t>(k, g_s_budget / per_vec));
    // Hd stage 2 runs one tile per CTA (in-CTA K accumulation): at most one wave of tiles
    if (hd && g_kacc) jmax = std::max<int64_t>(1, std::min<int64_t>(jmax, sm_count() * 128 / ct));
    const int64_t jc = ceil_div(k, ceil_div(k, jmax));  // equal chunks: no small remainder pass
    SplitBuf &T = hd ? m.S : m.U;
    T.ensure(jc * (hd ? ct : vt), m.Kg, s);
    for (int64_t j0 = 0; j0 < k; j0 += jc) {
      const int64_t kc = std::min(jc, k - j0);
      const uint16_t *xh = m.Xs.hi.get() + j0 * vt * m.Kc, *xl = m.Xs.lo.get() + j0 * vt * m.Kc;
      if (hd) {
        // stage 1: S[(j, c1)][(P, v)] = sum_c Xs[(j, v)][c] Mcc2[(P, c1)][c]: one GEMM whose N
        // runs over (P, c1), so N tiles pack across aux indices when ct is not a tile multiple
        const int bn = pick_bn(naux * ct);
        TcMat Xa = make_tc_mat(xh, xl, kc * vt, m.Kc, m.Kc, 128, bk_for(bn));
        TcMat Bm = make_tc_mat(m.Mcc2.hi.get(), m.Mcc2.lo.get(), naux * ct, m.Kc, m.Kc, bn, bk_for(bn));
        TcShape sh;
        sh.M = kc * vt; sh.N = naux * ct; sh.K = m.Kc; sh.products = g_products;
        TcEpilogue e;
        e.kind = TcEpilogue::SPLIT_BF16;
        e.rd = vt; e.ro1 = ct * m.Kg; e.ro2 = 1; e.rlim = vt;
        e.cd = ct; e.co1 = vt; e.co2 = m.Kg; e.clim = ct;
        e.out_hi = T.hi.get(); e.out_lo = T.lo.get();
        tc_gemm(Xa, Bm, sh, e, bn, err, s);
        op.timer.end(STAGE_TC_HD, s);
        op.timer.begin(STAGE_TC_HD_B, s);
        // stage 2: Y_j(c1, v1) += alpha sum_{(P,v)} S[(j, c1)][(P,v)] G2[v1][(P,v)]
        const int bn2 = pick_bn(vt);
        TcMat As = make_tc_mat(T.hi.get(), T.lo.get(), kc * ct, m.Kg, m.Kg, 128, bk_for(bn2));
        TcMat Bg = make_tc_mat(m.G2.hi.get(), m.G2.lo.get(), vt, m.Kg, m.Kg, bn2, bk_for(bn2));
        TcShape s2;
        s2.M = kc * ct; s2.N = vt; s2.K = m.Kg; s2.products = g_products;
        s2.ksplit = pick_ksplit(ceil_div(kc * ct, 128) * ceil_div(vt, bn2), m.Kg);
        const int64_t tiles2 = ceil_div(s2.M, 128) * ceil_div(s2.N, bn2);
        if (g_kacc && bn2 <= 64 && s2.ksplit > 1 && tiles2 * 2 >= sm_count()) {
          // enough tiles to keep the SMs busy: each CTA sums the K splits of its tile in FP64
          // and writes Y directly (no partials, no reduction launch; same numbers)
          s2.kacc = true;
          TcEpilogue r;
          r.kind = TcEpilogue::AXPBY_F64;
          r.rd = ct; r.ro1 = ldy; r.ro2 = 1; r.rlim = ct;
          r.cd = vt; r.co2 = ct; r.clim = vt;
          r.out_f64 = Y + j0 * ldy; r.alpha = alpha; r.beta = acc ? 1.0 : 0.0;
          tc_gemm(As, Bg, s2, r, bn2, err, s);
          op.timer.end(STAGE_TC_HD_B, s);
          if (j0 + jc < k) op.timer.begin(STAGE_TC_HD, s);
          continue;
        }
        m.part.resize((size_t)s2.ksplit * s2.M * s2.N);
        // partials column-major [split][v1][(j, c1)] (coalesced epilogue stores)
        TcEpilogue p;
        p.kind = TcEpilogue::STORE_F32;
        p.rd = s2.M; p.ro2 = 1; p.rlim = s2.M;
        p.cd = s2.N; p.co2 = s2.M; p.clim = s2.N;
        p.so = s2.M * s2.N;
        p.out_f32 = m.part.get();
        const int ks = tc_gemm(As, Bg, s2, p, bn2, err, s);
        // reduced as the transposed problem: rows v1, columns (j, c1)
        TcEpilogue r;
        r.kind = TcEpilogue::AXPBY_F64;
        r.rd = vt; r.ro2 = ct; r.rlim = vt;
        r.cd = ct; r.co1 = ldy; r.co2 = 1; r.clim = ct;
        r.out_f64 = Y + j0 * ldy; r.alpha = alpha; r.beta = acc ? 1.0 : 0.0;
        reduce_partials(m.part.get(), s2.N, s2.M, ks, r, s);
        op.timer.end(STAGE_TC_HD_B, s);
        if (j0 + jc < k) op.timer.begin(STAGE_TC_HD, s);
      } else {
        // stage 1: U[(j, v1)][(P, v)] = sum_c Xs[(j, v)][c] Bvc2[(P, v1)][c]
        const int bn = pick_bn(naux * vt);
        TcMat Xa = make_tc_mat(xh, xl, kc * vt, m.Kc, m.Kc, 128, bk_for(bn));
        TcMat Bm = make_tc_mat(m.Bvc2.hi.get(), m.Bvc2.lo.get(), naux * vt, m.Kc, m.Kc, bn, bk_for(bn));
        TcShape sh;
        sh.M = kc * vt; sh.N = naux * vt; sh.K = m.Kc; sh.products = g_products;
        TcEpilogue e;
        e.kind = TcEpilogue::SPLIT_BF16;
        e.rd = vt; e.ro1 = vt * m.Kg; e.ro2 = 1; e.rlim = vt;
        e.cd = vt; e.co1 = vt; e.co2 = m.Kg; e.clim = vt;
        e.out_hi = T.hi.get(); e.out_lo = T.lo.get();
        tc_gemm(Xa, Bm, sh, e, bn, err, s);
        op.timer.end(STAGE_TC_HD2, s);
        op.timer.begin(STAGE_TC_HD2_B, s);
        // stage 2: Y_j(c1, v1) += alpha sum_{(P,v)} McvT[c1][(P,v)] U[(j, v1)][(P,v)]
        const int bn2 = pick_bn(kc * vt);
        TcMat Am = make_tc_mat(m.McvT.hi.get(), m.McvT.lo.get(), ct, m.Kg, m.Kg, 128, bk_for(bn2));
        TcMat Bu = make_tc_mat(T.hi.get(), T.lo.get(), kc * vt, m.Kg, m.Kg, bn2, bk_for(bn2));
        TcShape s2;
        s2.M = ct; s2.N = kc * vt; s2.K = m.Kg; s2.products = g_products;
        s2.ksplit = pick_ksplit(ceil_div(ct, 128) * ceil_div(kc * vt, bn2), m.Kg);
        m.part.resize((size_t)s2.ksplit * s2.M * s2.N);
        // partials column-major [split][(j, v1)][c1] (coalesced epilogue stores)
        TcEpilogue p;
        p.kind = TcEpilogue::STORE_F32;
        p.rd = s2.M; p.ro2 = 1; p.rlim = s2.M;
        p.cd = s2.N; p.co2 = s2.M; p.clim = s2.N;
        p.so = s2.M * s2.N;
        p.out_f32 = m.part.get();
        const int ks = tc_gemm(Am, Bu, s2, p, bn2, err, s);
        // reduced as the transposed problem: rows (j, v1), columns c1
        TcEpilogue r;
        r.kind = TcEpilogue::AXPBY_F64;
        r.rd = vt; r.ro1 = ldy; r.ro2 = ct; r.rlim = vt;
        r.cd = ct; r.co2 = 1; r.clim = ct;
        r.out_f64 = Y + j0 * ldy; r.alpha = alpha; r.beta = acc ? 1.0 : 0.0;
        reduce_partials(m.part.get(), s2.N, s2.M, ks, r, s);
        op.timer.end(STAGE_TC_HD2_B, s);
        if (j0 + jc < k) op.timer.begin(STAGE_TC_HD2, s);
      }
    }
    acc = true;
  }
  if (!acc) {
    VGB_CUDA(cudaMemset2DAsync(Y, ldy * sizeof(double), 0, op.dim * sizeof(double), k, s));
  }
}

namespace {

// All pairs (a, b) of digit planes with a + b < nsl: the products kept by the Ozaki scheme (the
// dropped levels are below 2^(-7 nsl) of the row and column scales).
void set_pairs(TcShape &sh, int nsl) { sh.nslices = nsl; }

// One slice-mode product: C (M x N) = sum over pairs of A planes (rows a_plane apart, K-major,
// row stride K) times B planes, through the final FP64 epilogue fe.  When the tiles alone do
// not fill the SMs, the K splits of a tile are shared by several CTAs whose FP64 partials are
// added by a reduction launch.
// chain: the run of one digit scale along K in both operands (a multiple of 64 dividing K).
void sliced_gemm(const TcMat &A, int64_t a_plane, const TcMat &B, int64_t b_plane, int64_t M, int64_t N,
                 int64_t K, int64_t chain, int nsl, int bn, const TcEpilogue &fe, DeviceBuffer<double> &gpart,
                 int *err, cudaStream_t s) {
  TcShape sh;
  sh.M = M; sh.N = N; sh.K = K;
  set_pairs(sh, nsl);
  sh.a_plane = a_plane;
  sh.b_plane = b_plane;
  sh.chain = chain;
  sh.kacc = true;
  const int64_t tiles = ceil_div(M, 128) * ceil_div(N, bn);
  const int64_t runs = ceil_div(K / 64, sh.chain / 64);
  int groups = 1;  // float-pair outputs are written by the CTA that owns the tile
  for (int g = 2; g <= 64 && fe.kind == TcEpilogue::AXPBY_F64; ++g)
    if (runs % g == 0 && tiles * g <= sm_count()) groups = g;
  if (groups == 1) {
    tc_gemm(A, B, sh, fe, bn, err, s);
    return;
  }
  sh.kgroups = groups;
  gpart.resize((size_t)groups * M * N);
  TcEpilogue pe;  // FP64 partials, column-major per group
  pe.kind = TcEpilogue::AXPBY_F64;
  pe.rd = M; pe.ro2 = 1; pe.rlim = M;
  pe.cd = N; pe.co2 = M; pe.clim = N;
  pe.so = M * N;
  pe.out_f64 = gpart.get();
  pe.alpha = 1.0; pe.beta = 0.0;
  tc_gemm(A, B, sh, pe, bn, err, s);
  reduce_f64_groups(gpart.get(), M, N, groups, fe, s);
}

}  // namespace

void MixedEngine::apply_sliced(BseOperator &op, const Coef &c, const double *X, int64_t ldx, int64_t k,
                               double *Y, int64_t ldy, bool accumulate, cudaStream_t s) {
  Impl &m = *impl_;
  read_tuning();
  const int nsl = g_slices;
  const int64_t vt = m.vt, ct = m.ct, naux = m.naux, dim = m.dim;
  const int64_t chc = slice_chain(m.Kc), chg = slice_chain(m.Kg), chn = slice_chain(m.Kn);
  int *err = m.err.get();
  bool acc = accumulate;
  const bool hx = c.cx != 0, hd = c.cd != 0, hd2 = c.cd2 != 0;
  if (!hx && !hd && !hd2) {
    if (!acc) VGB_CUDA(cudaMemset2DAsync(Y, ldy * sizeof(double), 0, dim * sizeof(double), k, s));
    return;
  }
  // operator planes, built once per operand from the FP64 staged blocks
  op.timer.begin(STAGE_TC_SPLIT, s);
  auto build = [&](Planes &P, const double *src, int64_t rows, int64_t cols, int64_t ld, const SplitMap &sm,
                   int64_t chunk) {
    if (P.nsl == nsl && P.rows == rows && P.ld == ld) return;
    P.ensure(rows, ld, nsl, s);
    slice_f64(src, rows, cols, sm, nsl, chunk, P.get(), ld, P.plane(), s);
  };
  if (hd) {
    SplitMap a;  // Mcc planes [(P, c1)][c]
    a.rdiv = ct; a.rs1 = ct * ct; a.rs2 = 1; a.cs = ct; a.rlim = ct;
    build(m.pMcc, op.Mcc.get(), naux * ct, ct, m.Kc, a, chc);
    SplitMap g;  // G planes [v1][(P, v)]
    g.rdiv = vt; g.rs1 = 0; g.rs2 = naux * vt; g.cs = 1; g.rlim = vt;
    build(m.pG2, op.Gvv.get(), vt, naux * vt, m.Kg, g, chg);
  }
  if (hx || hd2) {
    SplitMap b;  // Bvc planes [(P, v)][c] (== [P][dimP] for Hx)
    b.rdiv = vt; b.rs1 = dim; b.rs2 = ct; b.cs = 1; b.rlim = vt;
    build(m.pBvc2, op.Bvc.get(), naux * vt, ct, m.Kc, b, chc);
  }
  if (hx) {
    SplitMap t;  // BvcT planes [(v, c')][P]
    t.rdiv = m.Kc; t.rs1 = ct; t.rs2 = 1; t.cs = dim; t.rlim = ct;
    build(m.pBvcT, op.Bvc.get(), m.dimP, naux, m.Kn, t, chn);
  }
  if (hd2) {
    SplitMap t;  // screened Mcv planes [c1][(P, v)]
    t.rdiv = ct; t.rs1 = 0; t.rs2 = 1; t.cs = ct; t.rlim = ct;
    build(m.pMcvT, op.Mcv.get(), ct, naux * vt, m.Kg, t, chg);
  }
  {  // X planes [(j, v)][c] (== [j][dimP] for Hx)
    m.pX.ensure(k * vt, m.Kc, nsl, s);
    SplitMap x;
    x.rdiv = vt; x.rs1 = ldx; x.rs2 = ct; x.cs = 1; x.rlim = vt;
    slice_f64(X, k * vt, ct, x, nsl, chc, m.pX.get(), m.Kc, m.pX.plane(), s);
  }
  op.timer.end(STAGE_TC_SPLIT, s);
  const uint16_t *px = m.pX.get();
  const int64_t xrows = nsl * k * vt;  // rows of the X planes as one matrix ([(j, v)] view)

  if (hx) {
    op.timer.begin(STAGE_TC_HX, s);
    const TcMat &Ab = m.mat(m.pBvc2.get(), m.pBvc2.get(), nsl * naux, m.dimP, 128, 64);
    m.fZ.resize(k * m.Kn);
    for (int64_t j0 = 0; j0 < k; j0 += 64) {  // Z[j][P] = sum_I' Bvc[P][I'] X_j[I']
      const int64_t kc = std::min<int64_t>(64, k - j0);
      const int bn = kc > 32 ? 64 : 32;
      TcMat Bx = make_tc_mat(px + j0 * m.dimP, px + j0 * m.dimP, nsl * k - j0, m.dimP, m.dimP, bn, 64);
      TcEpilogue e;
      e.kind = TcEpilogue::AXPBY_F64;
      e.rd = naux; e.ro2 = 1; e.rlim = naux;
      e.cd = kc; e.co2 = m.Kn; e.clim = kc;
      e.out_f64 = m.fZ.get() + j0 * m.Kn; e.alpha = 1.0; e.beta = 0.0;
      sliced_gemm(Ab, naux, Bx, k, naux, kc, m.dimP, chc, nsl, bn, e, m.gpart, err, s);
    }
    m.pZ.ensure(k, m.Kn, nsl, s);
    SplitMap z;
    z.rdiv = 1; z.rs1 = m.Kn; z.rs2 = 0; z.cs = 1; z.rlim = 1;
    slice_f64(m.fZ.get(), k, naux, z, nsl, chn, m.pZ.get(), m.Kn, m.pZ.plane(), s);
    const TcMat &At = m.mat(m.pBvcT.get(), m.pBvcT.get(), nsl * m.dimP, m.Kn, 128, 64);
    for (int64_t j0 = 0; j0 < k; j0 += 64) {  // Y(I, j) (+)= cx sum_P BvcT[I'][P] Z[j][P]
      const int64_t kc = std::min<int64_t>(64, k - j0);
      const int bn = kc > 32 ? 64 : 32;
      TcMat Bz = make_tc_mat(m.pZ.get() + j0 * m.Kn, m.pZ.get() + j0 * m.Kn, nsl * k - j0, m.Kn, m.Kn, bn, 64);
      TcEpilogue e;
      e.kind = TcEpilogue::AXPBY_F64;
      e.rd = m.Kc; e.ro1 = ct; e.ro2 = 1; e.rlim = ct;
      e.cd = kc; e.co2 = ldy; e.clim = kc;
      e.out_f64 = Y + j0 * ldy; e.alpha = c.cx; e.beta = acc ? 1.0 : 0.0;
      sliced_gemm(At, m.dimP, Bz, k, m.dimP, kc, m.Kn, chn, nsl, bn, e, m.gpart, err, s);
    }
    acc = true;
    op.timer.end(STAGE_TC_HX, s);
  }

  for (int pass = 0; pass < 2; ++pass) {
    const bool is_hd = pass == 0;
    if (is_hd ? !hd : !hd2) continue;
    const double alpha = is_hd ? -(double)c.cd : -(double)c.cd2;
    const int64_t rows_per_vec = is_hd ? ct : vt;  // rows of the intermediate per vector
    const int64_t per_vec = rows_per_vec * m.Kg * (8 + 2 * nsl);
    const int64_t jmax = std::max<int64_t>(1, std::min<int64_t>(k, g_s_budget / per_vec));
    const int64_t jc = ceil_div(k, ceil_div(k, jmax));
    m.fT.resize(jc * rows_per_vec * m.Kg);
    m.pT.ensure(jc * rows_per_vec, m.Kg, nsl, s);
    const int64_t tplane = m.pT.plane() / m.Kg;  // rows per plane of the intermediate
    for (int64_t j0 = 0; j0 < k; j0 += jc) {
      const int64_t kc = std::min(jc, k - j0);
      op.timer.begin(is_hd ? STAGE_TC_HD : STAGE_TC_HD2, s);
      TcMat Ax = make_tc_mat(px + j0 * vt * m.Kc, px + j0 * vt * m.Kc, xrows - j0 * vt, m.Kc, m.Kc, 128, 64);
      TcEpilogue e;  // stage 1 into the intermediate [(j, row)][(P, v)], FP64 sums as float pairs
      e.kind = TcEpilogue::PAIR_F32;
      e.rd = vt; e.ro2 = 1; e.rlim = vt;
      e.ro1 = rows_per_vec * m.Kg;
      e.cd = is_hd ? ct : vt; e.co1 = vt; e.co2 = m.Kg; e.clim = e.cd;
      e.out_f32 = reinterpret_cast<float *>(m.fT.get());
      if (is_hd) {  // S[(j, c1)][(P, v)] = sum_c X_j(v, c) M(c1, c, P)
        const TcMat &Bm = m.mat(m.pMcc.get(), m.pMcc.get(), nsl * naux * ct, m.Kc, 64, 64);
        sliced_gemm(Ax, k * vt, Bm, naux * ct, kc * vt, naux * ct, m.Kc, chc, nsl, 64, e, m.gpart, err, s);
      } else {      // U[(j, v1)][(P, v)] = sum_c X_j(v, c) M(v1, c, P)
        const TcMat &Bm = m.mat(m.pBvc2.get(), m.pBvc2.get(), nsl * naux * vt, m.Kc, 64, 64);
        sliced_gemm(Ax, k * vt, Bm, naux * vt, kc * vt, naux * vt, m.Kc, chc, nsl, 64, e, m.gpart, err, s);
      }
      op.timer.end(is_hd ? STAGE_TC_HD : STAGE_TC_HD2, s);
      op.timer.begin(STAGE_TC_SPLIT, s);
      SplitMap t;
      t.rdiv = 1; t.rs1 = m.Kg; t.rs2 = 0; t.cs = 1; t.rlim = 1;
      slice_pairs(reinterpret_cast<const float *>(m.fT.get()), kc * rows_per_vec, naux * vt, t, nsl, chg,
                  m.pT.get(), m.Kg, m.pT.plane(), s);
      op.timer.end(STAGE_TC_SPLIT, s);
      op.timer.begin(is_hd ? STAGE_TC_HD_B : STAGE_TC_HD2_B, s);
      if (is_hd) {  // Y_j(c1, v1) += alpha sum_{(P,v)} S[(j, c1)][(P,v)] G[v1][(P,v)]
        TcMat As = make_tc_mat(m.pT.get(), m.pT.get(), nsl * tplane, m.Kg, m.Kg, 128, 64);
        for (int64_t n0 = 0; n0 < vt; n0 += 64) {
          const int64_t nn = std::min<int64_t>(64, vt - n0);
          const int bn = nn > 32 ? 64 : 32;
          TcMat Bg = make_tc_mat(m.pG2.get() + n0 * m.Kg, m.pG2.get() + n0 * m.Kg, nsl * vt - n0, m.Kg, m.Kg,
                                 bn, 64);
          TcEpilogue r;
          r.kind = TcEpilogue::AXPBY_F64;
          r.rd = ct; r.ro1 = ldy; r.ro2 = 1; r.rlim = ct;
          r.cd = nn; r.co2 = ct; r.clim = nn;
          r.out_f64 = Y + j0 * ldy + n0 * ct; r.alpha = alpha; r.beta = acc ? 1.0 : 0.0;
          sliced_gemm(As, tplane, Bg, vt, kc * ct, nn, m.Kg, chg, nsl, bn, r, m.gpart, err, s);
        }
      } else {      // Y_j(c1, v1) += alpha sum_{(P,v)} McvT[c1][(P,v)] U[(j, v1)][(P,v)]
        const TcMat &Am = m.mat(m.pMcvT.get(), m.pMcvT.get(), nsl * ct, m.Kg, 128, 64);
        // column blocks of whole vectors (vt <= 64) or of 64 v1 of one vector
        const int64_t nv = vt <= 64 ? std::max<int64_t>(1, 64 / vt) : 1;
        for (int64_t j = 0; j < kc; j += nv) {
          const int64_t vj = std::min(nv, kc - j);
          for (int64_t v0 = 0; v0 < vt; v0 += 64) {
            const int64_t nn = vt <= 64 ? vj * vt : std::min<int64_t>(64, vt - v0);
            const int bn = nn > 32 ? 64 : 32;
            const int64_t r0 = j * vt + v0;  // first intermediate row of the block
            TcMat Bu = make_tc_mat(m.pT.get() + r0 * m.Kg, m.pT.get() + r0 * m.Kg, nsl * tplane - r0, m.Kg, m.Kg,
                                   bn, 64);
            TcEpilogue r;
            r.kind = TcEpilogue::AXPBY_F64;
            r.rd = ct; r.ro2 = 1; r.rlim = ct;
            r.cd = vt <= 64 ? vt : nn; r.co1 = ldy; r.co2 = ct; r.clim = r.cd;
            r.out_f64 = Y + (j0 + j) * ldy + v0 * ct; r.alpha = alpha; r.beta = acc ? 1.0 : 0.0;
            sliced_gemm(Am, ct, Bu, tplane, ct, nn, m.Kg, chg, nsl, bn, r, m.gpart, err, s);
            if (vt <= 64) break;
          }
        }
      }
      op.timer.end(is_hd ? STAGE_TC_HD_B : STAGE_TC_HD2_B, s);
    }
    acc = true;
  }
}

void MixedEngine::gemm_sliced(BseOperator &op, const double *A, const SplitMap &am, int64_t M, const double *B,
                              const SplitMap &bm, int64_t N, int64_t K, bool mcc_as_b, const TcEpilogue &e,
                              cudaStream_t s) {
  Impl &m = *impl_;
  read_tuning();
  if (M <= 0 || N <= 0 || K <= 0) return;
  VGB_REQUIRE(e.kind == TcEpilogue::AXPBY_F64, "gemm_sliced: FP64 epilogue expected");
  const int nsl = g_slices;
  const int64_t Kp = pad64(K), chain = slice_chain(Kp);
  const uint16_t *bp;
  int64_t bplane;
  if (mcc_as_b) {
    VGB_REQUIRE(K == m.ct && N == m.naux * m.ct, "gemm_sliced: cc block shape");
    if (!(m.pMcc.nsl == nsl && m.pMcc.rows == m.naux * m.ct && m.pMcc.ld == m.Kc)) {
      SplitMap a;  // Mcc planes [(P, c1)][c]
      a.rdiv = m.ct; a.rs1 = m.ct * m.ct; a.rs2 = 1; a.cs = m.ct; a.rlim = m.ct;
      m.pMcc.ensure(m.naux * m.ct, m.Kc, nsl, s);
      slice_f64(op.Mcc.get(), m.naux * m.ct, m.ct, a, nsl, chain, m.pMcc.get(), m.Kc, m.pMcc.plane(), s);
    }
    bp = m.pMcc.get();
    bplane = m.naux * m.ct;
  } else {
    m.pB.ensure(N, Kp, nsl, s);
    slice_f64(B, N, K, bm, nsl, chain, m.pB.get(), Kp, m.pB.plane(), s);
    bp = m.pB.get();
    bplane = N;
  }
  m.pA.ensure(M, Kp, nsl, s);
  slice_f64(A, M, K, am, nsl, chain, m.pA.get(), Kp, m.pA.plane(), s);
  const int bn = N > 32 ? 64 : 32;
  TcMat Am = make_tc_mat(m.pA.get(), m.pA.get(), nsl * M, Kp, Kp, 128, 64);
  TcMat Bm = make_tc_mat(bp, bp, nsl * bplane, Kp, Kp, bn, 64);
  sliced_gemm(Am, M, Bm, bplane, M, N, Kp, chain, nsl, bn, e, m.gpart, m.err.get(), s);
}

namespace {

// Grouped launches of one stage: problems bucketed by tile shape (bn, K box).
struct GemmBuckets {
  std::map<int, std::vector<const TcProblem *>> by_shape;
  std::map<int, std::vector<size_t>> owner;
  void add(const TcProblem *p, int bn, size_t item) {
    const int key = bn * 1000 + p->A.bk;
    by_shape[key].push_back(p);
    owner[key].push_back(item);
  }
  // launches every bucket; ks[item] = K splits of that item's problem
  void run(int *err, cudaStream_t s, std::vector<int> &ks, int group_max = 32, int nstreams = 1) {
    for (auto &kv : by_shape) {
      std::vector<int> k(kv.second.size(), 0);
      tc_gemm_grouped(kv.second, kv.first / 1000, err, s, k.data(), group_max, nstreams);
      const auto &own = owner[kv.first];
      for (size_t i = 0; i < own.size(); ++i) ks[own[i]] = k[i];
    }
  }
};

}  // namespace

namespace {

// Bc[(c1, c)][P] = split(M(c1, c, P)) from Mcc[P][c][c1] (= the [P][q] matrix, q = c ct + c1):
// a 32 x 32 tiled transpose through shared memory, so that reads run along q and writes
// along P.
__global__ void transpose_split_cc_kernel(const double *__restrict__ Mcc, int64_t naux, int64_t ct,
                                          uint16_t *__restrict__ hi, uint16_t *__restrict__ lo, int64_t ldo) {
  __shared__ double tile[32][33];
  const int64_t q0 = (int64_t)blockIdx.x * 32, p0 = (int64_t)blockIdx.y * 32;
  const int64_t nq = ct * ct;
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t P = p0 + r, q = q0 + threadIdx.x;
    tile[r][threadIdx.x] = (P < naux && q < nq) ? Mcc[P * nq + q] : 0.0;
  }
  __syncthreads();
  for (int r = threadIdx.y; r < 32; r += blockDim.y) {
    const int64_t q = q0 + r, P = p0 + threadIdx.x;
    if (q >= nq || P >= naux) continue;
    const int64_t c = q / ct, c1 = q % ct;
    const double v = tile[threadIdx.x][r];
    const __nv_bfloat16 h = __double2bfloat16(v);
    const __nv_bfloat16 l = __double2bfloat16(v - (double)__bfloat162float(h));
    const int64_t off = (c1 * ct + c) * ldo + P;
    hi[off] = __bfloat16_as_ushort(h);
    lo[off] = __bfloat16_as_ushort(l);
  }
}

// H = (H + H^T) / 2 off the diagonal: the two halves of the split products round differently
// (A_hi B_lo against A_lo B_hi), and a nonsymmetric operator leaves a floor on the Davidson
// residual.
// The diagonal is zeroed: the products add the exact FP64 diagonal of the whole operator
// beside the dense part, so the largest entries are not rounded to bf16 hi/lo.
__global__ void symmetrize_kernel(double *H, int64_t n) {
  const int64_t total = n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total; t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t i = t / n, j = t % n;
    if (j < i) continue;
    if (j == i) {
      H[i * n + i] = 0.0;
      continue;
    }
    const double a = 0.5 * (H[i * n + j] + H[j * n + i]);
    H[i * n + j] = a;
    H[j * n + i] = a;
  }
}

// the dense form holds cx Hx - cd Hd; Hqp is applied in FP64 beside it
bool same_coef(const Coef &a, const Coef &b) {
  return a.cx == b.cx && a.cd == b.cd && a.cd2 == b.cd2;
}

}  // namespace

bool MixedEngine::dense_ready(const Coef &c) const {
  return impl_->dense_ready && same_coef(impl_->dense_coef, c);
}

void MixedEngine::build_dense_grouped(const std::vector<BseOperator *> &ops, const Coef &c, cudaStream_t s) {
  read_tuning();
  VGB_REQUIRE(c.cd2 == 0, "dense form: TDA operators only");
  std::vector<BseOperator *> todo;
  for (BseOperator *op : ops) {
    VGB_REQUIRE(op->mixed && op->hqp_diagonal, "dense form: mixed-precision operators with a diagonal Hqp");
    if (!op->mixed->dense_ready(c)) todo.push_back(op);
  }
  int *err = todo.empty() ? nullptr : todo[0]->mixed->impl_->err.get();
  // slices of operators whose FP64 temporaries (H and the two K = Naux splits) fit 8 GB
  const int64_t budget = 8LL << 30;
  if (!todo.empty() && alloc_stream()) {
    // grow the stream-ordered pool once: the kept dense forms plus one slice of temporaries
    int64_t bytes = budget + (1LL << 20);
    for (BseOperator *op : todo) bytes += op->dim * pad64(op->dim) * 4 + 4096;
    void *p = nullptr;
    if (cudaMallocAsync(&p, (size_t)bytes, s) == cudaSuccess) VGB_CUDA(cudaFreeAsync(p, s));
    else cudaGetLastError();  // no headroom for one block: allocated piece by piece
  }
  size_t a = 0;
  while (a < todo.size()) {
    size_t b = a;
    int64_t used = 0;
    std::vector<int64_t> hoff, aoff, boff;
    while (b < todo.size()) {
      const BseOperator &op = *todo[b];
      const Impl &m = *op.mixed->impl_;
      const int64_t h = op.dim * op.dim * 8, av = op.vt * op.vt * m.Kn * 4, bc = op.ct * op.ct * m.Kn * 4;
      if (b > a && used + h + av + bc > budget) break;
      used += h + av + bc;
      ++b;
    }
    // temporaries of the slice
    int64_t nh = 0, na = 0, nb = 0;
    for (size_t t = a; t < b; ++t) {
      const BseOperator &op = *todo[t];
      const Impl &m = *op.mixed->impl_;
      hoff.push_back(nh); aoff.push_back(na); boff.push_back(nb);
      nh += op.dim * op.dim;
      na += pad64(op.vt * op.vt) * m.Kn;
      nb += pad64(op.ct * op.ct) * m.Kn;
    }
    DeviceBuffer<double> H(nh);
    SplitBuf Av, Bc;
    Av.ensure(1, na, s);  // zero-filled: K padding columns multiply as zeros
    Bc.ensure(1, nb, s);
    std::vector<SplitJob> sj;
    for (size_t t = a; t < b; ++t) {
      const BseOperator &op = *todo[t];
      const Impl &m = *op.mixed->impl_;
      const size_t q = t - a;
      // Av[(v1, v)][P] = w_P M(v1, v, P) = Gvv[v1][P][v]
      SplitJob j1;
      j1.x = op.Gvv.get(); j1.rows = op.vt * op.vt; j1.cols = op.naux;
      j1.map.rdiv = op.vt; j1.map.rs1 = op.naux * op.vt; j1.map.rs2 = 1; j1.map.cs = op.vt; j1.map.rlim = op.vt;
      j1.hi = Av.hi.get() + aoff[q]; j1.lo = Av.lo.get() + aoff[q]; j1.ldo = m.Kn;
      sj.push_back(j1);
      // Bc[(c1, c)][P] = M(c1, c, P) = Mcc[P][c][c1]: a transpose, done through shared memory
      const dim3 grid((unsigned)ceil_div(op.ct * op.ct, 32), (unsigned)ceil_div(op.naux, 32));
      transpose_split_cc_kernel<<<grid, dim3(32, 8), 0, s>>>(op.Mcc.get(), op.naux, op.ct, Bc.hi.get() + boff[q],
                                                            Bc.lo.get() + boff[q], m.Kn);
      VGB_LAUNCH_CHECK();
    }
    split_grouped(sj, s);
    std::vector<int> ks(b - a, 0);
    // Hx: H[(v, c)][(v', c')] = cx sum_P B(vc, P) B(v'c', P)  (rows/cols in the padded v*Kc + c index)
    if (c.cx != 0) {
      std::vector<TcProblem> px(b - a);
      GemmBuckets bx;
      for (size_t t = a; t < b; ++t) {
        const BseOperator &op = *todo[t];
        Impl &m = *op.mixed->impl_;
        const size_t q = t - a;
        const int bn = pick_bn(m.dimP);
        TcProblem &pr = px[q];
        pr.A = m.mat(m.BvcT.hi.get(), m.BvcT.lo.get(), m.dimP, m.Kn, 128, bk_for(bn));
        pr.B = m.mat(m.BvcT.hi.get(), m.BvcT.lo.get(), m.dimP, m.Kn, bn, bk_for(bn));
        pr.shape.M = m.dimP; pr.shape.N = m.dimP; pr.shape.K = m.Kn; pr.shape.products = g_products;
        pr.epi.kind = TcEpilogue::AXPBY_F64;
        pr.epi.rd = m.Kc; pr.epi.ro1 = op.ct * op.dim; pr.epi.ro2 = op.dim; pr.epi.rlim = op.ct;
        pr.epi.cd = m.Kc; pr.epi.co1 = op.ct; pr.epi.co2 = 1; pr.epi.clim = op.ct;
        pr.epi.out_f64 = H.get() + hoff[q]; pr.epi.alpha = c.cx; pr.epi.beta = 0.0;
        VGB_REQUIRE(m.Kn <= g_max_chain, "dense form: Naux above the FP32 chain bound");
        bx.add(&pr, bn, q);
      }
      bx.run(err, s, ks);
    }
    // Hd: H[(v1, c1)][(v, c)] -= cd sum_P w_P M(v1, v, P) M(c1, c, P): rows (v1, v), columns (c1, c)
    if (c.cd != 0) {
      std::vector<TcProblem> pd(b - a);
      GemmBuckets bd;
      for (size_t t = a; t < b; ++t) {
        const BseOperator &op = *todo[t];
        Impl &m = *op.mixed->impl_;
        const size_t q = t - a;
        const int bn = pick_bn(op.ct * op.ct);
        TcProblem &pr = pd[q];
        pr.A = make_tc_mat(Av.hi.get() + aoff[q], Av.lo.get() + aoff[q], op.vt * op.vt, m.Kn, m.Kn, 128, bk_for(bn));
        pr.B = make_tc_mat(Bc.hi.get() + boff[q], Bc.lo.get() + boff[q], op.ct * op.ct, m.Kn, m.Kn, bn, bk_for(bn));
        pr.shape.M = op.vt * op.vt; pr.shape.N = op.ct * op.ct; pr.shape.K = m.Kn; pr.shape.products = g_products;
        pr.epi.kind = TcEpilogue::AXPBY_F64;
        pr.epi.rd = op.vt; pr.epi.ro1 = op.ct * op.dim; pr.epi.ro2 = op.ct; pr.epi.rlim = op.vt;
        pr.epi.cd = op.ct; pr.epi.co1 = op.dim; pr.epi.co2 = 1; pr.epi.clim = op.ct;
        pr.epi.out_f64 = H.get() + hoff[q]; pr.epi.alpha = -(double)c.cd; pr.epi.beta = c.cx != 0 ? 1.0 : 0.0;
        bd.add(&pr, bn, q);
      }
      bd.run(err, s, ks);
    }
    for (size_t t = a; t < b; ++t) {
      BseOperator &op = *todo[t];
      Impl &m = *op.mixed->impl_;
      const size_t q = t - a;
      if (c.cx == 0 && c.cd == 0)
        VGB_CUDA(cudaMemsetAsync(H.get() + hoff[q], 0, op.dim * op.dim * sizeof(double), s));
      symmetrize_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(op.dim * op.dim, 256), 4096)),
                          256, 0, s>>>(H.get() + hoff[q], op.dim);
      VGB_LAUNCH_CHECK();
      m.Kd = pad64(op.dim);
      m.Hdense.ensure(op.dim, m.Kd, s);
    }
    std::vector<SplitJob> hj;
    for (size_t t = a; t < b; ++t) {
      const BseOperator &op = *todo[t];
      Impl &m = *op.mixed->impl_;
      SplitJob j;
      j.x = H.get() + hoff[t - a]; j.rows = op.dim; j.cols = op.dim;
      j.map.rdiv = 1; j.map.rs1 = op.dim; j.map.rs2 = 0; j.map.cs = 1; j.map.rlim = 1;
      j.hi = m.Hdense.hi.get(); j.lo = m.Hdense.lo.get(); j.ldo = m.Kd;
      hj.push_back(j);
    }
    split_grouped(hj, s);
    VGB_CUDA(cudaStreamSynchronize(s));  // the slice temporaries are freed next
    for (size_t t = a; t < b; ++t) {
      Impl &m = *todo[t]->mixed->impl_;
      m.dense_ready = true;
      m.dense_coef = c;
    }
    a = b;
  }
}

namespace {

// Empirical choice of the launch shape of the grouped dense products (the dominant launch of
// the lockstep batch): on the first product round with at least 16 operators of a tile width,
// every candidate (K box 32 or 64 bf16 elements, 8, 16 or 32 operators per launch, the launches
// on one stream or spread over four) runs the whole round twice into scratch outputs and the
// second run is timed with events; the fastest is kept for the process.  The candidates compute identical numbers (the same FP32 chains in
// the same order), so the choice affects time only.
struct DenseTuning {
  bool done = false;
  int bk = 64, group = 32, streams = 1;
  std::vector<std::array<double, 4>> table;  // bk, group, streams, ms
};
std::mutex g_tune_mu;
std::map<int, DenseTuning> g_dense_tuning;  // by tile width

}  // namespace

std::string autotune_report() {
  std::lock_guard<std::mutex> lk(g_tune_mu);
  std::string out = "[";
  bool first = true;
  for (const auto &kv : g_dense_tuning) {
    if (!kv.second.done) continue;
    if (!first) out += ", ";
    first = false;
    out += "{\"kernel\": \"grouped dense product\", \"bn\": " + std::to_string(kv.first) +
           ", \"chosen\": {\"bk\": " + std::to_string(kv.second.bk) + ", \"operators_per_launch\": " +
           std::to_string(kv.second.group) + ", \"streams\": " + std::to_string(kv.second.streams) +
           "}, \"candidates_ms\": [";
    for (size_t i = 0; i < kv.second.table.size(); ++i) {
      const auto &t = kv.second.table[i];
      char buf[112];
      snprintf(buf, sizeof(buf), "%s[%d, %d, %d, %.4f]", i ? ", " : "", (int)t[0], (int)t[1], (int)t[2], t[3]);
      out += buf;
    }
    out += "]}";
  }
  return out + "]";
}

void MixedEngine::apply_dense_grouped(const Coef &c, const std::vector<GroupedItem> &items, bool accumulate,
                                      cudaStream_t s) {
  read_tuning();
  const size_t n = items.size();
  if (n == 0) return;
  std::vector<Impl *> eng(n);
  for (size_t i = 0; i < n; ++i) {
    VGB_REQUIRE(items[i].op->mixed && items[i].op->mixed->dense_ready(c), "dense product: form not built");
    eng[i] = items[i].op->mixed->impl_;
  }
  int *err = eng[0]->err.get();
  // X -> Xd[j][I] (bf16 hi/lo, K = Kd)
  std::vector<SplitJob> jobs(n);
  for (size_t i = 0; i < n; ++i) {
    Impl &m = *eng[i];
    const GroupedItem &it = items[i];
    m.Xd.ensure(it.k, m.Kd, s);
    SplitJob &j = jobs[i];
    j.x = it.X; j.rows = it.k; j.cols = m.dim;
    j.map.rdiv = 1; j.map.rs1 = it.ldx; j.map.rs2 = 0; j.map.cs = 1; j.map.rlim = 1;
    j.hi = m.Xd.hi.get(); j.lo = m.Xd.lo.get(); j.ldo = m.Kd;
  }
  split_grouped(jobs, s);
  // Y[I + j ldy] (+)= (H X)(I, j).  With BN <= 64 a CTA runs all K splits of its tile and sums
  // their FP32 chains on the CTA, writing Y directly; otherwise FP32 partials [split][j][I] are
  // summed in FP64 by a reduction launch.
  std::vector<TcProblem> pr(n);
  std::vector<int> ks(n, 0);
  std::vector<char> direct(n, 0);
  // largest operators first: their long work items start early and the small ones fill the
  // tail of each launch
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return eng[x]->dim > eng[y]->dim; });
  int bn_all = 0;  // the tile width when every item has the same one and accumulates on the CTA
  bool tunable = g_autotune && n >= 16;
  for (size_t i = 0; i < n; ++i) {
    const int bn = pick_bn(items[i].k);
    tunable = tunable && g_kacc && bn <= 64 && (bn_all == 0 || bn == bn_all);
    bn_all = bn;
  }
  int use_bk = 0, use_group = 32, use_streams = 1;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_dense_tuning.find(bn_all);
    if (it != g_dense_tuning.end() && it->second.done) {
      use_bk = it->second.bk;
      use_group = it->second.group;
      use_streams = it->second.streams;
      tunable = false;
    }
  }
  // problems of one round; Ys: per-item outputs (scratch for the tuning runs)
  auto build = [&](int bk_override, const std::vector<double *> *Ys, GemmBuckets &b) {
    for (size_t i : order) {
      Impl &m = *eng[i];
      const GroupedItem &it = items[i];
      const int bn = pick_bn(it.k);
      const int bk = bk_override ? bk_override : bk_for(bn);
      TcProblem &q = pr[i];
      q = TcProblem();
      q.A = m.mat(m.Hdense.hi.get(), m.Hdense.lo.get(), m.dim, m.Kd, 128, bk);
      q.B = m.mat(m.Xd.hi.get(), m.Xd.lo.get(), (int64_t)m.Xd.hi.count / m.Kd, m.Kd, bn, bk);
      q.shape.M = m.dim; q.shape.N = it.k; q.shape.K = m.Kd; q.shape.products = g_products;
      direct[i] = (g_kacc && bn <= 64) ? 1 : 0;
      if (direct[i]) {
        // in-CTA accumulation adds no parallelism: only the chain bound sets the splits
        q.shape.ksplit = (int)ceil_div(m.Kd, g_dense_chain);
        q.shape.kacc = true;
        q.epi.kind = TcEpilogue::AXPBY_F64;
        q.epi.rd = m.dim; q.epi.ro2 = 1; q.epi.rlim = m.dim;
        q.epi.cd = it.k; q.epi.clim = it.k;
        if (Ys) {
          q.epi.co2 = m.dim; q.epi.out_f64 = (*Ys)[i]; q.epi.alpha = 1.0; q.epi.beta = 0.0;
        } else {
          q.epi.co2 = it.ldy; q.epi.out_f64 = it.Y; q.epi.alpha = 1.0; q.epi.beta = accumulate ? 1.0 : 0.0;
        }
      } else {
        q.shape.ksplit = pick_ksplit(ceil_div(m.dim, 128) * ceil_div(it.k, bn), m.Kd, g_dense_chain);
        m.part.resize((size_t)q.shape.ksplit * m.dim * it.k);
        q.epi.kind = TcEpilogue::STORE_F32;
        q.epi.rd = m.dim; q.epi.ro2 = 1; q.epi.rlim = m.dim;
        q.epi.cd = it.k; q.epi.co2 = m.dim; q.epi.clim = it.k;
        q.epi.so = m.dim * it.k;
        q.epi.out_f32 = m.part.get();
      }
      b.add(&q, bn, i);
    }
  };
  if (tunable) {
    DenseTuning t;
    int64_t tot = 0;
    for (size_t i = 0; i < n; ++i) tot += eng[i]->dim * items[i].k;
    DeviceBuffer<double> scratch(tot);
    std::vector<double *> Ys(n);
    for (size_t i = 0, off = 0; i < n; off += eng[i]->dim * items[i].k, ++i) Ys[i] = scratch.get() + off;
    cudaEvent_t e0, e1;
    VGB_CUDA(cudaEventCreate(&e0));
    VGB_CUDA(cudaEventCreate(&e1));
    double best = 1e30;
    for (int bk : {32, 64})
      for (int group : {8, 16, 32})
        for (int streams : {1, 4}) {
          float ms = 0.f;
          for (int rep = 0; rep < 2; ++rep) {
            GemmBuckets tb;
            build(bk, &Ys, tb);
            VGB_CUDA(cudaEventRecord(e0, s));
            tb.run(err, s, ks, group, streams);
            VGB_CUDA(cudaEventRecord(e1, s));
            VGB_CUDA(cudaEventSynchronize(e1));
            VGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          }
          t.table.push_back({(double)bk, (double)group, (double)streams, (double)ms});
          if (ms < best) { best = ms; t.bk = bk; t.group = group; t.streams = streams; }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    t.done = true;
    use_bk = t.bk;
    use_group = t.group;
    use_streams = t.streams;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_dense_tuning[bn_all] = t;
  }
  GemmBuckets b;
  build(use_bk, nullptr, b);
  b.run(err, s, ks, use_group, use_streams);
  std::vector<ReduceJob> rj;
  for (size_t i = 0; i < n; ++i) {
    if (direct[i]) continue;
    Impl &m = *eng[i];
    const GroupedItem &it = items[i];
    rj.emplace_back();
    ReduceJob &r = rj.back();
    r.part = m.part.get(); r.M = it.k; r.N = m.dim; r.ksplit = ks[i];
    r.epi.kind = TcEpilogue::AXPBY_F64;
    r.epi.rd = it.k; r.epi.ro2 = it.ldy; r.epi.rlim = it.k;
    r.epi.cd = m.dim; r.epi.co2 = 1; r.epi.clim = m.dim;
    r.epi.out_f64 = it.Y; r.epi.alpha = 1.0; r.epi.beta = accumulate ? 1.0 : 0.0;
  }
  reduce_grouped(rj, s);
}

void MixedEngine::prepare_grouped(const std::vector<BseOperator *> &ops, int64_t kmax, cudaStream_t s) {
  read_tuning();
  // sizes of every per-operator buffer a grouped product of <= kmax columns touches
  struct Need { Impl *m; int64_t xs, zs, part; };
  std::vector<Need> need;
  int64_t bytes = 0;
  for (BseOperator *op : ops) {
    if (!op->mixed) continue;
    Impl &m = *op->mixed->impl_;
    Need q;
    q.m = &m;
    q.xs = kmax * m.vt * m.Kc;
    q.zs = kmax * m.Kn;
    const int64_t ks1 = pick_ksplit(ceil_div(m.naux, 128) * ceil_div(kmax, pick_bn(kmax)), m.dimP);
    int64_t part = ks1 * m.naux * kmax;
    for (int64_t kc = 1; kc <= kmax; ++kc) {  // Hd stage 2 partials for any vector count
      const int64_t ks2 = pick_ksplit(ceil_div(kc * m.ct, 128) * ceil_div(m.vt, pick_bn(m.vt)), m.Kg);
      part = std::max(part, ks2 * kc * m.ct * m.vt);
    }
    if (m.dense_ready)
      part = std::max(part, pick_ksplit(ceil_div(m.dim, 128) * ceil_div(kmax, pick_bn(kmax)), m.Kd) * m.dim * kmax);
    q.part = part;
    need.push_back(q);
    bytes += 4 * (q.xs + q.zs + (m.dense_ready ? kmax * m.Kd : 0)) + 4 * q.part + 4096;
  }
  if (need.empty()) return;
  // grow the stream-ordered pool once instead of once per buffer
  if (alloc_stream()) {
    void *p = nullptr;
    if (cudaMallocAsync(&p, (size_t)bytes, s) == cudaSuccess) VGB_CUDA(cudaFreeAsync(p, s));
    else cudaGetLastError();  // no headroom for one block: the buffers are allocated one by one
  }
  for (Need &q : need) {
    if ((int64_t)q.m->Xs.hi.count < q.xs) q.m->Xs.ensure(q.xs / q.m->Kc, q.m->Kc, s);
    if (q.m->dense_ready) q.m->Xd.ensure(kmax, q.m->Kd, s);
    if ((int64_t)q.m->Zs.hi.count < q.zs) q.m->Zs.ensure(q.zs / q.m->Kn, q.m->Kn, s);
    q.m->part.resize((size_t)q.part);
  }
}

void MixedEngine::apply_grouped(const Coef &c, const std::vector<GroupedItem> &items,
                                bool accumulate, cudaStream_t s, GroupScratch *scratch) {
  read_tuning();
  const size_t n = items.size();
  if (n == 0) return;
  VGB_REQUIRE(c.cd2 == 0, "grouped products: Hd2 is not grouped");
  std::vector<Impl *> eng(n);
  for (size_t i = 0; i < n; ++i) {
    VGB_REQUIRE(items[i].op && items[i].op->mixed, "grouped products need mixed-precision operators");
    eng[i] = items[i].op->mixed->impl_;
  }
  int *err = eng[0]->err.get();  // one error flag for the whole group
  // X -> Xs[(j, v)][c]
  {
    std::vector<SplitJob> jobs(n);
    for (size_t i = 0; i < n; ++i) {
      Impl &m = *eng[i];
      const GroupedItem &it = items[i];
      m.Xs.ensure(it.k * m.vt, m.Kc, s);
      SplitJob &j = jobs[i];
      j.x = it.X; j.rows = it.k * m.vt; j.cols = m.ct;
      j.map.rdiv = m.vt; j.map.rs1 = it.ldx; j.map.rs2 = m.ct; j.map.cs = 1; j.map.rlim = m.vt;
      j.hi = m.Xs.hi.get(); j.lo = m.Xs.lo.get(); j.ldo = m.Kc;
    }
    split_grouped(jobs, s);
  }
  bool acc = accumulate;
  if (c.cx != 0) {
    // Z[P][j] = sum_I' Bvc2[P][I'] Xs[j][I']  (partials column-major), reduced into Zs[j][P]
    std::vector<TcProblem> pr(n);
    std::vector<int> ks(n, 0);
    GemmBuckets b;
    for (size_t i = 0; i < n; ++i) {
      Impl &m = *eng[i];
      const int64_t k = items[i].k;
      const int bn = pick_bn(k);
      TcProblem &q = pr[i];
      // descriptors over the whole (grown-only) buffers: rows past k are never stored
      q.A = m.mat(m.Bvc2.hi.get(), m.Bvc2.lo.get(), m.naux, m.dimP, 128, bk_for(bn));
      q.B = m.mat(m.Xs.hi.get(), m.Xs.lo.get(), (int64_t)m.Xs.hi.count / m.dimP, m.dimP, bn, bk_for(bn));
      q.shape.M = m.naux; q.shape.N = k; q.shape.K = m.dimP; q.shape.products = g_products;
      // the same K splits as the single product: identical FP32 chains, identical numbers
      q.shape.ksplit = pick_ksplit(ceil_div(m.naux, 128) * ceil_div(k, bn), m.dimP);
      m.part.resize((size_t)q.shape.ksplit * m.naux * k);
      q.epi.kind = TcEpilogue::STORE_F32;
      q.epi.rd = m.naux; q.epi.ro2 = 1; q.epi.rlim = m.naux;
      q.epi.cd = k; q.epi.co2 = m.naux; q.epi.clim = k;
      q.epi.so = m.naux * k;
      q.epi.out_f32 = m.part.get();
      m.Zs.ensure(k, m.Kn, s);
      b.add(&q, bn, i);
    }
    b.run(err, s, ks);
    std::vector<ReduceJob> rj(n);
    for (size_t i = 0; i < n; ++i) {
      Impl &m = *eng[i];
      const int64_t k = items[i].k;
      ReduceJob &r = rj[i];
      r.part = m.part.get(); r.M = k; r.N = m.naux; r.ksplit = ks[i];
      r.epi.kind = TcEpilogue::SPLIT_BF16;
      r.epi.rd = k; r.epi.ro2 = m.Kn; r.epi.rlim = k;
      r.epi.cd = m.naux; r.epi.co2 = 1; r.epi.clim = m.naux;
      r.epi.out_hi = m.Zs.hi.get(); r.epi.out_lo = m.Zs.lo.get();
    }
    reduce_grouped(rj, s);
    // Y(I, j) (+)= cx sum_P BvcT[I'][P] Zs[j][P]
    std::vector<TcProblem> p2(n);
    GemmBuckets b2;
    for (size_t i = 0; i < n; ++i) {
      Impl &m = *eng[i];
      const GroupedItem &it = items[i];
      const int bn = pick_bn(it.k);
      TcProblem &q = p2[i];
      q.A = m.mat(m.BvcT.hi.get(), m.BvcT.lo.get(), m.dimP, m.Kn, 128, bk_for(bn));
      q.B = m.mat(m.Zs.hi.get(), m.Zs.lo.get(), (int64_t)m.Zs.hi.count / m.Kn, m.Kn, bn, bk_for(bn));
      q.shape.M = m.dimP; q.shape.N = it.k; q.shape.K = m.Kn; q.shape.products = g_products;
      q.epi.kind = TcEpilogue::AXPBY_F64;
      q.epi.rd = m.Kc; q.epi.ro1 = m.ct; q.epi.ro2 = 1; q.epi.rlim = m.ct;
      q.epi.cd = it.k; q.epi.co2 = it.ldy; q.epi.clim = it.k;
      q.epi.out_f64 = it.Y; q.epi.alpha = c.cx; q.epi.beta = acc ? 1.0 : 0.0;
      b2.add(&q, bn, i);
    }
    b2.run(err, s, ks);
    acc = true;
  }
  if (c.cd != 0) {
    const double alpha = -(double)c.cd;
    // The Hd intermediates S live in one arena shared by the group: per round of vector
    // chunks the operators are taken in slices whose intermediates fit the arena, and
    // each slice runs stage 1, stage 2 and the reduction before the next reuses it.
    GroupScratch local;
    GroupScratch &arena = scratch ? *scratch : local;
    std::vector<int64_t> jc(n), need(n);
    int64_t rounds = 0, total = 0, largest = 0;
    for (size_t i = 0; i < n; ++i) {
      Impl &m = *eng[i];
      const int64_t per_vec = m.ct * m.Kg * 4;
      jc[i] = std::max<int64_t>(1, std::min<int64_t>(items[i].k, (4LL << 30) / per_vec));
      need[i] = jc[i] * m.ct * m.Kg;  // elements (a multiple of 64: regions stay 128-byte aligned)
      total += need[i];
      largest = std::max(largest, need[i]);
      rounds = std::max(rounds, ceil_div(items[i].k, jc[i]));
    }
    const int64_t want = std::max(largest, std::min(total, kGroupArenaElems));
    if (arena.elems < want) {
      arena.hi.resize(want);
      arena.lo.resize(want);
      // zero once: pad columns of S are read (times zero pads of G2) and must be finite
      VGB_CUDA(cudaMemsetAsync(arena.hi.get(), 0, want * sizeof(uint16_t), s));
      VGB_CUDA(cudaMemsetAsync(arena.lo.get(), 0, want * sizeof(uint16_t), s));
      arena.elems = want;
    }
    for (int64_t rd = 0; rd < rounds; ++rd) {
      std::vector<size_t> live;
      for (size_t i = 0; i < n; ++i)
        if (rd * jc[i] < items[i].k) live.push_back(i);
      size_t a = 0;
      while (a < live.size()) {
        // slice [a, b) of the live operators, regions packed in the arena
        std::vector<int64_t> off(n, 0);
        int64_t used = 0;
        size_t b = a;
        while (b < live.size() && (b == a || used + need[live[b]] <= arena.elems)) {
          off[live[b]] = used;
          used += need[live[b]];
          ++b;
        }
        std::vector<TcProblem> p1(n), p2(n);
        std::vector<int> ks(n, 0);
        GemmBuckets b1, b2;
        // stage 1: S[(j, c1)][(P, v)] = sum_c Xs[(j, v)][c] Mcc2[(P, c1)][c], N over (P, c1)
        for (size_t t = a; t < b; ++t) {
          const size_t i = live[t];
          Impl &m = *eng[i];
          const int64_t j0 = rd * jc[i];
          const int64_t kc = std::min(jc[i], items[i].k - j0);
          const uint16_t *xh = m.Xs.hi.get() + j0 * m.vt * m.Kc, *xl = m.Xs.lo.get() + j0 * m.vt * m.Kc;
          const int bn = pick_bn(m.naux * m.ct);
          TcProblem &q = p1[i];
          q.A = m.mat(xh, xl, ((int64_t)m.Xs.hi.count - j0 * m.vt * m.Kc) / m.Kc, m.Kc, 128, bk_for(bn));
          q.B = m.mat(m.Mcc2.hi.get(), m.Mcc2.lo.get(), m.naux * m.ct, m.Kc, bn, bk_for(bn));
          q.shape.M = kc * m.vt; q.shape.N = m.naux * m.ct; q.shape.K = m.Kc; q.shape.products = g_products;
          q.epi.kind = TcEpilogue::SPLIT_BF16;
          q.epi.rd = m.vt; q.epi.ro1 = m.ct * m.Kg; q.epi.ro2 = 1; q.epi.rlim = m.vt;
          q.epi.cd = m.ct; q.epi.co1 = m.vt; q.epi.co2 = m.Kg; q.epi.clim = m.ct;
          q.epi.out_hi = arena.hi.get() + off[i]; q.epi.out_lo = arena.lo.get() + off[i];
          b1.add(&q, bn, i);
        }
        b1.run(err, s, ks);
        // stage 2: partials [split][v1][(j, c1)] of sum_{(P,v)} S[(j, c1)][(P,v)] G2[v1][(P,v)]
        for (size_t t = a; t < b; ++t) {
          const size_t i = live[t];
          Impl &m = *eng[i];
          const int64_t kc = std::min(jc[i], items[i].k - rd * jc[i]);
          const int bn2 = pick_bn(m.vt);
          TcProblem &q = p2[i];
          q.A = m.mat(arena.hi.get() + off[i], arena.lo.get() + off[i], jc[i] * m.ct, m.Kg, 128, bk_for(bn2));
          q.B = m.mat(m.G2.hi.get(), m.G2.lo.get(), m.vt, m.Kg, bn2, bk_for(bn2));
          q.shape.M = kc * m.ct; q.shape.N = m.vt; q.shape.K = m.Kg; q.shape.products = g_products;
          q.shape.ksplit = pick_ksplit(ceil_div(kc * m.ct, 128) * ceil_div(m.vt, bn2), m.Kg);
          m.part.resize((size_t)q.shape.ksplit * q.shape.M * q.shape.N);
          q.epi.kind = TcEpilogue::STORE_F32;
          q.epi.rd = q.shape.M; q.epi.ro2 = 1; q.epi.rlim = q.shape.M;
          q.epi.cd = q.shape.N; q.epi.co2 = q.shape.M; q.epi.clim = q.shape.N;
          q.epi.so = q.shape.M * q.shape.N;
          q.epi.out_f32 = m.part.get();
          b2.add(&q, bn2, i);
        }
        b2.run(err, s, ks);
        std::vector<ReduceJob> rj;
        for (size_t t = a; t < b; ++t) {
          const size_t i = live[t];
          Impl &m = *eng[i];
          const int64_t j0 = rd * jc[i];
          const int64_t kc = std::min(jc[i], items[i].k - j0);
          ReduceJob r;
          r.part = m.part.get(); r.M = m.vt; r.N = kc * m.ct; r.ksplit = ks[i];
          r.epi.kind = TcEpilogue::AXPBY_F64;
          r.epi.rd = m.vt; r.epi.ro2 = m.ct; r.epi.rlim = m.vt;
          r.epi.cd = m.ct; r.epi.co1 = items[i].ldy; r.epi.co2 = 1; r.epi.clim = m.ct;
          r.epi.out_f64 = items[i].Y + j0 * items[i].ldy; r.epi.alpha = alpha; r.epi.beta = acc ? 1.0 : 0.0;
          rj.push_back(r);
        }
        reduce_grouped(rj, s);
        a = b;
      }
    }
    acc = true;
  }
  if (!acc) {
    for (const GroupedItem &it : items)
      VGB_CUDA(cudaMemset2DAsync(it.Y, it.ldy * sizeof(double), 0, it.op->dim * sizeof(double), it.k, s));
  }
}

}  // namespace vgb
