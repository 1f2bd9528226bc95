// Hellmann-Feynman adjoint of the BSE eigenvalues.
//
// TDA: for normalised eigenvectors x_k of A = cqp Hqp + cx Hx - cd Hd, every parameter
// derivative of Omega_k = x_k^T A x_k is x_k^T (dA) x_k.  Full BSE: for ([[A, B], [-B, -A]])
// = J S with S = [[A, B], [B, A]] symmetric and J = diag(I, -I), an eigenvector (X, Y) with
// X^T X - Y^T Y = 1 solves S z = Omega J z, so dOmega = z^T dS z = X^T dA X + Y^T dA Y +
// 2 X^T dB Y (the sum BSE::Analyze_eh_interaction forms, xtp/src/libxtp/gwbse/bse.cc:551-564);
// the bilinear term is the difference of two quadratic forms,
// 2 X^T dB Y = (1/2)(X+Y)^T dB (X+Y) - (1/2)(X-Y)^T dB (X-Y).
// Everything therefore reduces to quad_gradient: the gradient of sum_i g_i u_i^T H(c) u_i for
// a list of vectors and weights, returned for the Mmn blocks, the Hqp window and the screening
// (what a reverse-mode backward pass needs).  With X_k the v x c matrix of vector k
// (I = ct v + c):
//   Hqp:  dH(vt+c, vt+c') = cqp sum_k g_k sum_v X_k[v][c] X_k[v][c']
//         dH(v, v')       = -cqp sum_k g_k sum_c X_k[v'][c] X_k[v][c]
//   Hx:   dM(v,c,P)       = 2 cx sum_k g_k z_k[P] X_k[v][c],   z_k[P] = sum_I M(I,P) X_k[I]
//   Hd:   S_k^P[v'][c]    = sum_c' M(c,c',P) X_k[v'][c']          (the forward stage-1 product)
//         Q^P[v][v']      = sum_k g_k sum_c X_k[v][c] S_k^P[v'][c]
//         dM(v,v',P)      = -cd sum_Q W_QP Q^Q[v][v']             (diagonal W: -cd w_P Q^P)
//         dW_PQ           = -cd sum_{vv'} Q^P[v][v'] M(v,v',Q)    (diagonal: dw_P = -cd <Q^P, M_vv^P>)
//         dM(c,c',P)      = -cd sum_k g_k sum_v X_k[v][c] (G^P X_k)[v][c'],  G^P = screened vv block
//   Hd2 (a^P[v][c'] = M(v,c',P), b^P[c][v'] = M(c,v',P); Hd2 = sum_PQ W_PQ a^P b^Q as bilinear
//        pieces of x^T Hd2 x = sum x[v][c] a^P[v][c'] W_PQ b^Q[c][v'] x[v'][c']):
//         Yt^P[v][v']     = sum_c X_k[v][c] bw^P[c][v']       (bw = screened cv block, staged Mcv)
//         dM(v,c',P)      = -cd2 sum_k g_k sum_v' Yt^P[v][v'] X_k[v'][c']
//         Za^P[v][v']     = sum_c' a^P[v][c'] X_k[v'][c']
//         dM(c,v',P)      = -cd2 sum_k g_k sum_v X_k[v][c] (sum_Q W_QP Za^Q)[v][v']
//         dW_PQ           = -cd2 sum_k g_k <Za^P, Yb^Q>,  Yb^Q[v][v'] = sum_c X_k[v][c] b^Q[c][v']
// The forward analogue in the reference is the expectation-value analysis
// x^T H_part x (xtp/src/libxtp/gwbse/bse.cc:490-520, 565-606).
#include <algorithm>
#include <vector>

#include "bse_ops.cuh"
#include "tc_engine.cuh"

namespace vgb {

namespace {

unsigned gfor(int64_t n) {
  return (unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, 256), 16LL * 152));
}

__global__ void scale_cols_by_kernel(double *Z, int64_t ld, int64_t rows, int64_t ncols,
                                     const double *g) {
  const int64_t total = rows * ncols;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    Z[(t % rows) + ld * (t / rows)] *= g[t / rows];
}

// gH: (vt+ct)^2 column-major window gradient of Hqp
__global__ void hqp_grad_kernel(const double *X, int64_t ldx, int64_t nr, const double *g,
                                int64_t vt, int64_t ct, double cqp, double *gH) {
  const int64_t n = vt + ct, total = n * n;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t % n, col = t / n;
    double acc = 0.0;
    if (r >= vt && col >= vt) {  // (vt+c, vt+c')
      const int64_t c = r - vt, c2 = col - vt;
      for (int64_t k = 0; k < nr; ++k) {
        const double *x = X + k * ldx;
        double s = 0.0;
        for (int64_t v = 0; v < vt; ++v) s += x[v * ct + c] * x[v * ct + c2];
        acc += g[k] * s;
      }
      acc *= cqp;
    } else if (r < vt && col < vt) {  // (v, v')
      for (int64_t k = 0; k < nr; ++k) {
        const double *x = X + k * ldx;
        double s = 0.0;
        for (int64_t c = 0; c < ct; ++c) s += x[col * ct + c] * x[r * ct + c];
        acc += g[k] * s;
      }
      acc *= -cqp;
    }
    gH[t] += acc;
  }
}

// gw[P] = alpha * sum_{vv'} Q[P][v][v'] Mvv[P][v][v']
__global__ void dot_per_batch_kernel(const double *Q, const double *M, int64_t nb, int64_t len,
                                     double alpha, double *out) {
  for (int64_t b = blockIdx.x; b < nb; b += gridDim.x) {
    double s = 0.0;
    for (int64_t i = threadIdx.x; i < len; i += blockDim.x) s += Q[b * len + i] * M[b * len + i];
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) out[b] += alpha * red[0];
    __syncthreads();
  }
}

// out[P][...] (+)= alpha * w[P] * Q[P][...]
__global__ void scale_batches_kernel(const double *Q, const double *w, int64_t nb, int64_t len,
                                     double alpha, double *out, int accumulate) {
  const int64_t total = nb * len;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x)
    out[t] = alpha * w[t / len] * Q[t] + (accumulate ? out[t] : 0.0);
}

// One chunk [m0, m0 + cnt) of the Mmn-shaped gradient, slice layout out[(mi * naux + P) * nsize + n]:
// the vc, vv and cc block gradients at their window positions, zero elsewhere.
struct ScatterGradArgs {
  const double *gMvc, *gMcv, *gMvv, *gMcc;
  int64_t m0, cnt, naux, nsize, vt, ct, dim, m_v0, m_c0, n_v0, n_c0;
  double *out;
};
__global__ void scatter_grad_kernel(const ScatterGradArgs a) {
  const int64_t total = a.cnt * a.naux * a.nsize;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t n = t % a.nsize, P = (t / a.nsize) % a.naux, m = a.m0 + t / (a.nsize * a.naux);
    const int64_t v = m - a.m_v0, c1 = m - a.m_c0, nv = n - a.n_v0, nc = n - a.n_c0;
    double g = 0.0;
    if (v >= 0 && v < a.vt) {
      if (nc >= 0 && nc < a.ct) g = a.gMvc[P * a.dim + v * a.ct + nc];
      else if (nv >= 0 && nv < a.vt) g = a.gMvv[(P * a.vt + v) * a.vt + nv];
    } else if (c1 >= 0 && c1 < a.ct) {
      if (nc >= 0 && nc < a.ct) g = a.gMcc[(P * a.ct + c1) * a.ct + nc];
      else if (a.gMcv && nv >= 0 && nv < a.vt) g = a.gMcv[P * a.dim + nv * a.ct + c1];
    }
    a.out[t] = g;
  }
}

}  // namespace

void scatter_mmn_gradient(const BseOperator &op, const double *gMvc, const double *gMcv,
                          const double *gMvv, const double *gMcc, double *host_out, cudaStream_t s) {
  const int64_t slice = op.naux * op.nsize;
  const int64_t per = std::max<int64_t>(1, std::min<int64_t>(op.msize, (512LL << 20) / (slice * 8)));
  DeviceBuffer<double> buf(per * slice);
  for (int64_t m0 = 0; m0 < op.msize; m0 += per) {
    ScatterGradArgs a;
    a.gMvc = gMvc; a.gMcv = gMcv; a.gMvv = gMvv; a.gMcc = gMcc;
    a.m0 = m0; a.cnt = std::min(per, op.msize - m0);
    a.naux = op.naux; a.nsize = op.nsize; a.vt = op.vt; a.ct = op.ct; a.dim = op.dim;
    a.m_v0 = op.m_v0; a.m_c0 = op.m_c0; a.n_v0 = op.n_v0; a.n_c0 = op.n_c0;
    a.out = buf.get();
    const int64_t total = a.cnt * slice;
    scatter_grad_kernel<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, 256), 16LL * 152)),
                          256, 0, s>>>(a);
    VGB_LAUNCH_CHECK();
    VGB_CUDA(cudaMemcpyAsync(host_out + m0 * slice, buf.get(), total * sizeof(double),
                             cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));  // buf is reused by the next chunk
  }
}

void BseOperator::quad_gradient(const Coef &c, const double *X, int64_t ldx, int64_t nr,
                                const double *g_host, double *gMvc, double *gMcv, double *gMvv,
                                double *gMcc, double *gH, double *gW, bool accumulate, cudaStream_t s) {
  VGB_REQUIRE(nr >= 1 && ldx >= dim, "eig_gradient: bad eigenvector block");
  VGB_REQUIRE(!(c.cd != 0 && c.cd2 != 0), "Hamiltonian cannot contain Hd and Hd2 at the same time");
  const int64_t nW = dense_screening ? naux * naux : naux;
  if (!accumulate) {
    if (gMvc) VGB_CUDA(cudaMemsetAsync(gMvc, 0, naux * dim * sizeof(double), s));
    if (gMcv) VGB_CUDA(cudaMemsetAsync(gMcv, 0, naux * dim * sizeof(double), s));
    if (gMvv) VGB_CUDA(cudaMemsetAsync(gMvv, 0, naux * vt * vt * sizeof(double), s));
    if (gMcc) VGB_CUDA(cudaMemsetAsync(gMcc, 0, naux * ct * ct * sizeof(double), s));
    if (gH) VGB_CUDA(cudaMemsetAsync(gH, 0, (vt + ct) * (vt + ct) * sizeof(double), s));
    if (gW) VGB_CUDA(cudaMemsetAsync(gW, 0, nW * sizeof(double), s));
  }
  DeviceBuffer<double> g(nr);
  VGB_CUDA(cudaMemcpyAsync(g.get(), g_host, nr * sizeof(double), cudaMemcpyHostToDevice, s));
  const std::vector<double> gh(g_host, g_host + nr);
  if (gH && c.cqp != 0) {
    hqp_grad_kernel<<<gfor((vt + ct) * (vt + ct)), 256, 0, s>>>(X, ldx, nr, g.get(), vt, ct, c.cqp, gH);
    VGB_LAUNCH_CHECK();
  }
  if (gMvc && c.cx != 0) {
    DeviceBuffer<double> Zb(naux * nr);
    GemmDesc z;  // Z (naux x nr) = Bvc^T X
    z.M = naux; z.N = nr; z.K = dim;
    z.A = Bvc.get(); z.a_rs = dim; z.a_cs = 1;
    z.B = X; z.b_rs = 1; z.b_cs = ldx;
    z.C = Zb.get(); z.c_rs = 1; z.c_cs = naux;
    dgemm(z, s, &ws);
    scale_cols_by_kernel<<<gfor(naux * nr), 256, 0, s>>>(Zb.get(), naux, naux, nr, g.get());
    VGB_LAUNCH_CHECK();
    GemmDesc o;  // gMvc[P][I] += 2 cx sum_k Zg[P][k] X[I][k]
    o.M = naux; o.N = dim; o.K = nr;
    o.A = Zb.get(); o.a_rs = 1; o.a_cs = naux;
    o.B = X; o.b_rs = ldx; o.b_cs = 1;
    o.C = gMvc; o.c_rs = dim; o.c_cs = 1;
    o.alpha = 2.0 * c.cx; o.beta = 1.0;
    dgemm(o, s, &ws);
  }
  // Handles with a tensor-core engine (split-precision or slice-product handles) run the two
  // contractions of the cc block, 2 Naux v c^2 flops per vector each, as FP64-accurate slice
  // products (about 2e-10 of their scale); FP64 handles keep FP64 throughout.
  const bool sliced = mixed != nullptr;
  // vectors per slice-product chunk: the intermediates (Naux dim doubles per vector) within 4 GB
  const int64_t kch = std::max<int64_t>(1, std::min<int64_t>(nr, (4LL << 30) / (naux * dim * 8)));
  if (c.cd != 0 && (gMvv || gMcc || gW)) {
    const double cd = c.cd;
    DeviceBuffer<double> Sk(sliced ? kch * naux * dim : naux * dim), Q(naux * vt * vt);
    // ---- Q^P = sum_k g_k X_k S_k^P^T ----
    for (int64_t k = 0; k < nr; ++k) {
      const double *Skp = Sk.get();
      if (!sliced) {
        GemmDesc a;  // S_k[P](c1, v) = sum_c Mcc_P(c1, c) X_k(c, v)
        a.M = ct; a.N = vt; a.K = ct;
        a.A = Mcc.get(); a.a_rs = 1; a.a_cs = ct;
        a.B = X + k * ldx; a.b_rs = 1; a.b_cs = ct;
        a.C = Sk.get(); a.c_rs = 1; a.c_cs = ct;
        a.nb1 = naux; a.a_b1 = ct * ct; a.c_b1 = dim;
        dgemm(a, s, &ws);
      } else {
        if (k % kch == 0) {  // S of the next kch vectors, [k][P][v][c1], as one slice product
          const int64_t kc = std::min(kch, nr - k);
          SplitMap xm;  // rows (k, v), columns c
          xm.rdiv = vt; xm.rs1 = ldx; xm.rs2 = ct; xm.cs = 1; xm.rlim = vt;
          TcEpilogue e;
          e.kind = TcEpilogue::AXPBY_F64;
          e.rd = vt; e.ro1 = naux * dim; e.ro2 = ct; e.rlim = vt;
          e.cd = ct; e.co1 = dim; e.co2 = 1; e.clim = ct;
          e.out_f64 = Sk.get(); e.alpha = 1.0; e.beta = 0.0;
          mixed->gemm_sliced(*this, X + k * ldx, xm, kc * vt, nullptr, SplitMap(), naux * ct, ct, true, e, s);
        }
        Skp = Sk.get() + (k % kch) * naux * dim;
      }
      GemmDesc q;  // Q[P](v, v') += g_k sum_c X_k(v, c) S_k[P](c, v')
      q.M = vt; q.N = vt; q.K = ct;
      q.A = X + k * ldx; q.a_rs = ct; q.a_cs = 1;
      q.B = Skp; q.b_rs = 1; q.b_cs = ct; q.b_b1 = dim;
      q.C = Q.get(); q.c_rs = vt; q.c_cs = 1; q.c_b1 = vt * vt;
      q.nb1 = naux; q.alpha = gh[k]; q.beta = k > 0 ? 1.0 : 0.0;
      dgemm(q, s, &ws);
    }
    if (gMvv) {
      if (!dense_screening) {
        scale_batches_kernel<<<gfor(naux * vt * vt), 256, 0, s>>>(Q.get(), Wscr.get(), naux, vt * vt, -cd, gMvv,
                                                                   1);
        VGB_LAUNCH_CHECK();
      } else {
        GemmDesc d;  // gMvv[Q][e] += -cd sum_P W[P][Q] Q[P][e]
        d.M = naux; d.N = vt * vt; d.K = naux;
        d.A = Wscr.get(); d.a_rs = naux; d.a_cs = 1;
        d.B = Q.get(); d.b_rs = vt * vt; d.b_cs = 1;
        d.C = gMvv; d.c_rs = vt * vt; d.c_cs = 1;
        d.alpha = -cd; d.beta = 1.0;
        dgemm(d, s, &ws);
      }
    }
    if (gW) {
      if (!dense_screening) {
        dot_per_batch_kernel<<<(unsigned)std::min<int64_t>(naux, 4096), 256, 0, s>>>(Q.get(), Mvv.get(), naux,
                                                                                  vt * vt, -cd, gW);
        VGB_LAUNCH_CHECK();
      } else {
        GemmDesc d;  // gW[P][Q] += -cd sum_e Q[P][e] Mvv[Q][e]   (column-major naux x naux)
        d.M = naux; d.N = naux; d.K = vt * vt;
        d.A = Q.get(); d.a_rs = vt * vt; d.a_cs = 1;
        d.B = Mvv.get(); d.b_rs = 1; d.b_cs = vt * vt;
        d.C = gW; d.c_rs = 1; d.c_cs = naux;
        d.alpha = -cd; d.beta = 1.0;
        dgemm(d, s, &ws);
      }
    }
    if (gMcc && sliced) {
      // gMcc[(P, c)][c'] += -cd sum_{(k, v)} (g_k X_k(v, c)) T[(P, c')][(k, v)] as one slice product
      // per chunk of vectors, T = G^P X_k from FP64 GEMMs
      for (int64_t k0 = 0; k0 < nr; k0 += kch) {
        const int64_t kc = std::min(kch, nr - k0), Kt = kc * vt;
        DeviceBuffer<double> T(naux * ct * Kt), Xg(Kt * ct);
        for (int64_t k = k0; k < k0 + kc; ++k) {
          GemmDesc t;  // T[(P, c')][(k, v)] = sum_v' Gvv[v][P][v'] X_k(v', c')
          t.M = vt; t.N = ct; t.K = vt;
          t.A = Gvv.get(); t.a_rs = naux * vt; t.a_cs = 1; t.a_b1 = vt;
          t.B = X + k * ldx; t.b_rs = ct; t.b_cs = 1;
          t.C = T.get() + (k - k0) * vt; t.c_rs = 1; t.c_cs = Kt; t.c_b1 = ct * Kt;
          t.nb1 = naux;
          dgemm(t, s, &ws);
        }
        copy_cols(X + k0 * ldx, ldx, dim, kc, Xg.get(), dim, s);  // Xg[(k, v)][c] = g_k X_k(v, c)
        scale_cols_by_kernel<<<gfor(dim * kc), 256, 0, s>>>(Xg.get(), dim, dim, kc, g.get() + k0);
        VGB_LAUNCH_CHECK();
        SplitMap tm;  // rows (P, c'), columns (k, v)
        tm.rdiv = 1; tm.rs1 = Kt; tm.rs2 = 0; tm.cs = 1; tm.rlim = 1;
        SplitMap xm;  // rows c, columns (k, v): Xg[(k, v) ct + c]
        xm.rdiv = 1; xm.rs1 = 1; xm.rs2 = 0; xm.cs = ct; xm.rlim = 1;
        TcEpilogue e;  // gMcc[(P ct + c) ct + c'] for row (P, c'), column c
        e.kind = TcEpilogue::AXPBY_F64;
        e.rd = ct; e.ro1 = ct * ct; e.ro2 = 1; e.rlim = ct;
        e.cd = ct; e.co2 = ct; e.clim = ct;
        e.out_f64 = gMcc; e.alpha = -cd; e.beta = 1.0;
        mixed->gemm_sliced(*this, T.get(), tm, naux * ct, Xg.get(), xm, ct, Kt, false, e, s);
      }
    } else if (gMcc) {
      // gMcc[P][c][c'] += -cd sum_k g_k sum_v X_k(v, c) T_k[P](v, c'),  T_k[P] = G^P X_k
      for (int64_t k = 0; k < nr; ++k) {
        GemmDesc t;  // T[P](v, c') = sum_v' Gvv[v][P][v'] X_k(v', c')
        t.M = vt; t.N = ct; t.K = vt;
        t.A = Gvv.get(); t.a_rs = naux * vt; t.a_cs = 1; t.a_b1 = vt;
        t.B = X + k * ldx; t.b_rs = ct; t.b_cs = 1;
        t.C = Sk.get(); t.c_rs = ct; t.c_cs = 1; t.c_b1 = dim;
        t.nb1 = naux;
        dgemm(t, s, &ws);
        GemmDesc r;  // gMcc[P](c, c') += -cd g_k sum_v X_k(v, c) T[P](v, c')
        r.M = ct; r.N = ct; r.K = vt;
        r.A = X + k * ldx; r.a_rs = 1; r.a_cs = ct;
        r.B = Sk.get(); r.b_rs = ct; r.b_cs = 1; r.b_b1 = dim;
        r.C = gMcc; r.c_rs = ct; r.c_cs = 1; r.c_b1 = ct * ct;
        r.nb1 = naux; r.alpha = -cd * gh[k]; r.beta = 1.0;
        dgemm(r, s, &ws);
      }
    }
  }
  if (c.cd2 != 0 && (gMvc || gMcv || gW)) {
    const double cd2 = c.cd2;
    const int64_t vv = vt * vt;
    DeviceBuffer<double> T1(naux * vv), T2(naux * vv), T3;
    if (gW) T3.resize(naux * vv);
    for (int64_t k = 0; k < nr; ++k) {
      const double *x = X + k * ldx;
      const double alpha = -cd2 * gh[k];
      if (gMvc) {
        GemmDesc a;  // Yt[P](v, v') = sum_c x(v, c) bw[P](c, v'),  bw[P](c, v') = Mcv[P][v'][c]
        a.M = vt; a.N = vt; a.K = ct;
        a.A = x; a.a_rs = ct; a.a_cs = 1;
        a.B = Mcv.get(); a.b_rs = 1; a.b_cs = ct; a.b_b1 = dim;
        a.C = T1.get(); a.c_rs = vt; a.c_cs = 1; a.c_b1 = vv;
        a.nb1 = naux;
        dgemm(a, s, &ws);
        GemmDesc b;  // gMvc[P](v, c') += alpha sum_v' Yt[P](v, v') x(v', c')
        b.M = vt; b.N = ct; b.K = vt;
        b.A = T1.get(); b.a_rs = vt; b.a_cs = 1; b.a_b1 = vv;
        b.B = x; b.b_rs = ct; b.b_cs = 1;
        b.C = gMvc; b.c_rs = ct; b.c_cs = 1; b.c_b1 = dim;
        b.nb1 = naux; b.alpha = alpha; b.beta = 1.0;
        dgemm(b, s, &ws);
      }
      if (gMcv || gW) {
        GemmDesc a;  // Za[P](v, v') = sum_c' a[P](v, c') x(v', c'),  a[P] = Bvc block
        a.M = vt; a.N = vt; a.K = ct;
        a.A = Bvc.get(); a.a_rs = ct; a.a_cs = 1; a.a_b1 = dim;
        a.B = x; a.b_rs = 1; a.b_cs = ct;
        a.C = T2.get(); a.c_rs = vt; a.c_cs = 1; a.c_b1 = vv;
        a.nb1 = naux;
        dgemm(a, s, &ws);
      }
      if (gW) {
        GemmDesc a;  // Yb[Q](v, v') = sum_c x(v, c) b[Q](c, v'),  b[Q](c, v') = Mcv0[Q][v'][c]
        a.M = vt; a.N = vt; a.K = ct;
        a.A = x; a.a_rs = ct; a.a_cs = 1;
        a.B = Mcv0.get(); a.b_rs = 1; a.b_cs = ct; a.b_b1 = dim;
        a.C = T3.get(); a.c_rs = vt; a.c_cs = 1; a.c_b1 = vv;
        a.nb1 = naux;
        dgemm(a, s, &ws);
        if (!dense_screening) {
          dot_per_batch_kernel<<<(unsigned)std::min<int64_t>(naux, 4096), 256, 0, s>>>(T2.get(), T3.get(), naux,
                                                                                    vv, alpha, gW);
          VGB_LAUNCH_CHECK();
        } else {
          // the product pairs a^Q with bw^Q = sum_P b^P W(P, Q):  dW(P, Q) += alpha <Yb^P, Za^Q>
          GemmDesc d;
          d.M = naux; d.N = naux; d.K = vv;
          d.A = T3.get(); d.a_rs = vv; d.a_cs = 1;
          d.B = T2.get(); d.b_rs = 1; d.b_cs = vv;
          d.C = gW; d.c_rs = 1; d.c_cs = naux;
          d.alpha = alpha; d.beta = 1.0;
          dgemm(d, s, &ws);
        }
      }
      if (gMcv) {
        const double *Zw = T2.get();  // sum_Q W_QP Za^Q
        if (!dense_screening) {
          scale_batches_kernel<<<gfor(naux * vv), 256, 0, s>>>(T2.get(), Wscr.get(), naux, vv, 1.0, T1.get(), 0);
          VGB_LAUNCH_CHECK();
          Zw = T1.get();
        } else {
          GemmDesc d;  // Zw[P][e] = sum_Q W(P, Q) Za[Q][e]
          d.M = naux; d.N = vv; d.K = naux;
          d.A = Wscr.get(); d.a_rs = 1; d.a_cs = naux;
          d.B = T2.get(); d.b_rs = vv; d.b_cs = 1;
          d.C = T1.get(); d.c_rs = vv; d.c_cs = 1;
          dgemm(d, s, &ws);
          Zw = T1.get();
        }
        GemmDesc b;  // gMcv[P][v'][c] += alpha sum_v x(v, c) Zw[P](v, v')
        b.M = ct; b.N = vt; b.K = vt;
        b.A = x; b.a_rs = 1; b.a_cs = ct;
        b.B = Zw; b.b_rs = vt; b.b_cs = 1; b.b_b1 = vv;
        b.C = gMcv; b.c_rs = 1; b.c_cs = ct; b.c_b1 = dim;
        b.nb1 = naux; b.alpha = alpha; b.beta = 1.0;
        dgemm(b, s, &ws);
      }
    }
  }
  VGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace vgb
