// Producer side of the Mmn tensor (TCMatrix_gwbse::Fill, xtp/src/libxtp/threecenter.cc:79-95):
//   fill_3c_mo            TCMatrix_gwbse::Fill3cMO (xtp/src/libxtp/libint2_calls.cc:595-651):
//                         M(m, n, P) = sum_{mu,nu} C(mu, n) (P|mu nu) C(nu, m), with the AO
//                         three-centre integrals supplied by the caller (no integral engine
//                         here); two FP64 GEMMs per auxiliary function, batched over P.
//   aux_pseudo_inv_sqrt   AOCoulomb::Pseudo_InvSqrt (aomatrices/aomatrix.cc:88-102):
//                         V^-1/2 over the eigenvalues >= etol.
//   aux_pseudo_inv_sqrt_gwbse
//                         AOCoulomb::Pseudo_InvSqrt_GWBSE (aomatrix.cc:53-86): the metric the
//                         GW-BSE Mmn is multiplied with, (V'^-1/2 S^-1/2)^T with
//                         V' = S^-1/2 V S^-1/2, both inverse roots over eigenvalues >= etol.
//   transition_dipoles    Orbitals::CalcCoupledTransition_Dipoles (xtp/src/libxtp/orbitals.cc:
//                         740-877): the AO dipole matrices (caller-supplied, like the 3c
//                         integrals) in the MO basis of one spin block, contracted with the
//                         BSE states.
// The two eigenproblems are solved on the host, as the reference does (Eigen's
// SelfAdjointEigenSolver); the matrix products run on the device.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "dgemm.cuh"
#include "host_eig.hpp"

namespace vgb {

namespace {

// U diag(f) U^T for the host eigenvectors U (n x n, column-major) on the device.
void spectral_product(int64_t n, const std::vector<double> &U, const std::vector<double> &f, double *d_out,
                      cudaStream_t s, GemmWorkspace &ws) {
  std::vector<double> UF(n * n);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) UF[i + n * j] = U[i + n * j] * f[j];
  DeviceBuffer<double> dU(n * n), dUF(n * n);
  VGB_CUDA(cudaMemcpyAsync(dU.get(), U.data(), n * n * sizeof(double), cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaMemcpyAsync(dUF.get(), UF.data(), n * n * sizeof(double), cudaMemcpyHostToDevice, s));
  GemmDesc g;  // out = (U diag(f)) U^T
  g.M = n; g.N = n; g.K = n;
  g.A = dUF.get(); g.a_rs = 1; g.a_cs = n;
  g.B = dU.get(); g.b_rs = n; g.b_cs = 1;
  g.C = d_out; g.c_rs = 1; g.c_cs = n;
  dgemm(g, s, &ws);
  VGB_CUDA(cudaStreamSynchronize(s));  // the host staging goes out of scope
}

// f_i = 1/sqrt(lambda_i) for lambda_i >= etol, else 0 (the function is removed)
std::vector<double> inv_sqrt_weights(const std::vector<double> &lam, double etol, int64_t &removed) {
  std::vector<double> f(lam.size(), 0.0);
  for (size_t i = 0; i < lam.size(); ++i) {
    if (lam[i] < etol) ++removed;
    else f[i] = 1.0 / std::sqrt(lam[i]);
  }
  return f;
}

std::vector<double> copy_square(int64_t n, const double *a, int64_t lda) {
  std::vector<double> A(n * n);
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < n; ++i) A[i + n * j] = a[i + lda * j];
  return A;
}

void eig_or_fail(int64_t n, const std::vector<double> &A, std::vector<double> &lam, std::vector<double> &U) {
  if (!sym_eig(n, A.data(), lam, U)) fail(BSE_ERR_NUMERICAL, "auxiliary metric: eigenvalue problem failed");
}

}  // namespace

void aux_pseudo_inv_sqrt(int64_t n, const double *V, int64_t ldv, double etol, double *out, int64_t ldo,
                         int64_t *removed, cudaStream_t s) {
  VGB_REQUIRE(n >= 1 && ldv >= n && ldo >= n && V && out, "aux_pseudo_inv_sqrt: bad arguments");
  std::vector<double> lam, U;
  eig_or_fail(n, copy_square(n, V, ldv), lam, U);
  int64_t rem = 0;
  const std::vector<double> f = inv_sqrt_weights(lam, etol, rem);
  DeviceBuffer<double> d(n * n);
  GemmWorkspace ws;
  spectral_product(n, U, f, d.get(), s, ws);
  VGB_CUDA(cudaMemcpy2DAsync(out, ldo * sizeof(double), d.get(), n * sizeof(double), n * sizeof(double), n,
                             cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
  if (removed) *removed = rem;
}

void aux_pseudo_inv_sqrt_gwbse(int64_t n, const double *S, int64_t lds, const double *V, int64_t ldv,
                               double etol, double *out, int64_t ldo, int64_t *removed, cudaStream_t s) {
  VGB_REQUIRE(n >= 1 && lds >= n && ldv >= n && ldo >= n && S && V && out,
              "aux_pseudo_inv_sqrt_gwbse: bad arguments");
  GemmWorkspace ws;
  int64_t rem = 0;
  // S^-1/2 over the overlap eigenvalues >= etol
  std::vector<double> lam, U;
  eig_or_fail(n, copy_square(n, S, lds), lam, U);
  DeviceBuffer<double> Ssqrt(n * n), dV(n * n), T(n * n), ortho(n * n);
  spectral_product(n, U, inv_sqrt_weights(lam, etol, rem), Ssqrt.get(), s, ws);
  // ortho = S^-1/2 V S^-1/2
  VGB_CUDA(cudaMemcpy2DAsync(dV.get(), n * sizeof(double), V, ldv * sizeof(double), n * sizeof(double), n,
                             cudaMemcpyHostToDevice, s));
  GemmDesc a;
  a.M = n; a.N = n; a.K = n;
  a.a_colmajor(Ssqrt.get(), n, false).b_colmajor(dV.get(), n, false).c_colmajor(T.get(), n);
  dgemm(a, s, &ws);
  GemmDesc b;
  b.M = n; b.N = n; b.K = n;
  b.a_colmajor(T.get(), n, false).b_colmajor(Ssqrt.get(), n, false).c_colmajor(ortho.get(), n);
  dgemm(b, s, &ws);
  std::vector<double> O(n * n);
  VGB_CUDA(cudaMemcpyAsync(O.data(), ortho.get(), n * n * sizeof(double), cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
  // Vm1 = V'^-1/2 over its eigenvalues >= etol; result = (Vm1 S^-1/2)^T = S^-1/2 Vm1 (both symmetric)
  std::vector<double> lam2, U2;
  eig_or_fail(n, O, lam2, U2);
  DeviceBuffer<double> Vm1(n * n);
  spectral_product(n, U2, inv_sqrt_weights(lam2, etol, rem), Vm1.get(), s, ws);
  GemmDesc c;  // result(i, j) = (Vm1 Ssqrt)(j, i)
  c.M = n; c.N = n; c.K = n;
  c.a_colmajor(Vm1.get(), n, false).b_colmajor(Ssqrt.get(), n, false);
  c.C = T.get(); c.c_rs = n; c.c_cs = 1;  // stored transposed
  dgemm(c, s, &ws);
  VGB_CUDA(cudaMemcpy2DAsync(out, ldo * sizeof(double), T.get(), n * sizeof(double), n * sizeof(double), n,
                             cudaMemcpyDeviceToHost, s));
  VGB_CUDA(cudaStreamSynchronize(s));
  if (removed) *removed = rem;
}

void fill_3c_mo(const bse_mmn_desc &desc, double *const *slices, const double *ao3c, int64_t nbf,
                const double *C, int64_t ldc, int64_t nmo, cudaStream_t s) {
  const int64_t naux = desc.auxsize, mt = desc.mmax - desc.mmin + 1, nt = desc.nmax - desc.nmin + 1;
  VGB_REQUIRE(naux >= 1 && nbf >= 1 && mt >= 1 && nt >= 1 && ldc >= nbf, "fill_3c_mo: bad sizes");
  VGB_REQUIRE(desc.mmin >= 0 && desc.nmin >= 0 && desc.mmax < nmo && desc.nmax < nmo,
              "fill_3c_mo: MO window outside the orbital coefficients");
  VGB_REQUIRE(slices && ao3c && C, "fill_3c_mo: null input");
  for (int64_t m = 0; m < mt; ++m) VGB_REQUIRE(slices[m] != nullptr, "fill_3c_mo: null Mmn slice");
  // MO coefficients of the two windows, column-major nbf x mt and nbf x nt
  DeviceBuffer<double> Cm(nbf * mt), Cn(nbf * nt);
  VGB_CUDA(cudaMemcpy2DAsync(Cm.get(), nbf * sizeof(double), C + ldc * desc.mmin, ldc * sizeof(double),
                             nbf * sizeof(double), mt, cudaMemcpyHostToDevice, s));
  VGB_CUDA(cudaMemcpy2DAsync(Cn.get(), nbf * sizeof(double), C + ldc * desc.nmin, ldc * sizeof(double),
                             nbf * sizeof(double), nt, cudaMemcpyHostToDevice, s));
  // chunks of auxiliary functions: the AO block, T = A_P Cm and the output rows of <= 1 GB each
  const int64_t per_p = std::max(nbf * nbf, std::max(nbf * mt, nt * mt));
  int64_t pc = std::max<int64_t>(1, std::min<int64_t>(naux, (1LL << 27) / per_p));
  if (const char *e = getenv("VGB_FILL3C_MAX_P")) pc = std::max<int64_t>(1, std::min<int64_t>(pc, atoll(e)));
  DeviceBuffer<double> A(pc * nbf * nbf), T(pc * nbf * mt), R(pc * nt * mt);
  GemmWorkspace ws;
  for (int64_t p0 = 0; p0 < naux; p0 += pc) {
    const int64_t cnt = std::min(pc, naux - p0);
    VGB_CUDA(cudaMemcpyAsync(A.get(), ao3c + p0 * nbf * nbf, cnt * nbf * nbf * sizeof(double),
                             cudaMemcpyHostToDevice, s));
    GemmDesc g;  // T_P (nbf x mt) = A_P Cm
    g.M = nbf; g.N = mt; g.K = nbf;
    g.A = A.get(); g.a_rs = 1; g.a_cs = nbf;
    g.B = Cm.get(); g.b_rs = 1; g.b_cs = nbf;
    g.C = T.get(); g.c_rs = 1; g.c_cs = nbf;
    g.nb1 = cnt; g.a_b1 = nbf * nbf; g.c_b1 = nbf * mt;
    dgemm(g, s, &ws);
    GemmDesc h;  // R[m][p][n] = (Cn^T T_P)(n, m)
    h.M = nt; h.N = mt; h.K = nbf;
    h.A = Cn.get(); h.a_rs = nbf; h.a_cs = 1;
    h.B = T.get(); h.b_rs = 1; h.b_cs = nbf; h.b_b1 = nbf * mt;
    h.C = R.get(); h.c_rs = 1; h.c_cs = cnt * nt; h.c_b1 = nt;
    h.nb1 = cnt;
    dgemm(h, s, &ws);
    // slice m, columns p0 .. p0 + cnt (column-major nt x naux): one contiguous block each
    for (int64_t m = 0; m < mt; ++m)
      VGB_CUDA(cudaMemcpyAsync(slices[m] + p0 * nt, R.get() + m * cnt * nt, cnt * nt * sizeof(double),
                               cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));  // A, T and R are reused by the next chunk
  }
}

// Transition dipoles of BSE states from one spin block (Orbitals::CalcFreeTransition_Dipoles
// and CalcCoupledTransition_Dipoles, xtp/src/libxtp/orbitals.cc:740-800 and 804-877): the
// interlevel dipoles D_i = C_c^T dip_i C_v (ctotal x vtotal, i = x, y, z) as two GEMMs per
// component, then d(i, s) = prefactor sum_{v,c} (X + Y)(v ctotal + c, s) D_i(c, v) as one GEMM
// of the flattened D (dim x 3, the pair index of the eigenvectors) with the states.
void transition_dipoles(const double *ao_dip, int64_t nbf, const double *C, int64_t ldc, int64_t nmo,
                        int64_t vmin, int64_t vtotal, int64_t cmin, int64_t ctotal, const double *X,
                        const double *Y, int64_t ldx, int64_t nstates, double prefactor, bool accumulate,
                        double *dip, cudaStream_t s) {
  VGB_REQUIRE(ao_dip && C && X && dip, "transition_dipoles: null input");
  VGB_REQUIRE(nbf >= 1 && ldc >= nbf && vtotal >= 0 && ctotal >= 0 && nstates >= 0, "transition_dipoles: bad sizes");
  VGB_REQUIRE(vmin >= 0 && cmin >= 0 && vmin + vtotal <= nmo && cmin + ctotal <= nmo,
              "transition_dipoles: BSE window outside the orbital coefficients");
  const int64_t dim = vtotal * ctotal;
  VGB_REQUIRE(ldx >= dim, "transition_dipoles: leading dimension of the states too small");
  std::vector<double> out(3 * (size_t)nstates, 0.0);
  if (dim > 0 && nstates > 0) {
    DeviceBuffer<double> A(3 * nbf * nbf), Cv(nbf * vtotal), Cc(nbf * ctotal), T(nbf * vtotal),
        D(dim * 3), Xd(dim * nstates), R(3 * nstates);
    VGB_CUDA(cudaMemcpyAsync(A.get(), ao_dip, 3 * nbf * nbf * sizeof(double), cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpy2DAsync(Cv.get(), nbf * sizeof(double), C + ldc * vmin, ldc * sizeof(double),
                               nbf * sizeof(double), vtotal, cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpy2DAsync(Cc.get(), nbf * sizeof(double), C + ldc * cmin, ldc * sizeof(double),
                               nbf * sizeof(double), ctotal, cudaMemcpyHostToDevice, s));
    VGB_CUDA(cudaMemcpy2DAsync(Xd.get(), dim * sizeof(double), X, ldx * sizeof(double), dim * sizeof(double),
                               nstates, cudaMemcpyHostToDevice, s));
    GemmWorkspace ws;
    for (int i = 0; i < 3; ++i) {
      GemmDesc g;  // T (nbf x vtotal) = dip_i C_v
      g.M = nbf; g.N = vtotal; g.K = nbf;
      g.A = A.get() + i * nbf * nbf; g.a_rs = 1; g.a_cs = nbf;
      g.B = Cv.get(); g.b_rs = 1; g.b_cs = nbf;
      g.C = T.get(); g.c_rs = 1; g.c_cs = nbf;
      dgemm(g, s, &ws);
      GemmDesc h;  // D_i (ctotal x vtotal, column-major: the pair index c + ctotal v) = C_c^T T
      h.M = ctotal; h.N = vtotal; h.K = nbf;
      h.A = Cc.get(); h.a_rs = nbf; h.a_cs = 1;
      h.B = T.get(); h.b_rs = 1; h.b_cs = nbf;
      h.C = D.get() + i * dim; h.c_rs = 1; h.c_cs = ctotal;
      dgemm(h, s, &ws);
    }
    for (int pass = 0; pass < (Y ? 2 : 1); ++pass) {
      if (pass == 1)  // the full-BSE states enter as X + Y (orbitals.cc:780-782)
        VGB_CUDA(cudaMemcpy2DAsync(Xd.get(), dim * sizeof(double), Y, ldx * sizeof(double), dim * sizeof(double),
                                   nstates, cudaMemcpyHostToDevice, s));
      GemmDesc r;  // R (3 x nstates) += prefactor D^T (X or Y)
      r.M = 3; r.N = nstates; r.K = dim;
      r.A = D.get(); r.a_rs = dim; r.a_cs = 1;
      r.B = Xd.get(); r.b_rs = 1; r.b_cs = dim;
      r.C = R.get(); r.c_rs = 1; r.c_cs = 3;
      r.alpha = prefactor; r.beta = pass == 0 ? 0.0 : 1.0;
      dgemm(r, s, &ws);
    }
    VGB_CUDA(cudaMemcpyAsync(out.data(), R.get(), 3 * nstates * sizeof(double), cudaMemcpyDeviceToHost, s));
    VGB_CUDA(cudaStreamSynchronize(s));
  }
  for (int64_t t = 0; t < 3 * nstates; ++t) dip[t] = accumulate ? dip[t] + out[t] : out[t];
}

}  // namespace vgb
