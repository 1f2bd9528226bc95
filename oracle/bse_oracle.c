/*
 * CPU oracle for the BSE matrix-free Hamiltonian product.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this file; only the test-suite, the smoke check and the CPU-baseline
 * leg of the benchmark use it, and only to compare results against or as the
 * timed CPU reference.
 *
 * This is a plain-C restatement of VOTCA-XTP's CPU code path for
 *   BSE_OPERATOR<cqp,cx,cd,cd2>::matmul      xtp/src/libxtp/gwbse/bse_operator.cc:39-119
 *   BSE_OPERATOR<...>::Hqp_row               xtp/src/libxtp/gwbse/bse_operator.cc:121-131
 *   BSE_OPERATOR<...>::diagonal              xtp/src/libxtp/gwbse/bse_operator.cc:133-175
 * with the CPU branches of the OpenMP_CUDA helpers it drives
 *   PrepareMatrix1  xtp/src/libxtp/openmp_cuda.cc:299-316  (Temp *= diag(eps_inv))
 *   PrepareMatrix2  xtp/src/libxtp/openmp_cuda.cc:334-369  (row += Temp * M^T, Hd2 variant)
 *   Addvec          xtp/src/libxtp/openmp_cuda.cc:371-386
 *   MultiplyRow     xtp/src/libxtp/openmp_cuda.cc:388-407  (out.row(I) = row^T * X)
 *   MultiplyBlocks  xtp/src/libxtp/openmp_cuda.cc:442-478  (v1<=v2 c x c blocks of Hx)
 *   getReductionVar xtp/src/libxtp/openmp_cuda.cc:480-493  (sum of per-thread accumulators)
 * and the pair index of xtp/include/votca/xtp/vc2index.h:42-44 (I = ctotal*v + c).
 *
 * The loop nest is the reference's: every row of Hd (or Hd2) plus the Hqp row
 * is built explicitly for each (c1, v1) and multiplied with X; Hx is rebuilt as
 * c x c blocks for every v1 <= v2 pair.  A factorised product with the same
 * numbers is provided separately (oracle_bse_matmul_fact) for mid-size checks.
 *
 * Mmn layout (the reference's std::vector<Eigen::MatrixXd>, slices stored one
 * after another): element M(m, n, P) of slice m, row n, aux column P is
 *   mmn[m * (nn * naux) + P * nn + n]          (each slice column-major nn x naux)
 * with m, n counted from rpamin (TCMatrix_gwbse::Initialize, threecenter.cc:29-48).
 * Hqp is column-major with leading dimension ldh; only its leading
 * (vt + ct) x (vt + ct) window is read, occupied levels first.
 * X and Y are column-major dim x k with leading dimensions ldx, ldy.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef long long i64;

static inline double mget(const double *mmn, i64 nn, i64 naux, i64 m, i64 n,
                          i64 P) {
  return mmn[m * (nn * naux) + P * nn + n];
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

void oracle_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

/* Two doubles per vector register (SSE2 on x86-64, ASIMD on aarch64) through GCC's
 * portable vector extensions: no target intrinsics, unaligned loads through memcpy.  The
 * reference's CPU path runs Eigen's vectorised GEMM here; scalar dot products would
 * understate it several-fold. */
typedef double v2d __attribute__((vector_size(16)));
static inline v2d ld2(const double *p) {
  v2d r;
  memcpy(&r, p, sizeof r);
  return r;
}
static inline double hsum(v2d a) { return a[0] + a[1]; }

/* sum_p a[p] b[p], four independent vector partial sums */
static double dot(const double *a, const double *b, i64 n) {
  v2d s0 = {0.0, 0.0}, s1 = s0, s2 = s0, s3 = s0;
  i64 p = 0;
  for (; p + 8 <= n; p += 8) {
    s0 += ld2(a + p) * ld2(b + p);
    s1 += ld2(a + p + 2) * ld2(b + p + 2);
    s2 += ld2(a + p + 4) * ld2(b + p + 4);
    s3 += ld2(a + p + 6) * ld2(b + p + 6);
  }
  double s = hsum((s0 + s1) + (s2 + s3));
  for (; p < n; ++p) s += a[p] * b[p];
  return s;
}

/* C (rows_a x rows_b, column-major, ldc) += A * B^T with A (rows_a x K) and B (rows_b x K)
 * both row-major (K contiguous).  K is processed in chunks of KB so that a chunk of B stays in
 * the core's cache while the 4 x 4 register blocks sweep A; within a block, 16 vector partial
 * sums over K. */
enum { KB = 128 };
static void gemm_abt(i64 rows_a, i64 rows_b, i64 K, const double *A,
                     const double *B, double *C, i64 ldc) {
  for (i64 k0 = 0; k0 < K; k0 += KB) {
    const i64 kn = K - k0 < KB ? K - k0 : KB;
    i64 i = 0;
    for (; i + 4 <= rows_a; i += 4) {
      const double *a0 = A + (i + 0) * K + k0, *a1 = A + (i + 1) * K + k0,
                   *a2 = A + (i + 2) * K + k0, *a3 = A + (i + 3) * K + k0;
      i64 j = 0;
      for (; j + 4 <= rows_b; j += 4) {
        const double *b0 = B + (j + 0) * K + k0, *b1 = B + (j + 1) * K + k0,
                     *b2 = B + (j + 2) * K + k0, *b3 = B + (j + 3) * K + k0;
        v2d c00 = {0.0, 0.0}, c01 = c00, c02 = c00, c03 = c00, c10 = c00, c11 = c00,
            c12 = c00, c13 = c00, c20 = c00, c21 = c00, c22 = c00, c23 = c00, c30 = c00,
            c31 = c00, c32 = c00, c33 = c00;
        i64 p = 0;
        for (; p + 2 <= kn; p += 2) {
          const v2d x0 = ld2(a0 + p), x1 = ld2(a1 + p), x2 = ld2(a2 + p), x3 = ld2(a3 + p);
          const v2d y0 = ld2(b0 + p), y1 = ld2(b1 + p), y2 = ld2(b2 + p), y3 = ld2(b3 + p);
          c00 += x0 * y0; c01 += x0 * y1; c02 += x0 * y2; c03 += x0 * y3;
          c10 += x1 * y0; c11 += x1 * y1; c12 += x1 * y2; c13 += x1 * y3;
          c20 += x2 * y0; c21 += x2 * y1; c22 += x2 * y2; c23 += x2 * y3;
          c30 += x3 * y0; c31 += x3 * y1; c32 += x3 * y2; c33 += x3 * y3;
        }
        double r[4][4] = {{hsum(c00), hsum(c01), hsum(c02), hsum(c03)},
                          {hsum(c10), hsum(c11), hsum(c12), hsum(c13)},
                          {hsum(c20), hsum(c21), hsum(c22), hsum(c23)},
                          {hsum(c30), hsum(c31), hsum(c32), hsum(c33)}};
        for (; p < kn; ++p) {
          const double x[4] = {a0[p], a1[p], a2[p], a3[p]};
          const double y[4] = {b0[p], b1[p], b2[p], b3[p]};
          for (int ii = 0; ii < 4; ++ii)
            for (int jj = 0; jj < 4; ++jj) r[ii][jj] += x[ii] * y[jj];
        }
        for (int jj = 0; jj < 4; ++jj)
          for (int ii = 0; ii < 4; ++ii) C[(i + ii) + (j + jj) * ldc] += r[ii][jj];
      }
      for (; j < rows_b; ++j) {
        const double *b0 = B + j * K + k0;
        C[(i + 0) + j * ldc] += dot(a0, b0, kn);
        C[(i + 1) + j * ldc] += dot(a1, b0, kn);
        C[(i + 2) + j * ldc] += dot(a2, b0, kn);
        C[(i + 3) + j * ldc] += dot(a3, b0, kn);
      }
    }
    for (; i < rows_a; ++i)
      for (i64 j = 0; j < rows_b; ++j) C[i + j * ldc] += dot(A + i * K + k0, B + j * K + k0, kn);
  }
}

/* Copy the rows [n0, n0+cnt) of slice m into a P-contiguous buffer out[r*naux + P],
 * scaled by s (and by w[P] when w != NULL). */
static void slice_rows_T(const double *mmn, i64 nn, i64 naux, i64 m, i64 n0,
                         i64 cnt, double s, const double *w, double *out) {
  for (i64 P = 0; P < naux; ++P) {
    const double *col = mmn + m * (nn * naux) + P * nn + n0;
    double f = w ? s * w[P] : s;
    for (i64 r = 0; r < cnt; ++r) out[r * naux + P] = f * col[r];
  }
}

/*
 * Reference loop nest.  c1 in [c1_lo, c1_hi) for the Hd/Hd2/Hqp row stage and
 * v1 in [v1_lo, v1_hi) for the Hx block stage (full ranges reproduce the
 * reference; sub-ranges exist so that a bounded slice of the CPU work can be
 * timed).  Rows of Y outside the c1 range receive only the Hx contribution.
 */
void oracle_bse_matmul_ref(const double *mmn, i64 nm, i64 nn, i64 naux,
                           const double *w, const double *hqp, i64 ldh, i64 vt,
                           i64 ct, i64 voff, i64 coff, int cqp, int cx, int cd,
                           int cd2, const double *X, i64 ldx, i64 k, double *Y,
                           i64 ldy, i64 c1_lo, i64 c1_hi, i64 v1_lo,
                           i64 v1_hi) {
  (void)nm;
  const i64 dim = vt * ct;
  for (i64 j = 0; j < k; ++j) memset(Y + j * ldy, 0, sizeof(double) * dim);
  const int nthreads = oracle_num_threads();
  /* per-thread reduction buffers, summed at the end (getReductionVar) */
  double *reduce = (double *)calloc((size_t)nthreads * dim * k, sizeof(double));

#pragma omp parallel
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    double *red = reduce + (size_t)tid * dim * k;
    double *row = (double *)malloc(sizeof(double) * dim);
    /* Temp(c, P) (or Temp(v, P) for Hd2) after PrepareMatrix1 */
    i64 rows1 = cd != 0 ? ct : vt;
    double *temp = (double *)malloc(sizeof(double) * rows1 * naux);
    i64 rows2 = cd != 0 ? vt : ct;
    double *mat2 = (double *)malloc(sizeof(double) * rows2 * naux);

#pragma omp for schedule(dynamic)
    for (i64 c1 = c1_lo; c1 < c1_hi; ++c1) {
      if (cd != 0) /* Temp = -cd * Mmn[c1+cmin].middleRows(cmin, ct) * diag(w) */
        slice_rows_T(mmn, nn, naux, c1 + coff, coff, ct, -(double)cd, w, temp);
      else if (cd2 != 0) /* Temp = -cd2 * Mmn[c1+cmin].middleRows(vmin, vt) * diag(w) */
        slice_rows_T(mmn, nn, naux, c1 + coff, voff, vt, -(double)cd2, w, temp);

      for (i64 v1 = 0; v1 < vt; ++v1) {
        memset(row, 0, sizeof(double) * dim); /* SetTempZero */
        if (cd != 0) {
          /* row (ct x vt) += Temp * Mmn[v1+vmin].middleRows(vmin, vt)^T */
          slice_rows_T(mmn, nn, naux, v1 + voff, voff, vt, 1.0, NULL, mat2);
          gemm_abt(ct, vt, naux, temp, mat2, row, ct);
        }
        if (cd2 != 0) {
          /* row (ct x vt) += Mmn[v1+vmin].middleRows(cmin, ct) * Temp^T */
          slice_rows_T(mmn, nn, naux, v1 + voff, coff, ct, 1.0, NULL, mat2);
          gemm_abt(ct, vt, naux, mat2, temp, row, ct);
        }
        if (cqp != 0) {
          /* Hqp_row(v1, c1): column v1 gets +Hqp(vt+c, vt+c1), row c1 gets -Hqp(v, v1) */
          for (i64 c = 0; c < ct; ++c)
            row[c + ct * v1] += cqp * hqp[(vt + c) + (vt + c1) * ldh];
          for (i64 v = 0; v < vt; ++v)
            row[c1 + ct * v] -= cqp * hqp[v + v1 * ldh];
        }
        /* MultiplyRow: reduce.row(I(v1,c1)) = row^T * X */
        i64 I = ct * v1 + c1;
        for (i64 j = 0; j < k; ++j) {
          const double *xj = X + j * ldx;
          red[I + j * dim] = dot(row, xj, dim);
        }
      }
    }

    if (cx != 0) {
      double *m1 = (double *)malloc(sizeof(double) * ct * naux);
      double *m2 = (double *)malloc(sizeof(double) * ct * naux);
      double *blk = (double *)malloc(sizeof(double) * ct * ct);
#pragma omp for schedule(dynamic)
      for (i64 v1 = v1_lo; v1 < v1_hi; ++v1) {
        /* PushMatrix1: cx * Mmn[v1+vmin].middleRows(cmin, ct) */
        slice_rows_T(mmn, nn, naux, v1 + voff, coff, ct, (double)cx, NULL, m1);
        for (i64 v2 = v1; v2 < vt; ++v2) {
          slice_rows_T(mmn, nn, naux, v2 + voff, coff, ct, 1.0, NULL, m2);
          memset(blk, 0, sizeof(double) * ct * ct);
          gemm_abt(ct, ct, naux, m1, m2, blk, ct); /* blk(c,c') col-major */
          for (i64 j = 0; j < k; ++j) {
            const double *x2 = X + j * ldx + v2 * ct;
            const double *x1 = X + j * ldx + v1 * ct;
            double *r1 = red + j * dim + v1 * ct;
            double *r2 = red + j * dim + v2 * ct;
            for (i64 cc = 0; cc < ct; ++cc) { /* r1 += blk * x2 */
              double xv = x2[cc];
              const double *bcol = blk + cc * ct;
              for (i64 c = 0; c < ct; ++c) r1[c] += bcol[c] * xv;
            }
            if (v1 != v2) { /* r2 += blk^T * x1 */
              for (i64 cc = 0; cc < ct; ++cc) {
                r2[cc] += dot(blk + cc * ct, x1, ct);
              }
            }
          }
        }
      }
      free(m1); free(m2); free(blk);
    }
    free(row); free(temp); free(mat2);
  }
  /* getReductionVar */
  for (int t = 0; t < nthreads; ++t) {
    const double *red = reduce + (size_t)t * dim * k;
    for (i64 j = 0; j < k; ++j)
      for (i64 q = 0; q < dim; ++q) Y[q + j * ldy] += red[q + j * dim];
  }
  free(reduce);
}

/*
 * Selected rows of the same product: Yr(r, j) = (H X)(rows[r], j) for r < nrows,
 * Yr column-major nrows x k (ld nrows).  Each row is built as the reference builds
 * it: the Hd (or Hd2) row from PrepareMatrix1/PrepareMatrix2 and the Hqp row
 * (bse_operator.cc:61-93, openmp_cuda.cc:299-369), and the row of the Hx blocks
 * that MultiplyBlocks applies (bse_operator.cc:98-116, openmp_cuda.cc:442-478:
 * block (v1, v2) = cx Mmn[v1].middleRows(cmin, ct) Mmn[v2].middleRows(cmin, ct)^T,
 * row c1 of it for v2 >= v1 and of its transpose for v2 < v1, the same numbers);
 * then MultiplyRow's row^T X.  The cost per row is O(dim * naux), so rows of
 * products far too large for the full loop nest can be checked.
 */
void oracle_bse_matmul_rows(const double *mmn, i64 nm, i64 nn, i64 naux,
                            const double *w, const double *hqp, i64 ldh, i64 vt,
                            i64 ct, i64 voff, i64 coff, int cqp, int cx, int cd,
                            int cd2, const double *X, i64 ldx, i64 k,
                            const i64 *rows, i64 nrows, double *Yr) {
  (void)nm;
  const i64 dim = vt * ct;
#pragma omp parallel
  {
    double *row = (double *)malloc(sizeof(double) * dim);
    double *temp = (double *)malloc(sizeof(double) * (ct > vt ? ct : vt) * naux);
    double *mat2 = (double *)malloc(sizeof(double) * (ct > vt ? ct : vt) * naux);
    double *m1 = (double *)malloc(sizeof(double) * naux);
#pragma omp for schedule(dynamic)
    for (i64 r = 0; r < nrows; ++r) {
      const i64 I = rows[r], v1 = I / ct, c1 = I % ct;
      memset(row, 0, sizeof(double) * dim);
      if (cd != 0) {
        slice_rows_T(mmn, nn, naux, c1 + coff, coff, ct, -(double)cd, w, temp);
        slice_rows_T(mmn, nn, naux, v1 + voff, voff, vt, 1.0, NULL, mat2);
        gemm_abt(ct, vt, naux, temp, mat2, row, ct);
      }
      if (cd2 != 0) {
        slice_rows_T(mmn, nn, naux, c1 + coff, voff, vt, -(double)cd2, w, temp);
        slice_rows_T(mmn, nn, naux, v1 + voff, coff, ct, 1.0, NULL, mat2);
        gemm_abt(ct, vt, naux, mat2, temp, row, ct);
      }
      if (cqp != 0) {
        for (i64 c = 0; c < ct; ++c) row[c + ct * v1] += cqp * hqp[(vt + c) + (vt + c1) * ldh];
        for (i64 v = 0; v < vt; ++v) row[c1 + ct * v] -= cqp * hqp[v + v1 * ldh];
      }
      if (cx != 0) {
        slice_rows_T(mmn, nn, naux, v1 + voff, coff + c1, 1, (double)cx, NULL, m1);
        for (i64 v2 = 0; v2 < vt; ++v2) {
          slice_rows_T(mmn, nn, naux, v2 + voff, coff, ct, 1.0, NULL, mat2);
          gemm_abt(1, ct, naux, m1, mat2, row + ct * v2, 1);
        }
      }
      for (i64 j = 0; j < k; ++j) Yr[r + j * nrows] = dot(row, X + j * ldx, dim);
    }
    free(row); free(temp); free(mat2); free(m1);
  }
}

/* BSE_OPERATOR::diagonal, bse_operator.cc:133-175 */
void oracle_bse_diagonal(const double *mmn, i64 nm, i64 nn, i64 naux,
                         const double *w, const double *hqp, i64 ldh, i64 vt,
                         i64 ct, i64 voff, i64 coff, int cqp, int cx, int cd,
                         int cd2, double *D) {
  (void)nm;
#pragma omp parallel for schedule(dynamic)
  for (i64 v = 0; v < vt; ++v) {
    for (i64 c = 0; c < ct; ++c) {
      double entry = 0.0;
      if (cx != 0) {
        double s = 0;
        for (i64 P = 0; P < naux; ++P) {
          double x = mget(mmn, nn, naux, v + voff, coff + c, P);
          s += x * x;
        }
        entry += cx * s;
      }
      if (cqp != 0)
        entry += cqp * (hqp[(c + vt) + (c + vt) * ldh] - hqp[v + v * ldh]);
      if (cd != 0) {
        double s = 0;
        for (i64 P = 0; P < naux; ++P)
          s += mget(mmn, nn, naux, c + coff, c + coff, P) * w[P] *
               mget(mmn, nn, naux, v + voff, v + voff, P);
        entry -= cd * s;
      }
      if (cd2 != 0) {
        double s = 0;
        for (i64 P = 0; P < naux; ++P)
          s += mget(mmn, nn, naux, c + coff, v + voff, P) * w[P] *
               mget(mmn, nn, naux, v + voff, c + coff, P);
        entry -= cd2 * s;
      }
      D[ct * v + c] = entry;
    }
  }
}

/*
 * Factorised FP64 product with the same numbers as the loop nest above
 * (contraction over the auxiliary index first):
 *   (Hx X)_{v1 c1}  = sum_P M(v1,c1,P) * sum_{v c} M(v,c,P) X_{v c}
 *   (Hd X)_{v1 c1}  = sum_P w_P sum_v M(v1,v,P) sum_c M(c1,c,P) X_{v c}
 *   (Hd2 X)_{v1 c1} = sum_P w_P sum_v M(c1,v,P) sum_c M(v1,c,P) X_{v c}
 *   (Hqp X)_{v1 c1} = sum_c Hqp(vt+c, vt+c1) X_{v1 c} - sum_v Hqp(v, v1) X_{v c1}
 * out = cqp*Hqp + cx*Hx - cd*Hd - cd2*Hd2.
 */
void oracle_bse_matmul_fact(const double *mmn, i64 nm, i64 nn, i64 naux,
                            const double *w, const double *hqp, i64 ldh,
                            i64 vt, i64 ct, i64 voff, i64 coff, int cqp,
                            int cx, int cd, int cd2, const double *X, i64 ldx,
                            i64 k, double *Y, i64 ldy) {
  (void)nm;
  const i64 dim = vt * ct;
#pragma omp parallel for schedule(dynamic)
  for (i64 j = 0; j < k; ++j) {
    const double *x = X + j * ldx;
    double *y = Y + j * ldy;
    for (i64 q = 0; q < dim; ++q) y[q] = 0.0;
    double *t = (double *)malloc(sizeof(double) * dim);
    for (i64 P = 0; P < naux; ++P) {
      if (cx != 0) {
        double z = 0;
        for (i64 v = 0; v < vt; ++v)
          z += dot(&mmn[(v + voff) * (nn * naux) + P * nn + coff], x + ct * v, ct);
        z *= cx;
        for (i64 v = 0; v < vt; ++v)
          for (i64 c = 0; c < ct; ++c)
            y[ct * v + c] += mget(mmn, nn, naux, v + voff, c + coff, P) * z;
      }
      if (cd != 0) {
        /* t[v][c1] = sum_c M(c1,c,P) x[v][c]  (row c1 of slice P contiguous in c) */
        for (i64 v = 0; v < vt; ++v)
          for (i64 c1 = 0; c1 < ct; ++c1)
            t[ct * v + c1] = dot(&mmn[(c1 + coff) * (nn * naux) + P * nn + coff], x + ct * v, ct);
        double f = cd * w[P];
        for (i64 v1 = 0; v1 < vt; ++v1)
          for (i64 v = 0; v < vt; ++v) {
            double a = f * mget(mmn, nn, naux, v1 + voff, v + voff, P);
            for (i64 c1 = 0; c1 < ct; ++c1) y[ct * v1 + c1] -= a * t[ct * v + c1];
          }
      }
      if (cd2 != 0) {
        /* u[v1][v] = sum_c M(v1,c,P) x[v][c] */
        for (i64 v1 = 0; v1 < vt; ++v1)
          for (i64 v = 0; v < vt; ++v)
            t[vt * v1 + v] = dot(&mmn[(v1 + voff) * (nn * naux) + P * nn + coff], x + ct * v, ct);
        double f = cd2 * w[P];
        for (i64 v1 = 0; v1 < vt; ++v1)
          for (i64 c1 = 0; c1 < ct; ++c1)
            y[ct * v1 + c1] -= f * dot(&mmn[(c1 + coff) * (nn * naux) + P * nn + voff], t + vt * v1, vt);
      }
    }
    if (cqp != 0) {
      for (i64 v1 = 0; v1 < vt; ++v1)
        for (i64 c1 = 0; c1 < ct; ++c1) {
          double s = 0;
          for (i64 c = 0; c < ct; ++c)
            s += hqp[(vt + c) + (vt + c1) * ldh] * x[ct * v1 + c];
          for (i64 v = 0; v < vt; ++v) s -= hqp[v + v1 * ldh] * x[ct * v + c1];
          y[ct * v1 + c1] += cqp * s;
        }
    }
    free(t);
  }
}

/*
 * HamiltonianOperator product, xtp/include/votca/xtp/bseoperator_btda.h:116-149:
 * [[A, B], [-B, -A]] * [M1; M2] computed as A*[M1,M2] and B*[M1,M2] with the
 * input reinterpreted as dim x 2k (columns interleave M1_j, M2_j).
 * Both A and B are BSE operators over the same Mmn; their coefficient sets are
 * (aq, ax, ad, ad2) and (bq, bx, bd, bd2).  X, Y: (2*dim) x k, contiguous.
 */
void oracle_ham_matmul(const double *mmn, i64 nm, i64 nn, i64 naux,
                       const double *w, const double *hqp, i64 ldh, i64 vt,
                       i64 ct, i64 voff, i64 coff, const int *acoef,
                       const int *bcoef, const double *X, i64 k, double *Y,
                       int use_ref_loop) {
  const i64 dim = vt * ct;
  double *ta = (double *)malloc(sizeof(double) * dim * 2 * k);
  double *tb = (double *)malloc(sizeof(double) * dim * 2 * k);
  if (use_ref_loop) {
    oracle_bse_matmul_ref(mmn, nm, nn, naux, w, hqp, ldh, vt, ct, voff, coff,
                          acoef[0], acoef[1], acoef[2], acoef[3], X, dim, 2 * k,
                          ta, dim, 0, ct, 0, vt);
    oracle_bse_matmul_ref(mmn, nm, nn, naux, w, hqp, ldh, vt, ct, voff, coff,
                          bcoef[0], bcoef[1], bcoef[2], bcoef[3], X, dim, 2 * k,
                          tb, dim, 0, ct, 0, vt);
  } else {
    oracle_bse_matmul_fact(mmn, nm, nn, naux, w, hqp, ldh, vt, ct, voff, coff,
                           acoef[0], acoef[1], acoef[2], acoef[3], X, dim,
                           2 * k, ta, dim);
    oracle_bse_matmul_fact(mmn, nm, nn, naux, w, hqp, ldh, vt, ct, voff, coff,
                           bcoef[0], bcoef[1], bcoef[2], bcoef[3], X, dim,
                           2 * k, tb, dim);
  }
  /* temp_unshaped(2dim x k): column j = [T_{2j}; T_{2j+1}] */
  for (i64 j = 0; j < k; ++j) {
    const double *a_top = ta + (2 * j) * dim, *a_bot = ta + (2 * j + 1) * dim;
    const double *b_top = tb + (2 * j) * dim, *b_bot = tb + (2 * j + 1) * dim;
    double *y = Y + j * 2 * dim;
    for (i64 q = 0; q < dim; ++q) {
      y[q] = a_top[q] + b_bot[q];
      y[dim + q] = -a_bot[q] - b_top[q];
    }
  }
  free(ta);
  free(tb);
}
