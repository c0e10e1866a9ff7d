/*
 * CPU oracle for the LACE preconditioned-solve path.  TEST INFRASTRUCTURE:
 * see lace_oracle.h for who may use it.  Every routine cites the LACE source
 * lines (paths inside the LACE source tree) it restates.
 *
 * Built with -ffp-contract=off so that x86-64 and aarch64 produce identical
 * results, and so that the one-thread restatements reproduce LACE's own
 * arithmetic operation by operation.
 */
#include "lace_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static int g_threads = 1;

void orc_set_threads(int n) {
  g_threads = n > 0 ? n : 1;
#ifdef _OPENMP
  omp_set_num_threads(g_threads);
#endif
}
int orc_get_threads(void) { return g_threads; }

#define MINI(a, b) ((a) < (b) ? (a) : (b))

/* mysgn (include/sparse.h:1129-1133): +1 for v >= 0, -1 otherwise */
static double mysgn(double v) { return (double)(v >= 0.0) - (double)(v < 0.0); }

/* ================================================================ ParILU */

double orc_parilu_sweep(int mode, int nnzA, const int *Arowidx, const int *Acol,
                        const double *Aval, const int *Lrow, const int *Lcol,
                        const double *Lold, double *Lnew, const int *Ucolptr,
                        const int *Urowidx, const double *Uold, double *Unew) {
  double step = 0.0;
  if (mode == 0) {
    /* src/parilu_v0_3.cpp:70-102, executed in the one-thread order */
    double *Lv = Lnew, *Uv = Unew; /* in place: Lold/Uold are not read */
    (void)Lold;
    (void)Uold;
    double sp = 0.0;
    for (int k = 0; k < nnzA; k++) {
      int i = Arowidx[k], j = Acol[k];
      double s = Aval[k];
      int il = Lrow[i], iu = Ucolptr[j];
      while (il < Lrow[i + 1] && iu < Ucolptr[j + 1]) {
        sp = 0.0;
        int jl = Lcol[il], ju = Urowidx[iu];
        sp = (jl == ju) ? Lv[il] * Uv[iu] : sp;
        s = (jl == ju) ? s - sp : s;
        il = (jl <= ju) ? il + 1 : il;
        iu = (jl >= ju) ? iu + 1 : iu;
      }
      s += sp; /* :90, undo the last (diagonal) product */
      if (i > j) {
        double tmp = s / Uv[Ucolptr[j + 1] - 1];
        step += pow(Lv[il - 1] - tmp, 2);
        Lv[il - 1] = tmp;
      } else {
        double tmp = s;
        step += pow(Uv[iu - 1] - tmp, 2);
        Uv[iu - 1] = tmp;
      }
    }
    return step;
  }
  if (mode == 2) {
    /* src/parilu_v0_3.cpp:66-102 as LACE runs it: in place, entries split
     * statically over the OpenMP threads (racy across the threads' ranges,
     * as LACE's own loop) */
    double *Lv = Lnew, *Uv = Unew;
    (void)Lold;
    (void)Uold;
#pragma omp parallel for schedule(static) reduction(+ : step)
    for (int k = 0; k < nnzA; k++) {
      int i = Arowidx[k], j = Acol[k];
      double s = Aval[k], sp = 0.0;
      int il = Lrow[i], iu = Ucolptr[j];
      while (il < Lrow[i + 1] && iu < Ucolptr[j + 1]) {
        sp = 0.0;
        int jl = Lcol[il], ju = Urowidx[iu];
        sp = (jl == ju) ? Lv[il] * Uv[iu] : sp;
        s = (jl == ju) ? s - sp : s;
        il = (jl <= ju) ? il + 1 : il;
        iu = (jl >= ju) ? iu + 1 : iu;
      }
      s += sp;
      if (i > j) {
        double tmp = s / Uv[Ucolptr[j + 1] - 1];
        step += pow(Lv[il - 1] - tmp, 2);
        Lv[il - 1] = tmp;
      } else {
        double tmp = s;
        step += pow(Uv[iu - 1] - tmp, 2);
        Uv[iu - 1] = tmp;
      }
    }
    return step;
  }
  /* synchronous sweep: same update formula (:70-101) evaluated from the
   * previous iterate, sum over k < min(i,j) only */
#pragma omp parallel for schedule(static) reduction(+ : step)
  for (int k = 0; k < nnzA; k++) {
    int i = Arowidx[k], j = Acol[k];
    int kmax = i < j ? i : j;
    double s = Aval[k];
    int il = Lrow[i], iu = Ucolptr[j];
    const int le = Lrow[i + 1], ue = Ucolptr[j + 1];
    while (il < le && iu < ue) {
      int jl = Lcol[il], ju = Urowidx[iu];
      if (jl >= kmax || ju >= kmax) break;
      if (jl == ju) { s -= Lold[il] * Uold[iu]; il++; iu++; }
      else if (jl < ju) il++;
      else iu++;
    }
    if (i > j) {
      while (Lcol[il] != j) il++;
      double tmp = s / Uold[ue - 1];
      double d = Lold[il] - tmp;
      step += d * d;
      Lnew[il] = tmp;
    } else {
      while (Urowidx[iu] != i) iu++;
      double d = Uold[iu] - s;
      step += d * d;
      Unew[iu] = s;
    }
  }
  return step;
}

double orc_parilu_sweep_sync_f32(int nnzA, const int *Arowidx, const int *Acol,
                                 const double *Aval, const int *Lrow,
                                 const int *Lcol, const float *Lold, float *Lnew,
                                 const int *Ucolptr, const int *Urowidx,
                                 const float *Uold, float *Unew) {
  double step = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : step)
  for (int k = 0; k < nnzA; k++) {
    int i = Arowidx[k], j = Acol[k];
    int kmax = i < j ? i : j;
    float s = (float)Aval[k];
    int il = Lrow[i], iu = Ucolptr[j];
    const int le = Lrow[i + 1], ue = Ucolptr[j + 1];
    while (il < le && iu < ue) {
      int jl = Lcol[il], ju = Urowidx[iu];
      if (jl >= kmax || ju >= kmax) break;
      if (jl == ju) { s -= Lold[il] * Uold[iu]; il++; iu++; }
      else if (jl < ju) il++;
      else iu++;
    }
    if (i > j) {
      while (Lcol[il] != j) il++;
      float tmp = s / Uold[ue - 1];
      double d = (double)Lold[il] - (double)tmp;
      step += d * d;
      Lnew[il] = tmp;
    } else {
      while (Urowidx[iu] != i) iu++;
      double d = (double)Uold[iu] - (double)s;
      step += d * d;
      Unew[iu] = s;
    }
  }
  return step;
}

double orc_ilu_nonlinres(int nnzA, const int *Arowidx, const int *Acol,
                         const double *Aval, const int *Lrow, const int *Lcol,
                         const double *Lval, const int *Ucolptr,
                         const int *Urowidx, const double *Uval) {
  double acc = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : acc)
  for (int k = 0; k < nnzA; k++) {
    int i = Arowidx[k], j = Acol[k];
    double t = 0.0;
    int il = Lrow[i], iu = Ucolptr[j];
    while (il < Lrow[i + 1] && iu < Ucolptr[j + 1]) {
      int jl = Lcol[il], ju = Urowidx[iu];
      if (jl == ju) { t += Lval[il] * Uval[iu]; il++; iu++; }
      else if (jl < ju) il++;
      else iu++;
    }
    double d = t - Aval[k];
    acc += d * d;
  }
  return sqrt(acc);
}

void orc_zilures(int n, const int *Arow, const int *Acol, const double *Aval,
                 const int *Lrow, const int *Lcol, const double *Lval,
                 const int *Urow, const int *Ucol, const double *Uval,
                 double *res, double *nonlinres) {
  /* control/norms.cpp:301-405: LU = L*U (row by row), subtract A on its
   * pattern, res over all of LU's pattern, nonlinres over S(A) */
  double *acc = (double *)calloc((size_t)n, sizeof(double));
  int *mark = (int *)malloc(sizeof(int) * (size_t)n);
  int *list = (int *)malloc(sizeof(int) * (size_t)n);
  for (int c = 0; c < n; ++c) mark[c] = -1;
  double r = 0.0, nl = 0.0;
  for (int i = 0; i < n; ++i) {
    int cnt = 0;
    for (int p = Lrow[i]; p < Lrow[i + 1]; ++p) {
      int k = Lcol[p];
      double lik = (k == i) ? 1.0 : Lval[p];
      for (int q = Urow[k]; q < Urow[k + 1]; ++q) {
        int j = Ucol[q];
        if (mark[j] != i) { mark[j] = i; acc[j] = 0.0; list[cnt++] = j; }
        acc[j] += lik * Uval[q];
      }
    }
    for (int p = Arow[i]; p < Arow[i + 1]; ++p) {
      int j = Acol[p];
      if (mark[j] == i) {
        double t = acc[j] - Aval[p];
        acc[j] = t;
        nl += t * t;
      }
    }
    for (int a = 0; a < cnt; ++a) r += acc[list[a]] * acc[list[a]];
  }
  *res = sqrt(r);
  *nonlinres = sqrt(nl);
  free(acc);
  free(mark);
  free(list);
}

/* ================================================================== SpMV */

void orc_spmv(int n, const int *row, const int *col, const double *val,
              double alpha, const double *x, double beta, double *y) {
#pragma omp parallel for schedule(static)
  for (int i = 0; i < n; ++i) {
    double s = 0.0;
    for (int p = row[i]; p < row[i + 1]; ++p) s += val[p] * x[col[p]];
    y[i] = (beta == 0.0) ? alpha * s : alpha * s + beta * y[i];
  }
}

void orc_bcsr_spmv(int nbrows, int bs, const int *row, const int *col,
                   const double *val, const double *x, double *y) {
  const int ld = bs * bs;
#pragma omp parallel for schedule(static)
  for (int I = 0; I < nbrows; ++I) {
    for (int r = 0; r < bs; ++r) {
      double s = 0.0;
      for (int p = row[I]; p < row[I + 1]; ++p) {
        const double *blk = val + (size_t)p * ld + r * bs;
        const double *xj = x + (size_t)col[p] * bs;
        for (int c = 0; c < bs; ++c) s += blk[c] * xj[c];
      }
      y[(size_t)I * bs + r] = s;
    }
  }
}

/* ===================================================== triangular solves */

void orc_trsv(int n, const int *row, const int *col, const double *val,
              int lower, int unit, const double *b, double *x) {
  if (lower) {
    for (int i = 0; i < n; ++i) {
      double s = b[i], d = 1.0;
      for (int p = row[i]; p < row[i + 1]; ++p) {
        int j = col[p];
        if (j < i) s -= val[p] * x[j];
        else if (j == i) d = val[p];
      }
      x[i] = unit ? s : s / d;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      double s = b[i], d = 1.0;
      for (int p = row[i]; p < row[i + 1]; ++p) {
        int j = col[p];
        if (j > i) s -= val[p] * x[j];
        else if (j == i) d = val[p];
      }
      x[i] = unit ? s : s / d;
    }
  }
}

void orc_trsv_f32(int n, const int *row, const int *col, const float *val,
                  int lower, int unit, const float *b, float *x) {
  if (lower) {
    for (int i = 0; i < n; ++i) {
      float s = b[i], d = 1.0f;
      for (int p = row[i]; p < row[i + 1]; ++p) {
        int j = col[p];
        if (j < i) s -= val[p] * x[j];
        else if (j == i) d = val[p];
      }
      x[i] = unit ? s : s / d;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      float s = b[i], d = 1.0f;
      for (int p = row[i]; p < row[i + 1]; ++p) {
        int j = col[p];
        if (j > i) s -= val[p] * x[j];
        else if (j == i) d = val[p];
      }
      x[i] = unit ? s : s / d;
    }
  }
}

int orc_levels(int n, const int *row, const int *col, int lower, int *lev) {
  int nlev = 0;
  if (lower) {
    for (int i = 0; i < n; ++i) {
      int l = 0;
      for (int p = row[i]; p < row[i + 1]; ++p)
        if (col[p] < i && lev[col[p]] + 1 > l) l = lev[col[p]] + 1;
      lev[i] = l;
      if (l + 1 > nlev) nlev = l + 1;
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int l = 0;
      for (int p = row[i]; p < row[i + 1]; ++p)
        if (col[p] > i && lev[col[p]] + 1 > l) l = lev[col[p]] + 1;
      lev[i] = l;
      if (l + 1 > nlev) nlev = l + 1;
    }
  }
  return nlev;
}

int orc_parcsrtrsv(int uplo, int n, const double *val, const int *row,
                   const int *col, const double *rhs, double *y, double tol,
                   int *iter) {
  /* src/trisolve.cpp:264-297 (lower) and :306-340 (upper), one thread */
  *iter = 0;
  double step = 1.e8;
  if (uplo == 0) {
    while (step > tol && isfinite(step)) {
      step = 0.0;
      for (int i = 0; i < n; i++) {
        double tmp = 0.0;
        for (int k = row[i]; k < row[i + 1] - 1; k++) tmp += val[k] * y[col[k]];
        tmp = (rhs[i] - tmp) / val[row[i + 1] - 1];
        step += pow((y[i] - tmp), 2);
        y[i] = tmp;
      }
      *iter = *iter + 1;
    }
  } else {
    while (step > tol && isfinite(step)) {
      step = 0.0;
      for (int i = n - 1; i >= 0; i--) {
        double tmp = 0.0;
        for (int k = row[i] + 1; k < row[i + 1]; k++) tmp += val[k] * y[col[k]];
        tmp = (rhs[i] - tmp) / val[row[i]];
        step += pow((y[i] - tmp), 2);
        y[i] = tmp;
      }
      *iter = *iter + 1;
    }
  }
  return 0;
}

int orc_jacobi_trsv(int uplo, int n, const double *val, const int *row,
                    const int *col, const double *rhs, double *y, double tol,
                    int maxiter, int *iter) {
  /* synchronous counterpart of src/trisolve.cpp:256-351 */
  double *yn = (double *)malloc(sizeof(double) * (size_t)n);
  double step = 1.e8;
  *iter = 0;
  while (step > tol && isfinite(step) && *iter < maxiter) {
    step = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : step)
    for (int i = 0; i < n; i++) {
      double tmp = 0.0, d;
      if (uplo == 0) {
        for (int k = row[i]; k < row[i + 1] - 1; k++) tmp += val[k] * y[col[k]];
        d = val[row[i + 1] - 1];
      } else {
        for (int k = row[i] + 1; k < row[i + 1]; k++) tmp += val[k] * y[col[k]];
        d = val[row[i]];
      }
      tmp = (rhs[i] - tmp) / d;
      step += (y[i] - tmp) * (y[i] - tmp);
      yn[i] = tmp;
    }
    memcpy(y, yn, sizeof(double) * (size_t)n);
    *iter = *iter + 1;
  }
  free(yn);
  return 0;
}

/* ================================================================== BCSR */

int orc_block_inverse(int bs, const double *a, double *ainv) {
  double w[8 * 16];
  if (bs > 8) return -2;
  const int w2 = 2 * bs;
  for (int r = 0; r < bs; ++r)
    for (int c = 0; c < w2; ++c)
      w[r * w2 + c] = (c < bs) ? a[r * bs + c] : (c - bs == r ? 1.0 : 0.0);
  for (int p = 0; p < bs; ++p) {
    double piv = w[p * w2 + p];
    if (piv == 0.0) return -1;
    double rp = 1.0 / piv;
    for (int c = 0; c < w2; ++c) w[p * w2 + c] *= rp;
    for (int r = 0; r < bs; ++r) {
      if (r == p) continue;
      double f = w[r * w2 + p];
      for (int c = 0; c < w2; ++c) w[r * w2 + c] -= f * w[p * w2 + c];
    }
  }
  for (int r = 0; r < bs; ++r)
    for (int c = 0; c < bs; ++c) ainv[r * bs + c] = w[r * w2 + bs + c];
  return 0;
}

/* C = A*B for bs x bs row-major blocks (the data_dgemm_mkl call at
 * src/parilu_v0_3_bcsr.cpp:167-171 and :211-215) */
static void blk_gemm(int bs, const double *A, const double *B, double *C) {
  for (int r = 0; r < bs; ++r)
    for (int c = 0; c < bs; ++c) {
      double s = 0.0;
      for (int p = 0; p < bs; ++p) s += A[r * bs + p] * B[p * bs + c];
      C[r * bs + c] = s;
    }
}

double orc_bcsr_parilu_sweep(int mode, int bs, int nblkA, const int *Arowidx,
                             const int *Acol, const double *Aval,
                             const int *Lrow, const int *Lcol,
                             const double *Lold, double *Lnew,
                             const int *Ucolptr, const int *Urowidx,
                             const double *Uold, double *Unew) {
  const int ld = bs * bs;
  double step = 0.0;
  if (mode == 0) {
    /* src/parilu_v0_3_bcsr.cpp:129-249 in its (serial) COO order */
    double S[64], sp[64], tmp[64], inv[64];
    double *Lv = Lnew, *Uv = Unew; /* in place: Lold/Uold are not read */
    for (int kk = 0; kk < ld; kk++) sp[kk] = 0.0;
    for (int k = 0; k < nblkA; k++) {
      int i = Arowidx[k], j = Acol[k];
      for (int kk = 0; kk < ld; kk++) S[kk] = Aval[(size_t)k * ld + kk];
      int il = Lrow[i], iu = Ucolptr[j];
      while (il < Lrow[i + 1] && iu < Ucolptr[j + 1]) {
        for (int kk = 0; kk < ld; kk++) sp[kk] = 0.0;
        int jl = Lcol[il], ju = Urowidx[iu];
        if (jl == ju) {
          blk_gemm(bs, Lv + (size_t)il * ld, Uv + (size_t)iu * ld, sp);
          for (int kk = 0; kk < ld; kk++) S[kk] = S[kk] - sp[kk];
        }
        il = (jl <= ju) ? il + 1 : il;
        iu = (jl >= ju) ? iu + 1 : iu;
      }
      for (int kk = 0; kk < ld; kk++) S[kk] += sp[kk];
      if (i > j) {
        orc_block_inverse(bs, Uv + (size_t)(Ucolptr[j + 1] - 1) * ld, inv);
        blk_gemm(bs, S, inv, tmp);
        for (int kk = 0; kk < ld; kk++) {
          step += pow(Lv[(size_t)(il - 1) * ld + kk] - tmp[kk], 2);
          Lv[(size_t)(il - 1) * ld + kk] = tmp[kk];
        }
      } else {
        for (int kk = 0; kk < ld; kk++) {
          step += pow(Uv[(size_t)(iu - 1) * ld + kk] - S[kk], 2);
          Uv[(size_t)(iu - 1) * ld + kk] = S[kk];
        }
      }
    }
    return step;
  }
#pragma omp parallel for schedule(static) reduction(+ : step)
  for (int k = 0; k < nblkA; k++) {
    double S[64], pr[64], tmp[64], inv[64];
    int i = Arowidx[k], j = Acol[k];
    int kmax = i < j ? i : j;
    for (int kk = 0; kk < ld; kk++) S[kk] = Aval[(size_t)k * ld + kk];
    int il = Lrow[i], iu = Ucolptr[j];
    const int le = Lrow[i + 1], ue = Ucolptr[j + 1];
    while (il < le && iu < ue) {
      int jl = Lcol[il], ju = Urowidx[iu];
      if (jl >= kmax || ju >= kmax) break;
      if (jl == ju) {
        blk_gemm(bs, Lold + (size_t)il * ld, Uold + (size_t)iu * ld, pr);
        for (int kk = 0; kk < ld; kk++) S[kk] -= pr[kk];
        il++; iu++;
      } else if (jl < ju) il++;
      else iu++;
    }
    if (i > j) {
      while (Lcol[il] != j) il++;
      orc_block_inverse(bs, Uold + (size_t)(ue - 1) * ld, inv);
      blk_gemm(bs, S, inv, tmp);
      for (int kk = 0; kk < ld; kk++) {
        double d = Lold[(size_t)il * ld + kk] - tmp[kk];
        step += d * d;
        Lnew[(size_t)il * ld + kk] = tmp[kk];
      }
    } else {
      while (Urowidx[iu] != i) iu++;
      for (int kk = 0; kk < ld; kk++) {
        double d = Uold[(size_t)iu * ld + kk] - S[kk];
        step += d * d;
        Unew[(size_t)iu * ld + kk] = S[kk];
      }
    }
  }
  return step;
}

void orc_bcsr_trsv_lower_unit(int nbrows, int bs, const int *row,
                              const int *col, const double *val,
                              const double *b, double *x) {
  const int ld = bs * bs;
  double t[8];
  for (int I = 0; I < nbrows; ++I) {
    for (int r = 0; r < bs; ++r) t[r] = b[(size_t)I * bs + r];
    for (int p = row[I]; p < row[I + 1]; ++p) {
      int J = col[p];
      if (J >= I) continue;
      const double *blk = val + (size_t)p * ld;
      for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) t[r] -= blk[r * bs + c] * x[(size_t)J * bs + c];
    }
    for (int r = 0; r < bs; ++r) x[(size_t)I * bs + r] = t[r];
  }
}

void orc_bcsr_trsv_upper(int nbrows, int bs, const int *row, const int *col,
                         const double *val, const double *Dinv,
                         const double *b, double *x) {
  const int ld = bs * bs;
  double t[8];
  for (int I = nbrows - 1; I >= 0; --I) {
    for (int r = 0; r < bs; ++r) t[r] = b[(size_t)I * bs + r];
    for (int p = row[I]; p < row[I + 1]; ++p) {
      int J = col[p];
      if (J <= I) continue;
      const double *blk = val + (size_t)p * ld;
      for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) t[r] -= blk[r * bs + c] * x[(size_t)J * bs + c];
    }
    const double *D = Dinv + (size_t)I * ld;
    for (int r = 0; r < bs; ++r) {
      double s = 0.0;
      for (int c = 0; c < bs; ++c) s += D[r * bs + c] * t[c];
      x[(size_t)I * bs + r] = s;
    }
  }
}

void orc_bcsr_trsv_lower_unit_f32(int nbrows, int bs, const int *row,
                                  const int *col, const float *val,
                                  const float *b, float *x) {
  const int ld = bs * bs;
  float t[8];
  for (int I = 0; I < nbrows; ++I) {
    for (int r = 0; r < bs; ++r) t[r] = b[(size_t)I * bs + r];
    for (int p = row[I]; p < row[I + 1]; ++p) {
      int J = col[p];
      if (J >= I) continue;
      const float *blk = val + (size_t)p * ld;
      for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) t[r] -= blk[r * bs + c] * x[(size_t)J * bs + c];
    }
    for (int r = 0; r < bs; ++r) x[(size_t)I * bs + r] = t[r];
  }
}

void orc_bcsr_trsv_upper_f32(int nbrows, int bs, const int *row, const int *col,
                             const float *val, const float *Dinv,
                             const float *b, float *x) {
  const int ld = bs * bs;
  float t[8];
  for (int I = nbrows - 1; I >= 0; --I) {
    for (int r = 0; r < bs; ++r) t[r] = b[(size_t)I * bs + r];
    for (int p = row[I]; p < row[I + 1]; ++p) {
      int J = col[p];
      if (J <= I) continue;
      const float *blk = val + (size_t)p * ld;
      for (int r = 0; r < bs; ++r)
        for (int c = 0; c < bs; ++c) t[r] -= blk[r * bs + c] * x[(size_t)J * bs + c];
    }
    const float *D = Dinv + (size_t)I * ld;
    for (int r = 0; r < bs; ++r) {
      float s = 0.0f;
      for (int c = 0; c < bs; ++c) s += D[r * bs + c] * t[c];
      x[(size_t)I * bs + r] = s;
    }
  }
}

/* ===================================================== Householder/Givens */

void orc_givens(double a, double b, double tol, double *c, double *s) {
  /* src/givens.cpp:46-67 */
  if (fabs(b) <= tol) {
    *c = 1.0;
    *s = 0.0;
  } else if (fabs(b) > fabs(a)) {
    double temp = a / b;
    *s = 1.0 / sqrt(1.0 + temp * temp);
    *c = temp * (*s);
  } else {
    double temp = b / a;
    *c = 1.0 / sqrt(1.0 + temp * temp);
    *s = temp * (*c);
  }
}

static double seq_dot(int n, const double *x, const double *y) {
  /* cblas_ddot as the MKL stand-in computes it (sequential) */
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[i] * y[i];
  return s;
}

static double seq_nrm2(int n, const double *x) {
  double s = 0.0;
  for (int i = 0; i < n; ++i) s += x[i] * x[i];
  return sqrt(s);
}

double orc_orthogonality_error(int n, int ld, const double *Q, int search) {
  /* src/orthogonality_error.cpp:56-79 then data_infinity_norm */
  double *E = (double *)calloc((size_t)search * (size_t)search, sizeof(double));
  for (int e = 0; e < search; e++) E[e + e * search] = 1.0;
  for (int i = 0; i < search; i++)
    for (int j = 0; j < search; j++)
      E[i + j * search] -= seq_dot(n, Q + (size_t)i * ld, Q + (size_t)j * ld);
  double mx = 0.0;
  for (int i = 0; i < search; i++) {
    double t = 0.0;
    for (int j = 0; j < search; j++) t += fabs(E[i * search + j]);
    if (mx < t) mx = t;
  }
  free(E);
  return mx;
}

/* ===================================================== FGMRES-Householder */

#define DEV_STRIP 1024

/* 2*(v_j . w) over rows j..n-1 with LACE's strip-mined summation order
 * (src/fgmres_householder_restart.cpp:380-431 and :527-577): a head from j
 * to the next strip boundary, strips of 1024 summed individually and then in
 * order, and a tail.  Strips are independent, so they run in parallel
 * without changing a single rounding. */
static double strip_dot2(int n, int j, const double *v, const double *w,
                         double *bins) {
  const int STRIP = MINI(n, DEV_STRIP);
  const int BINS = n / STRIP;
  const int endStrip = BINS * STRIP;
  const int startStrip = (j / STRIP + 1) * STRIP;
  const int b0 = startStrip / STRIP;
#pragma omp parallel for schedule(static) if (BINS - b0 > 64)
  for (int b = b0; b < BINS; ++b) {
    double t = 0.0;
    for (int i = b * STRIP; i < (b + 1) * STRIP; ++i) t += v[i] * w[i];
    bins[b] = t;
  }
  double sumBegin = 0.0, sumEnd = 0.0, sum = 0.0;
  for (int i = j; i < startStrip && i < n; ++i) sumBegin += v[i] * w[i];
  for (int i = endStrip; i < n; ++i) sumEnd += v[i] * w[i];
  for (int b = 0; b < BINS; ++b) sum += (b >= b0) ? bins[b] : 0.0;
  return 2.0 * (sumBegin + sum + sumEnd);
}

static void op_apply(const orc_operator *A, const double *z, double *w) {
  /* inline SpMV of src/fgmres_householder_restart.cpp:362-367 accumulating
   * into the (zeroed) Krylov column */
  const int n = A->n;
  if (A->kind == ORC_OP_CSR) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      double s = w[i];
      for (int p = A->row[i]; p < A->row[i + 1]; ++p) s = s + A->val[p] * z[A->col[p]];
      w[i] = s;
    }
  } else {
    const int bs = A->bs, ld = bs * bs, nb = n / bs;
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nb; ++I)
      for (int r = 0; r < bs; ++r) {
        double s = w[(size_t)I * bs + r];
        for (int p = A->row[I]; p < A->row[I + 1]; ++p) {
          const double *blk = A->val + (size_t)p * ld + r * bs;
          const double *zj = z + (size_t)A->col[p] * bs;
          for (int c = 0; c < bs; ++c) s = s + blk[c] * zj[c];
        }
        w[(size_t)I * bs + r] = s;
      }
  }
}

static void op_residual(const orc_operator *A, const double *x, const double *b,
                        double *r) {
  /* :215-221: r = 0 - A x (row by row), then data_zaxpy(n, 1, b, r) */
  const int n = A->n;
  if (A->kind == ORC_OP_CSR) {
#pragma omp parallel for schedule(static)
    for (int i = 0; i < n; ++i) {
      double s = 0.0;
      for (int p = A->row[i]; p < A->row[i + 1]; ++p) s = s - A->val[p] * x[A->col[p]];
      r[i] = s + 1.0 * b[i];
    }
  } else {
    const int bs = A->bs, ld = bs * bs, nb = n / bs;
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nb; ++I)
      for (int rr = 0; rr < bs; ++rr) {
        double s = 0.0;
        for (int p = A->row[I]; p < A->row[I + 1]; ++p) {
          const double *blk = A->val + (size_t)p * ld + rr * bs;
          const double *xj = x + (size_t)A->col[p] * bs;
          for (int c = 0; c < bs; ++c) s = s - blk[c] * xj[c];
        }
        r[(size_t)I * bs + rr] = s + 1.0 * b[(size_t)I * bs + rr];
      }
  }
}

/* z = M^{-1} q (:320-349); tmp is LACE's zeroed r vector */
static void prec_apply(const orc_precond *M, int n, int bs, const double *q,
                       double *tmp, double *z, float *fa, float *fb) {
  int it = 0;
  switch (M->kind) {
    case ORC_PREC_NONE:
      memcpy(z, q, sizeof(double) * (size_t)n);
      break;
    case ORC_PREC_TRSV:
      orc_trsv(n, M->t1_row, M->t1_col, M->t1_val, M->t1_lower, M->t1_unit, q, tmp);
      orc_trsv(n, M->t2_row, M->t2_col, M->t2_val, M->t2_lower, M->t2_unit, tmp, z);
      break;
    case ORC_PREC_TRSV_F32:
      for (int i = 0; i < n; ++i) fa[i] = (float)q[i];
      orc_trsv_f32(n, M->t1_row, M->t1_col, M->t1_val32, M->t1_lower, M->t1_unit, fa, fb);
      orc_trsv_f32(n, M->t2_row, M->t2_col, M->t2_val32, M->t2_lower, M->t2_unit, fb, fa);
      for (int i = 0; i < n; ++i) z[i] = (double)fa[i];
      break;
    case ORC_PREC_PARTRSV:
      memset(tmp, 0, sizeof(double) * (size_t)n);
      orc_parcsrtrsv(0, n, M->t1_val, M->t1_row, M->t1_col, q, tmp, M->tol, &it);
      memset(z, 0, sizeof(double) * (size_t)n);
      orc_parcsrtrsv(1, n, M->t2_val, M->t2_row, M->t2_col, tmp, z, M->tol, &it);
      break;
    case ORC_PREC_JACOBI:
      memset(tmp, 0, sizeof(double) * (size_t)n);
      orc_jacobi_trsv(0, n, M->t1_val, M->t1_row, M->t1_col, q, tmp, M->tol,
                      M->max_sweeps, &it);
      memset(z, 0, sizeof(double) * (size_t)n);
      orc_jacobi_trsv(1, n, M->t2_val, M->t2_row, M->t2_col, tmp, z, M->tol,
                      M->max_sweeps, &it);
      break;
    case ORC_PREC_BCSR:
      orc_bcsr_trsv_lower_unit(n / bs, bs, M->t1_row, M->t1_col, M->t1_val, q, tmp);
      orc_bcsr_trsv_upper(n / bs, bs, M->t2_row, M->t2_col, M->t2_val, M->bdinv, tmp, z);
      break;
    case ORC_PREC_BCSR_F32:
      for (int i = 0; i < n; ++i) fa[i] = (float)q[i];
      orc_bcsr_trsv_lower_unit_f32(n / bs, bs, M->t1_row, M->t1_col, M->t1_val32, fa, fb);
      orc_bcsr_trsv_upper_f32(n / bs, bs, M->t2_row, M->t2_col, M->t2_val32, M->bdinv32, fb, fa);
      for (int i = 0; i < n; ++i) z[i] = (double)fa[i];
      break;
    default:
      memcpy(z, q, sizeof(double) * (size_t)n);
  }
}

#define K(i, j) krylov[(size_t)(i) + (size_t)(j) * (size_t)n]
#define Z(i, j) Minvvj[(size_t)(i) + (size_t)(j) * (size_t)n]

int orc_fgmres_householder(const orc_operator *A, const orc_precond *M,
                           const double *b, double *x0, const orc_gmres_par *par,
                           orc_gmres_log *log, double *resid_hist,
                           double *orth_hist) {
  const int n = A->n;
  const int m = par->search_max;
  const int restart_max = par->restart_max;
  int info = -205; /* DEV_NOTCONVERGED */
  double rtol = par->rtol;
  memset(log, 0, sizeof(*log));

  double *x = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(x, x0, sizeof(double) * (size_t)n);
  double *r = (double *)calloc((size_t)n, sizeof(double));
  double *q = (double *)calloc((size_t)n, sizeof(double));
  double *krylov = (double *)calloc((size_t)n * (size_t)(m + 1), sizeof(double));
  double *Minvvj = (double *)calloc((size_t)n * (size_t)m, sizeof(double));
  double *precondq = par->monitor_orthog
                         ? (double *)calloc((size_t)n * (size_t)(m + 1), sizeof(double))
                         : NULL;
  double *g = (double *)calloc((size_t)(m + 1), sizeof(double));
  double *gc = (double *)calloc((size_t)m, sizeof(double));
  double *gs = (double *)calloc((size_t)m, sizeof(double));
  double *bins = (double *)calloc((size_t)(n / MINI(n, DEV_STRIP) + 1), sizeof(double));
  float *fa = (float *)malloc(sizeof(float) * (size_t)n);
  float *fb = (float *)malloc(sizeof(float) * (size_t)n);
  const double eps = nextafter(0.0, 1.0);
  int total = 0;
  int early_return = 0;

  for (int restart = 0; restart < restart_max; ++restart) {
    if (restart > 0) { /* :197-207 */
      memset(r, 0, sizeof(double) * (size_t)n);
      memset(q, 0, sizeof(double) * (size_t)n);
      memset(krylov, 0, sizeof(double) * (size_t)n * (size_t)(m + 1));
      if (precondq) memset(precondq, 0, sizeof(double) * (size_t)n * (size_t)(m + 1));
      memset(Minvvj, 0, sizeof(double) * (size_t)n * (size_t)m);
      memset(g, 0, sizeof(double) * (size_t)(m + 1));
      memset(gc, 0, sizeof(double) * (size_t)m);
      memset(gs, 0, sizeof(double) * (size_t)m);
    }
    op_residual(A, x, b, r);
    double rnorm2 = seq_nrm2(n, r);
    if (restart == 0) { /* :223-230 */
      log->search_directions = 0;
      log->initial_residual = rnorm2;
      if (par->tol_type == 1) rtol = rtol * rnorm2;
    }
    if (rnorm2 < rtol) { /* :233-236: returns without copying x back */
      info = 0;
      log->converged = 1;
      log->lost_update = (restart > 0);
      early_return = 1;
      break;
    }
    /* first reflector, :239-308 */
    memcpy(&K(0, 0), r, sizeof(double) * (size_t)n);
    double dd = mysgn(K(0, 0)) * rnorm2;
    K(0, 0) = K(0, 0) + dd;
    double k1norm2 = 1.0 / seq_nrm2(n, &K(0, 0));
    for (int i = 0; i < n; ++i) K(i, 0) = K(i, 0) * k1norm2;
    for (int i = 0; i < n; ++i) {
      q[i] = -r[i] / dd;
      if (precondq) precondq[i] = q[i];
    }
    g[0] = -dd;

    for (int search = 0; search < m; ++search) { /* :311 */
      const int search1 = search + 1;
      memset(r, 0, sizeof(double) * (size_t)n);
      prec_apply(M, n, A->bs, q, r, &Z(0, search), fa, fb);
      op_apply(A, &Z(0, search), &K(0, search1));
      for (int j = 0; j <= search; ++j) { /* :376-469 */
        double sum = strip_dot2(n, j, &K(0, j), &K(0, search1), bins);
#pragma omp parallel for schedule(static) if (n - j > 65536)
        for (int i = j; i < n; ++i) K(i, search1) = K(i, search1) - sum * K(i, j);
      }
      if (search < n) { /* :476-617 */
        double snrm2 = seq_nrm2(n - search1, &K(search1, search1));
        dd = mysgn(K(search1, search1)) * snrm2;
        K(search1, search1) = K(search1, search1) + dd;
        snrm2 = 1.0 / seq_nrm2(n - search1, &K(search1, search1));
        for (int i = search1; i < n; ++i) K(i, search1) = K(i, search1) * snrm2;
        memset(q, 0, sizeof(double) * (size_t)n);
        q[search1] = 1.0;
        for (int j = search1; j >= 0; --j) {
          double sum = strip_dot2(n, j, &K(0, j), q, bins);
#pragma omp parallel for schedule(static) if (n - j > 65536)
          for (int i = j; i < n; ++i) q[i] = q[i] - sum * K(i, j);
        }
      }
      if (par->monitor_orthog) { /* :628-656 */
        memcpy(precondq + (size_t)search1 * n, q, sizeof(double) * (size_t)n);
        double oe = orc_orthogonality_error(n, n, precondq, search1);
        if (orth_hist) orth_hist[total] = oe;
      }
      for (int j = 0; j < search; ++j) { /* :661-679 */
        double t0 = K(j, search1), t1 = K(j + 1, search1);
        K(j + 1, search1) = -gs[j] * t0 + gc[j] * t1;
        K(j, search1) = gc[j] * t0 + gs[j] * t1;
      }
      if (search < n) { /* :686-701 */
        orc_givens(K(search, search1), -dd, eps, &gc[search], &gs[search]);
        K(search, search1) = gc[search] * K(search, search1) - gs[search] * dd;
        g[search1] = -gs[search] * g[search];
        g[search] = gc[search] * g[search];
      }
      if (resid_hist) resid_hist[total] = fabs(g[search1]);
      total++;
      if (fabs(g[search1]) < rtol || search == m - 1) { /* :714-757 */
        for (int i = 0; i <= search; ++i) r[i] = g[i] / K(i, i + 1);
        for (int j = search; j > 0; --j)
          for (int i = j - 1; i >= 0; --i)
            r[i] = r[i] - K(i, j + 1) * r[j] / K(i, i + 1);
        for (int j = 0; j <= search; j++) {
#pragma omp parallel for schedule(static) if (n > 65536)
          for (int i = 0; i < n; i++) x[i] = x[i] + Z(i, j) * r[j];
        }
        log->restarts = restart;
        log->search_directions = search1;
        log->final_residual = fabs(g[search1]);
        if (fabs(g[search1]) < rtol) {
          log->converged = 1;
          restart = restart_max;
        }
        break;
      }
    }
  }
  log->total_iterations = total;
  if (!early_return) {
    memcpy(x0, x, sizeof(double) * (size_t)n); /* :764-765 */
    if (log->final_residual > rtol) info = 0;   /* :768-770, as written */
  }
  log->info = info;
  free(x); free(r); free(q); free(krylov); free(Minvvj); free(precondq);
  free(g); free(gc); free(gs); free(bins); free(fa); free(fb);
  return info;
}

/* ========================================================= FGMRES-MGS */

#define H(i, j) h[(size_t)(i) + (size_t)(j) * (size_t)(m + 1)]

int orc_fgmres_mgs(const orc_operator *A, const orc_precond *M, const double *b,
                   double *x0, const orc_gmres_par *par, int restarted,
                   orc_gmres_log *log, double *resid_hist, double *orth_hist) {
  const int n = A->n;
  const int m = par->search_max;
  const int restart_max = restarted ? par->restart_max : 1;
  int info = -205; /* DEV_NOTCONVERGED */
  double rtol = par->rtol;
  memset(log, 0, sizeof(*log));

  double *x = (double *)malloc(sizeof(double) * (size_t)n);
  memcpy(x, x0, sizeof(double) * (size_t)n);
  double *r = (double *)calloc((size_t)n, sizeof(double));
  double *u = (double *)calloc((size_t)n, sizeof(double));
  double *tmp = (double *)calloc((size_t)n, sizeof(double));
  double *z = (double *)calloc((size_t)n, sizeof(double));
  double *krylov = (double *)calloc((size_t)n * (size_t)(m + 1), sizeof(double));
  double *Minvvj = (double *)calloc((size_t)n * (size_t)m, sizeof(double));
  double *h = (double *)calloc((size_t)(m + 1) * (size_t)m, sizeof(double));
  double *g = (double *)calloc((size_t)(m + 1), sizeof(double));
  double *gc = (double *)calloc((size_t)m, sizeof(double));
  double *gs = (double *)calloc((size_t)m, sizeof(double));
  double *alpha = (double *)calloc((size_t)m, sizeof(double));
  float *fa = (float *)malloc(sizeof(float) * (size_t)n);
  float *fb = (float *)malloc(sizeof(float) * (size_t)n);
  /* the Brown/Hindmarsh test's threshold (fgmres_restart.cpp:150) and the
   * happy-breakdown threshold (:363; fgmres.cpp:341 uses DBL_EPSILON) */
  const double eps = nextafter(0.0, 1.0);
  const double brk = restarted ? 0.0 : DBL_EPSILON;
  int total = 0;
  int early_return = 0;

  for (int restart = 0; restart < restart_max; ++restart) {
    if (restart > 0) { /* fgmres_restart.cpp:181-189 (h and alpha are kept) */
      memset(r, 0, sizeof(double) * (size_t)n);
      memset(u, 0, sizeof(double) * (size_t)n);
      memset(krylov, 0, sizeof(double) * (size_t)n * (size_t)(m + 1));
      memset(Minvvj, 0, sizeof(double) * (size_t)n * (size_t)m);
      memset(g, 0, sizeof(double) * (size_t)(m + 1));
      memset(gc, 0, sizeof(double) * (size_t)m);
      memset(gs, 0, sizeof(double) * (size_t)m);
    }
    op_residual(A, x, b, r); /* :192-194 */
    const double rnorm2 = seq_nrm2(n, r);
    if (restart == 0 && par->tol_type == 1) rtol = rtol * rnorm2; /* :195-201 */
    if (rnorm2 < rtol) { /* :205-208: returns without copying x back */
      info = 0;
      log->converged = 1;
      log->lost_update = (restart > 0);
      early_return = 1;
      break;
    }
    for (int i = 0; i < n; ++i) K(i, 0) = r[i] / rnorm2; /* :211-218 */
    g[0] = rnorm2;
    log->search_directions = 0; /* :221-223, every cycle */
    log->initial_residual = rnorm2;

    for (int search = 0; search < m; ++search) { /* :227 */
      const int search1 = search + 1;
      memset(u, 0, sizeof(double) * (size_t)n);
      memset(tmp, 0, sizeof(double) * (size_t)n);
      prec_apply(M, n, A->bs, &K(0, search), tmp, &Z(0, search), fa, fb); /* :239-270 */
      op_apply(A, &Z(0, search), u);                                        /* :284-290 */
      const double normav = seq_nrm2(n, u);                                 /* :291 */
      for (int j = 0; j <= search; ++j) { /* :302-328, modified Gram-Schmidt */
        double t = 0.0;
        for (int i = 0; i < n; ++i) t = t + K(i, j) * u[i];
        H(j, search) = t;
#pragma omp parallel for schedule(static) if (n > 65536)
        for (int i = 0; i < n; ++i) u[i] = u[i] - H(j, search) * K(i, j);
      }
      H(search1, search) = seq_nrm2(n, u); /* :329-330 */
      const double normav2 = H(search1, search);
      double hr = (normav + 0.001 * normav2) - normav; /* :336-360 */
      if ((par->reorth == 0 && hr <= eps) || par->reorth == 2) {
        for (int j = 0; j <= search; ++j) {
          hr = 0.0;
          for (int i = 0; i < n; ++i) hr = hr + K(i, j) * u[i];
          H(j, search) = H(j, search) + hr;
#pragma omp parallel for schedule(static) if (n > 65536)
          for (int i = 0; i < n; ++i) u[i] = u[i] - hr * K(i, j);
        }
        H(search1, search) = seq_nrm2(n, u);
      }
      if (fabs(H(search1, search)) > brk) /* :362-378 */
        for (int i = 0; i < n; ++i) K(i, search1) = u[i] / H(search1, search);
      if (par->monitor_orthog) { /* :380-387 */
        double oe = orc_orthogonality_error(n, n, krylov, search1);
        if (orth_hist) orth_hist[total] = oe;
      }
      for (int j = 0; j < search; ++j) { /* :406-415 */
        const double delta = H(j, search);
        H(j, search) = gc[j] * delta - gs[j] * H(j + 1, search);
        H(j + 1, search) = gs[j] * delta + gc[j] * H(j + 1, search);
      }
      const double gamma = sqrt(H(search, search) * H(search, search) +
                                H(search1, search) * H(search1, search)); /* :417-420 */
      if (gamma > 0.0) { /* :421-432 */
        gc[search] = H(search, search) / gamma;
        gs[search] = -H(search1, search) / gamma;
        H(search, search) = gc[search] * H(search, search) - gs[search] * H(search1, search);
        H(search1, search) = 0.0;
        const double delta = g[search];
        g[search] = gc[search] * delta - gs[search] * g[search1];
        g[search1] = gs[search] * delta + gc[search] * g[search1];
      }
      if (resid_hist) resid_hist[total] = fabs(g[search1]);
      total++;
      /* :459 (fgmres.cpp:440 also stops on a non-finite residual) */
      if (fabs(g[search1]) < rtol || search == m - 1 || (!restarted && !isfinite(g[search1]))) {
        for (int i = 0; i <= search; ++i) alpha[i] = g[i] / H(i, i); /* :461-469 */
        for (int j = search; j > 0; --j)
          for (int i = j - 1; i > -1; --i) alpha[i] = alpha[i] - H(i, j) * alpha[j] / H(i, i);
        if (restarted) { /* :472-481, column by column */
          for (int j = 0; j <= search; ++j) {
#pragma omp parallel for schedule(static) if (n > 65536)
            for (int i = 0; i < n; ++i) x[i] = x[i] + Z(i, j) * alpha[j];
          }
        } else { /* fgmres.cpp:453-474: z = sum_j Z_j alpha_j, then x += z */
#pragma omp parallel for schedule(static) if (n > 65536)
          for (int i = 0; i < n; ++i) {
            for (int j = 0; j <= search; ++j) z[i] = z[i] + Z(i, j) * alpha[j];
            x[i] = x[i] + z[i];
          }
        }
        if (restarted) log->restarts = restart;
        log->search_directions = search1;
        log->final_residual = fabs(g[search1]);
        if (fabs(g[search1]) < rtol) {
          log->converged = 1;
          restart = restart_max;
        }
        break;
      }
    }
  }
  log->total_iterations = total;
  if (!early_return) {
    memcpy(x0, x, sizeof(double) * (size_t)n); /* :506-507 */
    if (log->final_residual > rtol) info = 0;   /* :510-512, as written */
  }
  log->info = info;
  free(x); free(r); free(u); free(tmp); free(z); free(krylov); free(Minvvj);
  free(h); free(g); free(gc); free(gs); free(alpha); free(fa); free(fb);
  return info;
}
