/*
 * CPU re-implementation of the Intel MKL routines that LACE's hot path calls,
 * written from each routine's published mathematical definition.  It exists
 * only so that LACE's own unmodified sources can be compiled into the CPU
 * oracle (oracle/_ref).  Test infrastructure; not part of the product.
 *
 * Call sites in LACE (paths inside the LACE source tree):
 *   cblas_dnrm2   control/norms.cpp:12          (data_dnrm2)
 *   cblas_ddot    blas/zdot.cpp:75              (data_zdot_mkl)
 *   cblas_daxpy   blas/zaxpy.cpp:58             (data_zaxpy)
 *   cblas_dgemm   blas/zgemm.cpp:112            (data_dgemm_mkl, BCSR ParILU)
 *   mkl_dcsrmv    blas/zspmv.cpp:61             (data_z_spmv)
 *   mkl_dcsrtrsv  src/fgmres_householder_restart.cpp:325,330
 *   mkl_dcsrbsr   control/magma_zmconverter.cpp:654,664,836
 *   dcsrilu0      blas/zcsrilu0.cpp:58
 *   mkl_sparse_*  blas/zspmm.cpp:64-162         (data_z_spmm, used by data_zilures)
 *
 * Conventions chosen here (MKL's internal summation order is unpublished):
 *   - every reduction sums left to right in storage order;
 *   - dnrm2 is the unscaled definition sqrt(sum x_i^2);
 *   - SpMM output rows are emitted with ascending column indices.
 */
#include "mkl.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ CBLAS */

double cblas_dnrm2(const MKL_INT n, const double *x, const MKL_INT incx) {
  double s = 0.0;
  for (MKL_INT i = 0; i < n; ++i) s += x[(size_t)i * incx] * x[(size_t)i * incx];
  return sqrt(s);
}

double cblas_ddot(const MKL_INT n, const double *x, const MKL_INT incx,
                  const double *y, const MKL_INT incy) {
  double s = 0.0;
  for (MKL_INT i = 0; i < n; ++i) s += x[(size_t)i * incx] * y[(size_t)i * incy];
  return s;
}

void cblas_daxpy(const MKL_INT n, const double alpha, const double *x,
                 const MKL_INT incx, double *y, const MKL_INT incy) {
  for (MKL_INT i = 0; i < n; ++i) y[(size_t)i * incy] += alpha * x[(size_t)i * incx];
}

/* element (r,c) of an op(A) stored with the given layout / leading dim */
static double mat_at(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE tr, const double *a,
                     MKL_INT ld, MKL_INT r, MKL_INT c) {
  if (tr != CblasNoTrans) { MKL_INT t = r; r = c; c = t; }
  return layout == CblasRowMajor ? a[(size_t)r * ld + c] : a[(size_t)c * ld + r];
}

void cblas_dgemv(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE trans,
                 const MKL_INT m, const MKL_INT n, const double alpha,
                 const double *a, const MKL_INT lda, const double *x,
                 const MKL_INT incx, const double beta, double *y,
                 const MKL_INT incy) {
  MKL_INT rows = (trans == CblasNoTrans) ? m : n;
  MKL_INT cols = (trans == CblasNoTrans) ? n : m;
  for (MKL_INT i = 0; i < rows; ++i) {
    double s = 0.0;
    for (MKL_INT j = 0; j < cols; ++j)
      s += mat_at(layout, trans, a, lda, i, j) * x[(size_t)j * incx];
    double *yi = &y[(size_t)i * incy];
    *yi = (beta == 0.0) ? alpha * s : alpha * s + beta * (*yi);
  }
}

void cblas_dgemm(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const MKL_INT m, const MKL_INT n,
                 const MKL_INT k, const double alpha, const double *a,
                 const MKL_INT lda, const double *b, const MKL_INT ldb,
                 const double beta, double *c, const MKL_INT ldc) {
  for (MKL_INT i = 0; i < m; ++i) {
    for (MKL_INT j = 0; j < n; ++j) {
      double s = 0.0;
      for (MKL_INT p = 0; p < k; ++p)
        s += mat_at(layout, transa, a, lda, i, p) * mat_at(layout, transb, b, ldb, p, j);
      double *cij = (layout == CblasRowMajor) ? &c[(size_t)i * ldc + j] : &c[(size_t)j * ldc + i];
      *cij = (beta == 0.0) ? alpha * s : alpha * s + beta * (*cij);
    }
  }
}

/* ------------------------------------------------------- sparse BLAS (NIST) */

/* y = alpha*op(A)*x + beta*y, CSR given by (val, indx, pntrb, pntre).
 * matdescra[3] == 'F' -> one-based, otherwise zero-based. */
void mkl_dcsrmv(const char *transa, const MKL_INT *m, const MKL_INT *k,
                const double *alpha, const char *matdescra, const double *val,
                const MKL_INT *indx, const MKL_INT *pntrb, const MKL_INT *pntre,
                const double *x, const double *beta, double *y) {
  const MKL_INT base = (matdescra[3] == 'F' || matdescra[3] == 'f') ? 1 : 0;
  const int trans = !(transa[0] == 'N' || transa[0] == 'n');
  if (!trans) {
    for (MKL_INT i = 0; i < *m; ++i) {
      double s = 0.0;
      for (MKL_INT p = pntrb[i] - base; p < pntre[i] - base; ++p)
        s += val[p] * x[indx[p] - base];
      y[i] = (*beta == 0.0) ? (*alpha) * s : (*alpha) * s + (*beta) * y[i];
    }
  } else {
    for (MKL_INT j = 0; j < *k; ++j) y[j] = (*beta == 0.0) ? 0.0 : (*beta) * y[j];
    for (MKL_INT i = 0; i < *m; ++i)
      for (MKL_INT p = pntrb[i] - base; p < pntre[i] - base; ++p)
        y[indx[p] - base] += (*alpha) * val[p] * x[i];
  }
}

/* Triangular solve with the lower ('L') or upper ('U') triangle of a one-based
 * CSR matrix; diag 'U' means an implicit unit diagonal (stored diagonal
 * entries are ignored).  Only transa == 'N' is needed on LACE's path. */
void mkl_dcsrtrsv(const char *uplo, const char *transa, const char *diag,
                  const MKL_INT *m, const double *a, const MKL_INT *ia,
                  const MKL_INT *ja, const double *x, double *y) {
  (void)transa;
  const int lower = (uplo[0] == 'L' || uplo[0] == 'l');
  const int unit = (diag[0] == 'U' || diag[0] == 'u');
  const MKL_INT n = *m;
  if (lower) {
    for (MKL_INT i = 0; i < n; ++i) {
      double s = x[i], d = 1.0;
      for (MKL_INT p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
        MKL_INT j = ja[p] - 1;
        if (j < i) s -= a[p] * y[j];
        else if (j == i) d = a[p];
      }
      y[i] = unit ? s : s / d;
    }
  } else {
    for (MKL_INT i = n - 1; i >= 0; --i) {
      double s = x[i], d = 1.0;
      for (MKL_INT p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
        MKL_INT j = ja[p] - 1;
        if (j > i) s -= a[p] * y[j];
        else if (j == i) d = a[p];
      }
      y[i] = unit ? s : s / d;
    }
  }
}

/* CSR <-> BSR conversion.  job[0]: 0 CSR->BSR, 1 BSR->CSR; job[1]/job[2]:
 * index base of the CSR / BSR arrays; job[5]: -1 -> iab[0] receives the block
 * count only, 0 -> structure only, >0 -> structure and values.  With a
 * zero-based BSR the blocks are stored row-major (as LACE relies on,
 * control/magma_zmconverter.cpp:648-652). */
void mkl_dcsrbsr(const MKL_INT *job, const MKL_INT *m, const MKL_INT *mblk,
                 const MKL_INT *ldabsr, double *acsr, MKL_INT *ja, MKL_INT *ia,
                 double *absr, MKL_INT *jab, MKL_INT *iab, MKL_INT *info) {
  const MKL_INT bs = *mblk, ld = *ldabsr;
  const MKL_INT cb = job[1], bb = job[2];
  *info = 0;
  if (job[0] == 0) {
    const MKL_INT nrow = *m;
    const MKL_INT nbr = (nrow + bs - 1) / bs;
    MKL_INT ncolmax = 0;
    for (MKL_INT p = 0; p < ia[nrow] - cb; ++p)
      if (ja[p] - cb + 1 > ncolmax) ncolmax = ja[p] - cb + 1;
    MKL_INT nbc = (ncolmax + bs - 1) / bs;
    MKL_INT *mark = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)(nbc + 1));
    MKL_INT *slot = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)(nbc + 1));
    for (MKL_INT c = 0; c <= nbc; ++c) mark[c] = -1;
    MKL_INT nb = 0;
    for (MKL_INT I = 0; I < nbr; ++I) {
      MKL_INT rowstart = nb;
      /* collect block columns of this block row, in ascending order */
      for (MKL_INT r = I * bs; r < (I + 1) * bs && r < nrow; ++r)
        for (MKL_INT p = ia[r] - cb; p < ia[r + 1] - cb; ++p) {
          MKL_INT J = (ja[p] - cb) / bs;
          if (mark[J] != I) { mark[J] = I; ++nb; }
        }
      if (job[5] >= 0) {
        iab[I] = rowstart + bb;
        /* ascending block columns */
        MKL_INT cnt = 0;
        for (MKL_INT J = 0; J < nbc; ++J)
          if (mark[J] == I) { jab[rowstart + cnt] = J + bb; slot[J] = rowstart + cnt; ++cnt; }
        if (job[5] > 0) {
          for (MKL_INT q = rowstart; q < nb; ++q)
            for (MKL_INT e = 0; e < ld; ++e) absr[(size_t)q * ld + e] = 0.0;
          for (MKL_INT r = I * bs; r < (I + 1) * bs && r < nrow; ++r)
            for (MKL_INT p = ia[r] - cb; p < ia[r + 1] - cb; ++p) {
              MKL_INT c = ja[p] - cb, J = c / bs;
              absr[(size_t)slot[J] * ld + (r - I * bs) * bs + (c - J * bs)] = acsr[p];
            }
        }
      }
    }
    if (job[5] < 0) iab[0] = nb;
    else iab[nbr] = nb + bb;
    free(mark);
    free(slot);
  } else {
    const MKL_INT nbr = *m;
    MKL_INT z = 0;
    for (MKL_INT I = 0; I < nbr; ++I)
      for (MKL_INT ii = 0; ii < bs; ++ii) {
        ia[I * bs + ii] = z + cb;
        for (MKL_INT q = iab[I] - bb; q < iab[I + 1] - bb; ++q)
          for (MKL_INT jj = 0; jj < bs; ++jj) {
            if (job[5] > 0) acsr[z] = absr[(size_t)q * ld + ii * bs + jj];
            ja[z] = (jab[q] - bb) * bs + jj + cb;
            ++z;
          }
      }
    ia[nbr * bs] = z + cb;
  }
}

/* ------------------------------------------------------------------ ILU(0) */

/* ILU(0) of a one-based CSR matrix with sorted columns (Saad, "Iterative
 * Methods for Sparse Linear Systems", 2nd ed., Algorithm 10.4, IKJ variant).
 * bilu0 receives L (strict lower, unit diagonal implied) and U in A's pattern.
 * ipar[30] == 0: stop with ierr = -101 on a diagonal entry smaller in
 * magnitude than dpar[30]; otherwise replace it by dpar[31]. */
void dcsrilu0(const MKL_INT *n, const double *a, const MKL_INT *ia,
              const MKL_INT *ja, double *bilu0, const MKL_INT *ipar,
              const double *dpar, MKL_INT *ierr) {
  const MKL_INT N = *n;
  const MKL_INT nnz = ia[N] - 1;
  if (bilu0 != a) memmove(bilu0, a, sizeof(double) * (size_t)nnz);
  MKL_INT *iw = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)N);
  MKL_INT *dp = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)N);
  for (MKL_INT j = 0; j < N; ++j) { iw[j] = -1; dp[j] = -1; }
  for (MKL_INT i = 0; i < N; ++i)
    for (MKL_INT p = ia[i] - 1; p < ia[i + 1] - 1; ++p)
      if (ja[p] - 1 == i) dp[i] = p;
  *ierr = 0;
  for (MKL_INT i = 0; i < N; ++i) {
    for (MKL_INT p = ia[i] - 1; p < ia[i + 1] - 1; ++p) iw[ja[p] - 1] = p;
    for (MKL_INT p = ia[i] - 1; p < ia[i + 1] - 1; ++p) {
      MKL_INT k = ja[p] - 1;
      if (k >= i) break;
      if (dp[k] < 0) { *ierr = -101; goto done; }
      bilu0[p] = bilu0[p] / bilu0[dp[k]];
      double lik = bilu0[p];
      for (MKL_INT q = dp[k] + 1; q < ia[k + 1] - 1; ++q) {
        MKL_INT w = iw[ja[q] - 1];
        if (w >= 0) bilu0[w] -= lik * bilu0[q];
      }
    }
    if (dp[i] < 0) { *ierr = -101; goto done; }
    if (fabs(bilu0[dp[i]]) < dpar[30]) {
      if (ipar[30] == 0) { *ierr = -101; goto done; }
      bilu0[dp[i]] = dpar[31];
    }
    for (MKL_INT p = ia[i] - 1; p < ia[i + 1] - 1; ++p) iw[ja[p] - 1] = -1;
  }
done:
  free(iw);
  free(dp);
}

/* ---------------------------------------------------- sparse matrix handles */

struct lace_shim_sparse_matrix {
  MKL_INT rows, cols;
  sparse_index_base_t base;
  MKL_INT *rs, *re, *ci;
  double *v;
  int owned;
};

sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A,
                                        const sparse_index_base_t indexing,
                                        const MKL_INT rows, const MKL_INT cols,
                                        MKL_INT *rows_start, MKL_INT *rows_end,
                                        MKL_INT *col_indx, double *values) {
  struct lace_shim_sparse_matrix *h =
      (struct lace_shim_sparse_matrix *)calloc(1, sizeof(*h));
  if (!h) return SPARSE_STATUS_ALLOC_FAILED;
  h->rows = rows; h->cols = cols; h->base = indexing;
  h->rs = rows_start; h->re = rows_end; h->ci = col_indx; h->v = values;
  h->owned = 0;
  *A = h;
  return SPARSE_STATUS_SUCCESS;
}

/* C = A*B with a dense accumulator per row; C is zero-based, sorted. */
sparse_status_t mkl_sparse_spmm(const sparse_operation_t operation,
                                const sparse_matrix_t A, const sparse_matrix_t B,
                                sparse_matrix_t *C) {
  if (operation != SPARSE_OPERATION_NON_TRANSPOSE) return SPARSE_STATUS_NOT_SUPPORTED;
  if (A->cols != B->rows) return SPARSE_STATUS_INVALID_VALUE;
  const MKL_INT ab = A->base, bb = B->base;
  MKL_INT *mark = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)B->cols);
  double *acc = (double *)malloc(sizeof(double) * (size_t)B->cols);
  MKL_INT *rs = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)(A->rows + 1));
  for (MKL_INT j = 0; j < B->cols; ++j) mark[j] = -1;
  /* symbolic pass */
  MKL_INT nnz = 0;
  for (MKL_INT i = 0; i < A->rows; ++i) {
    rs[i] = nnz;
    for (MKL_INT p = A->rs[i] - ab; p < A->re[i] - ab; ++p) {
      MKL_INT k = A->ci[p] - ab;
      for (MKL_INT q = B->rs[k] - bb; q < B->re[k] - bb; ++q) {
        MKL_INT j = B->ci[q] - bb;
        if (mark[j] != i) { mark[j] = i; ++nnz; }
      }
    }
  }
  rs[A->rows] = nnz;
  MKL_INT *ci = (MKL_INT *)malloc(sizeof(MKL_INT) * (size_t)(nnz > 0 ? nnz : 1));
  double *v = (double *)malloc(sizeof(double) * (size_t)(nnz > 0 ? nnz : 1));
  for (MKL_INT j = 0; j < B->cols; ++j) mark[j] = -1;
  for (MKL_INT i = 0; i < A->rows; ++i) {
    MKL_INT cnt = 0;
    for (MKL_INT p = A->rs[i] - ab; p < A->re[i] - ab; ++p) {
      MKL_INT k = A->ci[p] - ab;
      for (MKL_INT q = B->rs[k] - bb; q < B->re[k] - bb; ++q) {
        MKL_INT j = B->ci[q] - bb;
        if (mark[j] != i) { mark[j] = i; acc[j] = 0.0; ci[rs[i] + cnt++] = j; }
        acc[j] += A->v[p] * B->v[q];
      }
    }
    /* insertion sort of this row's columns (rows are short) */
    MKL_INT *c0 = ci + rs[i];
    for (MKL_INT a = 1; a < cnt; ++a) {
      MKL_INT t = c0[a], b = a - 1;
      while (b >= 0 && c0[b] > t) { c0[b + 1] = c0[b]; --b; }
      c0[b + 1] = t;
    }
    for (MKL_INT a = 0; a < cnt; ++a) v[rs[i] + a] = acc[c0[a]];
  }
  free(mark);
  free(acc);
  struct lace_shim_sparse_matrix *h =
      (struct lace_shim_sparse_matrix *)calloc(1, sizeof(*h));
  h->rows = A->rows; h->cols = B->cols; h->base = SPARSE_INDEX_BASE_ZERO;
  h->rs = rs; h->re = rs + 1; h->ci = ci; h->v = v; h->owned = 1;
  *C = h;
  return SPARSE_STATUS_SUCCESS;
}

sparse_status_t mkl_sparse_d_export_csr(const sparse_matrix_t source,
                                        sparse_index_base_t *indexing,
                                        MKL_INT *rows, MKL_INT *cols,
                                        MKL_INT **rows_start, MKL_INT **rows_end,
                                        MKL_INT **col_indx, double **values) {
  if (!source) return SPARSE_STATUS_NOT_INITIALIZED;
  *indexing = source->base;
  *rows = source->rows;
  *cols = source->cols;
  *rows_start = source->rs;
  *rows_end = source->re;
  *col_indx = source->ci;
  *values = source->v;
  return SPARSE_STATUS_SUCCESS;
}

sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
  if (!A) return SPARSE_STATUS_SUCCESS;
  if (A->owned) { free(A->rs); free(A->ci); free(A->v); }
  free(A);
  return SPARSE_STATUS_SUCCESS;
}

/* ------------------------------------------- serial OpenMP runtime stand-in */
/* LACE is compiled without -fopenmp for the oracle (one-thread semantics);
 * these satisfy its calls into the OpenMP runtime. */
#include <time.h>

double omp_get_wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
int omp_get_num_threads(void) { return 1; }
int omp_get_max_threads(void) { return 1; }
int omp_get_num_procs(void) { return 1; }
int omp_get_thread_num(void) { return 0; }
void omp_set_num_threads(int n) { (void)n; }

/* zero-filled aligned allocation, padding included (see lace_ref_prelude.h) */
int lace_shim_posix_memalign(void **ptr, size_t alignment, size_t size) {
  size_t sz = (size + alignment - 1) / alignment * alignment + alignment;
  void *p = aligned_alloc(alignment, sz);
  if (!p) return 12; /* ENOMEM */
  memset(p, 0, sz);
  *ptr = p;
  return 0;
}
