/*
 * Minimal stand-in for the Intel MKL headers, used ONLY to compile LACE's own
 * hot-path sources into the CPU oracle (oracle/_ref).  Test infrastructure:
 * nothing in the lace_gb300 product links this.
 *
 * Intel MKL is not vendored by LACE and is absent from this image (LACE names
 * no version; its prospectus cites "Intel MKL 2017").  Every routine declared
 * here is re-implemented in mkl_shim.c from the published mathematical
 * definition of the routine (Intel MKL reference manual semantics, zero/one-
 * based CSR conventions as documented there).  Only the subset that LACE's
 * ParILU / trisolve / SpMV / FGMRES-Householder path calls is provided.
 */
#ifndef LACE_ORACLE_MKL_SHIM_H
#define LACE_ORACLE_MKL_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MKL_INT;

/* ---- CBLAS enums (standard CBLAS numbering) ---- */
typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef CBLAS_LAYOUT CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;
typedef enum { CblasNonUnit = 131, CblasUnit = 132 } CBLAS_DIAG;
typedef enum { CblasLeft = 141, CblasRight = 142 } CBLAS_SIDE;

double cblas_dnrm2(const MKL_INT n, const double *x, const MKL_INT incx);
double cblas_ddot(const MKL_INT n, const double *x, const MKL_INT incx,
                  const double *y, const MKL_INT incy);
void cblas_daxpy(const MKL_INT n, const double alpha, const double *x,
                 const MKL_INT incx, double *y, const MKL_INT incy);
void cblas_dgemv(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE trans,
                 const MKL_INT m, const MKL_INT n, const double alpha,
                 const double *a, const MKL_INT lda, const double *x,
                 const MKL_INT incx, const double beta, double *y,
                 const MKL_INT incy);
void cblas_dgemm(const CBLAS_LAYOUT layout, const CBLAS_TRANSPOSE transa,
                 const CBLAS_TRANSPOSE transb, const MKL_INT m, const MKL_INT n,
                 const MKL_INT k, const double alpha, const double *a,
                 const MKL_INT lda, const double *b, const MKL_INT ldb,
                 const double beta, double *c, const MKL_INT ldc);

/* ---- legacy NIST-style sparse BLAS ---- */
void mkl_dcsrmv(const char *transa, const MKL_INT *m, const MKL_INT *k,
                const double *alpha, const char *matdescra, const double *val,
                const MKL_INT *indx, const MKL_INT *pntrb, const MKL_INT *pntre,
                const double *x, const double *beta, double *y);
void mkl_dcsrtrsv(const char *uplo, const char *transa, const char *diag,
                  const MKL_INT *m, const double *a, const MKL_INT *ia,
                  const MKL_INT *ja, const double *x, double *y);
void mkl_dcsrbsr(const MKL_INT *job, const MKL_INT *m, const MKL_INT *mblk,
                 const MKL_INT *ldabsr, double *acsr, MKL_INT *ja, MKL_INT *ia,
                 double *absr, MKL_INT *jab, MKL_INT *iab, MKL_INT *info);

/* ---- RCI ILU(0) ---- */
void dcsrilu0(const MKL_INT *n, const double *a, const MKL_INT *ia,
              const MKL_INT *ja, double *bilu0, const MKL_INT *ipar,
              const double *dpar, MKL_INT *ierr);

/* ---- inspector-executor sparse handles (only what LACE's SpMM uses) ---- */
typedef enum {
  SPARSE_STATUS_SUCCESS = 0,
  SPARSE_STATUS_NOT_INITIALIZED = 1,
  SPARSE_STATUS_ALLOC_FAILED = 2,
  SPARSE_STATUS_INVALID_VALUE = 3,
  SPARSE_STATUS_EXECUTION_FAILED = 4,
  SPARSE_STATUS_INTERNAL_ERROR = 5,
  SPARSE_STATUS_NOT_SUPPORTED = 6
} sparse_status_t;
typedef enum { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 } sparse_index_base_t;
typedef enum {
  SPARSE_OPERATION_NON_TRANSPOSE = 10,
  SPARSE_OPERATION_TRANSPOSE = 11,
  SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12
} sparse_operation_t;
struct lace_shim_sparse_matrix;
typedef struct lace_shim_sparse_matrix *sparse_matrix_t;

sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A,
                                        const sparse_index_base_t indexing,
                                        const MKL_INT rows, const MKL_INT cols,
                                        MKL_INT *rows_start, MKL_INT *rows_end,
                                        MKL_INT *col_indx, double *values);
sparse_status_t mkl_sparse_spmm(const sparse_operation_t operation,
                                const sparse_matrix_t A, const sparse_matrix_t B,
                                sparse_matrix_t *C);
sparse_status_t mkl_sparse_d_export_csr(const sparse_matrix_t source,
                                        sparse_index_base_t *indexing,
                                        MKL_INT *rows, MKL_INT *cols,
                                        MKL_INT **rows_start, MKL_INT **rows_end,
                                        MKL_INT **col_indx, double **values);
sparse_status_t mkl_sparse_destroy(sparse_matrix_t A);

#ifdef __cplusplus
}
#endif

#endif
