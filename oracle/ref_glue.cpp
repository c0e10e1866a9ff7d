/*
 * Flat C entry points around LACE's own (unmodified) hot-path functions, so
 * that the test suite can drive the reference implementation through ctypes.
 * Compiled together with LACE's sources and the MKL stand-in into
 * oracle/_ref/liblace_ref.so by oracle/Makefile.  Test infrastructure only:
 * the lace_gb300 product never loads this library.
 *
 * Matrices cross this boundary as opaque handles to LACE's data_d_matrix.
 */
#include "sparse.h"

#include <stdlib.h>
#include <string.h>

extern "C" {

data_d_matrix *ref_vec_new(int n, const double *v);
void ref_mat_free(data_d_matrix *A);

/* ParILU v0.3 (reduction-driven, up to 20 sweeps) or the prescribed-sweeps
 * variant (max_sweeps >= 0).  log10 = {sweeps, tol, finalStep, A_Frobenius,
 * generation time, initial residual, initial nonlinear residual,
 * omp threads}. */
void ref_parilu(data_d_matrix *A, double reduction, int max_sweeps,
                data_d_matrix **L, data_d_matrix **U, double *log8) {
  *L = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  *U = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  (*L)->storage_type = Magma_CSRL;
  (*U)->storage_type = Magma_CSCU;
  data_d_preconditioner_log log;
  memset(&log, 0, sizeof(log));
  if (max_sweeps >= 0) {
    log.maxSweeps = max_sweeps;
    data_PariLU_v0_3_prescribedSweeps(A, *L, *U, reduction, &log);
  } else {
    data_PariLU_v0_3(A, *L, *U, reduction, &log);
  }
  log8[0] = log.sweeps;
  log8[1] = log.tol;
  log8[2] = log.finalStep;
  log8[3] = log.A_Frobenius;
  log8[4] = log.precond_generation_time;
  log8[5] = log.initial_residual;
  log8[6] = log.initial_nonlinear_residual;
  log8[7] = log.omp_num_threads;
}

int ref_zilures(const data_d_matrix *A, const data_d_matrix *L,
                const data_d_matrix *U, double *res, double *nonlinres) {
  data_d_matrix LU = {Magma_CSR};
  data_zmconvert(*A, &LU, Magma_CSR, Magma_CSR);
  int info = data_zilures(*A, *L, *U, &LU, res, nonlinres);
  data_zmfree(&LU);
  return info;
}

/* LACE's BCSR -> CSR conversion sizes the CSR row pointers by the block
 * rows (control/magma_zmconverter.cpp:250-255, 285) while mkl_dcsrbsr writes
 * one per scalar row (:836): with blocksize > 1 that overruns the array.
 * LACE's own pad_rows / pad_cols size it; the copies passed here carry the
 * scalar size so that the routine runs as written. */
int ref_zilures_bcsr(const data_d_matrix *A, const data_d_matrix *L,
                     const data_d_matrix *U, double *res, double *nonlinres) {
  data_d_matrix LU = {Magma_CSR};
  data_d_matrix Lc = *L, Uc = *U;
  Lc.pad_rows = Lc.pad_cols = L->num_rows * L->blocksize;
  Uc.pad_rows = Uc.pad_cols = U->num_rows * U->blocksize;
  int info = data_zilures_bcsr(*A, Lc, Uc, &LU, res, nonlinres);
  data_zmfree(&LU);
  return info;
}

int ref_spmv(double alpha, data_d_matrix *A, const double *x, double beta,
             double *y) {
  data_d_matrix *xv = ref_vec_new(A->num_cols, x);
  data_d_matrix *yv = ref_vec_new(A->num_rows, y);
  int info = data_z_spmv(alpha, A, xv, beta, yv);
  memcpy(y, yv->val, sizeof(double) * (size_t)A->num_rows);
  ref_mat_free(xv);
  ref_mat_free(yv);
  return info;
}

int ref_parcsrtrsv(int uplo, int storage, int diag, int n, const double *val,
                   const int *row, const int *col, const double *rhs,
                   double *y, double tol, int *iter) {
  return data_parcsrtrsv((data_uplo_t)uplo, (data_storage_t)storage,
                         (data_diagorder_t)diag, n, val, row, col, rhs, y, tol,
                         iter);
}

/* FGMRES-Householder with restarts.  par8 = {search_max, tol_type, rtol,
 * user_csrtrsv_choice, monitorOrthog, restart_max, precondition, reorth};
 * log7 = {restarts, search_directions, solve_time, initial_residual,
 * final_residual, scaled_residual, original_residual}.  x is in/out. */
typedef int (*ref_solver_fn)(data_d_matrix *, data_d_matrix *, data_d_matrix *,
                             data_d_matrix *, data_d_matrix *, data_d_gmres_param *,
                             data_d_gmres_log *);

static int ref_run_solver(ref_solver_fn solve, data_d_matrix *A, const double *b,
                          double *x, data_d_matrix *L, data_d_matrix *U,
                          const double *par8, double *log7) {
  data_d_matrix *bv = ref_vec_new(A->num_rows, b);
  data_d_matrix *xv = ref_vec_new(A->num_rows, x);
  data_d_gmres_param p;
  memset(&p, 0, sizeof(p));
  p.search_max = (int)par8[0];
  p.tol_type = (int)par8[1];
  p.rtol = par8[2];
  p.user_csrtrsv_choice = (int)par8[3];
  p.monitorOrthog = (int)par8[4];
  p.restart_max = (int)par8[5];
  p.precondition = (int)par8[6];
  p.reorth = (int)par8[7];
  data_d_gmres_log lg;
  memset(&lg, 0, sizeof(lg));
  int info = solve(A, bv, xv, L, U, &p, &lg);
  memcpy(x, xv->val, sizeof(double) * (size_t)A->num_rows);
  log7[0] = lg.restarts;
  log7[1] = lg.search_directions;
  log7[2] = lg.solve_time;
  log7[3] = lg.initial_residual;
  log7[4] = lg.final_residual;
  log7[5] = lg.scaled_residual;
  log7[6] = lg.original_residual;
  ref_mat_free(bv);
  ref_mat_free(xv);
  return info;
}

int ref_fgmres_householder_restart(data_d_matrix *A, const double *b, double *x,
                                   data_d_matrix *L, data_d_matrix *U,
                                   const double *par8, double *log7) {
  return ref_run_solver(data_fgmres_householder_restart, A, b, x, L, U, par8, log7);
}

/* FGMRES with modified Gram-Schmidt: data_fgmres_restart (restarted != 0)
 * or data_fgmres (one cycle); par8 and log7 as above. */
int ref_fgmres_mgs(data_d_matrix *A, const double *b, double *x, data_d_matrix *L,
                   data_d_matrix *U, const double *par8, double *log7, int restarted) {
  return ref_run_solver(restarted ? data_fgmres_restart : data_fgmres, A, b, x, L, U, par8,
                        log7);
}

void ref_givens(double a, double b, double tol, double *c, double *s) {
  givens_rotation(a, b, tol, c, s);
}

/* ||I - Q^T Q||_inf of the first `search` columns of the n x ncols
 * column-major Q */
double ref_orthogonality_error(int n, int ncols, const double *Q, int search) {
  data_d_matrix K = {Magma_DENSE};
  data_zvinit(&K, n, ncols, 0.0);
  memcpy(K.val, Q, sizeof(double) * (size_t)n * (size_t)ncols);
  double err = 0.0;
  int imax = 0;
  data_orthogonality_error(&K, &err, &imax, search);
  data_zmfree(&K);
  return err;
}

/* LACE's own Matrix Market reader (control/magma_zmio.cpp:92) into a new
 * CSR handle, and its writer (:587) */
data_d_matrix *ref_read_csr_mtx(const char *filename, int *info) {
  data_d_matrix *A = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  A->storage_type = Magma_CSR;
  data_storage_t st = Magma_CSR;
  *info = read_z_csr_from_mtx(&st, &A->num_rows, &A->num_cols, &A->nnz, &A->val, &A->row, &A->col,
                              filename);
  A->true_nnz = A->nnz;
  A->major = MagmaRowMajor;
  return A;
}

/* LACE's COO reader (:353) for non-symmetric files (it returns freed arrays
 * for symmetric ones): copies into caller-sized buffers, then releases */
int ref_read_coo_mtx(const char *filename, int *dims3, int cap, int *row, int *col, double *val) {
  data_storage_t st = Magma_COO;
  int *r = NULL, *c = NULL;
  double *v = NULL;
  int info = read_z_coo_from_mtx(&st, &dims3[0], &dims3[1], &dims3[2], &v, &r, &c, filename);
  if (info == 0 && dims3[2] <= cap) {
    memcpy(row, r, sizeof(int) * (size_t)dims3[2]);
    memcpy(col, c, sizeof(int) * (size_t)dims3[2]);
    memcpy(val, v, sizeof(double) * (size_t)dims3[2]);
  }
  free(r);
  free(c);
  free(v);
  return info;
}

int ref_write_csr_mtx(data_d_matrix *A, int major, const char *filename) {
  return data_zwrite_csr_mtx(*A, (data_order_t)major, filename);
}

/* MKL-semantics ILU(0) baseline (blas/zcsrilu0.cpp), in place on A's values */
int ref_csrilu0(data_d_matrix *A) { return data_dcsrilu0_mkl(A); }

}  /* extern "C" */
