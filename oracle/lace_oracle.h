/*
 * CPU oracle for the LACE preconditioned-solve path: a plain-C restatement of
 * LACE's ParILU(0), triangular solves, SpMV and FGMRES-Householder, plus the
 * variants LACE has no code for (synchronous sweeps, BCSR, FP32 factors).
 *
 * TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline leg may load this library, and only as the checker or the
 * timed CPU baseline - never as part of the lace_gb300 product path.
 *
 * Every function names the LACE source lines it follows (paths inside the
 * LACE source tree).  All index arrays are zero-based int32, values FP64
 * unless a name ends in _f32.
 */
#ifndef LACE_ORACLE_H
#define LACE_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* OpenMP thread count used by the loops LACE itself runs in parallel. */
void orc_set_threads(int n);
int orc_get_threads(void);

/* ---------------------------------------------------------------- ParILU */

/* One ParILU(0) sweep over A's pattern (COO order, rowidx/col).
 * L: CSR, unit diagonal stored last in each row (CSRL).
 * U: CSC (colptr/rowidx), diagonal stored last in each column (CSCU).
 * mode 0 (asynchronous, LACE's own semantics, src/parilu_v0_3.cpp:67-103):
 *   in place on Lnew/Unew (Lold/Uold are not read), sequential COO order, with
 *   LACE's exact arithmetic (including the subtract-then-restore of the last
 *   product, :84-90).  One thread gives LACE's deterministic result.
 * mode 1 (synchronous / Jacobi): reads Lold/Uold, writes Lnew/Unew; each
 *   entry uses s = a_ij - sum_{k<min(i,j)} l_ik u_kj summed in merge order.
 * Returns the un-normalised step sum (new-old)^2 (:94,99). */
double orc_parilu_sweep(int mode, int nnzA, const int *Arowidx, const int *Acol,
                        const double *Aval, const int *Lrow, const int *Lcol,
                        const double *Lold, double *Lnew, const int *Ucolptr,
                        const int *Urowidx, const double *Uold, double *Unew);

/* FP32 synchronous sweep (factors and arithmetic in float, A rounded to
 * float), the mixed-precision variant. */
double orc_parilu_sweep_sync_f32(int nnzA, const int *Arowidx, const int *Acol,
                                 const double *Aval, const int *Lrow,
                                 const int *Lcol, const float *Lold, float *Lnew,
                                 const int *Ucolptr, const int *Urowidx,
                                 const float *Uold, float *Unew);

/* ||(A - L U)|_S(A)||_F (the "nonlinear" residual, control/norms.cpp:375-387)
 * computed directly on A's pattern with L CSRL / U CSCU. */
double orc_ilu_nonlinres(int nnzA, const int *Arowidx, const int *Acol,
                         const double *Aval, const int *Lrow, const int *Lcol,
                         const double *Lval, const int *Ucolptr,
                         const int *Urowidx, const double *Uval);

/* data_zilures (control/norms.cpp:301-405): res = ||LU - A|| over pattern(LU)
 * (fill-in included), nonlinres over S(A).  L CSR with unit diagonal, U CSR. */
void orc_zilures(int n, const int *Arow, const int *Acol, const double *Aval,
                 const int *Lrow, const int *Lcol, const double *Lval,
                 const int *Urow, const int *Ucol, const double *Uval,
                 double *res, double *nonlinres);

/* ------------------------------------------------------------------ SpMV */

/* y = alpha*A*x + beta*y (blas/zspmv.cpp:61 semantics; beta==0 ignores y) */
void orc_spmv(int n, const int *row, const int *col, const double *val,
              double alpha, const double *x, double beta, double *y);

/* BCSR (row-major bs x bs blocks) y = A*x */
void orc_bcsr_spmv(int nbrows, int bs, const int *row, const int *col,
                   const double *val, const double *x, double *y);

/* ------------------------------------------------------ triangular solves */

/* Exact CSR triangular solve, x = T^{-1} b, using only the entries of the
 * requested triangle: lower uses col<i, upper col>i, the diagonal entry is
 * used unless unit != 0.  Sums in storage order - the semantics of
 * mkl_dcsrtrsv as called at src/fgmres_householder_restart.cpp:322-331. */
void orc_trsv(int n, const int *row, const int *col, const double *val,
              int lower, int unit, const double *b, double *x);
void orc_trsv_f32(int n, const int *row, const int *col, const float *val,
                  int lower, int unit, const float *b, float *x);

/* level of every row of a lower (or upper) triangular pattern:
 * lev[i] = 1 + max lev[j] over off-diagonal j in row i (0 if none).
 * Returns the number of levels. */
int orc_levels(int n, const int *row, const int *col, int lower, int *lev);

/* data_parcsrtrsv mirror (src/trisolve.cpp:256-351): in-place sweeps in
 * LACE's one-thread order until step <= tol or non-finite.
 * uplo 0 lower (diag last in row), 1 upper (diag first in row). */
int orc_parcsrtrsv(int uplo, int n, const double *val, const int *row,
                   const int *col, const double *rhs, double *y, double tol,
                   int *iter);

/* synchronous (Jacobi) variant: every sweep reads the previous iterate only.
 * Stops at step <= tol, non-finite step, or maxiter sweeps. */
int orc_jacobi_trsv(int uplo, int n, const double *val, const int *row,
                    const int *col, const double *rhs, double *y, double tol,
                    int maxiter, int *iter);

/* ------------------------------------------------------------------- BCSR */

/* One block ParILU(0) sweep (src/parilu_v0_3_bcsr.cpp:129-249).  L BCSR with
 * identity diagonal blocks stored last in each block row; U BCSC (blocks kept
 * untransposed, diagonal block last in each block column).  mode 0 in place
 * in COO order, mode 1 synchronous.  The U_jj inverse is exact Gauss-Jordan
 * without pivoting (LACE's data_inverse is LU without pivoting,
 * src/inverse.cpp:46).  Returns the un-normalised step. */
double orc_bcsr_parilu_sweep(int mode, int bs, int nblkA, const int *Arowidx,
                             const int *Acol, const double *Aval,
                             const int *Lrow, const int *Lcol,
                             const double *Lold, double *Lnew,
                             const int *Ucolptr, const int *Urowidx,
                             const double *Uold, double *Unew);

/* dense bs x bs row-major inverse, Gauss-Jordan without pivoting;
 * returns 0, or -1 on a zero pivot */
int orc_block_inverse(int bs, const double *a, double *ainv);

/* Block triangular solves.  Lower: unit (identity) diagonal blocks, uses
 * block columns < block row.  Upper: block row's diagonal block is applied
 * through its inverse Dinv (nbrows * bs*bs, row-major). */
void orc_bcsr_trsv_lower_unit(int nbrows, int bs, const int *row,
                              const int *col, const double *val,
                              const double *b, double *x);
void orc_bcsr_trsv_upper(int nbrows, int bs, const int *row, const int *col,
                         const double *val, const double *Dinv,
                         const double *b, double *x);
void orc_bcsr_trsv_lower_unit_f32(int nbrows, int bs, const int *row,
                                  const int *col, const float *val,
                                  const float *b, float *x);
void orc_bcsr_trsv_upper_f32(int nbrows, int bs, const int *row, const int *col,
                             const float *val, const float *Dinv,
                             const float *b, float *x);

/* --------------------------------------------------- Householder / Givens */

/* src/givens.cpp:46-67 */
void orc_givens(double a, double b, double tol, double *c, double *s);

/* ||I - Q^T Q||_inf over the first `search` columns of the column-major n x *
 * ld Q (src/orthogonality_error.cpp:46-83, control/norms.cpp:473-494) */
double orc_orthogonality_error(int n, int ld, const double *Q, int search);

/* ----------------------------------------------------- FGMRES-Householder */

/* operator kinds */
enum { ORC_OP_CSR = 0, ORC_OP_BCSR = 1 };
/* preconditioner kinds (choice numbers 0..2 are LACE's user_csrtrsv_choice) */
enum {
  ORC_PREC_TRSV = 0,     /* two exact triangular solves, FP64           */
  ORC_PREC_PARTRSV = 1,  /* data_parcsrtrsv L then U, tol (LACE mirror) */
  ORC_PREC_NONE = 2,     /* identity                                     */
  ORC_PREC_TRSV_F32 = 3, /* two exact triangular solves in FP32          */
  ORC_PREC_JACOBI = 4,   /* synchronous Jacobi sweeps, tol / max sweeps  */
  ORC_PREC_BCSR = 5,     /* block solves FP64                            */
  ORC_PREC_BCSR_F32 = 6  /* block solves FP32                            */
};

typedef struct {
  int kind;  /* ORC_OP_* */
  int n;     /* scalar rows */
  int bs;    /* block size for BCSR */
  const int *row, *col;
  const double *val;
} orc_operator;

/* M^{-1} q = T2^{-1} T1^{-1} q.  For the forward solve T1 = L (lower, unit),
 * T2 = U (upper); for the adjoint T1 = U^T (lower, non-unit: U's CSC image)
 * and T2 = L^T (upper, unit: L's CSC image). */
typedef struct {
  int kind;                      /* ORC_PREC_* */
  const int *t1_row, *t1_col;    /* first solve  */
  const double *t1_val;
  const float *t1_val32;
  int t1_lower, t1_unit;
  const int *t2_row, *t2_col;    /* second solve */
  const double *t2_val;
  const float *t2_val32;
  int t2_lower, t2_unit;
  const double *bdinv;           /* BCSR: inverted diagonal blocks of U */
  const float *bdinv32;
  double tol;                    /* PARTRSV / JACOBI */
  int max_sweeps;                /* JACOBI */
} orc_precond;

typedef struct {
  int search_max, restart_max, tol_type;  /* sparse_types.h:158-176 */
  double rtol;
  int monitor_orthog;
  int reorth;  /* MGS only: 0 Brown/Hindmarsh test, 1 never, 2 always */
} orc_gmres_par;

typedef struct {
  int restarts, search_directions;  /* as data_d_gmres_log (final cycle) */
  int total_iterations;             /* search directions over all cycles */
  double initial_residual, final_residual;
  int converged;                    /* |g| < rtol reached */
  int lost_update;                  /* LACE early-return path taken (see .c) */
  int info;                         /* LACE's return value */
} orc_gmres_log;

/* Right-preconditioned FGMRES with Householder Arnoldi and restarts, a
 * statement-by-statement mirror of src/fgmres_householder_restart.cpp:63-788
 * (one-thread order).  x is in/out.  resid_hist receives |g_{j+1}| per
 * search direction (restart_max*search_max entries, may be NULL);
 * orth_hist the monitor value per direction when monitor_orthog (may be
 * NULL). */
int orc_fgmres_householder(const orc_operator *A, const orc_precond *M,
                           const double *b, double *x, const orc_gmres_par *par,
                           orc_gmres_log *log, double *resid_hist,
                           double *orth_hist);

/* Right-preconditioned FGMRES with modified Gram-Schmidt Arnoldi, a
 * statement-by-statement mirror of src/fgmres_restart.cpp:63-532
 * (restarted != 0) or src/fgmres.cpp:64-517 (restarted == 0: one cycle,
 * breakdown threshold DBL_EPSILON, a non-finite residual stops, the update
 * summed into z before x += z).  Same in/out conventions as
 * orc_fgmres_householder; orth_hist holds the orthogonality error of the
 * Krylov basis v_0..v_j. */
int orc_fgmres_mgs(const orc_operator *A, const orc_precond *M, const double *b,
                   double *x, const orc_gmres_par *par, int restarted,
                   orc_gmres_log *log, double *resid_hist, double *orth_hist);

#ifdef __cplusplus
}
#endif

#endif
