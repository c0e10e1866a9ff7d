/*
 * lace_gb300 - GB300 (sm_103a) implementation of LACE's preconditioned-solve
 * path: ParILU(0) -> sparse triangular solves -> FGMRES-Householder.
 *
 * Two layers, both plain C ABI (no C++ or torch types in any signature):
 *
 *  1. Drop-in entry points with LACE's own names and signatures
 *     (include/sparse.h of LACE).  A program built against LACE links this
 *     library in place of LACE's src/parilu_v0_3*.cpp, src/trisolve.cpp's
 *     data_parcsrtrsv, blas/zspmv.cpp and src/fgmres_householder*.cpp; the
 *     rest of LACE (IO, conversions, free) stays as it is.  Containers are
 *     LACE's data_d_matrix (host memory); every call uploads, runs on the
 *     GPU and downloads.  Unlike LACE, nothing here calls exit(): failures
 *     return DEV_ERR_* codes (ParILU, which LACE declares void, reports
 *     through log->sweeps = -1 and sets lace_gpu_last_error()).
 *
 *  2. GPU-resident entry points (lace_gpu_*) that keep a matrix, its factors
 *     and the Krylov workspace in HBM across calls.  All return DEV_SUCCESS
 *     (0) or a DEV_ERR_* code.
 *
 * The container and log structs below are byte-compatible with LACE's
 * include/sparse_types.h:14-176 (same members, same 64-byte alignment);
 * when LACE's own headers are included first they are used instead.
 */
#ifndef LACE_GB300_H
#define LACE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* everything declared here is exported from liblace_gb300.so (the library
 * is built with hidden visibility by default) */
#if defined(__GNUC__)
#pragma GCC visibility push(default)
#endif

/* ------------------------------------------------------------------------
 * LACE types (include/dense_types.h, include/sparse_types.h)
 * ---------------------------------------------------------------------- */
#ifndef DEV_TYPES_H
#define LACE_GB300_DEFINES_DEV_TYPES 1
#define DEV_ALIGN 64
typedef int data_int_t;
typedef double dataType;
/* error codes, include/dense_types.h:134-160 */
#define DEV_SUCCESS 0
#define DEV_ERR -100
#define DEV_ERR_NOT_INITIALIZED -101
#define DEV_ERR_NOT_SUPPORTED -103
#define DEV_ERR_ILLEGAL_VALUE -104
#define DEV_ERR_NOT_FOUND -105
#define DEV_ERR_ALLOCATION -106
#define DEV_ERR_INTERNAL_LIMIT -107
#define DEV_ERR_HOST_ALLOC -112
#define DEV_ERR_DEVICE_ALLOC -113
#define DEV_ERR_INVALID_PTR -115
#define DEV_ERR_UNKNOWN -116
#define DEV_ERR_NOT_IMPLEMENTED -117
#define DEV_ERR_NAN -118
#define DEV_ERR_BADPRECOND -204
#define DEV_NOTCONVERGED -205
typedef enum { MagmaRowMajor = 101, MagmaColMajor = 102 } data_order_t;
typedef enum { MagmaUpper = 121, MagmaLower = 122, MagmaFull = 123, MagmaHessenberg = 124 } data_uplo_t;
typedef enum {
  Magma_CSR = 611, Magma_ELLPACKT = 612, Magma_ELL = 613, Magma_DENSE = 614,
  Magma_BCSR = 615, Magma_CSC = 616, Magma_HYB = 617, Magma_COO = 618,
  Magma_ELLRT = 619, Magma_SPMVFUNCTION = 620, Magma_SELLP = 621,
  Magma_ELLD = 622, Magma_CSRLIST = 623, Magma_CSRD = 624, Magma_CSRL = 627,
  Magma_CSRU = 628, Magma_CSRCOO = 629, Magma_CUCSR = 630, Magma_COOLIST = 631,
  Magma_CSR5 = 632, Magma_CSCD = 633, Magma_CSCL = 634, Magma_CSCU = 635,
  Magma_CSCCOO = 636, Magma_DENSEL = 637, Magma_DENSEU = 638,
  Magma_DENSED = 639, Magma_BCSRD = 640, Magma_BCSRL = 641, Magma_BCSRU = 642,
  Magma_BCSC = 643, Magma_BCSCD = 644, Magma_BCSCL = 645, Magma_BCSCU = 646
} data_storage_t;
typedef enum { Magma_GENERAL = 581, Magma_SYMMETRIC = 582 } data_symmetry_t;
typedef enum {
  Magma_ORDERED = 591, Magma_DIAGFIRST = 592, Magma_UNITY = 593,
  Magma_VALUE = 594, Magma_ZERO = 595, Magma_NODIAG = 596
} data_diagorder_t;
#endif /* DEV_TYPES_H */

#ifndef SPARSE_TYPES_H
#define LACE_GB300_DEFINES_SPARSE_TYPES 1
/* include/sparse_types.h:14-41 */
typedef struct data_d_matrix {
  data_storage_t storage_type;
  data_symmetry_t sym;
  data_diagorder_t diagorder_type;
  data_uplo_t fill_mode;
  data_int_t num_rows;
  data_int_t num_cols;
  data_int_t nnz;
  data_int_t max_nnz_row;
  data_int_t diameter;
  data_int_t true_nnz;
  dataType *val __attribute__((aligned(DEV_ALIGN)));
  dataType *diag __attribute__((aligned(DEV_ALIGN)));
  data_int_t *row __attribute__((aligned(DEV_ALIGN)));
  data_int_t *rowidx __attribute__((aligned(DEV_ALIGN)));
  data_int_t *col __attribute__((aligned(DEV_ALIGN)));
  data_int_t *list;
  data_int_t *blockinfo;
  data_int_t blocksize;
  data_int_t ldblock;
  data_int_t numblocks;
  data_int_t alignment;
  data_order_t major;
  data_int_t ld;
  data_int_t pad_rows;
  data_int_t pad_cols;
} __attribute__((aligned(DEV_ALIGN))) data_d_matrix;

/* include/sparse_types.h:131-144 */
typedef struct data_z_preconditioner_log {
  data_int_t sweeps;
  data_int_t maxSweeps;
  dataType tol;
  dataType finalStep;
  dataType A_Frobenius;
  dataType precond_generation_time;
  dataType initial_residual;
  dataType initial_nonlinear_residual;
  dataType residual;
  dataType nonlinear_residual;
  data_int_t omp_num_threads;
} __attribute__((aligned(DEV_ALIGN))) data_d_preconditioner_log;

/* include/sparse_types.h:147-156 */
typedef struct data_z_gmres_log {
  data_int_t restarts;
  data_int_t search_directions;
  dataType solve_time;
  dataType initial_residual;
  dataType final_residual;
  dataType scaled_residual;
  dataType original_residual;
} __attribute__((aligned(DEV_ALIGN))) data_d_gmres_log;

/* include/sparse_types.h:158-176 */
typedef struct data_z_gmres_param {
  data_int_t search_max;
  data_int_t tol_type;
  dataType rtol;
  data_int_t reorth;
  data_int_t user_csrtrsv_choice;
  data_int_t monitorOrthog;
  data_int_t restart_max;
  data_int_t precondition;
  dataType parilu_reduction;
  data_int_t reorder;
} __attribute__((aligned(DEV_ALIGN))) data_d_gmres_param;
#endif /* SPARSE_TYPES_H */

/* ------------------------------------------------------------------------
 * 1. Drop-in entry points (LACE names and signatures)
 * ---------------------------------------------------------------------- */

/* Replaces src/parilu_v0_3.cpp:16 (CSR, and src/parilu_v0_3_bcsr.cpp:16 when
 * A->storage_type == Magma_BCSR).  Synchronous ParILU(0) sweeps on the GPU
 * until step <= reduction * initial residual or 20 sweeps.  Outputs L as
 * Magma_CSRL (unit diagonal last in each row) and U as Magma_CSCU
 * (diagonal last in each column), host arrays allocated with
 * posix_memalign(64) so data_zmfree() releases them. */
void data_PariLU_v0_3(data_d_matrix *A, data_d_matrix *L, data_d_matrix *U,
                      dataType reduction, data_d_preconditioner_log *log);

/* Replaces src/parilu_v0_3_prescribedSweeps.cpp:17: stops after
 * log->maxSweeps sweeps or step <= 4*eps. */
void data_PariLU_v0_3_prescribedSweeps(data_d_matrix *A, data_d_matrix *L,
                                       data_d_matrix *U, dataType reduction,
                                       data_d_preconditioner_log *log);

/* Replaces src/parilu_v0_3_gpu.cpp:110 (nthreads is accepted and ignored:
 * the launch shape is chosen for the GPU). */
void data_PariLU_v0_3_gpu(data_d_matrix *A, data_d_matrix *L, data_d_matrix *U,
                          dataType reduction, data_d_preconditioner_log *log,
                          int nthreads);

/* Replaces src/parilu_v0_3_gpu_prescribedSweeps.cpp:111 */
void data_PariLU_v0_3_gpu_prescribedSweeps(data_d_matrix *A, data_d_matrix *L,
                                           data_d_matrix *U, dataType reduction,
                                           data_d_preconditioner_log *log);

/* Replaces src/trisolve.cpp:256.  LACE's in-place sweeps in LACE's order
 * (L rows from the first, U rows from the last; each row's off-diagonal
 * products summed in storage order, then divided by the stored diagonal)
 * until sum (y_new - y_old)^2 <= tol or a non-finite step; the iterate and
 * *iter equal LACE's one-thread run bit for bit.  uplo MagmaLower needs
 * storage Magma_CSRL (diagonal last), MagmaUpper needs Magma_CSRU (diagonal
 * first); otherwise returns -1 as LACE does.  A column outside the matrix or
 * a diagonal position outside the arrays (where LACE would read outside
 * them) returns DEV_ERR_ILLEGAL_VALUE.  LACE loops forever for a negative
 * tol; here the loop also ends at a sweep that changes nothing.  Host
 * arrays. */
int data_parcsrtrsv(const data_uplo_t uplo, const data_storage_t storage,
                    const data_diagorder_t diag, const int num_rows,
                    const dataType *Aval, const int *row, const int *col,
                    const dataType *rhsval, dataType *yval, const dataType tol,
                    int *iter);

/* Replaces blas/zspmv.cpp:48: y = alpha*A*x + beta*y for CSR/CSRL/CSRU,
 * and (beyond LACE) Magma_BCSR; DEV_ERR_NOT_SUPPORTED otherwise. */
int data_z_spmv(dataType alpha, data_d_matrix *A, data_d_matrix *x,
                dataType beta, data_d_matrix *y);

/* Replaces src/fgmres_householder_restart.cpp:63.  Right-preconditioned
 * restarted FGMRES with Householder Arnoldi; preconditioner M = L*U given as
 * L (Magma_CSRL) and U (Magma_CSRU, or Magma_CSCU as ParILU returns it).
 * gmres_par->user_csrtrsv_choice: 0 exact triangular solves (sync-free
 * SpTRSV), 1 ParCSRTRSV with tol 1.0 (in LACE's sweep order the first sweep
 * is the exact substitution and the second changes nothing, so the
 * preconditioned vectors are the exact solves'), 2 no preconditioner.
 * Beyond LACE (whose data_z_spmv and solves take CSR only): A may be
 * Magma_BCSR (num_rows = block rows; b, x0 of num_rows * blocksize rows)
 * with the factors data_PariLU_v0_3 returns for it, L Magma_BCSR and U
 * Magma_BCSCU of the same block pattern (other factor layouts:
 * DEV_ERR_NOT_SUPPORTED); this holds for every FGMRES entry point below.
 * x0 is overwritten with the solution (LACE frees and re-allocates
 * x0->val; this replacement writes into the existing array).  Returns
 * DEV_SUCCESS when the residual target was reached, DEV_NOTCONVERGED
 * otherwise (LACE's own return value is inverted, see
 * src/fgmres_householder_restart.cpp:768-770). */
int data_fgmres_householder_restart(data_d_matrix *A, data_d_matrix *b,
                                    data_d_matrix *x0, data_d_matrix *L,
                                    data_d_matrix *U,
                                    data_d_gmres_param *gmres_par,
                                    data_d_gmres_log *gmres_log);

/* Replaces src/fgmres_householder_opt4.cpp:63 (one cycle, no restarts).
 * The FGMRES entry points hold at most 128 search directions per cycle on
 * the device: a larger search_max (LACE's tests pass 2000) runs cycles of
 * 128 and returns DEV_ERR_NOT_SUPPORTED if a cycle needs more. */
int data_fgmres_householder(data_d_matrix *A, data_d_matrix *b,
                            data_d_matrix *x0, data_d_matrix *L,
                            data_d_matrix *U, data_d_gmres_param *gmres_par,
                            data_d_gmres_log *gmres_log);

/* Replaces src/fgmres_restart.cpp:63 (declared include/sparse.h:1034).
 * Right-preconditioned restarted FGMRES with modified Gram-Schmidt Arnoldi;
 * arguments, preconditioner choices and x0 handling as
 * data_fgmres_householder_restart.  gmres_par->reorth: 0 reorthogonalise
 * when the Brown/Hindmarsh test asks (:336), 2 always, other values never.
 * Returns DEV_SUCCESS when the residual target was reached, DEV_NOTCONVERGED
 * otherwise (LACE's own value is inverted, :510-512). */
int data_fgmres_restart(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0,
                        data_d_matrix *L, data_d_matrix *U,
                        data_d_gmres_param *gmres_par, data_d_gmres_log *gmres_log);

/* Replaces src/fgmres.cpp:64 (declared include/sparse.h:1027): one cycle of
 * the same (happy breakdown below DBL_EPSILON, a non-finite residual stops,
 * x += sum_j z_j y_j). */
int data_fgmres(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0,
                data_d_matrix *L, data_d_matrix *U, data_d_gmres_param *gmres_par,
                data_d_gmres_log *gmres_log);

/* Matrix Market files (replace control/magma_zmio.cpp:92, 941 and 587;
 * declared in include/sparse.h).  Same results as LACE's: entries in file
 * order, symmetric and hermitian files expanded entry by entry, each row
 * sorted by column; output lines "%d %d %.16g" in row order (or, for
 * MagmaColMajor from a row-major matrix, column order), byte for byte.
 * Parsed and formatted on host threads.  Arrays allocated like LACE_CALLOC
 * (data_zmfree releases them).  Returns DEV_ERR_NOT_FOUND for a missing
 * file, DEV_ERR_NOT_SUPPORTED for a banner LACE rejects (only coordinate
 * real, integer, pattern or complex matrices), DEV_ERR_UNKNOWN for a
 * malformed size line or missing entries, DEV_ERR_ILLEGAL_VALUE for an index
 * outside the declared size (LACE writes out of bounds there); -1 when the
 * output file cannot be opened, as LACE. */
int read_z_csr_from_mtx(data_storage_t *type, int *n_row, int *n_col, int *nnz,
                        dataType **val, int **row, int **col, const char *filename);
int data_z_csr_mtx(data_d_matrix *A, const char *filename);
int data_zwrite_csr_mtx(data_d_matrix A, data_order_t MajorType, const char *filename);
/* Replace control/magma_zmio.cpp:353-557 and 957-967: the entries in file order
 * (symmetric and hermitian files expanded; LACE returns freed arrays for
 * those), *type set to Magma_CSR as LACE sets it. */
int read_z_coo_from_mtx(data_storage_t *type, int *n_row, int *n_col, int *nnz,
                        dataType **coo_val, int **coo_row, int **coo_col, const char *filename);
int data_z_coo_mtx(data_d_matrix *A, const char *filename);

/* The setup conversions, on host threads, with LACE's results:
 * data_zmconvert (control/magma_zmconverter.cpp:199) for CSR, CSRL or CSRU
 * sources to CSR, CUCSR, CSRL, CSRU, COO, CSRCOO, CSC, CSCL, CSCU, CSCCOO and
 * BCSR (B->blocksize set), COO to CSR, and BCSR to BCSRL, BCSRU, BCSCU; B->diagorder_type
 * selects the diagonal of a split as in LACE.  Other pairs return
 * DEV_ERR_NOT_SUPPORTED with B untouched.  data_zmtranspose
 * (control/magma_zmtranspose.cpp:484) and data_rowindex
 * (control/magma_zmconverter.cpp:145).  Output arrays are posix_memalign(64)
 * and zeroed, so data_zmfree releases them. */
int data_zmconvert(data_d_matrix A, data_d_matrix *B, data_storage_t old_format, data_storage_t new_format);
int data_zmtranspose(data_d_matrix A, data_d_matrix *B);
int data_rowindex(data_d_matrix *A, int **rowidx);

/* Cuthill-McKee orderings (src/cuthill_mckee.cpp:53), on the host:
 * nn_map[old] = new.  The seed is the lowest-numbered node of maximum degree
 * (off-diagonal entries of its row), nodes are numbered breadth first over
 * A's rows, each node's unnumbered neighbours in order of decreasing degree
 * (lower index first among equals), each further component from its own
 * seed; reverse gives new' = n - 1 - new.  This is the ordering LACE's
 * source describes; LACE's routine itself reads outside its arrays on
 * ordinary meshes, so its results are not reproducible (a null argument or a
 * malformed pattern sets lace_gpu_last_error() and leaves nn_map alone). */
#if defined(__cplusplus) && !defined(SPARSE_Z_H)
void data_reorder_cuthill_mckee(data_d_matrix *A, int *nn_map, bool reverse = false);
#elif defined(__cplusplus)
void data_reorder_cuthill_mckee(data_d_matrix *A, int *nn_map, bool reverse);
#else
void data_reorder_cuthill_mckee(data_d_matrix *A, int *nn_map, _Bool reverse);
#endif

/* src/reorder.cpp:167: reorder 1 Cuthill-McKee, 2 reverse Cuthill-McKee,
 * anything else but 3 none; A (Magma_CSR, or Magma_BCSR by block rows) is
 * replaced in place by A in the new numbering, rows sorted by column, its
 * arrays reallocated as LACE's are.  P[new] = old and Pinv[old] = new (LACE
 * hands the old-to-new map to its permutation as P and so applies the inverse
 * ordering).  3 (AMD, SuiteSparse in LACE) returns DEV_ERR_NOT_SUPPORTED with
 * A untouched.  Nothing is printed. */
int data_sparse_reorder(data_d_matrix *A, int *P, int *Pinv, int reorder);

/* Replaces control/norms.cpp:301: *res = ||A - L U||_F over the product's
 * pattern (fill-in included) and *nonlinres = the same over the entries of
 * A the product holds, on the GPU without forming L U.  L: CSRL with its
 * unit diagonal stored (L.row[1] == 1) or strictly lower (L.row[1] == 0),
 * U: Magma_CSCU or Magma_CSRU.  LU is not formed; the caller's matrix is
 * left as passed. */
int data_zilures(data_d_matrix A, data_d_matrix L, data_d_matrix U,
                 data_d_matrix *LU, dataType *res, dataType *nonlinres);

/* Replaces control/norms.cpp:409 (data_zilures_bcsr): L and U read as BCSR
 * (num_rows block rows of blocksize^2 row-major blocks), every block entry
 * expanded to scalar CSR as LACE's BCSR -> CSR conversion does, their
 * product measured against A (scalar CSR, num_rows = blocks x blocksize)
 * as data_zilures does, L's values as stored.  LACE reads both factors with
 * the BCSR reader whatever their storage tag, and so does this.  LU is not
 * formed. */
int data_zilures_bcsr(data_d_matrix A, data_d_matrix L, data_d_matrix U,
                      data_d_matrix *LU, dataType *res, dataType *nonlinres);

/* ------------------------------------------------------------------------
 * 2. GPU-resident API
 * ---------------------------------------------------------------------- */

typedef struct lace_gpu_ctx lace_gpu_ctx;

/* precision of the ParILU factors and of both triangular solves; the outer
 * FGMRES, its SpMV and the reflectors are FP64-class: FP64, or in the
 * one-kernel Householder step of FP32/BF16 runs double-float pairs (about 48
 * bits, on the FP32 pipe); each cycle's true residual is FP64 */
enum { LACE_PREC_FP64 = 0, LACE_PREC_FP32 = 1, LACE_PREC_BF16_STORE = 2 };
/* how M^{-1} is applied */
enum {
  LACE_TRSV_SYNCFREE = 0, /* exact, sync-free (ready flags per row chunk) */
  LACE_TRSV_LEVELS = 1,   /* exact, level-scheduled                       */
  LACE_TRSV_JACOBI = 2,   /* synchronous Jacobi sweeps (not LACE's order: */
                          /* inexact; jacobi_sweeps / jacobi_tol)         */
  LACE_TRSV_NONE = 3      /* identity                                     */
};

typedef struct lace_gpu_options {
  int precision;        /* LACE_PREC_*                                   */
  int trsv_mode;        /* LACE_TRSV_*                                   */
  int jacobi_sweeps;    /* sweeps per triangle for LACE_TRSV_JACOBI      */
  double jacobi_tol;    /* ... or stop when sum (dy)^2 <= tol            */
  int use_graph;        /* capture each Arnoldi cycle in a CUDA graph    */
  int spmv_lanes;       /* lanes per CSR row; 0 = autotune               */
  int trsv_rows_per_lane; /* sync-free chunk = 32 * this rows; 0 = auto  */
  int monitor_orthog;   /* ||I - Q^T Q||_inf after every step (slow)     */
  /* Sync-free solve schedule.  0 = autotune; trsv_chunks_per_block > 0 pins
   * it (with trsv_rows_per_lane, 0 meaning 1): chunks per block (<= 1024),
   * warps per CTA (1-16, 0 = 16) and CTAs per thread-block cluster (1, 2, 4,
   * 8 or 16; 0 = 1; a cluster the device or the shared memory cannot hold runs
   * as 1). */
  int trsv_chunks_per_block;
  int trsv_warps;
  int trsv_cluster;
} lace_gpu_options;

void lace_gpu_default_options(lace_gpu_options *opt);

/* Options used by the drop-in (LACE-named) entry points of section 1, e.g.
 * FP32 factors for data_PariLU_v0_3 / data_fgmres_householder_restart.
 * NULL restores the defaults (FP64, sync-free solves, CUDA graphs).
 * No counterpart in LACE, whose calls carry no precision or mode knobs. */
int lace_gpu_dropin_set_options(const lace_gpu_options *opt);

/* stream: a cudaStream_t (NULL = a stream owned by the context) */
int lace_gpu_ctx_create(lace_gpu_ctx **ctx, int device, void *stream);
int lace_gpu_ctx_destroy(lace_gpu_ctx *ctx);
int lace_gpu_set_options(lace_gpu_ctx *ctx, const lace_gpu_options *opt);
void *lace_gpu_stream(lace_gpu_ctx *ctx);

/* Upload A (zero-based CSR, sorted columns, every diagonal present) and run
 * the structural analysis: L/U split, CSC image of U, A->factor position
 * maps, SpTRSV chunk classification and level sets, SpMV autotuning.
 * _host: arrays in host memory; _device: arrays already in device memory. */
int lace_gpu_upload_csr_host(lace_gpu_ctx *ctx, int n, int nnz, const int *row,
                             const int *col, const double *val);
int lace_gpu_upload_csr_device(lace_gpu_ctx *ctx, int n, int nnz,
                               const int *row, const int *col,
                               const double *val);
/* BCSR with row-major bs x bs blocks (host arrays); nblk blocks */
int lace_gpu_upload_bcsr_host(lace_gpu_ctx *ctx, int nbrows, int bs, int nblk,
                              const int *row, const int *col, const double *val);
/* refresh only the values of A (same pattern), device array */
int lace_gpu_update_values_device(lace_gpu_ctx *ctx, const double *val);

/* ParILU(0): `sweeps` synchronous sweeps from the A-initial guess.
 * step_out (may be NULL): step of the last sweep, normalised by ||A||_F.
 * nonlinres_out (may be NULL): ||(A-LU)|_S||_F / ||A||_F after the sweeps.
 * Returns DEV_ERR_BADPRECOND when the last step is not finite (a zero or
 * non-finite pivot); the factors are then left as the sweeps made them. */
int lace_gpu_parilu0(lace_gpu_ctx *ctx, int sweeps, double *step_out,
                     double *nonlinres_out);

/* y = alpha*A*x + beta*y, device vectors (FP64) */
int lace_gpu_spmv(lace_gpu_ctx *ctx, double alpha, const double *x,
                  double beta, double *y);

/* z = M^{-1} q with the current factors and options (device FP64) */
int lace_gpu_apply_precond(lace_gpu_ctx *ctx, const double *q, double *z);

/* The sync-free solve schedule in use, once the first solve has tuned it:
 * out[0] rows per lane, out[1] chunks per block, out[2] warps per CTA,
 * out[3] CTAs per thread-block cluster (1: none).  DEV_ERR_NOT_INITIALIZED
 * before.  No counterpart in LACE. */
int lace_gpu_get_trsv_schedule(lace_gpu_ctx *ctx, int *out);

/* z = M^{-1} q as one step of the FGMRES cycle applies it, enqueued on the
 * context's stream without waiting: q and z are device vectors in the
 * vector type of the factor precision (float for FP32/BF16 factors, double
 * for FP64).  For timing the preconditioner kernels; the preconditioner must
 * have been applied once (lace_gpu_apply_precond) since the factors changed,
 * and a spin-wait timeout shows in the next lace_gpu_apply_precond or solve. */
int lace_gpu_precond_enqueue(lace_gpu_ctx *ctx, const void *q, void *z);

/* Largest num_rows lace_gpu_parcsrtrsv_noalloc accepts. */
#define LACE_GPU_NOALLOC_MAX_ROWS 262144

/* data_parcsrtrsv on DEVICE arrays, allocating no memory.  No counterpart in
 * the reference: it is for callers that cannot allocate device memory - code
 * whose device memory belongs to its own pool or arena, which forbids further
 * allocations, and code in a latency-critical loop, where cudaMalloc/cudaFree
 * would synchronise the whole device.  Same arguments, rule for uplo /
 * storage / diag, sweeps and result as data_parcsrtrsv (LACE's sweep order,
 * bit for bit), but Aval, row, col, rhsval and yval (start vector in,
 * solution out) are device pointers, and the sweeps run on `stream` (NULL:
 * the default stream), which must belong to the current device
 * (DEV_ERR_ILLEGAL_VALUE otherwise); the call returns when the solve is done,
 * after one host synchronisation per two sweeps.  Its scratch is one fixed
 * device array (about 2 MB, held by every GPU that loads the library):
 * num_rows above LACE_GPU_NOALLOC_MAX_ROWS returns DEV_ERR_NOT_SUPPORTED.
 * The first call on a device looks the scratch's address up and should come
 * before any stream capture.  Every call clears the scratch's counters
 * itself, but all calls use the same scratch: calls that overlap on the GPU
 * (from several threads or streams) race and give wrong results. */
int lace_gpu_parcsrtrsv_noalloc(const data_uplo_t uplo, const data_storage_t storage,
                                const data_diagorder_t diag, const int num_rows,
                                const dataType *Aval, const int *row, const int *col,
                                const dataType *rhsval, dataType *yval, const dataType tol,
                                int *iter, void *stream);

/* ------------------------------------------------------------------------
 * Failure handling (no counterpart in LACE, which exits or returns codes)
 * ---------------------------------------------------------------------- */

/* Self-test of the bounded device waits.  Runs data_parcsrtrsv's sweep
 * kernel on a built-in 4096-row bidiagonal triangle with its first row group
 * withheld (its ticket is never handed out), so the rows after it wait for
 * values nothing writes; each wait gives up after max_polls polls (<= 0: the
 * library's limit, about a second), sets a status bit and returns, which the
 * host reads into *status_out (may be NULL; bit 1 = a wait gave up).  Then
 * the same sweep runs with every row group on the same device (with the
 * library's own limit).  Returns
 * DEV_SUCCESS when the first sweep reported the timeout and the second is
 * the exact substitution with no status bit (the device stayed usable). */
int lace_gpu_selftest_wait_limit(int max_polls, int *status_out);

/* Fault injection for the host side: the next `after` device allocations of
 * the library succeed and every one after them fails as if cudaMalloc had
 * (the call that needed it returns DEV_ERR_DEVICE_ALLOC); after < 0 turns
 * the injection off.  Process-wide. */
void lace_gpu_inject_alloc_failure(int after);

/* one triangle: which 0 = L (unit lower), 1 = U (upper), 2 = U^T (lower),
 * 3 = L^T (unit upper); device FP64 in/out (converted internally) */
int lace_gpu_sptrsv(lace_gpu_ctx *ctx, int which, const double *b, double *x);

/* FGMRES-Householder on device vectors b, x (x: initial guess in, solution
 * out).  par: LACE's parameter struct (search_max, restart_max, tol_type,
 * rtol, user_csrtrsv_choice is ignored here: the context options decide);
 * log: LACE's log struct (search_directions = directions of the final
 * cycle, restarts = index of the final cycle, as LACE fills it).
 * total_iters (may be NULL): search directions over all cycles. */
int lace_gpu_fgmres_householder(lace_gpu_ctx *ctx, const double *b, double *x,
                                const data_d_gmres_param *par,
                                data_d_gmres_log *log, int *total_iters);

/* FGMRES with modified Gram-Schmidt Arnoldi on device vectors (LACE's
 * data_fgmres_restart when restarted != 0, else data_fgmres); par and log
 * as lace_gpu_fgmres_householder, par->reorth as LACE's. */
int lace_gpu_fgmres_mgs(lace_gpu_ctx *ctx, const double *b, double *x,
                        const data_d_gmres_param *par, int restarted,
                        data_d_gmres_log *log, int *total_iters);

/* Facts about the last FGMRES solve of this context: out[0] = directions
 * that the Gram-Schmidt FGMRES reorthogonalised (LACE prints
 * "Reorthogonalize" for each); out[1] = 1 when conditional CUDA graph nodes
 * are available (the separate-kernel step puts its second pass in one);
 * out[2] = 1 when each Gram-Schmidt Arnoldi step after the solves runs as
 * one cooperative kernel (environment LACE_GB300_MGS_STEP=0 at context
 * creation selects the separate kernels); out[3] = the same for the
 * Householder step (LACE_GB300_HH_STEP=0: passes A, B, C).  out: 4 ints. */
int lace_gpu_get_solve_stats(lace_gpu_ctx *ctx, int *out);

/* The orthogonality monitor of the last FGMRES solve on ctx (options
 * monitor_orthog = 1): LACE's data_orthogonality_error
 * (src/orthogonality_error.cpp:46-83), ||I - Q^T Q||_inf of the Krylov
 * vectors after every search direction, over all cycles in order, which LACE
 * prints as it goes.  ctx NULL: the context of the LACE-named calls
 * (data_fgmres_householder_restart with gmres_par->monitorOrthog = 1).
 * Writes min(capacity, *count) values to out; *count is the number of
 * directions (0 when the monitor was off). */
int lace_gpu_get_orthog_history(lace_gpu_ctx *ctx, double *out, int capacity, int *count);

/* Measurement: the mean device time of one launch of the one-kernel Arnoldi
 * step j (method 0 Householder, 1 Gram-Schmidt), replayed reps times on the
 * basis the last FGMRES solve of this context left (j + 2 <= its
 * search_max), timed with CUDA events on the context's stream.  The replays
 * overwrite that solve's cycle state; the next solve starts afresh.
 * DEV_ERR_NOT_SUPPORTED when that step runs as separate kernels. */
int lace_gpu_time_arnoldi_step(lace_gpu_ctx *ctx, int method, int j, int reps, double *seconds);

/* Adjoint of the solve x = A^{-1} b for a loss L(x): given dL/dx (device),
 * solves A^T lambda = dL/dx with FGMRES-Householder preconditioned by the
 * transposed factors (U^T then L^T), and returns dL/db = lambda and
 * dL/dA_ij = -lambda_i x_j on A's pattern (nnz values, CSR order).
 * x is the forward solution (device).  Either output may be NULL. */
int lace_gpu_solve_backward(lace_gpu_ctx *ctx, const double *x,
                            const double *dLdx, const data_d_gmres_param *par,
                            double *dLdb, double *dLdA_val, int *total_iters);

/* Last error recorded on this thread (for the void drop-in calls). */
int lace_gpu_last_error(void);
const char *lace_gpu_error_string(int code);

/* ------------------------------------------------------------------------
 * GPU-side setup conversions on device arrays (zero-based CSR), the GPU form
 * of the conversions the factorisation path runs: data_rowindex
 * (control/magma_zmconverter.cpp:145), the CSR -> CSRL/CSRU split (:304),
 * the CSR transpose (control/magma_zmtranspose.cpp:85) and CSR -> BCSR
 * (:614).  Results equal the host data_zmconvert / data_zmtranspose /
 * data_rowindex array for array; work runs on the context's stream and the
 * calls return once it is done.
 * ---------------------------------------------------------------------- */
/* rowidx[p] = the row of entry p */
int lace_gpu_rowindex_device(lace_gpu_ctx *ctx, int n, const int *row, int *rowidx);
/* lower = 1: CSRL, 0: CSRU, with data_diagorder_t diagorder as LACE's
 * B->diagorder_type (Magma_UNITY, Magma_VALUE, Magma_ZERO, Magma_NODIAG or
 * another value for LACE's default).  *nnz_out = the entries the rows hold
 * (LACE's nnz field also counts a lower split's default diagonal, which no
 * row holds).  brow (n + 1 ints) may be NULL for a size query; bcol and bval
 * (nnz_out entries) NULL skip the fill. */
int lace_gpu_csr_split_device(lace_gpu_ctx *ctx, int n, const int *row, const int *col, const double *val,
                              int lower, int diagorder, int *nnz_out, int *brow, int *bcol, double *bval);
/* the transpose as CSR (tptr: ncols + 1; tidx, tval: nnz), each row of the
 * transpose by ascending column; DEV_ERR_ILLEGAL_VALUE for a column index
 * outside [0, ncols) */
int lace_gpu_csr_transpose_device(lace_gpu_ctx *ctx, int n, int ncols, const int *row, const int *col,
                                  const double *val, int *tptr, int *tidx, double *tval);
/* CSR -> BCSR with bs x bs row-major blocks, block columns ascending in each
 * block row, zero-filled; *nblocks_out = blocks; brow ((n+bs-1)/bs + 1 ints)
 * may be NULL for a size query; bcol, bval (nblocks, nblocks*bs*bs) NULL skip
 * the fill.  DEV_ERR_NOT_SUPPORTED for a block row with more than 256 block
 * columns. */
int lace_gpu_csr_to_bcsr_device(lace_gpu_ctx *ctx, int n, const int *row, const int *col, const double *val,
                                int bs, int *nblocks_out, int *brow, int *bcol, double *bval);

/* ------------------------------------------------------------------------
 * Batched solves: many independent CSR systems, several right-hand sides
 * each; every system's ParILU sweeps and FGMRES-Householder for every
 * (system, rhs) pair in one persistent launch (captured in a CUDA graph when
 * the context's use_graph option is on).  Each row of a system's triangles
 * may hold at most 4 off-diagonal entries (DEV_ERR_NOT_SUPPORTED otherwise).
 * ---------------------------------------------------------------------- */
typedef struct lace_gpu_batch lace_gpu_batch;

/* Host arrays: system s has n[s] rows starting at global row row_off[s]
 * (row_off[0] = 0, row_off[s+1] = row_off[s] + n[s]); `row` concatenates
 * the systems' local row-pointer arrays (n[s]+1 entries each, so system s's
 * starts at row + row_off[s] + s); its column indices and values start at
 * col + nnz_off[s] / val + nnz_off[s] and are local to the system.  nrhs
 * right-hand sides per system (1..64).  The context `ctx` becomes the
 * batch's working context (its options decide the factor precision). */
int lace_gpu_batch_create(lace_gpu_batch **batch, lace_gpu_ctx *ctx, int nsys,
                          const int *n, const int *row_off, const int *nnz_off,
                          const int *row, const int *col, const double *val,
                          int nrhs);
int lace_gpu_batch_destroy(lace_gpu_batch *batch);
/* ParILU sweeps for every system, then FGMRES-Householder(search_max <= 64)
 * on every (system, rhs) pair to its own relative tolerance rtol.  b, x:
 * device arrays of nrhs vectors of length N = sum n[s], rhs-major: entry i of
 * system s for right-hand side r is at [r*N + row_off[s] + i].  x holds the
 * initial guesses.  iters_out (host, nsys*nrhs, system-major, may be NULL):
 * search directions used per (system, rhs). */
int lace_gpu_batch_solve(lace_gpu_batch *batch, int sweeps, int search_max,
                         int restart_max, double rtol, const double *b,
                         double *x, int *iters_out);

/* ABI self-description for bindings: sizeof and member offsets of the
 * LACE structs as compiled into this library. */
int lace_gpu_abi_layout(int *out, int cap);

#if defined(__GNUC__)
#pragma GCC visibility pop
#endif

#ifdef __cplusplus
}
#endif

#endif /* LACE_GB300_H */
