/*
 * Flat C entry point around LACE's BCSR ParILU (src/parilu_v0_3_bcsr.cpp,
 * which exports the same data_PariLU_v0_3 symbol as the CSR version and is
 * therefore linked into its own library, oracle/_ref/liblace_ref_bcsr.so).
 * Test infrastructure only.
 */
#include "sparse.h"

#include <stdlib.h>
#include <string.h>

extern "C" {

/* A: BCSR handle (row-major blocks).  Returns L (BCSR lower, identity
 * diagonal blocks) and U (BCSC upper, blocks stored untransposed).
 * Iterates until the un-normalised step is <= reduction
 * (src/parilu_v0_3_bcsr.cpp:118). log2 = {sweeps, generation time}. */
void ref_bcsr_parilu(data_d_matrix *A, double reduction, data_d_matrix **L,
                     data_d_matrix **U, double *log2) {
  *L = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  *U = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  (*L)->storage_type = Magma_BCSRL;
  (*U)->storage_type = Magma_BCSCU;
  (*L)->blocksize = A->blocksize;
  (*U)->blocksize = A->blocksize;
  data_d_preconditioner_log log;
  memset(&log, 0, sizeof(log));
  data_PariLU_v0_3(A, *L, *U, reduction, &log);
  log2[0] = log.sweeps;
  log2[1] = log.precond_generation_time;
}

/* dense block inverse as LACE computes it (src/inverse.cpp:17): ParLU
 * without pivoting followed by iterative triangular solves */
int ref_dense_inverse(int bs, const double *a_rowmajor, double *ainv_rowmajor) {
  data_d_matrix A = {Magma_DENSE};
  A.num_rows = bs;
  A.num_cols = bs;
  A.ld = bs;
  A.nnz = bs * bs;
  A.true_nnz = A.nnz;
  A.major = MagmaRowMajor;
  A.blocksize = bs;
  LACE_CALLOC(A.val, A.nnz);
  memcpy(A.val, a_rowmajor, sizeof(double) * (size_t)A.nnz);
  data_d_matrix Ai = {Magma_DENSE};
  Ai.num_rows = bs;
  Ai.num_cols = bs;
  Ai.ld = bs;
  Ai.nnz = bs * bs;
  Ai.major = MagmaRowMajor;
  LACE_CALLOC(Ai.val, Ai.nnz);
  int info = data_inverse(&A, &Ai);
  memcpy(ainv_rowmajor, Ai.val, sizeof(double) * (size_t)Ai.nnz);
  data_zmfree(&A);
  data_zmfree(&Ai);
  return info;
}

}  /* extern "C" */
