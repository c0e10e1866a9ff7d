/*
 * Handle helpers shared by the two reference glue libraries (ref_glue.cpp for
 * the CSR path, ref_glue_bcsr.cpp for LACE's BCSR ParILU, which reuses the
 * data_PariLU_v0_3 symbol and so links separately).  Test infrastructure only.
 *
 * Matrices cross this boundary as opaque handles to LACE's data_d_matrix.
 */
#include "sparse.h"

#include <stdlib.h>
#include <string.h>

extern "C" {

/* handle <- copies of (row, col, val); storage is a data_storage_t value.
 * For a BCSR matrix pass blocksize > 0: nnz then counts blocks and val holds
 * nnz*blocksize^2 row-major block values. */
data_d_matrix *ref_mat_new(int storage, int nrows, int ncols, int nnz,
                           const int *row, const int *col, const double *val,
                           int blocksize) {
  data_d_matrix *A = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  A->storage_type = (data_storage_t)storage;
  A->num_rows = nrows;
  A->num_cols = ncols;
  A->fill_mode = MagmaFull;
  A->major = MagmaRowMajor;
  int nval = nnz;
  if (blocksize > 0) {
    A->blocksize = blocksize;
    A->ldblock = blocksize * blocksize;
    A->numblocks = nnz;
    nval = nnz * A->ldblock;
    A->nnz = nval;
  } else {
    A->nnz = nnz;
  }
  A->true_nnz = A->nnz;
  LACE_CALLOC(A->row, nrows + 1);
  LACE_CALLOC(A->col, (nnz > 0 ? nnz : 1));
  LACE_CALLOC(A->val, (nval > 0 ? nval : 1));
  memcpy(A->row, row, sizeof(int) * (size_t)(nrows + 1));
  memcpy(A->col, col, sizeof(int) * (size_t)nnz);
  memcpy(A->val, val, sizeof(double) * (size_t)nval);
  return A;
}

/* COO handle: row, col and val each nnz long */
data_d_matrix *ref_coo_new(int nrows, int ncols, int nnz, const int *row,
                           const int *col, const double *val) {
  data_d_matrix *A = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  A->storage_type = Magma_COO;
  A->num_rows = nrows;
  A->num_cols = ncols;
  A->fill_mode = MagmaFull;
  A->major = MagmaRowMajor;
  A->nnz = A->true_nnz = nnz;
  LACE_CALLOC(A->row, (nnz > 0 ? nnz : 1));
  LACE_CALLOC(A->col, (nnz > 0 ? nnz : 1));
  LACE_CALLOC(A->val, (nnz > 0 ? nnz : 1));
  memcpy(A->row, row, sizeof(int) * (size_t)nnz);
  memcpy(A->col, col, sizeof(int) * (size_t)nnz);
  memcpy(A->val, val, sizeof(double) * (size_t)nnz);
  return A;
}

/* dense column vector handle (n x 1, Magma_DENSE) */
data_d_matrix *ref_vec_new(int n, const double *v) {
  data_d_matrix *x = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  data_zvinit(x, n, 1, 0.0);
  memcpy(x->val, v, sizeof(double) * (size_t)n);
  return x;
}

void ref_mat_info(const data_d_matrix *A, int *info6) {
  info6[0] = A->storage_type;
  info6[1] = A->num_rows;
  info6[2] = A->num_cols;
  info6[3] = A->nnz;
  info6[4] = A->numblocks;
  info6[5] = A->blocksize;
}

/* copy out; nrow_ptr = number of row (or column) pointers, nidx = number of
 * index entries, nval = number of values */
void ref_mat_copy(const data_d_matrix *A, int nrow_ptr, int nidx, int nval,
                  int *row, int *col, double *val) {
  if (row) memcpy(row, A->row, sizeof(int) * (size_t)nrow_ptr);
  if (col) memcpy(col, A->col, sizeof(int) * (size_t)nidx);
  if (val) memcpy(val, A->val, sizeof(double) * (size_t)nval);
}

void ref_mat_free(data_d_matrix *A) {
  if (!A) return;
  data_zmfree(A);
  free(A);
}

/* B = convert(A) with B->diagorder_type preset (data_zmconvert reads it) */
data_d_matrix *ref_convert(const data_d_matrix *A, int old_format,
                           int new_format, int diagorder) {
  data_d_matrix *B = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  B->diagorder_type = (data_diagorder_t)diagorder;
  B->blocksize = A->blocksize;
  data_zmconvert(*A, B, (data_storage_t)old_format, (data_storage_t)new_format);
  return B;
}

/* the same with B->blocksize preset (CSR -> BCSR reads it) */
data_d_matrix *ref_convert_bs(const data_d_matrix *A, int old_format,
                              int new_format, int diagorder, int blocksize) {
  data_d_matrix *B = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  B->diagorder_type = (data_diagorder_t)diagorder;
  B->blocksize = blocksize;
  data_zmconvert(*A, B, (data_storage_t)old_format, (data_storage_t)new_format);
  return B;
}

data_d_matrix *ref_transpose(const data_d_matrix *A) {
  data_d_matrix *B = (data_d_matrix *)calloc(1, sizeof(data_d_matrix));
  data_zmtranspose(*A, B);
  return B;
}

}  /* extern "C" */
