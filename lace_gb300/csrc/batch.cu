// Batched solves over many independent systems (lace_gpu_batch_*).
#include "context.h"

struct lace_gpu_batch {
  int dummy;
};

extern "C" int lace_gpu_batch_create(lace_gpu_batch **batch, lace_gpu_ctx *ctx, int nsys, const int *n,
                                     const int *row_off, const int *nnz_off, const int *row,
                                     const int *col, const double *val, int nrhs) {
  (void)batch; (void)ctx; (void)nsys; (void)n; (void)row_off; (void)nnz_off; (void)row; (void)col;
  (void)val; (void)nrhs;
  return lace::set_err(DEV_ERR_NOT_IMPLEMENTED);
}
extern "C" int lace_gpu_batch_destroy(lace_gpu_batch *batch) {
  delete batch;
  return DEV_SUCCESS;
}
extern "C" int lace_gpu_batch_solve(lace_gpu_batch *batch, int sweeps, int search_max, int restart_max,
                                    double rtol, const double *b, double *x, int *iters_out) {
  (void)batch; (void)sweeps; (void)search_max; (void)restart_max; (void)rtol; (void)b; (void)x;
  (void)iters_out;
  return lace::set_err(DEV_ERR_NOT_IMPLEMENTED);
}
