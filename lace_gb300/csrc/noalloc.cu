// data_parcsrtrsv on device arrays, without allocating any memory.
//
// data_parcsrtrsv takes host arrays and copies them into device buffers it
// allocates on every call.  Some callers cannot allocate device memory at
// all: code that has handed the device's memory to its own pool or arena and
// forbids further allocations, and code in a latency-critical loop, where a
// cudaMalloc or cudaFree would synchronise the whole device and stall work on
// other streams.  lace_gpu_parcsrtrsv_noalloc serves them: the caller passes
// device arrays, and the scratch of the sweeps - the second iterate, the
// partial sums of the step reduction, the counters and the steps - sits in
// one file-scope device array of fixed size, so a call allocates nothing.
// The sweeps are the same kernels, in the same order, as in data_parcsrtrsv
// (LACE's sweep order, partrsv.cu), so both return the same iterate.
#include <cmath>
#include <mutex>
#include <utility>

#include "context.h"

namespace lace {
namespace {

constexpr int kNaMaxRows = LACE_GPU_NOALLOC_MAX_ROWS;
constexpr int kNaMaxPartials = 4096;  // blocks of the step reduction (4 per SM)
constexpr int kNaMaxDevices = 64;
// layout in doubles: the second iterate, the partial sums, the two steps of
// a round and four int counters (two tickets, the reduction's arrival
// counter, the status bits) in the last two slots
constexpr size_t kNaPartials = kNaMaxRows;
constexpr size_t kNaSteps = kNaPartials + kNaMaxPartials;
constexpr size_t kNaCounters = kNaSteps + 2;
constexpr size_t kNaWords = kNaCounters + 2;

// About 2 MB, held by every GPU that loads the library until the process
// exits.  In host code this name is a host-side stand-in, not a device
// address: host code uses the address cudaGetSymbolAddress returns.
static __device__ __align__(256) double g_noalloc_scratch[kNaWords];

std::mutex g_na_mu;
double *g_na_addr[kNaMaxDevices] = {};

// Device address of the scratch on the current device, looked up (with that
// device current) by the first call on the device.  Every call clears the
// counters itself on its own stream, so nothing depends on how an earlier
// call ended.
int noalloc_scratch(double **out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return DEV_ERR_NOT_INITIALIZED;
  }
  if (dev < 0 || dev >= kNaMaxDevices) return DEV_ERR_NOT_SUPPORTED;
  std::lock_guard<std::mutex> lk(g_na_mu);
  if (g_na_addr[dev] == nullptr) {
    double *p = nullptr;
    if (cudaGetSymbolAddress((void **)&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
      cudaGetLastError();
      return DEV_ERR_UNKNOWN;
    }
    g_na_addr[dev] = p;
  }
  *out = g_na_addr[dev];
  return 0;
}

}  // namespace
}  // namespace lace

using namespace lace;

extern "C" int lace_gpu_parcsrtrsv_noalloc(const data_uplo_t uplo, const data_storage_t storage,
                                           const data_diagorder_t diag, const int num_rows,
                                           const double *Aval, const int *row, const int *col,
                                           const double *rhsval, double *yval, const double tol, int *iter,
                                           void *stream) {
  // the storage / fill rule of data_parcsrtrsv (src/trisolve.cpp:262-345)
  bool lower;
  if (storage == Magma_CSRL && uplo == MagmaLower && diag != Magma_NODIAG) lower = true;
  else if (storage == Magma_CSRL || uplo == MagmaLower) return -1;
  else if (storage == Magma_CSRU && uplo == MagmaUpper && diag != Magma_NODIAG) lower = false;
  else if (storage == Magma_CSRU || uplo == MagmaUpper) return -1;
  else return 0;
  if (!iter) return set_err(DEV_ERR_INVALID_PTR);
  *iter = 0;
  if (num_rows < 0 || num_rows > kNaMaxRows) return set_err(DEV_ERR_NOT_SUPPORTED);
  if (num_rows == 0) return 0;
  if (!Aval || !row || !col || !rhsval || !yval) return set_err(DEV_ERR_INVALID_PTR);
  if (partrsv_partials_needed() > kNaMaxPartials) return set_err(DEV_ERR_NOT_SUPPORTED);
  cudaStream_t s = (cudaStream_t)stream;
  // the stream must belong to the current device, where the scratch address
  // is looked up
  int cur_dev = 0, stream_dev = 0;
  if (cudaGetDevice(&cur_dev) != cudaSuccess || cudaStreamGetDevice(s, &stream_dev) != cudaSuccess) {
    cudaGetLastError();
    return set_err(DEV_ERR_ILLEGAL_VALUE);
  }
  if (cur_dev != stream_dev) return set_err(DEV_ERR_ILLEGAL_VALUE);
  double *scr = nullptr;
  int rc = noalloc_scratch(&scr);
  if (rc) return set_err(rc);
  double h_steps[2] = {0.0, 0.0};
  int h_status = 0;
  PartrsvScratch sc;
  sc.a = scr;
  sc.partials = scr + kNaPartials;
  sc.steps = scr + kNaSteps;
  sc.counters = (int *)(scr + kNaCounters);
  sc.h_steps = h_steps;
  sc.h_status = &h_status;
  rc = partrsv_solve(s, lower, num_rows, row, col, Aval, rhsval, yval, tol, iter, sc);
  return rc ? set_err(rc) : 0;
}
