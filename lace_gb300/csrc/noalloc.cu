// The Jacobi triangular solve of data_parcsrtrsv on device arrays, without
// allocating any memory.
//
// data_parcsrtrsv takes host arrays and copies them into device buffers it
// allocates on every call.  Some callers cannot allocate device memory at
// all: code that has handed the device's memory to its own pool or arena and
// forbids further allocations, and code in a latency-critical loop, where a
// cudaMalloc or cudaFree would synchronise the whole device and stall work on
// other streams.  lace_gpu_parcsrtrsv_noalloc serves them: the caller passes
// device arrays, and the scratch of the sweeps - the second iterate, the
// partial sums of the step reduction, its arrival counter and the step itself
// - sits in one file-scope device array of fixed size, so a call allocates
// nothing.  The sweeps are the same kernels, in the same order, as in
// data_parcsrtrsv, so both return the same iterate.
#include <cmath>
#include <mutex>
#include <utility>

#include "context.h"

namespace lace {
namespace {

constexpr int kNaMaxRows = LACE_GPU_NOALLOC_MAX_ROWS;
constexpr int kNaMaxPartials = 4096;  // blocks of the step reduction (4 per SM)
constexpr int kNaMaxDevices = 64;
// layout in doubles: the second iterate, the partial sums, the step, and the
// arrival counter (an int in the last slot)
constexpr size_t kNaPartials = kNaMaxRows;
constexpr size_t kNaStep = kNaPartials + kNaMaxPartials;
constexpr size_t kNaCounter = kNaStep + 1;
constexpr size_t kNaWords = kNaCounter + 1;

// About 2 MB, held by every GPU that loads the library until the process
// exits.  In host code this name is a host-side stand-in, not a device
// address: host code uses the address cudaGetSymbolAddress returns.
static __device__ __align__(256) double g_noalloc_scratch[kNaWords];

std::mutex g_na_mu;
double *g_na_addr[kNaMaxDevices] = {};

// Device address of the scratch on the current device.  The first call on a
// device looks it up (with that device current) and clears the counter on
// stream s, then waits for that clear.
int noalloc_scratch(cudaStream_t s, double **out) {
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
    // the reduction's arrival counter must start at zero; its last block
    // puts it back to zero after every reduction
    if (cudaMemsetAsync(p + kNaCounter, 0, sizeof(double), s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return DEV_ERR_UNKNOWN;
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
  if (num_sms() * 4 > kNaMaxPartials) return set_err(DEV_ERR_NOT_SUPPORTED);
  cudaStream_t s = (cudaStream_t)stream;
  double *scr = nullptr;
  int rc = noalloc_scratch(s, &scr);
  if (rc) return set_err(rc);
  TriDev t;
  t.n = num_rows;
  t.row = row;
  t.col = col;
  t.val = Aval;
  t.lower = lower ? 1 : 0;
  t.unit = 0;  // LACE divides by the stored diagonal
  double *cur = yval, *nxt = scr;
  double step = 1.e8;
  // Jacobi sweeps converge in at most (number of levels) sweeps; bound the loop
  const int cap = num_rows + 2;
  while (step > tol && std::isfinite(step) && *iter < cap) {
    launch_jacobi_sweep(s, t, VType::F64, rhsval, 0, cur, nxt, 0, nullptr, false);
    launch_sqdiff(s, num_rows, nxt, cur, 0, scr + kNaPartials, (int *)(scr + kNaCounter), scr + kNaStep);
    if (cudaMemcpyAsync(&step, scr + kNaStep, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return set_err(DEV_ERR_UNKNOWN);
    std::swap(cur, nxt);
    *iter = *iter + 1;
  }
  if (cur != yval) {
    if (cudaMemcpyAsync(yval, cur, sizeof(double) * (size_t)num_rows, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return set_err(DEV_ERR_UNKNOWN);
  }
  return 0;
}
