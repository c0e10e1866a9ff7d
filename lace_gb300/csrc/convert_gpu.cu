// The setup conversions of the factorisation path on the GPU, for callers
// whose matrices are already in device memory: data_rowindex
// (control/magma_zmconverter.cpp:145-167), the CSR -> CSRL / CSRU split
// (:304-461), the CSR transpose (control/magma_zmtranspose.cpp:85-185) and
// CSR -> BCSR (:614-668, LACE's zero-based mkl_dcsrbsr call).  Outputs equal
// the host forms in convert.cu (and so LACE's) array for array on zero-based
// input: rows keep their entries' order, a transposed column lists its rows
// ascending, a block row its block columns ascending, blocks row-major.
//
// Counts run a thread per row (or block row), offsets come from a three-phase
// exclusive scan written here, and rows are filled a thread per row; the
// transpose scatters with one atomic per entry and then orders each column by
// row, so the result does not depend on scheduling.
#include <algorithm>

#include "context.h"

namespace lace {

constexpr int kScanT = 1024, kScanPer = 4, kScanChunk = kScanT * kScanPer;

// in-block exclusive scan of kScanChunk values; block totals to bsum
__global__ void __launch_bounds__(kScanT) k_scan_chunks(const int *__restrict__ in, int n, int *__restrict__ out,
                                                        int *__restrict__ bsum) {
  __shared__ int sw[kScanT / 32];
  const int base = blockIdx.x * kScanChunk + threadIdx.x * kScanPer;
  int v[kScanPer], t = 0;
#pragma unroll
  for (int u = 0; u < kScanPer; ++u) {
    v[u] = base + u < n ? in[base + u] : 0;
    t += v[u];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = t;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sw[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int s = lane < kScanT / 32 ? sw[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    if (lane < kScanT / 32) sw[lane] = s;
  }
  __syncthreads();
  int run = x - t + (wid > 0 ? sw[wid - 1] : 0);
#pragma unroll
  for (int u = 0; u < kScanPer; ++u) {
    if (base + u < n) out[base + u] = run;
    run += v[u];
  }
  if (threadIdx.x == kScanT - 1) bsum[blockIdx.x] = run;
}

// exclusive scan of the block totals, one block, in chunks of kScanT;
// bsum[nb] gets the grand total
__global__ void __launch_bounds__(kScanT) k_scan_sums(int *bsum, int nb) {
  __shared__ int sw[kScanT / 32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c0 = 0; c0 < nb; c0 += kScanT) {
    const int i = c0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) sw[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int s = sw[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      sw[lane] = s;
    }
    __syncthreads();
    const int excl = carry + x - v + (wid > 0 ? sw[wid - 1] : 0);
    __syncthreads();
    if (i < nb) bsum[i] = excl;
    if (threadIdx.x == kScanT - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) bsum[nb] = carry;
}

__global__ void k_scan_add(int n, int *__restrict__ out, const int *__restrict__ bsum, int nb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += bsum[i / kScanChunk];
  if (i == 0) out[n] = bsum[nb];
}

// out[0..n] = exclusive scan of in[0..n), out[n] = the total (also to *total)
static int dev_scan(cudaStream_t s, const int *in, int n, int *out, DBuf &scratch, int *total) {
  const int nb = std::max(1, (n + kScanChunk - 1) / kScanChunk);
  if (scratch.ensure(4 * ((size_t)nb + 1))) return DEV_ERR_DEVICE_ALLOC;
  int *bsum = (int *)scratch.p;
  k_scan_chunks<<<nb, kScanT, 0, s>>>(in, n, out, bsum);
  k_scan_sums<<<1, kScanT, 0, s>>>(bsum, nb);
  k_scan_add<<<(n + 255) / 256 + 1, 256, 0, s>>>(n, out, bsum, nb);
  if (cudaMemcpyAsync(total, out + n, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return DEV_ERR_UNKNOWN;
  return 0;
}

__global__ void k_rowindex(int n, const int *__restrict__ row, int *__restrict__ ridx) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int p = row[i]; p < row[i + 1]; ++p) ridx[p] = i;
}

// CSR -> CSRL (lower) / CSRU: what a row keeps (convert.cu split, bs = 0)
__device__ __forceinline__ int split_keep(int col, int i, bool lower, int d) {
  if (lower ? col < i : col > i) return 1;  // off-diagonal on the kept side
  if (col != i || d == Magma_NODIAG) return 0;
  if (d == Magma_UNITY || d == Magma_VALUE || d == Magma_ZERO || !lower) return d == Magma_UNITY ? 2 : 3;
  return 0;  // a lower split's diagonal by default: counted by LACE, not stored
}

__global__ void k_split_count(int n, const int *__restrict__ row, const int *__restrict__ col, int lower, int d,
                              int *__restrict__ kept) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int k = 0;
    for (int p = row[i]; p < row[i + 1]; ++p) k += split_keep(col[p], i, lower != 0, d) != 0;
    kept[i] = k;
  }
}

__global__ void k_split_fill(int n, const int *__restrict__ row, const int *__restrict__ col,
                             const double *__restrict__ val, int lower, int d, const int *__restrict__ brow,
                             int *__restrict__ bcol, double *__restrict__ bval) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    int o = brow[i];
    for (int p = row[i]; p < row[i + 1]; ++p) {
      const int c = col[p];
      const int k = split_keep(c, i, lower != 0, d);
      if (!k) continue;
      // 1: off-diagonal; 2: UNITY diagonal; 3: VALUE (or the upper default) / ZERO diagonal
      bval[o] = k == 1 ? val[p] : (k == 2 ? 1.0 : (d == Magma_ZERO ? 0.0 : val[p]));
      bcol[o++] = c;
    }
  }
}

// column counts; an index outside [0, ncols) is not counted (the caller
// sees the totals disagree)
__global__ void k_col_count(int nnz, int ncols, const int *__restrict__ col, int *__restrict__ cnt) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < nnz; p += gridDim.x * blockDim.x) {
    const int c = col[p];
    if (c >= 0 && c < ncols) atomicAdd(cnt + c, 1);
  }
}

__global__ void k_transpose_scatter(int n, const int *__restrict__ row, const int *__restrict__ col,
                                    const double *__restrict__ val, int *__restrict__ cursor, int *__restrict__ tidx,
                                    double *__restrict__ tval) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    for (int p = row[i]; p < row[i + 1]; ++p) {
      const int q = atomicAdd(cursor + col[p], 1);
      tidx[q] = i;
      tval[q] = val[p];
    }
}

// each column's entries by ascending row (insertion sort: a column of a
// sparse matrix holds a handful)
__global__ void k_transpose_order(int ncols, const int *__restrict__ tptr, int *__restrict__ tidx,
                                  double *__restrict__ tval) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ncols; c += gridDim.x * blockDim.x) {
    const int b = tptr[c], e = tptr[c + 1];
    for (int q = b + 1; q < e; ++q) {
      const int r = tidx[q];
      const double v = tval[q];
      int t = q - 1;
      while (t >= b && tidx[t] > r) {
        tidx[t + 1] = tidx[t];
        tval[t + 1] = tval[t];
        --t;
      }
      tidx[t + 1] = r;
      tval[t + 1] = v;
    }
  }
}

constexpr int kBcsrMaxCols = 256;  // distinct block columns a block row may hold

// the ascending distinct block columns of block row I into cols; count, or
// -1 when more than kBcsrMaxCols
__device__ int bcsr_block_cols(int I, int bs, int n, const int *__restrict__ row, const int *__restrict__ col,
                               int *cols) {
  int m = 0;
  for (int r = I * bs; r < min(n, (I + 1) * bs); ++r)
    for (int p = row[r]; p < row[r + 1]; ++p) {
      const int J = col[p] / bs;
      int t = m - 1;
      while (t >= 0 && cols[t] > J) --t;
      if (t >= 0 && cols[t] == J) continue;  // already listed
      if (m == kBcsrMaxCols) return -1;
      for (int u = m; u > t + 1; --u) cols[u] = cols[u - 1];
      cols[t + 1] = J;
      ++m;
    }
  return m;
}

__global__ void k_bcsr_count(int nbr, int bs, int n, const int *__restrict__ row, const int *__restrict__ col,
                             int *__restrict__ cnt, int *__restrict__ err) {
  int cols[kBcsrMaxCols];
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nbr; I += gridDim.x * blockDim.x) {
    const int m = bcsr_block_cols(I, bs, n, row, col, cols);
    if (m < 0) atomicOr(err, 1);
    cnt[I] = max(m, 0);
  }
}

__global__ void k_bcsr_fill(int nbr, int bs, int n, const int *__restrict__ row, const int *__restrict__ col,
                            const double *__restrict__ val, const int *__restrict__ brow, int *__restrict__ bcol,
                            double *__restrict__ bval) {
  int cols[kBcsrMaxCols];
  const int ld = bs * bs;
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nbr; I += gridDim.x * blockDim.x) {
    const int m = bcsr_block_cols(I, bs, n, row, col, cols);
    if (m < 0) continue;
    const int o = brow[I];
    for (int q = 0; q < m; ++q) bcol[o + q] = cols[q];
    for (int r = I * bs; r < min(n, (I + 1) * bs); ++r)
      for (int p = row[r]; p < row[r + 1]; ++p) {
        const int c = col[p], J = c / bs;
        int lo = 0, hi = m - 1;  // J's slot
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (cols[mid] < J) lo = mid + 1;
          else hi = mid;
        }
        bval[(size_t)(o + lo) * ld + (size_t)(r - I * bs) * bs + (c - J * bs)] = val[p];
      }
  }
}

static int conv_grid(int items) { return std::max(1, std::min((items + 255) / 256, num_sms() * 16)); }

// row pointers start at 0 and do not decrease (else *err = 1)
__global__ void k_check_rows(int n, const int *__restrict__ row, int *__restrict__ err) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    if (row[i + 1] < row[i] || (i == 0 && row[0] != 0)) atomicOr(err, 1);
}

static int check_rows(cudaStream_t s, int n, const int *row) {
  if (n == 0) return 0;
  DBuf err;
  int h = 0;
  if (err.ensure(4)) return DEV_ERR_DEVICE_ALLOC;
  cudaMemsetAsync(err.p, 0, 4, s);
  k_check_rows<<<conv_grid(n), 256, 0, s>>>(n, row, (int *)err.p);
  if (cudaMemcpyAsync(&h, err.p, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
    return DEV_ERR_UNKNOWN;
  return h ? DEV_ERR_ILLEGAL_VALUE : 0;
}

}  // namespace lace

using namespace lace;

extern "C" int lace_gpu_rowindex_device(lace_gpu_ctx *c, int n, const int *row, int *rowidx) {
  if (!c || !row || !rowidx) return set_err(DEV_ERR_INVALID_PTR);
  if (n < 0) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(c->device);
  if (int rc = check_rows(c->stream, n, row)) return set_err(rc);
  if (n > 0) k_rowindex<<<conv_grid(n), 256, 0, c->stream>>>(n, row, rowidx);
  return cudaGetLastError() == cudaSuccess ? DEV_SUCCESS : set_err(DEV_ERR_UNKNOWN);
}

extern "C" int lace_gpu_csr_split_device(lace_gpu_ctx *c, int n, const int *row, const int *col, const double *val,
                                         int lower, int diagorder, int *nnz_out, int *brow, int *bcol, double *bval) {
  if (!c || !row || !col || !nnz_out) return set_err(DEV_ERR_INVALID_PTR);
  if (n < 0) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  if (int rc = check_rows(s, n, row)) return set_err(rc);
  DBuf kept, own, scr;
  int *rp = brow;
  if (!rp) {  // the size query without the caller's pointer array
    if (own.ensure(4 * ((size_t)n + 1))) return set_err(DEV_ERR_DEVICE_ALLOC);
    rp = (int *)own.p;
  }
  if (kept.ensure(4 * ((size_t)n + 1))) return set_err(DEV_ERR_DEVICE_ALLOC);
  k_split_count<<<conv_grid(n), 256, 0, s>>>(n, row, col, lower, diagorder, (int *)kept.p);
  int total = 0;
  int rc = dev_scan(s, (const int *)kept.p, n, rp, scr, &total);
  if (rc) return set_err(rc);
  *nnz_out = total;
  if (bcol && bval) {
    if (!val) return set_err(DEV_ERR_INVALID_PTR);
    k_split_fill<<<conv_grid(n), 256, 0, s>>>(n, row, col, val, lower, diagorder, rp, bcol, bval);
  }
  return (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess) ? DEV_SUCCESS
                                                                                          : set_err(DEV_ERR_UNKNOWN);
}

extern "C" int lace_gpu_csr_transpose_device(lace_gpu_ctx *c, int n, int ncols, const int *row, const int *col,
                                             const double *val, int *tptr, int *tidx, double *tval) {
  if (!c || !row || !col || !val || !tptr || !tidx || !tval) return set_err(DEV_ERR_INVALID_PTR);
  if (n < 0 || ncols < 0) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  if (int rc = check_rows(s, n, row)) return set_err(rc);
  int nnz = 0;
  if (cudaMemcpyAsync(&nnz, row + n, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return set_err(DEV_ERR_UNKNOWN);
  DBuf cnt, scr, cursor;
  if (cnt.ensure(4 * ((size_t)ncols + 1)) || cursor.ensure(4 * ((size_t)ncols + 1))) return set_err(DEV_ERR_DEVICE_ALLOC);
  cudaMemsetAsync(cnt.p, 0, 4 * ((size_t)ncols + 1), s);
  if (nnz > 0) k_col_count<<<conv_grid(nnz), 256, 0, s>>>(nnz, ncols, col, (int *)cnt.p);
  int total = 0;
  int rc = dev_scan(s, (const int *)cnt.p, ncols, tptr, scr, &total);
  if (rc) return set_err(rc);
  if (total != nnz) return set_err(DEV_ERR_ILLEGAL_VALUE);  // a column index outside [0, ncols)
  cudaMemcpyAsync(cursor.p, tptr, 4 * (size_t)ncols, cudaMemcpyDeviceToDevice, s);
  k_transpose_scatter<<<conv_grid(n), 256, 0, s>>>(n, row, col, val, (int *)cursor.p, tidx, tval);
  k_transpose_order<<<conv_grid(ncols), 256, 0, s>>>(ncols, tptr, tidx, tval);
  return (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess) ? DEV_SUCCESS
                                                                                          : set_err(DEV_ERR_UNKNOWN);
}

extern "C" int lace_gpu_csr_to_bcsr_device(lace_gpu_ctx *c, int n, const int *row, const int *col, const double *val,
                                           int bs, int *nblocks_out, int *brow, int *bcol, double *bval) {
  if (!c || !row || !col || !nblocks_out) return set_err(DEV_ERR_INVALID_PTR);
  if (n < 0 || bs < 1) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  if (int rc = check_rows(s, n, row)) return set_err(rc);
  const int nbr = (n + bs - 1) / bs;
  DBuf cnt, own, scr, err;
  int *rp = brow;
  if (!rp) {
    if (own.ensure(4 * ((size_t)nbr + 1))) return set_err(DEV_ERR_DEVICE_ALLOC);
    rp = (int *)own.p;
  }
  if (cnt.ensure(4 * ((size_t)nbr + 1)) || err.ensure(4)) return set_err(DEV_ERR_DEVICE_ALLOC);
  cudaMemsetAsync(err.p, 0, 4, s);
  k_bcsr_count<<<conv_grid(nbr), 256, 0, s>>>(nbr, bs, n, row, col, (int *)cnt.p, (int *)err.p);
  int total = 0, herr = 0;
  int rc = dev_scan(s, (const int *)cnt.p, nbr, rp, scr, &total);
  if (rc) return set_err(rc);
  if (cudaMemcpy(&herr, err.p, 4, cudaMemcpyDeviceToHost) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
  if (herr) return set_err(DEV_ERR_NOT_SUPPORTED);  // a block row with more than kBcsrMaxCols block columns
  *nblocks_out = total;
  if (bcol && bval) {
    if (!val) return set_err(DEV_ERR_INVALID_PTR);
    cudaMemsetAsync(bval, 0, 8 * (size_t)total * bs * bs, s);
    k_bcsr_fill<<<conv_grid(nbr), 256, 0, s>>>(nbr, bs, n, row, col, val, rp, bcol, bval);
  }
  return (cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(s) == cudaSuccess) ? DEV_SUCCESS
                                                                                          : set_err(DEV_ERR_UNKNOWN);
}
