// Sparse triangular solves x = T^{-1} b on the GPU.
//
// Exact solves replace LACE's mkl_dcsrtrsv calls
// (src/fgmres_householder_restart.cpp:320-332); the Jacobi sweep replaces
// data_parcsrtrsv (src/trisolve.cpp:256-351) in synchronous form.
//
// Here: the level-scheduled solve, the Jacobi sweeps and the BCSR solve (the
// default CSR solve, block-scheduled and sync-free, is in sptrsv_blk.cu).  The
// BCSR solve takes block rows in dependency order from an atomic ticket, so a
// warp only ever waits for block rows already held by running warps, and
// waits for them through per-block-row ready flags (acquire/release, bounded
// spin) that carry an epoch advancing every launch, so they are never reset.
#include "internal.h"

namespace lace {

constexpr int kSTPB = 256;

template <typename CT, typename VT>
struct EntryLoad {
  __device__ __forceinline__ static CT get(const VT *v, int p) { return cvt<CT>(v[p]); }
};

template <typename T> __device__ __forceinline__ T ldcg(const T *p) { return __ldcg(p); }

template <typename T>
__device__ __forceinline__ T ldin(const void *b, int in_f32, int i) {
  return in_f32 ? (T)((const float *)b)[i] : (T)((const double *)b)[i];
}

template <typename T>
__device__ __forceinline__ void stout(void *x, int out_f32, int i, T v) {
  if (out_f32) ((float *)x)[i] = (float)v;
  else ((double *)x)[i] = (double)v;
}

template <typename T>
__device__ __forceinline__ T ldx(const void *x, int out_f32, int i) {
  return out_f32 ? (T)__ldcg(((const float *)x) + i) : (T)__ldcg(((const double *)x) + i);
}

// bounded wait for chunk flag == epoch
__device__ __forceinline__ void wait_flag(const int *flag, int epoch, int *status) {
  if (ld_acquire(flag) == epoch) return;
  int spins = 0;
  while (ld_acquire(flag) != epoch) {
    if (++spins > kMaxSpins) {
      atomicOr(status, kStatusSpinTimeout);
      return;
    }
    if (spins > 64) __nanosleep(64);
  }
}

// ------------------------------------------------------ level scheduled
// Rows grouped by level (host analysis); one cooperative launch walks the
// levels with a grid-wide barrier (bounded spin) between them.  Thread per
// row within a level.
template <typename CT, typename VT>
__global__ void __launch_bounds__(kSTPB) k_sptrsv_levels(int nlevels, const int *__restrict__ lvl_ptr,
                                                         const int *__restrict__ lvl_rows,
                                                         const int *__restrict__ row,
                                                         const int *__restrict__ col,
                                                         const VT *__restrict__ val, int lower,
                                                         int unit, const void *b, int in_f32, void *x,
                                                         int out_f32, int *bar, const int *done_flag,
                                                         int *status) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nth = gridDim.x * blockDim.x;
  const unsigned nb = gridDim.x;
  for (int L = 0; L < nlevels; ++L) {
    for (int k = lvl_ptr[L] + tid; k < lvl_ptr[L + 1]; k += nth) {
      const int i = lvl_rows[k];
      CT acc = ldin<CT>(b, in_f32, i), d = (CT)1;
      for (int e = row[i]; e < row[i + 1]; ++e) {
        const int jc = col[e];
        if (jc == i) {
          if (!unit) d = cvt<CT>(val[e]);
        } else if (lower ? jc < i : jc > i) {
          acc -= cvt<CT>(val[e]) * ldx<CT>(x, out_f32, jc);
        }
      }
      stout<CT>(x, out_f32, i, acc / d);
    }
    // grid barrier: monotonically increasing arrival counter
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
      const unsigned target = (unsigned)(L + 1) * nb;
      atomicAdd((unsigned *)bar, 1u);
      int spins = 0;
      while (ld_acquire(bar) < (int)target) {
        if (++spins > kMaxSpins) {
          atomicOr(status, kStatusSpinTimeout);
          break;
        }
      }
    }
    __syncthreads();
  }
  // reset the barrier counter: the last block to finish does it
  if (threadIdx.x == 0) {
    const unsigned done = atomicAdd((unsigned *)(bar + 1), 1u);
    if (done == nb - 1) {
      bar[0] = 0;
      bar[1] = 0;
      __threadfence();
    }
  }
}

void launch_sptrsv_levels(cudaStream_t s, const TriDev &t, VType vt, const void *b, int in_f32,
                          void *x, int out_f32, Control *ctrl, bool honor_done) {
  // co-residency: one block per SM is always resident for this kernel's
  // resources; cooperative launch enforces it
  int grid = num_sms();
  int *bar = ctrl->tickets[t.slot];
  void *args[15];
  const int *df = honor_done ? &ctrl->done : nullptr;
  int *st = &ctrl->status;
  int nl = t.nlevels;
  const int *lp = t.lvl_ptr, *lr = t.lvl_rows, *rw = t.row, *cl = t.col;
  const void *vv = t.val;
  int lower = t.lower, unit = t.unit;
  const void *bb = b;
  void *xx = x;
  args[0] = &nl; args[1] = &lp; args[2] = &lr; args[3] = &rw; args[4] = &cl; args[5] = &vv;
  args[6] = &lower; args[7] = &unit; args[8] = &bb; args[9] = &in_f32; args[10] = &xx;
  args[11] = &out_f32; args[12] = &bar; args[13] = &df; args[14] = &st;
  const void *fn = nullptr;
  switch (vt) {
    case VType::F64: fn = (const void *)k_sptrsv_levels<double, double>; break;
    case VType::F32: fn = (const void *)k_sptrsv_levels<float, float>; break;
    case VType::BF16: fn = (const void *)k_sptrsv_levels<float, __nv_bfloat16>; break;
  }
  cudaLaunchCooperativeKernel(fn, dim3(grid), dim3(kSTPB), args, 0, s);
}

// ------------------------------------------------------------- Jacobi
template <typename CT, typename VT>
__global__ void __launch_bounds__(kSTPB) k_jacobi(int n, const int *__restrict__ row,
                                                  const int *__restrict__ col,
                                                  const VT *__restrict__ val, int lower, int unit,
                                                  const void *b, int in_f32, const void *yold,
                                                  void *ynew, int y_f32, const int *done_flag) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    CT acc = ldin<CT>(b, in_f32, i), d = (CT)1;
    for (int e = row[i]; e < row[i + 1]; ++e) {
      const int jc = col[e];
      if (jc == i) {
        if (!unit) d = cvt<CT>(val[e]);
      } else if (lower ? jc < i : jc > i) {
        acc -= cvt<CT>(val[e]) * (yold ? ldx<CT>(yold, y_f32, jc) : (CT)0);
      }
    }
    stout<CT>(ynew, y_f32, i, acc / d);
  }
}

void launch_jacobi_sweep(cudaStream_t s, const TriDev &t, VType vt, const void *b, int in_f32,
                         const void *yold, void *ynew, int y_f32, Control *ctrl, bool honor_done) {
  const int *dfl = (honor_done && ctrl) ? &ctrl->done : nullptr;
  int grid = min((t.n + kSTPB - 1) / kSTPB, num_sms() * 8);
  if (grid < 1) return;
  switch (vt) {
    case VType::F64: k_jacobi<double, double><<<grid, kSTPB, 0, s>>>(t.n, t.row, t.col, (const double *)t.val, t.lower, t.unit, b, in_f32, yold, ynew, y_f32, dfl); break;
    case VType::F32: k_jacobi<float, float><<<grid, kSTPB, 0, s>>>(t.n, t.row, t.col, (const float *)t.val, t.lower, t.unit, b, in_f32, yold, ynew, y_f32, dfl); break;
    case VType::BF16: k_jacobi<float, __nv_bfloat16><<<grid, kSTPB, 0, s>>>(t.n, t.row, t.col, (const __nv_bfloat16 *)t.val, t.lower, t.unit, b, in_f32, yold, ynew, y_f32, dfl); break;
  }
}

// ------------------------------------------------------------- BCSR
// Block rows in chunks of 32 block rows per warp is not needed for the
// block-stencil systems: one thread per scalar row of a block row, the bs
// threads of a block row sit in one warp segment.  Block rows are taken by
// ticket in dependency order; the block row's diagonal block is applied
// through its precomputed inverse (upper) or is the identity (lower).
template <typename CT, typename VT, bool LOWER>
__global__ void __launch_bounds__(kSTPB) k_bcsr_sptrsv(int nb, int bs, const int *__restrict__ row,
                                                       const int *__restrict__ col,
                                                       const VT *__restrict__ val,
                                                       const VT *__restrict__ dinv, const void *b,
                                                       int in_f32, void *x, int out_f32, int *ready,
                                                       int *tickets, int *epoch_slot, const int *done_flag,
                                                       int *status) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int epoch = *(volatile int *)epoch_slot + 1;
  const int per = 32 / bs;          // block rows per warp pass
  const int ld = bs * bs;
  const int sub = lane / bs, r = lane % bs;
  const int nch = (nb + per - 1) / per;  // chunks of `per` block rows
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&tickets[0], 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= nch) break;
    const int c = LOWER ? t : nch - 1 - t;
    // block rows of the chunk are processed one after the other (in solve
    // order) by the whole warp; lanes sub*bs + r hold scalar row r
    const int first = c * per;
    const int cnt = min(per, nb - first);
    for (int q = 0; q < cnt; ++q) {
      const int I = LOWER ? first + q : first + cnt - 1 - q;
      CT acc = (CT)0;
      if (sub == 0) acc = ldin<CT>(b, in_f32, I * bs + r);
      // lanes with sub > 0 help: each sub-group takes every per-th block
      if (lane < per * bs) {
        int k = 0;
        for (int p = row[I]; p < row[I + 1]; ++p) {
          const int J = col[p];
          if (LOWER ? J >= I : J <= I) continue;
          if ((k++ % per) != sub) continue;
          const int cj = J / per;
          if (cj != c) wait_flag(&ready[cj], epoch, status);
          const VT *blk = val + (size_t)p * ld + r * bs;
          CT s = (CT)0;
          for (int cc = 0; cc < bs; ++cc) s += cvt<CT>(blk[cc]) * ldx<CT>(x, out_f32, J * bs + cc);
          acc -= s;
        }
      }
      // sum the sub-groups' partials onto sub 0
      for (int g = 1; g < per; ++g) {
        CT v = __shfl_sync(0xffffffffu, acc, (g * bs + r) & 31);
        if (sub == 0 && g * bs + r < 32) acc += v;
      }
      // apply the diagonal: identity (lower) or dinv (upper); row r of dinv
      CT xr = acc;
      if (!LOWER) {
        CT t2 = (CT)0;
        for (int cc = 0; cc < bs; ++cc) {
          CT ac = __shfl_sync(0xffffffffu, acc, cc);
          t2 += cvt<CT>(dinv[(size_t)I * ld + r * bs + cc]) * ac;
        }
        xr = t2;
      }
      if (sub == 0) stout<CT>(x, out_f32, I * bs + r, xr);
      __threadfence();
      __syncwarp();
    }
    if (lane == 0) st_release(&ready[c], epoch);
  }
  if (lane == 0) {
    const int e = atomicAdd(&tickets[1], 1);
    if (e == nwarps - 1) {
      tickets[0] = 0;
      tickets[1] = 0;
      *epoch_slot = epoch;
      __threadfence();
    }
  }
}

void launch_bcsr_sptrsv(cudaStream_t s, const TriDev &t, int bs, VType vt, const void *dinv,
                        const void *b, int in_f32, void *x, int out_f32, Control *ctrl,
                        int grid_hint, bool honor_done) {
  const int nb = t.n / bs;
  const int *dfl = honor_done ? &ctrl->done : nullptr;
  const int per = 32 / bs;
  const int nch = (nb + per - 1) / per;
  int grid = grid_hint > 0 ? grid_hint : num_sms() * 8;
  int maxgrid = (nch * 32 + kSTPB - 1) / kSTPB;
  if (grid > maxgrid) grid = maxgrid;
  if (grid < 1) grid = 1;
  int *tickets = ctrl->tickets[t.slot];
  int *epoch_slot = &ctrl->trsv_epoch[t.slot];
  int *status = &ctrl->status;
#define LACE_BCSR_LAUNCH(CT, VT)                                                                   \
  if (t.lower)                                                                                     \
    k_bcsr_sptrsv<CT, VT, true><<<grid, kSTPB, 0, s>>>(nb, bs, t.row, t.col, (const VT *)t.val,  \
                                                       (const VT *)dinv, b, in_f32, x, out_f32,    \
                                                       t.ready, tickets, epoch_slot, dfl, status);  \
  else                                                                                             \
    k_bcsr_sptrsv<CT, VT, false><<<grid, kSTPB, 0, s>>>(nb, bs, t.row, t.col, (const VT *)t.val, \
                                                        (const VT *)dinv, b, in_f32, x, out_f32,   \
                                                        t.ready, tickets, epoch_slot, dfl, status);
  switch (vt) {
    case VType::F64: LACE_BCSR_LAUNCH(double, double); break;
    case VType::F32: LACE_BCSR_LAUNCH(float, float); break;
    case VType::BF16: LACE_BCSR_LAUNCH(float, __nv_bfloat16); break;
  }
#undef LACE_BCSR_LAUNCH
}

}  // namespace lace

namespace lace {
// sum (a_i - b_i)^2 over two typed vectors into *out (device), last block folds
__global__ void k_sqdiff(int n, const void *a, const void *b, int f32, double *partials, int *counter,
                         double *out) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double d = ldx<double>(a, f32, i) - ldx<double>(b, f32, i);
    acc = fma(d, d, acc);
  }
  __shared__ double scratch[kSTPB / 32];
  acc = warp_sum(acc);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kSTPB / 32; ++w) t += scratch[w];
    partials[blockIdx.x] = t;
  }
  if (!arrive_last(counter)) return;
  const double s = block_fold(partials, 1, (int)gridDim.x);
  if (threadIdx.x == 0) *out = s;
}

// sum of squares of count FP64 values (||A||_F^2 of the resident values):
// 16-byte loads, one FMA per value, two accumulators; the last block folds
// the blocks' partial sums in a fixed order
__global__ void __launch_bounds__(kSTPB) k_sumsq(size_t count, const double *__restrict__ a, double *partials,
                                                 int *counter, double *out) {
  double acc0 = 0.0, acc1 = 0.0;
  const size_t npair = count / 2;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += stride) {
    const double2 v = __ldcs(reinterpret_cast<const double2 *>(a) + p);
    acc0 = fma(v.x, v.x, acc0);
    acc1 = fma(v.y, v.y, acc1);
  }
  if ((count & 1) && blockIdx.x == 0 && threadIdx.x == 0) acc0 = fma(a[count - 1], a[count - 1], acc0);
  __shared__ double scratch[kSTPB / 32];
  const double acc = warp_sum(acc0 + acc1);
  if ((threadIdx.x & 31) == 0) scratch[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kSTPB / 32; ++w) t += scratch[w];
    partials[blockIdx.x] = t;
  }
  if (!arrive_last(counter)) return;
  const double s = block_fold(partials, 1, (int)gridDim.x);
  if (threadIdx.x == 0) *out = s;
}

void launch_sumsq(cudaStream_t s, size_t count, const double *a, double *partials, int *counter, double *out) {
  const int grid = (int)std::max<size_t>(1, std::min<size_t>((size_t)num_sms() * 4, (count / 2 + kSTPB - 1) / kSTPB));
  k_sumsq<<<grid, kSTPB, 0, s>>>(count, a, partials, counter, out);
}

void launch_sqdiff(cudaStream_t s, int n, const void *a, const void *b, int f32, double *partials,
                   int *counter, double *out) {
  int grid = min((n + kSTPB - 1) / kSTPB, num_sms() * 4);
  if (grid < 1) grid = 1;
  k_sqdiff<<<grid, kSTPB, 0, s>>>(n, a, b, f32, partials, counter, out);
}
}  // namespace lace
