// Sparse triangular solves x = T^{-1} b on the GPU.
//
// Exact solves replace LACE's mkl_dcsrtrsv calls
// (src/fgmres_householder_restart.cpp:320-332).  The Jacobi sweeps are a
// GPU-native inexact mode (LACE_TRSV_JACOBI), not LACE's data_parcsrtrsv,
// whose in-place order partrsv.cu reproduces.
//
// Here: the level-scheduled solve, the Jacobi sweeps and the BCSR solve (the
// default CSR solve, block-scheduled and sync-free, is in sptrsv_blk.cu).  The
// BCSR solve takes chunks of block rows in solve order from an atomic ticket,
// so a warp only ever waits for rows already held by running warps, and
// waits for their values themselves (bounded spin).
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
// One warp per chunk of consecutive block rows in solve order (rows upwards
// for L, downwards for U), chunks taken by atomic ticket in solve order, so a
// warp only ever waits for rows that earlier tickets hold.  A chunk holds at
// most 64 block rows and never crosses a place where a block row does not
// depend on the one solved before it (host-built chunk table), so chunks
// follow the grid lines: a chunk that straddled the end of one line and the
// start of the next would make every line wait for the whole previous one.
// A solved value is its own ready flag: the output starts as an all-ones bit
// pattern (a NaN arithmetic does not produce; a result with those bits is
// stored as a quiet NaN), so no flags, fences or epochs.  Lanes sub*BS + r
// work on scalar row r of a block: sub-group `sub` takes the row's
// off-diagonal blocks sub, sub + 32/BS, ...; lane r of a sub-group waits for
// entry r of the block's x segment and the sub-group shares the segment by
// shuffles; the previous block row of the chunk (the chain along a grid
// line) comes from registers.  While a row waits and computes, the warp
// loads the next row's structure, block values and far dependencies.  The
// diagonal block is the identity (lower) or applied through its precomputed
// inverse (upper).
template <typename XT> struct Unsolved;
template <> struct Unsolved<float> {
  __device__ static bool is(float v) { return __float_as_uint(v) == 0xffffffffu; }
  __device__ static float fix(float v) { return is(v) ? __uint_as_float(0x7fc00000u) : v; }
  __device__ static float load(const float *p) {
    float v;
    asm volatile("ld.relaxed.gpu.global.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
  }
  __device__ static void store(float *p, float v) {
    asm volatile("st.relaxed.gpu.global.f32 [%0], %1;" ::"l"(p), "f"(v) : "memory");
  }
};
template <> struct Unsolved<double> {
  __device__ static bool is(double v) { return (unsigned long long)__double_as_longlong(v) == ~0ull; }
  __device__ static double fix(double v) { return is(v) ? __longlong_as_double(0x7ff8000000000000ll) : v; }
  __device__ static double load(const double *p) {
    double v;
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
  }
  __device__ static void store(double *p, double v) {
    asm volatile("st.relaxed.gpu.global.f64 [%0], %1;" ::"l"(p), "d"(v) : "memory");
  }
};

// What a lane needs for one block row: its off-diagonal block (the k-th of
// the row for k = k0 + sub), that block's row r, entry r of the block's x
// segment if it is already there, the right-hand side and (upper) row r of
// the diagonal block's inverse.
template <typename CT, typename XT, int BS>
struct BcsrRow {
  int I, J, p;
  bool more;  // more off-diagonal blocks than this round
  CT a[BS];
  XT xv;
  bool have;  // xv holds a solved value (or is not needed)
  CT bv;
  CT d[BS];
};

template <typename CT, typename VT, typename XT, int BS, bool LOWER>
__device__ __forceinline__ void bcsr_fetch(BcsrRow<CT, XT, BS> &w, int I, int prevI, int k0,
                                           const int *__restrict__ row, const int *__restrict__ col,
                                           const VT *__restrict__ val, const VT *__restrict__ dinv,
                                           const void *b, int in_f32, const XT *x, int sub, int r,
                                           bool active) {
  constexpr int PER = 32 / BS;
  constexpr int LD = BS * BS;
  w.I = I;
  const int rb = __ldg(row + I), re = __ldg(row + I + 1);
  w.J = -1;
  w.p = -1;
  w.more = false;
  int k = 0;
  for (int e = rb; e < re; ++e) {
    const int c = __ldg(col + e);
    if (LOWER ? c >= I : c <= I) continue;
    if (k == k0 + sub) {
      w.J = c;
      w.p = e;
    }
    if (k >= k0 + PER) w.more = true;
    ++k;
  }
  const bool mine = active && w.J >= 0;
#pragma unroll
  for (int cc = 0; cc < BS; ++cc) w.a[cc] = mine ? cvt<CT>(__ldg(val + (size_t)w.p * LD + r * BS + cc)) : (CT)0;
  w.have = !mine || w.J == prevI;  // the previous row comes from registers
  w.xv = (XT)0;
  if (mine && w.J != prevI) {
    w.xv = Unsolved<XT>::load(x + (size_t)w.J * BS + r);
    w.have = !Unsolved<XT>::is(w.xv);
  }
  w.bv = sub == 0 ? ldin<CT>(b, in_f32, I * BS + r) : (CT)0;
  if (!LOWER) {
#pragma unroll
    for (int cc = 0; cc < BS; ++cc) w.d[cc] = cvt<CT>(__ldg(dinv + (size_t)I * LD + r * BS + cc));
  }
}

template <typename CT, typename VT, typename XT, int BS, bool LOWER>
__global__ void __launch_bounds__(kSTPB) k_bcsr_sptrsv(int nb, const int *__restrict__ row,
                                                       const int *__restrict__ col,
                                                       const VT *__restrict__ val,
                                                       const VT *__restrict__ dinv,
                                                       const int *__restrict__ chunk_first, int nch,
                                                       const void *b, int in_f32, XT *x, int *tickets,
                                                       const int *done_flag, int *status) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  constexpr int PER = 32 / BS;  // sub-groups
  const int lane = threadIdx.x & 31;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int sub = lane / BS, r = lane % BS;
  const bool active = sub < PER;
  const int src0 = lane - r;  // lane 0 of this lane's sub-group
  bool gave_up = false;
  // bounded warp-uniform wait until every lane's x entry is solved
  auto wait_x = [&](XT &xv, bool &have, int J) {
    int spins = 0;
    while (!__all_sync(0xffffffffu, have)) {
      if (!have) {
        xv = Unsolved<XT>::load(x + (size_t)J * BS + r);
        have = !Unsolved<XT>::is(xv);
      }
      ++spins;
      if ((spins & 1023) == 1023 && (ld_relaxed(status) & kStatusSpinTimeout)) gave_up = true;
      if (spins > kMaxSpins) {
        if (lane == 0) atomicOr(status, kStatusSpinTimeout);
        gave_up = true;
      }
      if (gave_up) have = true;  // the solve is reported as failed
      if (spins > 16) __nanosleep(32);
    }
  };
  BcsrRow<CT, XT, BS> cur, nxt;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&tickets[0], 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= nch) break;
    const int first = __ldg(chunk_first + t), cnt = __ldg(chunk_first + t + 1) - first;
    CT prev = (CT)0;  // lanes 0..BS-1: the previous block row of the chunk
    int prevI = -1;
    bcsr_fetch<CT, VT, XT, BS, LOWER>(nxt, LOWER ? first : nb - 1 - first, -1, 0, row, col, val, dinv, b, in_f32,
                                      x, sub, r, active);
    for (int q = 0; q < cnt; ++q) {
      cur = nxt;
      if (q + 1 < cnt)
        bcsr_fetch<CT, VT, XT, BS, LOWER>(nxt, LOWER ? first + q + 1 : nb - 2 - (first + q), cur.I, 0, row, col,
                                          val, dinv, b, in_f32, x, sub, r, active);
      const CT fromprev = __shfl_sync(0xffffffffu, prev, r);
      if (cur.J >= 0 && cur.J == prevI && active) cur.xv = (XT)fromprev;
      wait_x(cur.xv, cur.have, cur.J);
      CT acc = (CT)0;
      {
        CT s = (CT)0;
#pragma unroll
        for (int cc = 0; cc < BS; ++cc) s = fma(cur.a[cc], (CT)__shfl_sync(0xffffffffu, cur.xv, src0 + cc), s);
        if (active && cur.J >= 0) acc -= s;
      }
      // further rounds of off-diagonal blocks (none on a 7-point stencil)
      for (int k0 = PER; __any_sync(0xffffffffu, cur.more); k0 += PER) {
        BcsrRow<CT, XT, BS> extra;
        bcsr_fetch<CT, VT, XT, BS, LOWER>(extra, cur.I, prevI, k0, row, col, val, dinv, b, in_f32, x, sub, r,
                                          active);
        if (extra.J >= 0 && extra.J == prevI && active) extra.xv = (XT)fromprev;
        wait_x(extra.xv, extra.have, extra.J);
        CT s = (CT)0;
#pragma unroll
        for (int cc = 0; cc < BS; ++cc) s = fma(extra.a[cc], (CT)__shfl_sync(0xffffffffu, extra.xv, src0 + cc), s);
        if (active && extra.J >= 0) acc -= s;
        cur.more = extra.more;
      }
      // the sub-groups' partial sums onto sub-group 0
#pragma unroll
      for (int g = 1; g < PER; ++g) {
        const CT v = __shfl_sync(0xffffffffu, acc, (g * BS + r) & 31);
        if (sub == 0) acc += v;
      }
      acc += cur.bv;
      CT xr = acc;
      if (!LOWER) {
        CT t2 = (CT)0;
#pragma unroll
        for (int cc = 0; cc < BS; ++cc) t2 = fma(cur.d[cc], __shfl_sync(0xffffffffu, acc, cc), t2);
        xr = t2;
      }
      if (lane < BS) {
        const XT out = Unsolved<XT>::fix((XT)xr);
        Unsolved<XT>::store(x + (size_t)cur.I * BS + r, out);
        prev = (CT)out;
      }
      prevI = cur.I;
    }
  }
  if (lane == 0) {
    const int e = atomicAdd(&tickets[1], 1);
    if (e == nwarps - 1) {
      tickets[0] = 0;
      tickets[1] = 0;
      __threadfence();
    }
  }
}

template <typename CT, typename VT, typename XT, int BS>
static void bcsr_launch(cudaStream_t s, int grid, const TriDev &t, const void *dinv, const void *b, int in_f32,
                        void *x, int *tickets, const int *dfl, int *status) {
  const int nb = t.n / BS;
  if (t.lower)
    k_bcsr_sptrsv<CT, VT, XT, BS, true><<<grid, kSTPB, 0, s>>>(nb, t.row, t.col, (const VT *)t.val,
                                                              (const VT *)dinv, t.bchunk_first, t.bnch, b,
                                                              in_f32, (XT *)x, tickets, dfl, status);
  else
    k_bcsr_sptrsv<CT, VT, XT, BS, false><<<grid, kSTPB, 0, s>>>(nb, t.row, t.col, (const VT *)t.val,
                                                               (const VT *)dinv, t.bchunk_first, t.bnch, b,
                                                               in_f32, (XT *)x, tickets, dfl, status);
}

template <typename CT, typename VT, typename XT>
static void bcsr_launch_bs(cudaStream_t s, int grid, int bs, const TriDev &t, const void *dinv, const void *b,
                           int in_f32, void *x, int *tickets, const int *dfl, int *status) {
  switch (bs) {
    case 1: bcsr_launch<CT, VT, XT, 1>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    case 2: bcsr_launch<CT, VT, XT, 2>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    case 3: bcsr_launch<CT, VT, XT, 3>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    case 4: bcsr_launch<CT, VT, XT, 4>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    case 5: bcsr_launch<CT, VT, XT, 5>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    case 6: bcsr_launch<CT, VT, XT, 6>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    case 7: bcsr_launch<CT, VT, XT, 7>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    default: bcsr_launch<CT, VT, XT, 8>(s, grid, t, dinv, b, in_f32, x, tickets, dfl, status); break;
  }
}

void launch_bcsr_sptrsv(cudaStream_t s, const TriDev &t, int bs, VType vt, const void *dinv,
                        const void *b, int in_f32, void *x, int out_f32, Control *ctrl,
                        int grid_hint, bool honor_done) {
  const int nch = t.bnch;
  const int *dfl = honor_done ? &ctrl->done : nullptr;
  int grid = grid_hint > 0 ? grid_hint : num_sms() * 8;
  int maxgrid = (nch * 32 + kSTPB - 1) / kSTPB;
  if (grid > maxgrid) grid = maxgrid;
  if (grid < 1) grid = 1;
  int *tickets = ctrl->tickets[t.slot];
  int *status = &ctrl->status;
  // the output starts unsolved (x must not overlap b)
  cudaMemsetAsync(x, 0xFF, (size_t)t.n * (out_f32 ? 4 : 8), s);
  if (out_f32) {
    switch (vt) {
      case VType::F64: bcsr_launch_bs<double, double, float>(s, grid, bs, t, dinv, b, in_f32, x, tickets, dfl, status); break;
      case VType::F32: bcsr_launch_bs<float, float, float>(s, grid, bs, t, dinv, b, in_f32, x, tickets, dfl, status); break;
      case VType::BF16: bcsr_launch_bs<float, __nv_bfloat16, float>(s, grid, bs, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    }
  } else {
    switch (vt) {
      case VType::F64: bcsr_launch_bs<double, double, double>(s, grid, bs, t, dinv, b, in_f32, x, tickets, dfl, status); break;
      case VType::F32: bcsr_launch_bs<float, float, double>(s, grid, bs, t, dinv, b, in_f32, x, tickets, dfl, status); break;
      case VType::BF16: bcsr_launch_bs<float, __nv_bfloat16, double>(s, grid, bs, t, dinv, b, in_f32, x, tickets, dfl, status); break;
    }
  }
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
