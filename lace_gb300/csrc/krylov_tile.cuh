// Row-tile machinery shared by the two Arnoldi variants (Householder in
// krylov.cu, modified Gram-Schmidt in krylov_mgs.cu): the operator applied
// to a tile of rows, deterministic block and grid reductions, FP32<->FP64
// conversions on the integer pipes, and the unsolved-pattern prefill of the
// sync-free solves' outputs.
#pragma once

#include <algorithm>

#include "internal.h"

namespace lace {

constexpr int kTPB = 256;   // threads per block of the row-tile kernels

// operator row i of the tile: CSR (LPR lanes per row) or BCSR (thread/row)
struct OpView {
  int bs;
  const int *row, *col;
  const double *val;
  const int *sell_ptr, *sell_col;  // sliced ELL (CSR row pointers give the row lengths)
  const double *sell_val;
};

template <int LPR, typename ZT>
__device__ __forceinline__ void tile_apply(const OpView &op, int n, int base, int tr,
                                           const ZT *__restrict__ z, double *sw) {
  if (op.bs == 0 && op.sell_ptr != nullptr) {
    // sliced ELL: warp w takes the 32-row slices w, w+8, ... of the tile; entry
    // t of the slice's rows is one coalesced load, four entries in flight
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t0 = wid * 32; t0 < tr; t0 += kTPB) {
      const int i = base + t0 + lane;
      double s = 0.0;
      if (i < n) {
        const int len = op.row[i + 1] - op.row[i];
        const int *cp = op.sell_col + op.sell_ptr[(base + t0) >> 5] + lane;
        const double *vp = op.sell_val + (cp - op.sell_col);
        for (int t = 0; t < len; t += 4) {
          int c[4];
          double v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (t + u < len) {
              c[u] = cp[32 * (t + u)];
              v[u] = vp[32 * (t + u)];
            }
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (t + u < len) s = fma(v[u], to_f64(z[c[u]]), s);
        }
      }
      sw[t0 + lane] = s;
    }
  } else if (op.bs == 0) {
    const int sub = threadIdx.x & (LPR - 1);
    const int grp = threadIdx.x / LPR;
    constexpr int G = kTPB / LPR;
    for (int t = grp; t < tr; t += G) {
      const int i = base + t;
      double s = 0.0;
      if (i < n) {
        const int e = op.row[i + 1];
        for (int p = op.row[i] + sub; p < e; p += LPR) s = fma(op.val[p], to_f64(z[op.col[p]]), s);
      }
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
      if (sub == 0) sw[t] = s;
    }
  } else {
    const int bs = op.bs, ld = bs * bs;
    for (int t = threadIdx.x; t < tr; t += kTPB) {
      const int i = base + t;
      double s = 0.0;
      if (i < n) {
        const int I = i / bs, r = i - I * bs;
        for (int p = op.row[I]; p < op.row[I + 1]; ++p) {
          const double *blk = op.val + (size_t)p * ld + r * bs;
          const ZT *zj = z + (size_t)op.col[p] * bs;
          for (int c = 0; c < bs; ++c) s = fma(blk[c], to_f64(zj[c]), s);
        }
      }
      sw[t] = s;
    }
  }
}

__device__ __forceinline__ double block_sum(double v, double *scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kTPB / 32; ++w) t += scratch[w];
  return t;  // valid in thread 0
}

// last block: sred[k] = sum over blocks of partials[b*kLdT + k], k < count;
// warp w takes k = w, w+8, ..., its lanes stride over the blocks (fixed
// order, so the result is deterministic)
__device__ __forceinline__ void fold_partials(const double *partials, int count, double *sred) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = wid; k < count; k += kTPB / 32) {
    double s = strided_sum(partials + k, kLdT, lane, 32, (int)gridDim.x);
    s = warp_sum(s);
    if (lane == 0) sred[k] = s;
  }
}

// FP64 -> FP32 with integer operations, rounding toward zero (the FP64 unit,
// which also converts, is the scarce one).  Finite values only: below the
// FP32 normal range they become 0, above it NaN.
__device__ __forceinline__ float dtof_rz(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const unsigned hi = (unsigned)(b >> 32);
  const int e = (int)((hi >> 20) & 0x7ffu) - 896;
  const unsigned m = ((hi & 0xfffffu) << 3) | ((unsigned)b >> 29);
  const unsigned mag = e <= 0 ? 0u : (e >= 255 ? 0x7fc00000u : (((unsigned)e << 23) | m));
  return __uint_as_float((hi & 0x80000000u) | mag);
}

// Double-float values: an FP64 value x as hi = dtof_rz(x) and lo =
// dtof_rz(x - hi), about 48 bits together (finite |x| < 2^128; lo of values
// near the FP32 underflow flushes to 0), so that products and sums of FP64
// data run on the FP32 unit - 64 times the FP64 unit's rate on this part -
// with FP64-like accuracy.  Conversions use integer operations.
__device__ __forceinline__ float2 df_split(double x) {
  const float h = dtof_rz(x);
  return make_float2(h, dtof_rz(x - to_f64(h)));
}
__device__ __forceinline__ double df_join(float2 v) { return to_f64(v.x) + to_f64(v.y); }
// (sh, sl) += (ah + al) * (bh + bl): the high product exactly (an FMA gives
// its rounding error), the cross terms in FP32, al*bl dropped (2^-48
// relative), the high parts summed error-free (TwoSum), the rest into sl
__device__ __forceinline__ void df_mac(float ah, float al, float bh, float bl, float &sh, float &sl) {
  const float p = ah * bh;
  const float pe = fmaf(ah, bl, fmaf(al, bh, fmaf(ah, bh, -p)));
  const float t = sh + p;
  const float z = t - sh;
  const float e = (sh - (t - z)) + (p - z);
  sh = t;
  sl += e + pe;
}// (sh, sl) += (ah + al) * b for an FP32 b
__device__ __forceinline__ void df_mac1(float ah, float al, float b, float &sh, float &sl) {
  const float p = ah * b;
  const float pe = fmaf(al, b, fmaf(ah, b, -p));
  const float t = sh + p;
  const float z = t - sh;
  const float e = (sh - (t - z)) + (p - z);
  sh = t;
  sl += e + pe;
}

// pair arithmetic for values kept as pairs: h + l as an unevaluated sum
// renormalised (TwoSum: exact for any magnitudes), a + b (the high parts
// summed error-free, the low parts added) and a * b (the high product
// exactly, the cross terms in FP32, a.lo * b.lo dropped)
__device__ __forceinline__ float2 df_renorm(float h, float l) {
  const float t = h + l, z = t - h;
  return make_float2(t, (h - (t - z)) + (l - z));
}
__device__ __forceinline__ float2 df_add(float2 a, float2 b) {
  const float t = a.x + b.x, z = t - a.x;
  const float e = (a.x - (t - z)) + (b.x - z);
  return df_renorm(t, e + (a.y + b.y));
}
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float p = a.x * b.x;
  const float e = fmaf(a.x, b.y, fmaf(a.y, b.x, fmaf(a.x, b.x, -p)));
  const float s = p + e;  // |e| <= |p| up to rounding: Fast2Sum
  return make_float2(s, e - (s - p));
}

// the unsolved pattern (all ones) into row i of an FP32 or FP64 vector: the
// sync-free solve that writes the vector polls it until the pattern is gone
__device__ __forceinline__ void mark_unsolved(void *x, int f32, size_t i) {
  if (f32) reinterpret_cast<unsigned *>(x)[i] = ~0u;
  else reinterpret_cast<unsigned long long *>(x)[i] = ~0ull;
}

// the vectors the next step's two solves write, marked unsolved (null: none)
struct Prefill {
  void *t, *z;
  int t_f32, z_f32;
};

__device__ __forceinline__ void prefill_row(const Prefill &f, size_t i) {
  if (f.t) mark_unsolved(f.t, f.t_f32, i);
  if (f.z) mark_unsolved(f.z, f.z_f32, i);
}

// ------------------------------------- persistent (cooperative) kernels

// Grid barrier over a cooperatively launched grid (Control::block_count[3]
// arrivals, [4] generation).  Bounded: a wait that gives up sets
// kStatusSpinTimeout, and every block leaves at its next barrier.
__device__ __forceinline__ bool grid_barrier(Control *ctrl) {
  __shared__ int s_ok;
  __threadfence();  // every thread's writes before the arrival (partial sums)
  __syncthreads();
  if (threadIdx.x == 0) {
    int *count = &ctrl->block_count[3];
    int *gen = &ctrl->block_count[4];
    const int g = ld_acquire(gen);
    __threadfence();
    int ok = 1;
    if (atomicAdd(count, 1) == (int)gridDim.x - 1) {
      *count = 0;
      st_release(gen, g + 1);
    } else {
      for (int spins = 0;; ++spins) {
        if (ld_acquire(gen) != g) break;
        if (spins > kMaxSpins || ((spins & 1023) == 1023 && (ld_relaxed(&ctrl->status) & kStatusSpinTimeout))) {
          atomicOr(&ctrl->status, kStatusSpinTimeout);
          ok = 0;
          break;
        }
        if (spins > 32) __nanosleep(32);
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// ------------------------------------------------------------ host side

static inline OpView opview(const ArnoldiArgs &a) {
  return OpView{a.bs, a.row, a.col, a.val, a.sell_ptr, a.sell_col, a.sell_val};
}

static inline int rowgrid(int n) {
  int g = (n + kTPB - 1) / kTPB;
  return std::min(g, num_sms() * 8);
}

// the outputs of step j's two solves (the L solve's vector and column j of Z)
static inline Prefill prefill_for(const ArnoldiArgs &a, int j) {
  if (!a.prefill || j >= a.m) return Prefill{nullptr, nullptr, 0, 0};
  void *zj = (char *)a.Z + (size_t)j * a.ldz * (a.z_f32 ? 4 : 8);
  return Prefill{a.fill_t, zj, a.fill_t_f32, a.z_f32};
}

// One wave: as many blocks as are resident at once (the passes loop over
// their row tiles), so no partly filled last wave, and the last block folds
// few partial sums.  Never more than the ArnoldiArgs grid the partial-sum
// buffer is sized for.
template <typename K>
static inline int wave_grid(K kernel, int cap) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kTPB, 0) != cudaSuccess || per_sm <= 0) {
    cudaGetLastError();
    return cap;
  }
  return std::max(1, std::min(cap, per_sm * num_sms()));
}

}  // namespace lace
