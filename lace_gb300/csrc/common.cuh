// Device-side helpers shared by the lace_gb300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

namespace lace {

constexpr int kWarp = 32;

// Bit set in Control::status when a bounded wait gave up.
constexpr int kStatusSpinTimeout = 1;
// Bit set when a kernel met a non-finite value it must not divide by.
constexpr int kStatusBreakdown = 2;
// Bit set when a kernel met an index it must not follow (a column outside the
// matrix, a diagonal entry outside the value array).
constexpr int kStatusBadInput = 4;
// Upper bound on polls of one ready flag before a wait gives up.  A poll is
// one L2 round trip (~0.5 us), so this is ~1 s - far above any correct wait.
constexpr int kMaxSpins = 1 << 21;

// Per-solve device control block (lives in device memory; every kernel of an
// Arnoldi cycle reads `done` first and returns at once when it is set).
struct Control {
  int done;           // cycle finished (converged or search_max reached)
  int converged;      // |g_{j+1}| < rtol reached
  int nsteps;         // search directions in the finished cycle
  int status;         // kStatus* bits
  int trsv_epoch[4];  // last epoch published per triangle (L, U, U^T, L^T)
  int tickets[4][2];  // per-triangle {next chunk ticket, warps exited}
  int block_count[8]; // last-block counters, one per reducing kernel
  double rtol_abs;    // absolute tolerance of the current solve
  double rnorm0;      // initial residual of the solve
  double resid;       // |g_{j+1}| of the latest step
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ int ld_acquire(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(int *p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// value conversions for the factor storage types
template <typename T> __device__ __forceinline__ float to_f(T v);
template <> __device__ __forceinline__ float to_f<float>(float v) { return v; }
template <> __device__ __forceinline__ float to_f<double>(double v) { return (float)v; }
template <> __device__ __forceinline__ float to_f<__nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }

template <typename C, typename T> __device__ __forceinline__ C cvt(T v) { return (C)v; }
template <> __device__ __forceinline__ float cvt<float, __nv_bfloat16>(__nv_bfloat16 v) { return __bfloat162float(v); }
template <> __device__ __forceinline__ double cvt<double, __nv_bfloat16>(__nv_bfloat16 v) { return (double)__bfloat162float(v); }
template <> __device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16, float>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 cvt<__nv_bfloat16, double>(double v) { return __float2bfloat16_rn((float)v); }

// Deterministic grid reduction helper: every block writes its partials to
// partials[blockIdx.x * stride + k]; the block that arrives last (counter
// protocol with a fence) returns true and may then read all partials.  The
// counter is reset by that block.
__device__ __forceinline__ bool arrive_last(int *counter) {
  __shared__ int s_last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) {
    int prev = atomicAdd(counter, 1);
    s_last = (prev == (int)gridDim.x - 1);
    if (s_last) *counter = 0;
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last != 0;
}

// sum of p[b * step] over b = first, first + stride, ... < end, added in
// that order with eight loads in flight (a serial walk over a grid's
// partial sums costs one L2 round trip per block).  L2 loads: the partials
// were written by other blocks of the same grid.
__device__ __forceinline__ double strided_sum(const double *p, size_t step, int first, int stride, int end) {
  double s = 0.0;
  int b = first;
  for (; b + 7 * stride < end; b += 8 * stride) {
    double v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = __ldcg(p + (size_t)(b + u * stride) * step);
#pragma unroll
    for (int u = 0; u < 8; ++u) s += v[u];
  }
  for (; b < end; b += stride) s += __ldcg(p + (size_t)b * step);
  return s;
}

// the last block's fold of count partial sums p[b * step], by all of its
// threads: thread t adds b = t, t + blockDim.x, ..., then the warps and the
// warp sums in a fixed order (deterministic for a given grid).  Every thread
// of the block calls it; the sum is valid in thread 0.
__device__ __forceinline__ double block_fold(const double *p, size_t step, int count) {
  __shared__ double s_fold[32];
  double s = strided_sum(p, step, threadIdx.x, blockDim.x, count);
  s = warp_sum(s);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_fold[threadIdx.x >> 5] = s;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += s_fold[w];
  return t;
}

// FP32 -> FP64 exactly, with integer operations (conversions run on the FP64
// unit, the scarce one on this part)
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xffu;
  unsigned m = b & 0x7fffffu;
  unsigned long long ef;
  if (e == 0) {
    if (m == 0) {
      ef = 0;
    } else {  // subnormal: normalise
      const int sh = __clz((int)m) - 8;
      m = (m << sh) & 0x7fffffu;
      ef = (unsigned long long)(897 - sh) << 52;
    }
  } else {
    ef = (unsigned long long)(e == 255 ? 2047u : e + 896u) << 52;
  }
  return __longlong_as_double(
      (long long)(((unsigned long long)(b & 0x80000000u) << 32) | ef | ((unsigned long long)m << 29)));
}

// a stored factor value in FP64, exactly, without an FP64-pipe conversion
template <typename T> __device__ __forceinline__ double fval(T v);
template <> __device__ __forceinline__ double fval<double>(double v) { return v; }
template <> __device__ __forceinline__ double fval<float>(float v) { return to_f64(v); }
template <> __device__ __forceinline__ double fval<__nv_bfloat16>(__nv_bfloat16 v) {
  return to_f64(__bfloat162float(v));
}

// mysgn of LACE (include/sparse.h:1129-1133): +1 for v >= 0, -1 otherwise
__device__ __forceinline__ double mysgn(double v) { return v >= 0.0 ? 1.0 : -1.0; }

// LACE's Givens rotation (src/givens.cpp:46-67): (c, s) with
// [c s; -s c]^T-style sign convention of the reference
__device__ __forceinline__ void givens_rot(double a, double b, double tol, double *c, double *s) {
  if (fabs(b) <= tol) {
    *c = 1.0;
    *s = 0.0;
  } else if (fabs(b) > fabs(a)) {
    const double temp = a / b;
    *s = 1.0 / sqrt(1.0 + temp * temp);
    *c = temp * (*s);
  } else {
    const double temp = b / a;
    *c = 1.0 / sqrt(1.0 + temp * temp);
    *s = temp * (*c);
  }
}

}  // namespace lace
