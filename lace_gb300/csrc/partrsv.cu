// ParCSRTRSV (data_parcsrtrsv, src/trisolve.cpp:256-351) in LACE's own sweep
// order.
//
// LACE sweeps in place: the lower triangle row by row upwards from row 0
// (:276-292), the upper one from the last row down (:319-335), each row
//   tmp = sum_k a_k * y[col_k]   (off-diagonal entries, in storage order)
//   y_i = (rhs_i - tmp) / diag   (diag: last entry of an L row, first of a U row)
// and the step is sum (y_old - y_new)^2; sweeps repeat while step > tol and
// the step is finite.  Run by one thread, an entry whose column comes earlier
// in the sweep reads the value this sweep already wrote, any other entry the
// previous sweep's value.  On a well-formed triangle the first sweep is
// therefore the exact substitution, and the second changes nothing.
//
// The GPU reproduces that order without a serial loop: one warp per row,
// rows taken in sweep order by groups of kPtGroup from an atomic ticket.  A
// value written in this sweep is its own ready flag (the output starts as an
// all-ones bit pattern, a NaN no arithmetic produces), so a row waits only for
// the rows before it in the sweep, which earlier tickets hold (no deadlock for
// any input).  Values of the warp's own group come from shared memory.  Each
// row's sum is formed in storage order with separately rounded multiplies and
// adds and an IEEE division, as LACE's loop compiles without contraction, so
// an iterate equals LACE's one-thread iterate bit for bit.
//
// A call runs rounds of two sweeps with no host round trip between them: the
// second sweep, the fill before it and the copy after it read the first
// sweep's step on the device and do nothing when LACE would have stopped.
#include <cmath>
#include <vector>

#include "context.h"

namespace lace {

namespace {

constexpr int kPtWarps = 8;   // warps per block
constexpr int kPtGroup = 32;  // rows per ticket, solved in order by one warp
constexpr unsigned long long kUnsolvedBits = 0xFFFFFFFFFFFFFFFFull;
constexpr unsigned long long kQuietNaNBits = 0x7FF8000000000000ull;

__device__ __forceinline__ double ld_relaxed_f64(const double *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return __longlong_as_double((long long)v);
}
__device__ __forceinline__ void st_relaxed_f64(double *p, double v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"((unsigned long long)__double_as_longlong(v))
               : "memory");
}

// true when the previous sweep of the round leaves LACE's loop running
__device__ __forceinline__ bool keep_going(const double *step, double tol) {
  const double v = *step;
  return v > tol && isfinite(v);
}

template <bool LOWER>
__global__ void __launch_bounds__(kPtWarps * 32)
    k_partrsv_sweep(int n, const int *__restrict__ row, const int *__restrict__ col,
                    const double *__restrict__ val, const double *__restrict__ rhs,
                    const double *__restrict__ yold, double *ynew, int *ticket, int *status,
                    const double *guard, double tol, int max_polls) {
  if (guard != nullptr && !keep_going(guard, tol)) return;
  __shared__ double win[kPtWarps][kPtGroup];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int ngroups = (n + kPtGroup - 1) / kPtGroup;
  const int nnz = __ldg(row + n);
  bool gave_up = false;
  while (true) {
    int t = 0;
    if (lane == 0) t = atomicAdd(ticket, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= ngroups) break;
    const int p0 = t * kPtGroup;  // sweep position of the group's first row
    const int cnt = min(kPtGroup, n - p0);
    // lane r holds the row pointers and right-hand side of the group's row r
    int rs = 0, re = 0;
    double bv = 0.0;
    if (lane < cnt) {
      const int i = LOWER ? p0 + lane : n - 1 - (p0 + lane);
      rs = __ldg(row + i);
      re = __ldg(row + i + 1);
      bv = __ldg(rhs + i);
    }
    for (int r = 0; r < cnt; ++r) {
      const int i = LOWER ? p0 + r : n - 1 - (p0 + r);
      const int s = __shfl_sync(0xffffffffu, rs, r), e = __shfl_sync(0xffffffffu, re, r);
      // row pointers outside the arrays: LACE would read outside them
      const bool rows_ok = s >= 0 && e <= nnz;
      if (!rows_ok && lane == 0) atomicOr(status, kStatusBadInput);
      const int kb = LOWER ? s : s + 1;  // off-diagonal entries [kb, ke)
      const int ke = rows_ok ? (LOWER ? e - 1 : e) : kb;
      const int dp = LOWER ? e - 1 : s;  // the entry LACE divides by
      double tmp = 0.0;
      for (int base = kb; base < ke; base += 32) {
        const int k = base + lane;
        double a = 0.0, v = 0.0;
        bool have = false, ready = true;
        int c = 0;
        if (k < ke) {
          c = __ldg(col + k);
          a = __ldg(val + k);
          if (c < 0 || c >= n) {
            atomicOr(status, kStatusBadInput);  // LACE would read outside y
          } else if (LOWER ? c < i : c > i) {   // written earlier in this sweep
            const int pc = LOWER ? c : n - 1 - c;
            if (pc >= p0) {
              v = win[wid][pc - p0];
            } else {
              v = ld_relaxed_f64(ynew + c);
              ready = (unsigned long long)__double_as_longlong(v) != kUnsolvedBits;
            }
            have = true;
          } else {  // not yet reached in this sweep: the previous sweep's value
            v = __ldg(yold + c);
            have = true;
          }
        }
        // warp-uniform bounded wait for the values other warps still owe
        int spins = 0;
        while (!__all_sync(0xffffffffu, ready)) {
          if (!ready && !gave_up) {
            v = ld_relaxed_f64(ynew + c);
            ready = (unsigned long long)__double_as_longlong(v) != kUnsolvedBits;
          }
          ++spins;
          if ((spins & 255) == 0 && (ld_relaxed(status) & kStatusSpinTimeout)) gave_up = true;
          if (spins > max_polls) {
            if (lane == 0) atomicOr(status, kStatusSpinTimeout);
            gave_up = true;
          }
          if (gave_up) ready = true;  // the call reports the timeout; finish without waiting
          if (spins > 32) __nanosleep(32);
        }
        const double prod = have ? __dmul_rn(a, v) : 0.0;
        const int m = min(32, ke - base);
        for (int q = 0; q < m; ++q) tmp = __dadd_rn(tmp, __shfl_sync(0xffffffffu, prod, q));
      }
      const double b = __shfl_sync(0xffffffffu, bv, r);
      double y;
      if (dp < 0 || dp >= nnz) {  // an empty first L row / last U row: LACE reads outside val
        if (lane == 0) atomicOr(status, kStatusBadInput);
        y = __longlong_as_double((long long)kQuietNaNBits);
      } else {
        y = __ddiv_rn(__dsub_rn(b, tmp), __ldg(val + dp));
      }
      if ((unsigned long long)__double_as_longlong(y) == kUnsolvedBits) y = __longlong_as_double((long long)kQuietNaNBits);
      if (lane == 0) {
        win[wid][r] = y;
        st_relaxed_f64(ynew + i, y);
      }
      __syncwarp();
    }
  }
}

// y <- unsolved pattern, when the round's second sweep will run
__global__ void k_partrsv_fill_if(int n, double *y, const double *guard, double tol) {
  if (!keep_going(guard, tol)) return;
  const double pat = __longlong_as_double((long long)kUnsolvedBits);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = pat;
}

// y <- a, when the round's second sweep did not run (LACE stopped after the
// first: its iterate is in a)
__global__ void k_partrsv_copy_unless(int n, double *y, const double *a, const double *guard, double tol) {
  if (keep_going(guard, tol)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = a[i];
}

int plain_grid(int n) {
  int g = (n + 255) / 256;
  const int cap = num_sms() * 4;
  return g < 1 ? 1 : (g > cap ? cap : g);
}

}  // namespace

int partrsv_partials_needed() { return num_sms() * 4; }

void launch_partrsv_sweep(cudaStream_t s, bool lower, int n, const int *row, const int *col, const double *val,
                          const double *rhs, const double *yold, double *ynew, int *ticket, int *status,
                          const double *guard, double tol, int max_polls) {
  if (max_polls <= 0) max_polls = kMaxSpins;
  const int ngroups = (n + kPtGroup - 1) / kPtGroup;
  int grid = (ngroups + kPtWarps - 1) / kPtWarps;
  const int cap = num_sms() * 8;
  if (grid > cap) grid = cap;
  if (grid < 1) grid = 1;
  if (lower)
    k_partrsv_sweep<true><<<grid, kPtWarps * 32, 0, s>>>(n, row, col, val, rhs, yold, ynew, ticket, status, guard, tol,
                                                                   max_polls);
  else
    k_partrsv_sweep<false><<<grid, kPtWarps * 32, 0, s>>>(n, row, col, val, rhs, yold, ynew, ticket, status, guard, tol,
                                                                    max_polls);
}

int partrsv_solve(cudaStream_t s, bool lower, int n, const int *row, const int *col, const double *val,
                  const double *rhs, double *y, double tol, int *iter, const PartrsvScratch &sc) {
  *iter = 0;
  if (n <= 0) return 0;
  // LACE loops while step > tol; a sweep that changes nothing changes
  // nothing again, so the loop also ends there (LACE's would not end for a
  // negative tol).  Well-formed triangles finish in two sweeps; the cap only
  // bounds a malformed triangle's Gauss-Seidel iteration.
  const int cap = 1000;
  const int pg = plain_grid(n);
  while (true) {
    // counters: two sweep tickets, the step reduction's arrival counter, status
    if (cudaMemsetAsync(sc.counters, 0, 4 * sizeof(int), s) != cudaSuccess) return DEV_ERR_UNKNOWN;
    if (cudaMemsetAsync(sc.a, 0xFF, sizeof(double) * (size_t)n, s) != cudaSuccess) return DEV_ERR_UNKNOWN;
    launch_partrsv_sweep(s, lower, n, row, col, val, rhs, y, sc.a, sc.counters + 0, sc.counters + 3, nullptr, tol, 0);
    launch_sqdiff(s, n, sc.a, y, 0, sc.partials, sc.counters + 2, sc.steps + 0);
    k_partrsv_fill_if<<<pg, 256, 0, s>>>(n, y, sc.steps + 0, tol);
    launch_partrsv_sweep(s, lower, n, row, col, val, rhs, sc.a, y, sc.counters + 1, sc.counters + 3, sc.steps + 0,
                         tol, 0);
    launch_sqdiff(s, n, y, sc.a, 0, sc.partials, sc.counters + 2, sc.steps + 1);
    k_partrsv_copy_unless<<<pg, 256, 0, s>>>(n, y, sc.a, sc.steps + 0, tol);
    if (cudaGetLastError() != cudaSuccess) return DEV_ERR_UNKNOWN;
    if (cudaMemcpyAsync(sc.h_steps, sc.steps, 2 * sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaMemcpyAsync(sc.h_status, sc.counters + 3, sizeof(int), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      return DEV_ERR_UNKNOWN;
    const int st = *sc.h_status;
    if (st & kStatusBadInput) return DEV_ERR_ILLEGAL_VALUE;
    if (st & kStatusSpinTimeout) return DEV_ERR_INTERNAL_LIMIT;
    double step = sc.h_steps[0];
    *iter += 1;
    if (!(step > tol && std::isfinite(step))) return 0;
    step = sc.h_steps[1];
    *iter += 1;
    if (!(step > tol && std::isfinite(step)) || step == 0.0) return 0;
    if (*iter >= cap) return DEV_ERR_INTERNAL_LIMIT;
  }
}

}  // namespace lace

using namespace lace;

extern "C" int lace_gpu_selftest_wait_limit(int max_polls, int *status_out) {
  // a 4096-row lower bidiagonal triangle: y_i = 1 + y_{i-1} / 2
  const int n = 4096;
  std::vector<int> hrow(n + 1), hcol;
  std::vector<double> hval;
  for (int i = 0; i < n; ++i) {
    hrow[i] = (int)hcol.size();
    if (i > 0) {
      hcol.push_back(i - 1);
      hval.push_back(-0.5);
    }
    hcol.push_back(i);
    hval.push_back(1.0);
  }
  hrow[n] = (int)hcol.size();
  const int nnz = hrow[n];
  std::vector<double> ref(n);
  for (int i = 0; i < n; ++i) {
    const double tmp = i > 0 ? 0.0 + (-0.5 * ref[i - 1]) : 0.0;
    ref[i] = (1.0 - tmp) / 1.0;
  }
  if (status_out) *status_out = 0;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return set_err(DEV_ERR_NOT_INITIALIZED);
  }
  cudaStream_t s = nullptr;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
  int rc = 0;
  {
    DBuf drow, dcol, dval, drhs, dold, dnew, dcnt;
    std::vector<double> ones(n, 1.0), zeros(n, 0.0);
    if (drow.upload(hrow.data(), 4 * (size_t)(n + 1), s) || dcol.upload(hcol.data(), 4 * (size_t)nnz, s) ||
        dval.upload(hval.data(), 8 * (size_t)nnz, s) || drhs.upload(ones.data(), 8 * (size_t)n, s) ||
        dold.upload(zeros.data(), 8 * (size_t)n, s) || dnew.ensure(8 * (size_t)n) || dcnt.ensure(4 * sizeof(int))) {
      rc = DEV_ERR_DEVICE_ALLOC;
    } else {
      int *cnt = (int *)dcnt.p;
      // 1. the first row group's ticket is never handed out (the counter
      //    starts past it), so the rows after it wait for values nothing
      //    writes until their waits give up
      const int start[4] = {1, 0, 0, 0};
      int st = 0;
      cudaMemcpyAsync(cnt, start, sizeof(start), cudaMemcpyHostToDevice, s);
      cudaMemsetAsync(dnew.p, 0xFF, 8 * (size_t)n, s);
      launch_partrsv_sweep(s, true, n, (const int *)drow.p, (const int *)dcol.p, (const double *)dval.p,
                           (const double *)drhs.p, (const double *)dold.p, (double *)dnew.p, cnt, cnt + 3,
                           nullptr, 0.0, max_polls);
      cudaMemcpyAsync(&st, cnt + 3, sizeof(int), cudaMemcpyDeviceToHost, s);
      if (cudaStreamSynchronize(s) != cudaSuccess) {
        cudaGetLastError();
        rc = DEV_ERR_UNKNOWN;
      } else {
        if (status_out) *status_out = st;
        if (!(st & kStatusSpinTimeout)) rc = DEV_ERR_UNKNOWN;  // the waits should have run out
      }
      // 2. the same sweep with every ticket handed out, on the same device,
      //    with the library's own wait limit (the rows of this chain wait
      //    for all the rows before them): the exact substitution, and no
      //    status bit
      if (!rc) {
        std::vector<double> y(n);
        cudaMemsetAsync(cnt, 0, 4 * sizeof(int), s);
        cudaMemsetAsync(dnew.p, 0xFF, 8 * (size_t)n, s);
        launch_partrsv_sweep(s, true, n, (const int *)drow.p, (const int *)dcol.p, (const double *)dval.p,
                             (const double *)drhs.p, (const double *)dold.p, (double *)dnew.p, cnt, cnt + 3,
                             nullptr, 0.0, 0);
        cudaMemcpyAsync(&st, cnt + 3, sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(y.data(), dnew.p, 8 * (size_t)n, cudaMemcpyDeviceToHost, s);
        if (cudaStreamSynchronize(s) != cudaSuccess) {
          cudaGetLastError();
          rc = DEV_ERR_UNKNOWN;
        } else if (st != 0 || y != ref) {
          rc = DEV_ERR_UNKNOWN;
        }
      }
    }
  }
  cudaStreamDestroy(s);
  return rc ? set_err(rc) : 0;
}
