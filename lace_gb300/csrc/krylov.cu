// SpMV and the FGMRES-Householder Arnoldi kernels.
//
// The Arnoldi step follows LACE's FGMRES-Householder
// (src/fgmres_householder_restart.cpp:311-757) but applies the reflectors in
// compact-WY form: P_0 P_1 ... P_j = I - V T V^T with T upper triangular.
//   pass A : w = A z_j fused with s = V^T w (one read of V)
//   pass B : w <- w - V (T^T s)  (LACE :376-469, all reflectors at once),
//            fused with d' = V^T w over rows > j and ||w_{j+1:}||^2; the last
//            block forms the new reflector scalars (LACE :476-511), extends T,
//            applies the Givens rotations, updates g and tests convergence
//            (LACE :658-714)
//   pass C : v_{j+1} and q = P_0...P_{j+1} e_{j+1} (LACE :519-617) in one read
//   x update (end of cycle): small least-squares solve + x += Z y (:721-744)
// k_hh_step runs passes A, B and C of a step as one cooperative kernel (w in
// shared memory, two grid reductions) where the operator is CSR and w fits;
// the separate passes serve the rest (BCSR, the adjoint, large n).
// Every kernel returns at once when Control::done is set, so a whole cycle can
// be launched (or replayed from a CUDA graph) without host round trips.
#include <math.h>
#include <stdio.h>

#include <algorithm>

#include "krylov_tile.cuh"

namespace lace {
constexpr int kSlots = (kMaxM + 2 + 7) / 8;  // k-slots per warp (8 warps)

// ------------------------------------------------------------------ SpMV

// LPR lanes per row, 32/LPR rows per warp; the loop bound is warp-uniform so
// every lane takes part in the segmented shuffle reduction.
template <int LPR, typename XT>
__global__ void __launch_bounds__(kTPB) k_spmv(int n, const int *__restrict__ row,
                                               const int *__restrict__ col,
                                               const double *__restrict__ val,
                                               const XT *__restrict__ x, double alpha,
                                               double beta, double *__restrict__ y) {
  constexpr int GPW = 32 / LPR;
  const int lane = threadIdx.x & 31;
  const int sub = lane & (LPR - 1);
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int wb = gw * GPW; wb < n; wb += nw * GPW) {
    const int i = wb + lane / LPR;
    double s = 0.0;
    if (i < n) {
      const int e = row[i + 1];
      for (int p = row[i] + sub; p < e; p += LPR) s = fma(val[p], (double)x[col[p]], s);
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
    if (sub == 0 && i < n) y[i] = (beta == 0.0) ? alpha * s : fma(beta, y[i], alpha * s);
  }
}

template <typename XT>
static void spmv_dispatch(cudaStream_t s, int lanes, int n, const int *row, const int *col,
                          const double *val, const XT *x, double alpha, double beta, double *y) {
  if (n <= 0) return;
  long long threads = (long long)n * lanes;
  long long g = (threads + kTPB - 1) / kTPB;
  if (g > (long long)num_sms() * 16) g = (long long)num_sms() * 16;
  int grid = (int)g;
  grid = grid < 1 ? 1 : grid;
  switch (lanes) {
    case 1: k_spmv<1, XT><<<grid, kTPB, 0, s>>>(n, row, col, val, x, alpha, beta, y); break;
    case 2: k_spmv<2, XT><<<grid, kTPB, 0, s>>>(n, row, col, val, x, alpha, beta, y); break;
    case 4: k_spmv<4, XT><<<grid, kTPB, 0, s>>>(n, row, col, val, x, alpha, beta, y); break;
    case 16: k_spmv<16, XT><<<grid, kTPB, 0, s>>>(n, row, col, val, x, alpha, beta, y); break;
    case 32: k_spmv<32, XT><<<grid, kTPB, 0, s>>>(n, row, col, val, x, alpha, beta, y); break;
    default: k_spmv<8, XT><<<grid, kTPB, 0, s>>>(n, row, col, val, x, alpha, beta, y); break;
  }
}

void launch_spmv_f64x(cudaStream_t s, int lanes, int n, const int *row, const int *col,
                      const double *val, const double *x, double alpha, double beta, double *y) {
  spmv_dispatch<double>(s, lanes, n, row, col, val, x, alpha, beta, y);
}
void launch_spmv_f32x(cudaStream_t s, int lanes, int n, const int *row, const int *col,
                      const double *val, const float *x, double alpha, double beta, double *y) {
  spmv_dispatch<float>(s, lanes, n, row, col, val, x, alpha, beta, y);
}

// y = alpha*A*x + beta*y on the sliced-ELL copy of A (slices of 32 rows,
// entry t of a slice's rows stored together): a warp per slice, a lane per
// row, so every column and value load is one coalesced 128- or 256-byte
// segment; a row's entries are loaded eight at a time (a 7-point row in one
// round) before their x gathers, with the entries summed in CSR order.
__global__ void __launch_bounds__(kTPB) k_sell_spmv(int n, const int *__restrict__ row,
                                                    const int *__restrict__ sell_ptr,
                                                    const int *__restrict__ sell_col,
                                                    const double *__restrict__ sell_val,
                                                    const double *__restrict__ x, double alpha, double beta,
                                                    double *__restrict__ y) {
  const int lane = threadIdx.x & 31;
  const int nsl = (n + 31) >> 5;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int sl = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; sl < nsl; sl += nw) {
    const int i = 32 * sl + lane;
    if (i >= n) continue;
    const int len = __ldg(row + i + 1) - __ldg(row + i);
    const int *cp = sell_col + __ldg(sell_ptr + sl) + lane;
    const double *vp = sell_val + (cp - sell_col);
    double s = 0.0;
    for (int t = 0; t < len; t += 8) {
      int c[8];
      double v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (t + u < len) {
          c[u] = __ldcs(cp + 32 * (t + u));
          v[u] = __ldcs(vp + 32 * (t + u));
        }
      double xv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (t + u < len) xv[u] = __ldg(x + c[u]);
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (t + u < len) s = fma(v[u], xv[u], s);
    }
    y[i] = (beta == 0.0) ? alpha * s : fma(beta, y[i], alpha * s);
  }
}

void launch_sell_spmv(cudaStream_t s, int n, const int *row, const int *sell_ptr, const int *sell_col,
                      const double *sell_val, const double *x, double alpha, double beta, double *y) {
  if (n <= 0) return;
  const int nsl = (n + 31) / 32;
  int grid = (nsl + kTPB / 32 - 1) / (kTPB / 32);
  const int cap = num_sms() * (2048 / kTPB);
  if (grid > cap) grid = cap;
  k_sell_spmv<<<grid, kTPB, 0, s>>>(n, row, sell_ptr, sell_col, sell_val, x, alpha, beta, y);
}

// BCSR: one thread per scalar row, the bs threads of a block row read the
// same blocks (row-major bs x bs)
__global__ void __launch_bounds__(kTPB) k_bcsr_spmv(int nb, int bs, const int *__restrict__ row,
                                                    const int *__restrict__ col,
                                                    const double *__restrict__ val,
                                                    const double *__restrict__ x, double alpha,
                                                    double beta, double *__restrict__ y) {
  const int n = nb * bs;
  const int ld = bs * bs;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int I = i / bs, r = i - I * bs;
    double s = 0.0;
    for (int p = row[I]; p < row[I + 1]; ++p) {
      const double *blk = val + (size_t)p * ld + r * bs;
      const double *xj = x + (size_t)col[p] * bs;
      for (int c = 0; c < bs; ++c) s = fma(blk[c], xj[c], s);
    }
    y[i] = (beta == 0.0) ? alpha * s : fma(beta, y[i], alpha * s);
  }
}

void launch_bcsr_spmv(cudaStream_t s, int nb, int bs, const int *row, const int *col,
                      const double *val, const double *x, double alpha, double beta, double *y) {
  int n = nb * bs;
  if (n <= 0) return;
  int grid = min((n + kTPB - 1) / kTPB, num_sms() * 16);
  k_bcsr_spmv<<<grid, kTPB, 0, s>>>(nb, bs, row, col, val, x, alpha, beta, y);
}

// --------------------------------------------------- row-tile machinery


// acc[slot] += sum over tile rows (masked by lo) of V[k][i] * sw[t]  with
// k = slot*8 + warp.  Lanes walk rows, warps walk columns: every V load is a
// coalesced 256-byte row segment of one column.
template <int NS>
__device__ __forceinline__ void tile_dots(const double *__restrict__ V, size_t ldv, int ncols,
                                          int n, int base, int tr, int lo, const double *sw,
                                          double (&acc)[NS]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  // the 8 rows of this lane, masked rows contribute 0 (their load address is
  // redirected to the tile's first row, which is always valid)
  double wv[8];
  int iv[8];
#pragma unroll
  for (int r = 0; r < 8; ++r) {
    const int t = lane + 32 * r;
    const int i = base + t;
    const bool ok = t < tr && i < n && i >= lo;
    wv[r] = ok ? sw[t] : 0.0;
    iv[r] = ok ? i : base;
  }
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    if (sl * 8 >= ncols) break;  // uniform over the block
    const int k = sl * 8 + wid;
    if (k < ncols) {
      // straight into the slot: FP64 additions cost as much as the products
      const double *Vk = V + (size_t)k * ldv;
      double v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) v[r] = Vk[iv[r]];
#pragma unroll
      for (int r = 0; r < 8; ++r) acc[sl] = fma(v[r], wv[r], acc[sl]);
    }
  }
}

// block-reduce acc into sred[k] (k < ncols); plus optional extra scalar
template <int NS>
__device__ __forceinline__ void block_reduce_slots(double (&acc)[NS], int ncols, double *sred) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) {
    const int k = sl * 8 + wid;
    if (sl * 8 < ncols) {  // warp-uniform
      double v = warp_sum(acc[sl]);
      if (lane == 0 && k < ncols) sred[k] = v;
    }
  }
}



// ------------------------------------------------------- cycle start

// r = b - A x (into a.w) and ||r||; last block sets up the first reflector
// scalars (LACE :209-236, :239-308) and the convergence test at cycle start.
// mgs: the Gram-Schmidt cycle instead (src/fgmres_restart.cpp:181-219):
// g = ||r|| e_0 and the rotations cleared, 1/||r|| for v_0.
template <int LPR>
__global__ void __launch_bounds__(kTPB) k_cycle_residual(int n, OpView op, const double *__restrict__ b,
                                                         const double *__restrict__ x,
                                                         double *__restrict__ r, double *partials,
                                                         Cycle *cy, Control *ctrl, int mgs, int m) {
  __shared__ double sw[kTPB];
  __shared__ double scratch[kTPB / 32];
  const int tr = (op.bs == 0) ? kTPB : (kTPB / op.bs) * op.bs;
  double nrm = 0.0;
  for (int base = blockIdx.x * tr; base < n; base += gridDim.x * tr) {
    tile_apply<LPR, double>(op, n, base, tr, x, sw);
    __syncthreads();
    for (int t = threadIdx.x; t < tr; t += kTPB) {
      const int i = base + t;
      if (i < n) {
        double ri = b[i] - sw[t];
        r[i] = ri;
        nrm = fma(ri, ri, nrm);
      }
    }
    __syncthreads();
  }
  double tot = block_sum(nrm, scratch);
  if (threadIdx.x == 0) partials[blockIdx.x] = tot;
  if (!arrive_last(&ctrl->block_count[0])) return;
  const double s = block_fold(partials, 1, (int)gridDim.x);
  if (threadIdx.x == 0) {
    const double rnorm = sqrt(s);
    cy->rnorm = rnorm;
    if (cy->first_cycle) {
      ctrl->rnorm0 = rnorm;
      ctrl->rtol_abs = cy->tol_type == 1 ? cy->rtol * rnorm : cy->rtol;
    }
    ctrl->nsteps = 0;
    ctrl->status = ctrl->status;  // keep earlier bits
    if (!(rnorm >= ctrl->rtol_abs)) {  // LACE :233 (also catches NaN: stop)
      ctrl->done = 1;
      ctrl->converged = (rnorm < ctrl->rtol_abs) ? 1 : 0;
      if (!(rnorm == rnorm)) ctrl->status |= kStatusBreakdown;
    } else if (mgs) {
      for (int k = 0; k <= m; ++k) cy->g[k] = 0.0;
      for (int k = 0; k < m; ++k) cy->cs[k] = cy->sn[k] = 0.0;
      cy->g[0] = rnorm;
      cy->hinv = 1.0 / rnorm;
      cy->nreorth = 0;
      ctrl->done = 0;
      ctrl->converged = 0;
    } else {
      const double r0 = r[0];
      const double dd = mysgn(r0) * rnorm;
      const double alpha = sqrt(2.0 * (s + fabs(r0) * rnorm));
      cy->dd0 = dd;
      cy->inv_alpha0 = alpha > 0.0 ? 1.0 / alpha : 0.0;
      cy->g[0] = -dd;
      cy->T[0] = 2.0;
      cy->G[0] = 1.0;
      ctrl->done = 0;
      ctrl->converged = 0;
    }
  }
}

// V[:,0] = (r + dd e_0)/alpha,  q = -r/dd
template <typename QT>
__global__ void __launch_bounds__(kTPB) k_cycle_init(int n, const double *__restrict__ r,
                                                     double *__restrict__ V, float *__restrict__ Vf,
                                                     float *__restrict__ Vlo, QT *__restrict__ q, const Cycle *cy,
                                                     const Control *ctrl, Prefill pf) {
  if (ctrl->done) return;
  const double dd = cy->dd0, ia = cy->inv_alpha0;
  const double rdd = 1.0 / dd;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double ri = r[i];
    const double v = (i == 0 ? ri + dd : ri) * ia;
    V[i] = v;
    if (Vf) {
      const float2 d = df_split(v);
      Vf[i] = d.x;
      if (Vlo) Vlo[i] = d.y;
    }
    q[i] = (QT)(-ri * rdd);
    prefill_row(pf, i);
  }
}

// sum_k V[k][i] c[k] over k < ncols: eight independent loads in flight
__device__ __forceinline__ double vcomb8(const double *__restrict__ V, size_t ldv, int i, int ncols,
                                         const double *c) {
  double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  int k = 0;
  for (; k + 8 <= ncols; k += 8) {
#pragma unroll
    for (int u = 0; u < 8; ++u) a[u] = fma(V[(size_t)(k + u) * ldv + i], c[k + u], a[u]);
  }
#pragma unroll
  for (int u = 0; u < 8; ++u)
    if (k + u < ncols) a[u] = fma(V[(size_t)(k + u) * ldv + i], c[k + u], a[u]);
  return ((a[0] + a[1]) + (a[2] + a[3])) + ((a[4] + a[5]) + (a[6] + a[7]));
}


// rows i, i+1 (i even): sum_k Vf[k][i..i+1] c[k] in FP32 from the FP32 copy
// of the reflectors, for vectors that only feed the FP32 preconditioner
__device__ __forceinline__ float2 vcomb8x2f(const float *__restrict__ Vf, size_t ldv, int i, int ncols,
                                           const float *c) {
  float2 a[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
  for (int k = 0; k < ncols; k += 8) {
    float2 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k + u < ncols) v[u] = __ldg(reinterpret_cast<const float2 *>(Vf + (size_t)(k + u) * ldv + i));
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k + u < ncols) {
        a[u & 3].x = fmaf(v[u].x, c[k + u], a[u & 3].x);
        a[u & 3].y = fmaf(v[u].y, c[k + u], a[u & 3].y);
      }
  }
  return make_float2((a[0].x + a[1].x) + (a[2].x + a[3].x), (a[0].y + a[1].y) + (a[2].y + a[3].y));
}

// rows i, i+1 (i even, i+1 < n): sum_k V[k][i..i+1] c[k] over k < ncols with
// 16-byte loads, a batch of eight columns in flight before any use
__device__ __forceinline__ double2 vcomb8x2(const double *__restrict__ V, size_t ldv, int i, int ncols,
                                           const double *c) {
  // two accumulators per row: the FP64 unit is the scarce one, so few
  // closing additions matter more than a short dependency chain
  double2 a[2] = {{0.0, 0.0}, {0.0, 0.0}};
  for (int k = 0; k < ncols; k += 8) {
    // a partial batch skips its missing columns
    double2 v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k + u < ncols) v[u] = __ldg(reinterpret_cast<const double2 *>(V + (size_t)(k + u) * ldv + i));
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k + u < ncols) {
        a[u & 1].x = fma(v[u].x, c[k + u], a[u & 1].x);
        a[u & 1].y = fma(v[u].y, c[k + u], a[u & 1].y);
      }
  }
  return make_double2(a[0].x + a[1].x, a[0].y + a[1].y);
}

// ------------------------------------------------------------- pass A

// NS: dot-product slots per warp (8 NS >= j + 1), so that short bases keep
// few accumulators in registers
// five blocks per SM for up to 16 basis columns (a few bytes of spill;
// measured slightly faster than four)
template <int LPR, typename ZT, int NS>
__global__ void __launch_bounds__(kTPB, NS <= 2 ? 5 : 1) k_passA(int n, OpView op, const ZT *__restrict__ z,
                                                double *__restrict__ w, const double *__restrict__ V,
                                                size_t ldv, int jp1, double *partials, Cycle *cy,
                                                Control *ctrl) {
  if (ctrl->done) return;
  // two tile buffers: a tile's products are written while slower warps still
  // read the previous tile's, so one barrier per tile
  __shared__ double swb[2][kTPB];
  int buf = 0;
  __shared__ double sred[kLdT];
  const int tr = (op.bs == 0) ? kTPB : (kTPB / op.bs) * op.bs;
  double acc[NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) acc[sl] = 0.0;
  for (int base = blockIdx.x * tr; base < n; base += gridDim.x * tr, buf ^= 1) {
    double *sw = swb[buf];
    tile_apply<LPR, ZT>(op, n, base, tr, z, sw);
    __syncthreads();
    for (int t = threadIdx.x; t < tr; t += kTPB)
      if (base + t < n) w[base + t] = sw[t];
    tile_dots<NS>(V, ldv, jp1, n, base, tr, 0, sw, acc);
  }
  __syncthreads();
  block_reduce_slots<NS>(acc, jp1, sred);
  __syncthreads();
  for (int k = threadIdx.x; k < jp1; k += kTPB) partials[(size_t)blockIdx.x * kLdT + k] = sred[k];
  if (!arrive_last(&ctrl->block_count[1])) return;
  // s = V^T w  -> y = T^T s
  fold_partials(partials, jp1, sred);
  __syncthreads();
  for (int k = threadIdx.x; k < jp1; k += kTPB) {
    double y = 0.0;
    for (int l = 0; l <= k; ++l) y = fma(cy->T[l + k * kLdT], sred[l], y);
    cy->y[k] = y;
  }
}

// ------------------------------------------------------------- pass B

// three blocks per SM for up to 32 basis columns (a few bytes of spill; the
// occupancy matters more: measured 2.8 % faster FGMRES)
template <int NS>
__global__ void __launch_bounds__(kTPB, NS <= 4 ? 3 : 1) k_passB(int n, const double *__restrict__ V, size_t ldv,
                                                int j, int m, double *__restrict__ w,
                                                double *partials, Cycle *cy, Control *ctrl) {
  if (ctrl->done) return;
  __shared__ double swb[2][2 * kTPB];  // two tile buffers, one barrier per tile (as in pass A)
  int buf = 0;
  __shared__ double sy[kLdT];
  __shared__ double sred[kLdT + 1];
  __shared__ double scratch[kTPB / 32];
  const int jp1 = j + 1;
  for (int k = threadIdx.x; k < jp1; k += kTPB) sy[k] = cy->y[k];
  __syncthreads();
  double acc[NS];
#pragma unroll
  for (int sl = 0; sl < NS; ++sl) acc[sl] = 0.0;
  double nrm = 0.0;
  // w -= V y over tiles of 2*kTPB rows (a row pair per thread, 16-byte
  // loads), then the tile's dot products with V for rows > j
  for (int base = blockIdx.x * 2 * kTPB; base < n; base += gridDim.x * 2 * kTPB, buf ^= 1) {
    double *sw = swb[buf];
    const int i = base + 2 * threadIdx.x;
    if (i + 1 < n) {
      const double2 wv = *reinterpret_cast<const double2 *>(w + i);
      const double2 c = vcomb8x2(V, ldv, i, jp1, sy);
      const double s0 = wv.x - c.x, s1 = wv.y - c.y;
      *reinterpret_cast<double2 *>(w + i) = make_double2(s0, s1);
      sw[2 * threadIdx.x] = s0;
      sw[2 * threadIdx.x + 1] = s1;
      if (i > j) nrm = fma(s0, s0, nrm);
      if (i + 1 > j) nrm = fma(s1, s1, nrm);
    } else if (i < n) {
      const double s0 = w[i] - vcomb8(V, ldv, i, jp1, sy);
      w[i] = s0;
      sw[2 * threadIdx.x] = s0;
      if (i > j) nrm = fma(s0, s0, nrm);
    }
    __syncthreads();
    tile_dots<NS>(V, ldv, jp1, n, base, kTPB, jp1, sw, acc);
    tile_dots<NS>(V, ldv, jp1, n, base + kTPB, kTPB, jp1, sw + kTPB, acc);
  }
  block_reduce_slots<NS>(acc, jp1, sred);
  double tot = block_sum(nrm, scratch);
  if (threadIdx.x == 0) sred[jp1] = tot;
  __syncthreads();
  for (int k = threadIdx.x; k <= jp1; k += kTPB) partials[(size_t)blockIdx.x * kLdT + k] = sred[k];
  if (!arrive_last(&ctrl->block_count[2])) return;

  // ---- last block: new reflector, T extension, Givens rotations
  __shared__ double sd[kLdT];
  __shared__ double srho[kLdT];
  __shared__ double sh[kLdT], scs[kLdT], ssn[kLdT];
  __shared__ double s_dd, s_ia, s_vjj;
  fold_partials(partials, jp1 + 1, sred);
  // Hessenberg column j and the rotations so far, staged in shared memory
  for (int k = threadIdx.x; k <= j; k += kTPB) {
    sh[k] = w[k];
    scs[k] = cy->cs[k];
    ssn[k] = cy->sn[k];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    // j+1 == n: the Krylov space is exhausted (LACE guards with search < n,
    // :476); the new reflector is empty and H(j+1,j) = 0
    const double nrm2 = jp1 < n ? sred[jp1] : 0.0;
    const double wn = sqrt(nrm2);
    const double wj1 = jp1 < n ? w[jp1] : 0.0;
    const double dd = mysgn(wj1) * wn;  // LACE :477-478
    const double alpha = sqrt(2.0 * (nrm2 + fabs(wj1) * wn));
    const double ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
    s_dd = dd;
    s_ia = ia;
    s_vjj = (wj1 + dd) * ia;
    cy->dd = dd;
    cy->inv_alpha = ia;
  }
  __syncthreads();
  // d = V_j^T v_{j+1}; rho = row j+1 of V_{j+1}
  for (int k = threadIdx.x; k < jp1; k += kTPB) {
    const double vk = jp1 < n ? V[(size_t)k * ldv + jp1] : 0.0;
    sd[k] = (sred[k] + s_dd * vk) * s_ia;
    srho[k] = vk;
  }
  if (threadIdx.x == 0) srho[jp1] = s_vjj;
  __syncthreads();
  // T(:, j+1) = [-2 T_j d ; 2]
  double *T = cy->T;
  for (int k = threadIdx.x; k < jp1; k += kTPB) {
    double t = 0.0;
    for (int l = k; l < jp1; ++l) t = fma(T[k + l * kLdT], sd[l], t);
    T[k + jp1 * kLdT] = -2.0 * t;
  }
  if (threadIdx.x == 0) {
    T[jp1 + jp1 * kLdT] = 2.0;
    for (int k = jp1 + 1; k < kLdT; ++k) T[k + jp1 * kLdT] = 0.0;
  }
  __syncthreads();
  // c = T_{j+1} rho  (consumed by pass C)
  for (int k = threadIdx.x; k <= jp1; k += kTPB) {
    double t = 0.0;
    for (int l = k; l <= jp1; ++l) t = fma(T[k + l * kLdT], srho[l], t);
    cy->c[k] = t;
  }
  if (threadIdx.x == 0) {
    // Hessenberg column j: h_k = w_k (k <= j), h_{j+1} = -dd  (LACE :658-701)
    for (int k = 0; k < j; ++k) {
      const double t0 = sh[k], t1 = sh[k + 1];
      sh[k + 1] = -ssn[k] * t0 + scs[k] * t1;
      sh[k] = scs[k] * t0 + ssn[k] * t1;
    }
    const double dd = s_dd;
    double c, s;
    givens_rot(sh[j], -dd, 4.9406564584124654e-324, &c, &s);
    cy->cs[j] = c;
    cy->sn[j] = s;
    sh[j] = c * sh[j] - s * dd;
    const double gj = cy->g[j];
    cy->g[jp1] = -s * gj;
    cy->g[j] = c * gj;
    const double resid = fabs(-s * gj);
    cy->hist[j] = resid;
    ctrl->resid = resid;
    const bool conv = resid < ctrl->rtol_abs;
    if (conv || j == m - 1 || !(resid == resid)) {  // LACE :714 (+ opt4's non-finite stop)
      ctrl->nsteps = jp1;  // the least-squares solve runs in the x update
      ctrl->converged = conv ? 1 : 0;
      if (!(resid == resid)) ctrl->status |= kStatusBreakdown;
      ctrl->done = 1;
    }
  }
  __syncthreads();
  double *R = cy->R + (size_t)j * kLdT;
  for (int k = threadIdx.x; k <= j; k += kTPB) R[k] = sh[k];
}

// ------------------------------------------------------------- pass C

// v_{j+1} (FP64) and q = e_{j+1} - V_{j+1} c, two rows per thread.  With an
// FP32 q (mixed precision: q only feeds the FP32 preconditioner, which
// rounds it to FP32 on its first read) the combination runs in FP32.
template <typename QT>
__global__ void __launch_bounds__(kTPB) k_passC(int n, double *__restrict__ V, float *__restrict__ Vf,
                                                float *__restrict__ Vlo, size_t ldv, int j, const double *__restrict__ w,
                                                QT *__restrict__ q, const Cycle *cy, const Control *ctrl,
                                                Prefill pf) {
  if (ctrl->done) return;
  constexpr bool kF32 = sizeof(QT) == 4;
  __shared__ double sc[kLdT];
  __shared__ float scf[kLdT];
  const int jp1 = j + 1;
  for (int k = threadIdx.x; k <= jp1; k += kTPB) {
    sc[k] = cy->c[k];
    scf[k] = (float)sc[k];
  }
  __syncthreads();
  const double dd = cy->dd, ia = cy->inv_alpha;
  double *vn = V + (size_t)jp1 * ldv;
  const int npair = n / 2;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += gridDim.x * blockDim.x) {
    const int i = 2 * p;
    const double2 wv = *reinterpret_cast<const double2 *>(w + i);
    const double v0 = (i > j) ? (i == jp1 ? wv.x + dd : wv.x) * ia : 0.0;
    const double v1 = (i + 1 > j) ? (i + 1 == jp1 ? wv.y + dd : wv.y) * ia : 0.0;
    *reinterpret_cast<double2 *>(vn + i) = make_double2(v0, v1);
    if constexpr (kF32) {
      const float2 d0 = df_split(v0), d1 = df_split(v1);
      const float2 vf = make_float2(d0.x, d1.x);
      *reinterpret_cast<float2 *>(Vf + (size_t)jp1 * ldv + i) = vf;  // the FP32 copy of v_{j+1}
      if (Vlo) *reinterpret_cast<float2 *>(Vlo + (size_t)jp1 * ldv + i) = make_float2(d0.y, d1.y);
      const float2 s = vcomb8x2f(Vf, ldv, i, jp1, scf);
      *reinterpret_cast<float2 *>(q + i) = make_float2(((i == jp1 ? 1.f : 0.f) - vf.x * scf[jp1]) - s.x,
                                                       ((i + 1 == jp1 ? 1.f : 0.f) - vf.y * scf[jp1]) - s.y);
    } else {
      const double2 s = vcomb8x2(V, ldv, i, jp1, sc);
      *reinterpret_cast<double2 *>(q + i) = make_double2(((i == jp1 ? 1.0 : 0.0) - v0 * sc[jp1]) - s.x,
                                                         ((i + 1 == jp1 ? 1.0 : 0.0) - v1 * sc[jp1]) - s.y);
    }
    prefill_row(pf, i);
    prefill_row(pf, i + 1);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {  // the last row of an odd n
    const int i = n - 1;
    const double v = (i > j) ? (i == jp1 ? w[i] + dd : w[i]) * ia : 0.0;
    vn[i] = v;
    if (kF32) {
      const float2 d = df_split(v);
      Vf[(size_t)jp1 * ldv + i] = d.x;
      if (Vlo) Vlo[(size_t)jp1 * ldv + i] = d.y;
    }
    q[i] = (QT)(((i == jp1 ? 1.0 : 0.0) - v * sc[jp1]) - vcomb8(V, ldv, i, jp1, sc));
    prefill_row(pf, i);
  }
}

// ------------------------------------------- one persistent kernel per step

// Passes A, B and C of step j in one cooperative launch of one block per SM:
// block b keeps rows [b*RB, (b+1)*RB) of w in shared memory through the step,
// the two sets of dot products (V^T w, then V^T w over rows > j with ||w||^2)
// are grid reductions (block partials, grid barrier, a fold every block
// performs in the same order), and the small-matrix work of pass B's last
// block (new reflector, T column, c = T rho) is done by every block
// identically, so pass C's combination follows without another barrier.
// The formulas and summation orders are the passes' own.
constexpr int kHHTPB = 1024;
constexpr int kHHSmemMax = 200 * 1024;  // rows of w per block: at most 25,600

struct HHStep {
  int n, rb;
  OpView op;  // sliced ELL
  const void *z;
  double *V;
  float *Vf;
  size_t ldv;
  void *q;
  double *partials;  // 2 phases x kLdT x gridDim.x
  Cycle *cy;
  Control *ctrl;
  int m;
  Prefill pf;
};

// block partial sums sacc[k] = sum over this block's rows i > lo of
// V[k][i] w[i], k < jp1: up to 32 columns as (column, row group) pairs over
// the 32 warps, more as up to five columns per warp; lanes walk rows
__device__ __forceinline__ void hh_block_dots(const double *__restrict__ V, size_t ldv, int jp1, int r0, int r1,
                                              int lo, const double *sw, double *swarp, double *sacc) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nsl = r1 > r0 ? (r1 - r0 + 31) >> 5 : 0;
  if (jp1 <= 32) {
    const int G = 32 / jp1;
    double acc = 0.0;
    if (wid < G * jp1) {
      // a warp streams its column over 1/G of the rows: eight rows per lane
      // in flight (one block per SM has few warps to hide the latency)
      const int k = wid % jp1, g = wid / jp1;
      const double *Vk = V + (size_t)k * ldv + r0;
      for (int sl0 = g; sl0 < nsl; sl0 += 8 * G) {
        double v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int t = 32 * (sl0 + u * G) + lane;
          v[u] = (sl0 + u * G < nsl && r0 + t < r1) ? Vk[t] : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int t = 32 * (sl0 + u * G) + lane;
          const int i = r0 + t;
          acc = fma(v[u], (sl0 + u * G < nsl && i < r1 && i > lo) ? sw[t] : 0.0, acc);
        }
      }
      acc = warp_sum(acc);
    }
    if (lane == 0) swarp[wid] = acc;
    __syncthreads();
    if (threadIdx.x < jp1) {
      double t = 0.0;
      for (int g = 0; g < G; ++g) t += swarp[g * jp1 + threadIdx.x];
      sacc[threadIdx.x] = t;
    }
  } else {
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    for (int sl0 = 0; sl0 < nsl; sl0 += 4) {
      // four rows per lane for each of the warp's columns in flight
      double wv[4];
      int ii[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int t = 32 * (sl0 + u) + lane;
        const int i = r0 + t;
        const bool ok = sl0 + u < nsl && i < r1 && i > lo;
        wv[u] = ok ? sw[t] : 0.0;
        ii[u] = ok ? i : r0;
      }
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        const int k = wid + 32 * c;
        if (32 * c < jp1 && k < jp1) {
          double v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) v[u] = V[(size_t)k * ldv + ii[u]];
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[c] = fma(v[u], wv[u], acc[c]);
        }
      }
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      const int k = wid + 32 * c;
      if (32 * c < jp1) {  // warp-uniform
        const double v = warp_sum(acc[c]);
        if (lane == 0 && k < jp1) swarp[k] = v;
      }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < jp1; k += blockDim.x) sacc[k] = swarp[k];
  }
  __syncthreads();
}

// sres[k] = sum over the grid of the blocks' sacc[k], k < nv, the same in
// every block (warp w folds k = w, w+32, ...; lanes stride over the blocks)
__device__ __forceinline__ bool hh_grid_fold(const double *sacc, int nv, double *partials, int &phase,
                                             Control *ctrl, double *sres, int cap = kLdT) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int G = gridDim.x;
  double *P = partials + (size_t)phase * cap * G;
  for (int k = threadIdx.x; k < nv; k += blockDim.x) P[(size_t)k * G + blockIdx.x] = sacc[k];
  if (!grid_barrier(ctrl)) return false;
  for (int k = wid; k < nv; k += (int)(blockDim.x >> 5)) {
    double t = strided_sum(P + (size_t)k * G, 1, lane, 32, G);
    t = warp_sum(t);
    if (lane == 0) sres[k] = t;
  }
  __syncthreads();
  phase ^= 1;
  return true;
}

template <typename ZT, typename QT>
__global__ void __launch_bounds__(kHHTPB, 1) k_hh_step(HHStep a, int j) {
  if (a.ctrl->done) return;
  constexpr bool kF32 = sizeof(QT) == 4;
  extern __shared__ double sw[];
  __shared__ double swarp[5 * 32];
  __shared__ double sacc[kLdT + 1], sres[kLdT + 1];
  __shared__ double sy[kLdT], sd[kLdT], srho[kLdT], sc[kLdT];
  __shared__ float scf[kLdT];
  __shared__ double sbuf[kHHTPB];
  __shared__ double s_dd, s_ia, s_vjj;
  const int n = a.n, jp1 = j + 1, T = blockDim.x;
  const int r0 = blockIdx.x * a.rb, r1 = min(n, r0 + a.rb);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t ldv = a.ldv;
  const double *__restrict__ V = a.V;
  Cycle *cy = a.cy;
  int phase = 0;
  // ---- pass A: w = A z_j (a warp per 32-row slice), s = V^T w
  {
    const ZT *z = (const ZT *)a.z;
    for (int sl = (r0 >> 5) + wid; 32 * sl < r1; sl += (T >> 5)) {
      const int i = 32 * sl + lane;
      if (i < r1) {
        const int len = a.op.row[i + 1] - a.op.row[i];
        const int *cp = a.op.sell_col + a.op.sell_ptr[sl] + lane;
        const double *vp = a.op.sell_val + (cp - a.op.sell_col);
        double s = 0.0;
        for (int t = 0; t < len; t += 8) {  // a 7-point row in one round of loads
          int c[8];
          double v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t + u < len) {
              c[u] = cp[32 * (t + u)];
              v[u] = vp[32 * (t + u)];
            }
          ZT zv[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t + u < len) zv[u] = z[c[u]];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t + u < len) s = fma(v[u], to_f64(zv[u]), s);
        }
        sw[i - r0] = s;
      }
    }
  }
  __syncthreads();
  hh_block_dots(V, ldv, jp1, r0, r1, -1, sw, swarp, sacc);
  if (!hh_grid_fold(sacc, jp1, a.partials, phase, a.ctrl, sres)) return;
  // y = T^T s
  for (int k = threadIdx.x; k < jp1; k += T) {
    double y = 0.0;
    for (int l = 0; l <= k; ++l) y = fma(cy->T[l + k * kLdT], sres[l], y);
    sy[k] = y;
  }
  __syncthreads();
  // ---- pass B: w -= V y (a row pair per thread), then V^T w over rows > j
  // and ||w_{j+1:}||^2; rows 0..j+1 of w published for every block
  double nrm = 0.0;
  {
    const int p0 = r0 >> 1, p1 = r1 >> 1;
    for (int p = p0 + threadIdx.x; p < p1; p += T) {
      const int i = 2 * p;
      const double2 c = vcomb8x2(V, ldv, i, jp1, sy);
      const double s0 = sw[i - r0] - c.x, s1 = sw[i + 1 - r0] - c.y;
      sw[i - r0] = s0;
      sw[i + 1 - r0] = s1;
      if (i > j) nrm = fma(s0, s0, nrm);
      if (i + 1 > j) nrm = fma(s1, s1, nrm);
      if (i <= jp1) cy->wtop[i] = s0;
      if (i + 1 <= jp1) cy->wtop[i + 1] = s1;
    }
    if ((r1 & 1) && r1 > r0 && threadIdx.x == 0) {  // the last row of an odd n
      const int i = r1 - 1;
      const double s0 = sw[i - r0] - vcomb8(V, ldv, i, jp1, sy);
      sw[i - r0] = s0;
      if (i > j) nrm = fma(s0, s0, nrm);
      if (i <= jp1) cy->wtop[i] = s0;
    }
  }
  sbuf[threadIdx.x] = nrm;
  __syncthreads();  // w and the norm terms in place
  hh_block_dots(V, ldv, jp1, r0, r1, j, sw, swarp, sacc);
  if (wid < 4) {  // the norm: four warps add a quarter each (few FP64 adds)
    const int quarter = T >> 2;
    double t = 0.0;
    for (int k = wid * quarter + lane; k < (wid + 1) * quarter; k += 32) t += sbuf[k];
    t = warp_sum(t);
    if (lane == 0) swarp[wid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) sacc[jp1] = ((swarp[0] + swarp[1]) + swarp[2]) + swarp[3];
  __syncthreads();
  if (!hh_grid_fold(sacc, jp1 + 1, a.partials, phase, a.ctrl, sres)) return;
  // ---- pass B's last-block work, in every block: new reflector, T column,
  // c = T_{j+1} rho (LACE :476-511)
  if (threadIdx.x == 0) {
    const double nrm2 = jp1 < n ? sres[jp1] : 0.0;
    const double wn = sqrt(nrm2);
    const double wj1 = jp1 < n ? __ldcg(&cy->wtop[jp1]) : 0.0;
    const double dd = mysgn(wj1) * wn;
    const double alpha = sqrt(2.0 * (nrm2 + fabs(wj1) * wn));
    const double ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
    s_dd = dd;
    s_ia = ia;
    s_vjj = (wj1 + dd) * ia;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < jp1; k += T) {
    const double vk = jp1 < n ? V[(size_t)k * ldv + jp1] : 0.0;
    sd[k] = (sres[k] + s_dd * vk) * s_ia;
    srho[k] = vk;
  }
  if (threadIdx.x == 0) srho[jp1] = s_vjj;
  __syncthreads();
  // the new column of T (kept in sacc) and c
  for (int k = threadIdx.x; k < jp1; k += T) {
    double t = 0.0;
    for (int l = k; l < jp1; ++l) t = fma(cy->T[k + l * kLdT], sd[l], t);
    sacc[k] = -2.0 * t;
  }
  if (threadIdx.x == 0) sacc[jp1] = 2.0;
  __syncthreads();
  for (int k = threadIdx.x; k <= jp1; k += T) {
    double t = 0.0;
    for (int l = k; l < jp1; ++l) t = fma(cy->T[k + l * kLdT], srho[l], t);
    t = fma(sacc[k], srho[jp1], t);
    sc[k] = t;
    scf[k] = (float)t;
  }
  __syncthreads();
  if (blockIdx.x == 0) {
    // the record: T column, reflector scalars, c; rotations and the test
    double *Tg = cy->T;
    for (int k = threadIdx.x; k < kLdT; k += T) Tg[k + jp1 * kLdT] = k <= jp1 ? sacc[k] : 0.0;
    for (int k = threadIdx.x; k <= jp1; k += T) cy->c[k] = sc[k];
    if (threadIdx.x == 0) {
      cy->dd = s_dd;
      cy->inv_alpha = s_ia;
      // Hessenberg column j: h_k = w_k (k <= j), h_{j+1} = -dd (LACE :658-701)
      double *sh = sbuf;
      for (int k = 0; k <= j; ++k) sh[k] = __ldcg(&cy->wtop[k]);
      for (int k = 0; k < j; ++k) {
        const double t0 = sh[k], t1 = sh[k + 1];
        sh[k + 1] = -cy->sn[k] * t0 + cy->cs[k] * t1;
        sh[k] = cy->cs[k] * t0 + cy->sn[k] * t1;
      }
      const double dd = s_dd;
      double c, sn;
      givens_rot(sh[j], -dd, 4.9406564584124654e-324, &c, &sn);
      cy->cs[j] = c;
      cy->sn[j] = sn;
      sh[j] = c * sh[j] - sn * dd;
      const double gj = cy->g[j];
      cy->g[jp1] = -sn * gj;
      cy->g[j] = c * gj;
      const double resid = fabs(-sn * gj);
      cy->hist[j] = resid;
      a.ctrl->resid = resid;
      const bool conv = resid < a.ctrl->rtol_abs;
      double *R = cy->R + (size_t)j * kLdT;
      for (int k = 0; k <= j; ++k) R[k] = sh[k];
      if (conv || j == a.m - 1 || !(resid == resid)) {  // LACE :714 (+ opt4's non-finite stop)
        a.ctrl->nsteps = jp1;
        a.ctrl->converged = conv ? 1 : 0;
        if (!(resid == resid)) a.ctrl->status |= kStatusBreakdown;
        a.ctrl->done = 1;
      }
    }
  }
  // ---- pass C: v_{j+1} and q = e_{j+1} - V_{j+1} c for this block's rows
  const double dd = s_dd, ia = s_ia;
  double *vn = a.V + (size_t)jp1 * ldv;
  QT *q = (QT *)a.q;
  const int p0 = r0 >> 1, p1 = r1 >> 1;
  for (int p = p0 + threadIdx.x; p < p1; p += T) {
    const int i = 2 * p;
    const double w0 = sw[i - r0], w1 = sw[i + 1 - r0];
    const double v0 = (i > j) ? (i == jp1 ? w0 + dd : w0) * ia : 0.0;
    const double v1 = (i + 1 > j) ? (i + 1 == jp1 ? w1 + dd : w1) * ia : 0.0;
    *reinterpret_cast<double2 *>(vn + i) = make_double2(v0, v1);
    if constexpr (kF32) {
      const float2 vf = make_float2(dtof_rz(v0), dtof_rz(v1));
      *reinterpret_cast<float2 *>(a.Vf + (size_t)jp1 * ldv + i) = vf;
      const float2 sm = vcomb8x2f(a.Vf, ldv, i, jp1, scf);
      *reinterpret_cast<float2 *>(q + i) = make_float2(((i == jp1 ? 1.f : 0.f) - vf.x * scf[jp1]) - sm.x,
                                                       ((i + 1 == jp1 ? 1.f : 0.f) - vf.y * scf[jp1]) - sm.y);
    } else {
      const double2 sm = vcomb8x2(V, ldv, i, jp1, sc);
      *reinterpret_cast<double2 *>(q + i) = make_double2(((i == jp1 ? 1.0 : 0.0) - v0 * sc[jp1]) - sm.x,
                                                         ((i + 1 == jp1 ? 1.0 : 0.0) - v1 * sc[jp1]) - sm.y);
    }
    prefill_row(a.pf, i);
    prefill_row(a.pf, i + 1);
  }
  if ((r1 & 1) && r1 > r0 && threadIdx.x == 0) {
    const int i = r1 - 1;
    const double v = (i > j) ? (i == jp1 ? sw[i - r0] + dd : sw[i - r0]) * ia : 0.0;
    vn[i] = v;
    if (kF32) a.Vf[(size_t)jp1 * ldv + i] = dtof_rz(v);
    q[i] = (QT)(((i == jp1 ? 1.0 : 0.0) - v * sc[jp1]) - vcomb8(V, ldv, i, jp1, sc));
    prefill_row(a.pf, i);
  }
}

// --------------------------- the one-kernel step in double-float arithmetic
// Mixed precision (FP32 preconditioner) on this part: the step's (j+1)-column
// dot products and its w -= V y update, 3(j+1) FP64 FMAs per row in the FP64
// form, run as double-float arithmetic on the FP32 unit from the reflectors'
// (Vf, Vlo) pair and a (hi, lo) copy of w in shared memory.  FP64 stays in
// the operator (A z), in w itself between the phases (rebuilt from its pair
// where it is needed: the update, the norm, the published top rows, the new
// reflector) and in everything after the grid reductions, which fold FP64
// partial sums as before.  A lane's double-float sum goes into an FP64
// accumulator every 32 terms, so its rounding stays at the level of a short
// FP64 sum.  Same phases, barriers and small-matrix work as k_hh_step.

// operand of the block dot products: the block's rows of a vector as
// pairs in shared memory
struct DfShared {
  const float2 *sw;
  __device__ __forceinline__ float2 get(int t, int) const { return sw[t]; }
};

// block partial sums sacc[k] = sum over this block's rows i > lo of
// V[k][i] x[i], k < ncols, from the double-float pairs (ncols >= 1)
template <class OP>
__device__ __forceinline__ void hh_block_dots_df(const float *__restrict__ Vf, const float *__restrict__ Vlo,
                                                 size_t ldv, int ncols, int r0, int r1, int lo, OP x,
                                                 double *swarp, double *sacc) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int nsl = r1 > r0 ? (r1 - r0 + 31) >> 5 : 0;
  if (ncols <= 32) {
    const int G = 32 / ncols;
    double acc = 0.0;
    if (wid < G * ncols) {
      const int k = wid % ncols, g = wid / ncols;
      const float *Hk = Vf + (size_t)k * ldv + r0, *Lk = Vlo + (size_t)k * ldv + r0;
      int batch = 0;
      float sh = 0.f, sl = 0.f;
      for (int sl0 = g; sl0 < nsl; sl0 += 8 * G) {
        float vh[8], vl[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int t = 32 * (sl0 + u * G) + lane;
          const bool ok = sl0 + u * G < nsl && r0 + t < r1;
          vh[u] = ok ? Hk[t] : 0.f;
          vl[u] = ok ? Lk[t] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int t = 32 * (sl0 + u * G) + lane;
          const int i = r0 + t;
          const float2 wv = (sl0 + u * G < nsl && i < r1 && i > lo) ? x.get(t, i) : make_float2(0.f, 0.f);
          df_mac(vh[u], vl[u], wv.x, wv.y, sh, sl);
        }
        if (++batch == 4) {  // 32 terms per lane: into the FP64 sum
          acc += to_f64(sh) + to_f64(sl);
          sh = sl = 0.f;
          batch = 0;
        }
      }
      acc += to_f64(sh) + to_f64(sl);
      acc = warp_sum(acc);
    }
    if (lane == 0) swarp[wid] = acc;
    __syncthreads();
    if (threadIdx.x < ncols) {
      double t = 0.0;
      for (int g = 0; g < G; ++g) t += swarp[g * ncols + threadIdx.x];
      sacc[threadIdx.x] = t;
    }
  } else {
    double acc[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    float sh[5] = {0.f, 0.f, 0.f, 0.f, 0.f}, sl[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    int batch = 0;
    for (int sl0 = 0; sl0 < nsl; sl0 += 4) {
      float2 wv[4];
      int ii[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int t = 32 * (sl0 + u) + lane;
        const int i = r0 + t;
        const bool ok = sl0 + u < nsl && i < r1 && i > lo;
        wv[u] = ok ? x.get(t, i) : make_float2(0.f, 0.f);
        ii[u] = ok ? i : r0;
      }
#pragma unroll
      for (int c = 0; c < 5; ++c) {
        const int k = wid + 32 * c;
        if (32 * c < ncols && k < ncols) {
          float vh[4], vl[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            vh[u] = Vf[(size_t)k * ldv + ii[u]];
            vl[u] = Vlo[(size_t)k * ldv + ii[u]];
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) df_mac(vh[u], vl[u], wv[u].x, wv[u].y, sh[c], sl[c]);
        }
      }
      if (++batch == 8) {
#pragma unroll
        for (int c = 0; c < 5; ++c) {
          acc[c] += to_f64(sh[c]) + to_f64(sl[c]);
          sh[c] = sl[c] = 0.f;
        }
        batch = 0;
      }
    }
#pragma unroll
    for (int c = 0; c < 5; ++c) {
      acc[c] += to_f64(sh[c]) + to_f64(sl[c]);
      const int k = wid + 32 * c;
      if (32 * c < ncols) {  // warp-uniform
        const double v = warp_sum(acc[c]);
        if (lane == 0 && k < ncols) swarp[k] = v;
      }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < ncols; k += blockDim.x) sacc[k] = swarp[k];
  }
  __syncthreads();
}

// (h, l) summed over the warp in double-float (TwoSum at each level; every
// lane ends with the same pair)
__device__ __forceinline__ void warp_sum_df(float &h, float &l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, h, o), l2 = __shfl_xor_sync(0xffffffffu, l, o);
    const float t = h + h2, z = t - h;
    const float e = (h - (t - z)) + (h2 - z);
    h = t;
    l = (l + l2) + e;
  }
}

// pass C's sweep over the basis, a thread per row, eight columns at a
// time: sgx[k] = sum over the block's rows of V[k][i] x[i] (k < ncols, x =
// v_{j+1} as pairs in sx; double-float per thread, then over the warp, then
// over the warps in FP64 in a fixed order) and q[i] = q0_i - sum_k V[k][i]
// c[k] in FP32, the columns in ascending order (q0_i = e_{j+1} - v_{j+1,i}
// c_{j+1}): each thread keeps its rows from chunk to chunk, so q is
// deterministic.  swarp2 holds 32 x 8 pairs.
__device__ __forceinline__ void hh_passC_rows(const float *__restrict__ Vf, const float *__restrict__ Vlo,
                                              size_t ldv, int ncols, int r0, int r1, int jp1, const float2 *sx,
                                              const float *scf, float *q, float2 *swarp2, double *sgx) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, T = blockDim.x;
  const float cj1 = scf[jp1];
  for (int k0 = 0; k0 < ncols; k0 += 8) {
    float cf[8];
#pragma unroll
    for (int c = 0; c < 8; ++c) cf[c] = k0 + c < ncols ? scf[k0 + c] : 0.f;
    float sh[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f}, sl[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int i = r0 + threadIdx.x; i < r1; i += T) {
      float vh[8], vl[8];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        const bool ok = k0 + c < ncols;
        vh[c] = ok ? Vf[(size_t)(k0 + c) * ldv + i] : 0.f;
        vl[c] = ok ? Vlo[(size_t)(k0 + c) * ldv + i] : 0.f;
      }
      const float2 x = sx[i - r0];
      float qp = k0 == 0 ? (i == jp1 ? 1.f : 0.f) - x.x * cj1 : q[i];
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        df_mac(vh[c], vl[c], x.x, x.y, sh[c], sl[c]);
        qp = fmaf(-vh[c], cf[c], qp);
      }
      q[i] = qp;
    }
#pragma unroll
    for (int c = 0; c < 8; ++c) {
      warp_sum_df(sh[c], sl[c]);
      if (lane == 0) swarp2[wid * 8 + c] = make_float2(sh[c], sl[c]);
    }
    __syncthreads();
    if (threadIdx.x < 8 && k0 + (int)threadIdx.x < ncols) {
      double t = 0.0;
      for (int w = 0; w < (T >> 5); ++w) {
        const float2 v = swarp2[w * 8 + threadIdx.x];
        t += to_f64(v.x) + to_f64(v.y);
      }
      sgx[k0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

// rows i, i+1 (i even): sum_k V[k][i..i+1] y[k] over k < ncols in
// double-float from the (Vf, Vlo) pairs and y's pair (yh, yl), as two pairs
__device__ __forceinline__ float4 vcomb_df_x2(const float *__restrict__ Vf, const float *__restrict__ Vlo,
                                              size_t ldv, int i, int ncols, const float *yh, const float *yl) {
  float h0 = 0.f, l0 = 0.f, h1 = 0.f, l1 = 0.f;
  for (int k = 0; k < ncols; k += 8) {
    float2 vh[8], vl[8];
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k + u < ncols) {
        vh[u] = __ldg(reinterpret_cast<const float2 *>(Vf + (size_t)(k + u) * ldv + i));
        vl[u] = __ldg(reinterpret_cast<const float2 *>(Vlo + (size_t)(k + u) * ldv + i));
      }
#pragma unroll
    for (int u = 0; u < 8; ++u)
      if (k + u < ncols) {
        df_mac(vh[u].x, vl[u].x, yh[k + u], yl[k + u], h0, l0);
        df_mac(vh[u].y, vl[u].y, yh[k + u], yl[k + u], h1, l1);
      }
  }
  return make_float4(h0, l0, h1, l1);
}

__device__ __forceinline__ float2 vcomb_df(const float *__restrict__ Vf, const float *__restrict__ Vlo, size_t ldv,
                                           int i, int ncols, const float *yh, const float *yl) {
  float h = 0.f, l = 0.f;
  for (int k = 0; k < ncols; ++k) df_mac(Vf[(size_t)k * ldv + i], Vlo[(size_t)k * ldv + i], yh[k], yl[k], h, l);
  return make_float2(h, l);
}

struct HHStepDF {
  HHStep base;
  float *Vlo;
  const float2 *sell_pair;  // the operator's sliced-ELL values as pairs
  double *carry;  // block partials of V_j^T v_{j+1}, left for the next step
};

// One Arnoldi step as one cooperative kernel, double-float dot products.
// Pass A: w = A z_j and s = V^T w.  With g = V_j^T v_j (its block partials
// left by the previous step), one grid fold gives s and the exact column j
// of T and of the Gram matrix G = V^T V; y = T^T s.  Pass B: w -= V y and
// ||w_{j+1:}||^2 (a second fold).  Then the new reflector and a
// provisional column j+1 of T from V^T w_{j+1:} = s - G y - V_top^T w_top
// (no pass over V, but its rounding grows with ||w|| / ||w_{j+1:}||): it
// only forms this step's q = e_{j+1} - V T V^T e_{j+1}, the vector the
// preconditioner is applied to next, which need not be exact - the Arnoldi
// relation holds for any q.  Pass C: v_{j+1}, then one sweep over V forms q
// and the exact V_j^T v_{j+1} for the next step.  The Hessenberg column and
// its Givens rotation run last, in the block with the fewest rows.
__global__ void __launch_bounds__(kHHTPB, 1) k_hh_step_df(HHStepDF ad, int j) {
  const HHStep &a = ad.base;
  if (a.ctrl->done) return;
  extern __shared__ float2 swd[];  // this block's rows of w, then of v_{j+1}, as (hi, lo)
  constexpr int kCap = 2 * kLdT;   // values per grid fold
  __shared__ double swarp[5 * 32];
  __shared__ double sacc[kCap], sres[kCap];
  __shared__ double sd[kLdT], srho[kLdT], sc[kLdT];
  __shared__ double sy[kLdT], ss[kLdT], stc[kLdT], sg[kLdT], s2[kLdT];
  __shared__ float syh[kLdT], syl[kLdT];
  __shared__ float scf[kLdT];
  __shared__ double sbuf[kHHTPB];
  __shared__ double s_dd, s_ia, s_vjj;
  const int n = a.n, jp1 = j + 1, T = blockDim.x, nw = T >> 5;
  const int r0 = blockIdx.x * a.rb, r1 = min(n, r0 + a.rb);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const size_t ldv = a.ldv;
  const float *__restrict__ Vf = a.Vf;
  const float *__restrict__ Vlo = ad.Vlo;
  Cycle *cy = a.cy;
  const int G = gridDim.x;
  int phase = 0;
  // g's block partials from the previous step, folded with s below
  for (int k = threadIdx.x; k < j; k += T) sacc[jp1 + k] = __ldcg(&ad.carry[(size_t)k * G + blockIdx.x]);
  // ---- pass A: w = A z_j in pair arithmetic (the operator's values as
  // pairs, z in FP32: each product's high part exact), a warp per 32-row
  // slice
  {
    const float *z = (const float *)a.z;
    for (int sl = (r0 >> 5) + wid; 32 * sl < r1; sl += nw) {
      const int i = 32 * sl + lane;
      if (i < r1) {
        const int len = a.op.row[i + 1] - a.op.row[i];
        const int *cp = a.op.sell_col + a.op.sell_ptr[sl] + lane;
        const float2 *vp = ad.sell_pair + (cp - a.op.sell_col);
        float sh = 0.f, sl2 = 0.f;
        for (int t = 0; t < len; t += 8) {
          int c[8];
          float2 v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t + u < len) {
              c[u] = cp[32 * (t + u)];
              v[u] = vp[32 * (t + u)];
            }
          float zv[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t + u < len) zv[u] = z[c[u]];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (t + u < len) df_mac1(v[u].x, v[u].y, zv[u], sh, sl2);
        }
        swd[i - r0] = df_renorm(sh, sl2);
      }
    }
  }
  __syncthreads();
  hh_block_dots_df(Vf, Vlo, ldv, jp1, r0, r1, -1, DfShared{swd}, swarp, sacc);
  if (!hh_grid_fold(sacc, jp1 + j, a.partials, phase, a.ctrl, sres, kCap)) return;
  // T(:, j) = [-2 T_j g ; 2] and G(:, j) = [g ; 1] (a warp per entry)
  for (int k = wid; k <= j; k += nw) {
    double t = 0.0;
    for (int l = k + lane; l < j; l += 32) t = fma(cy->T[k + l * kLdT], sres[jp1 + l], t);
    t = warp_sum(t);
    if (lane == 0) {
      stc[k] = k < j ? -2.0 * t : 2.0;
      sg[k] = k < j ? sres[jp1 + k] : 1.0;
    }
  }
  __syncthreads();
  // y = T^T s, as a pair (and in FP64); s kept for the second dot set
  for (int k = wid; k < jp1; k += nw) {
    double t = 0.0;
    for (int l = lane; l <= k; l += 32) t = fma(k < j ? cy->T[l + k * kLdT] : stc[l], sres[l], t);
    t = warp_sum(t);
    if (lane == 0) {
      const float2 d = df_split(t);
      syh[k] = d.x;
      syl[k] = d.y;
      sy[k] = t;
      ss[k] = sres[k];
    }
  }
  if (blockIdx.x == 0) {  // read by the later steps only
    for (int k = threadIdx.x; k < kLdT; k += T) cy->T[k + j * kLdT] = k <= j ? stc[k] : 0.0;
    for (int k = threadIdx.x; k <= j; k += T) {
      cy->G[k + j * kLdT] = sg[k];
      cy->G[j + k * kLdT] = sg[k];
    }
  }
  __syncthreads();
  // ---- pass B: w -= V y (a row pair per thread) and ||w_{j+1:}||^2, in
  // pair arithmetic; rows 0..j+1 of w published for every block
  double nrm;
  {
    float nh = 0.f, nl = 0.f;
    const int p0 = r0 >> 1, p1 = r1 >> 1;
    for (int p = p0 + threadIdx.x; p < p1; p += T) {
      const int i = 2 * p;
      const float4 c = vcomb_df_x2(Vf, Vlo, ldv, i, jp1, syh, syl);
      const float2 s0 = df_add(swd[i - r0], make_float2(-c.x, -c.y));
      const float2 s1 = df_add(swd[i + 1 - r0], make_float2(-c.z, -c.w));
      swd[i - r0] = s0;
      swd[i + 1 - r0] = s1;
      if (i > j) df_mac(s0.x, s0.y, s0.x, s0.y, nh, nl);
      if (i + 1 > j) df_mac(s1.x, s1.y, s1.x, s1.y, nh, nl);
      if (i <= jp1) cy->wtop[i] = df_join(s0);
      if (i + 1 <= jp1) cy->wtop[i + 1] = df_join(s1);
    }
    if ((r1 & 1) && r1 > r0 && threadIdx.x == 0) {  // the last row of an odd n
      const int i = r1 - 1;
      const float2 c = vcomb_df(Vf, Vlo, ldv, i, jp1, syh, syl);
      const float2 s0 = df_add(swd[i - r0], make_float2(-c.x, -c.y));
      swd[i - r0] = s0;
      if (i > j) df_mac(s0.x, s0.y, s0.x, s0.y, nh, nl);
      if (i <= jp1) cy->wtop[i] = df_join(s0);
    }
    nrm = to_f64(nh) + to_f64(nl);
  }
  sbuf[threadIdx.x] = nrm;
  __syncthreads();
  if (wid < 4) {
    const int quarter = T >> 2;
    double t = 0.0;
    for (int k = wid * quarter + lane; k < (wid + 1) * quarter; k += 32) t += sbuf[k];
    t = warp_sum(t);
    if (lane == 0) swarp[wid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) sacc[0] = ((swarp[0] + swarp[1]) + swarp[2]) + swarp[3];
  __syncthreads();
  if (!hh_grid_fold(sacc, 1, a.partials, phase, a.ctrl, sres, kCap)) return;
  const double nrm2 = jp1 < n ? sres[0] : 0.0;
  // V^T w over rows > j after the update, without a pass over V:
  // s - G y over all rows, less the rows <= j that their owners published
  for (int k = wid; k < jp1; k += nw) {
    double t = 0.0;
    for (int l = lane; l < jp1; l += 32) {
      const double gkl = l == j ? sg[k] : (k == j ? sg[l] : cy->G[k + l * kLdT]);
      t = fma(gkl, sy[l], t);
    }
    for (int i = k + lane; i <= j; i += 32) t = fma(a.V[(size_t)k * ldv + i], __ldcg(&cy->wtop[i]), t);
    t = warp_sum(t);
    if (lane == 0) s2[k] = ss[k] - t;
  }
  if (threadIdx.x == 0) {
    const double wn = sqrt(nrm2);
    const double wj1 = jp1 < n ? __ldcg(&cy->wtop[jp1]) : 0.0;
    const double dd = mysgn(wj1) * wn;
    const double alpha = sqrt(2.0 * (nrm2 + fabs(wj1) * wn));
    const double ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
    s_dd = dd;
    s_ia = ia;
    s_vjj = (wj1 + dd) * ia;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < jp1; k += T) {
    const double vk = jp1 < n ? a.V[(size_t)k * ldv + jp1] : 0.0;
    sd[k] = (s2[k] + s_dd * vk) * s_ia;
    srho[k] = vk;
  }
  if (threadIdx.x == 0) srho[jp1] = s_vjj;
  __syncthreads();
  // T's column j+1 (provisional, see above), then c = T_{j+1} rho
  for (int k = wid; k < jp1; k += nw) {
    double t = 0.0;
    for (int l = k + lane; l <= j; l += 32) t = fma(l == j ? stc[k] : cy->T[k + l * kLdT], sd[l], t);
    t = warp_sum(t);
    if (lane == 0) sacc[k] = -2.0 * t;
  }
  if (threadIdx.x == 0) sacc[jp1] = 2.0;
  __syncthreads();
  for (int k = wid; k <= jp1; k += nw) {
    double t = 0.0;
    for (int l = k + lane; l <= j; l += 32) t = fma(l == j ? stc[k] : cy->T[k + l * kLdT], srho[l], t);
    t = warp_sum(t);
    if (lane == 0) {
      t = fma(sacc[k], srho[jp1], t);
      sc[k] = t;
      scf[k] = (float)t;
    }
  }
  __syncthreads();
  if (blockIdx.x == 0) {
    double *Tg = cy->T;
    for (int k = threadIdx.x; k < kLdT; k += T) Tg[k + jp1 * kLdT] = k <= jp1 ? sacc[k] : 0.0;
    for (int k = threadIdx.x; k <= jp1; k += T) cy->c[k] = sc[k];
    if (threadIdx.x == 0) {
      cy->dd = s_dd;
      cy->inv_alpha = s_ia;
    }
  }
  // ---- pass C: v_{j+1} (pairs; FP64 for the top rows the small-matrix
  // work reads; its pairs replace w in shared memory), then q and
  // V_j^T v_{j+1} from one sweep over V
  const double dd = s_dd, ia = s_ia;
  const int ntop = a.m + 2;
  double *vn = a.V + (size_t)jp1 * ldv;
  float *vfn = a.Vf + (size_t)jp1 * ldv, *vln = ad.Vlo + (size_t)jp1 * ldv;
  {
    const float2 iad = df_split(ia);
    const int p0 = r0 >> 1, p1 = r1 >> 1;
    for (int p = p0 + threadIdx.x; p < p1; p += T) {
      const int i = 2 * p;
      const float2 z2 = make_float2(0.f, 0.f);
      const float2 d0 = i > j ? (i == jp1 ? df_split((df_join(swd[i - r0]) + dd) * ia) : df_mul(swd[i - r0], iad)) : z2;
      const float2 d1 =
          i + 1 > j ? (i + 1 == jp1 ? df_split((df_join(swd[i + 1 - r0]) + dd) * ia) : df_mul(swd[i + 1 - r0], iad))
                    : z2;
      if (i < ntop) *reinterpret_cast<double2 *>(vn + i) = make_double2(df_join(d0), df_join(d1));
      *reinterpret_cast<float2 *>(vfn + i) = make_float2(d0.x, d1.x);
      *reinterpret_cast<float2 *>(vln + i) = make_float2(d0.y, d1.y);
      swd[i - r0] = d0;
      swd[i + 1 - r0] = d1;
      prefill_row(a.pf, i);
      prefill_row(a.pf, i + 1);
    }
    if ((r1 & 1) && r1 > r0 && threadIdx.x == 0) {
      const int i = r1 - 1;
      const float2 d = i > j ? (i == jp1 ? df_split((df_join(swd[i - r0]) + dd) * ia) : df_mul(swd[i - r0], iad))
                             : make_float2(0.f, 0.f);
      if (i < ntop) vn[i] = df_join(d);
      vfn[i] = d.x;
      vln[i] = d.y;
      swd[i - r0] = d;
      prefill_row(a.pf, i);
    }
  }
  __syncthreads();
  hh_passC_rows(Vf, Vlo, ldv, jp1, r0, r1, jp1, swd, scf, (float *)a.q, reinterpret_cast<float2 *>(sbuf), sg);
  for (int k = threadIdx.x; k < jp1; k += T) ad.carry[(size_t)k * G + blockIdx.x] = sg[k];
  // ---- the Hessenberg column j (rows 0..j of w, -dd below), its Givens
  // rotation and the convergence test, in the last block (the fewest rows)
  if (blockIdx.x == G - 1) {
    double *sh = sbuf, *scs = sbuf + 256, *ssn = sbuf + 512;
    if (wid == 0) {
      for (int k = lane; k <= j; k += 32) sh[k] = __ldcg(&cy->wtop[k]);
      for (int k = lane; k < j; k += 32) {
        scs[k] = cy->cs[k];
        ssn[k] = cy->sn[k];
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int k = 0; k < j; ++k) {
        const double t0 = sh[k], t1 = sh[k + 1];
        sh[k + 1] = -ssn[k] * t0 + scs[k] * t1;
        sh[k] = scs[k] * t0 + ssn[k] * t1;
      }
      double c, sn;
      givens_rot(sh[j], -dd, 4.9406564584124654e-324, &c, &sn);
      cy->cs[j] = c;
      cy->sn[j] = sn;
      sh[j] = c * sh[j] - sn * dd;
      const double gj = cy->g[j];
      cy->g[jp1] = -sn * gj;
      cy->g[j] = c * gj;
      const double resid = fabs(-sn * gj);
      cy->hist[j] = resid;
      a.ctrl->resid = resid;
      const bool conv = resid < a.ctrl->rtol_abs;
      double *R = cy->R + (size_t)j * kLdT;
      for (int k = 0; k <= j; ++k) R[k] = sh[k];
      if (conv || j == a.m - 1 || !(resid == resid)) {
        a.ctrl->nsteps = jp1;
        a.ctrl->converged = conv ? 1 : 0;
        if (!(resid == resid)) a.ctrl->status |= kStatusBreakdown;
        a.ctrl->done = 1;
      }
    }
  }
}

// ----------------------------------------------- orthogonality monitor
// orth[j+1] = ||I - Q^T Q||_inf over q_0..q_{j} (LACE :628-656 evaluates it on
// the first search+1 stored vectors); Q columns stored by the host driver.
__global__ void k_orthog(int n, const double *__restrict__ Q, size_t ldq, int ncols, double *G) {
  // G[a*ncols+b] = q_a . q_b, one block per (a,b) pair with a <= b
  const int a = blockIdx.x, bcol = blockIdx.y;
  if (a > bcol || bcol >= ncols) return;
  __shared__ double scratch[kTPB / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += kTPB) s = fma(Q[(size_t)a * ldq + i], Q[(size_t)bcol * ldq + i], s);
  double t = block_sum(s, scratch);
  if (threadIdx.x == 0) {
    G[a * ncols + bcol] = t;
    G[bcol * ncols + a] = t;
  }
}
__global__ void k_orthog_norm(const double *G, int ncols, double *out) {
  if (threadIdx.x != 0) return;
  double mx = 0.0;
  for (int i = 0; i < ncols; ++i) {
    double t = 0.0;
    for (int jj = 0; jj < ncols; ++jj) t += fabs((i == jj ? 1.0 : 0.0) - G[i * ncols + jj]);
    if (mx < t) mx = t;
  }
  *out = mx;
}

void launch_orthog_monitor(cudaStream_t s, const ArnoldiArgs &a, int j, double *Q, size_t ldq) {
  const int ncols = j + 1;
  dim3 grid(ncols, ncols);
  k_orthog<<<grid, kTPB, 0, s>>>(a.n, Q, ldq, ncols, a.partials);
  k_orthog_norm<<<1, 32, 0, s>>>(a.partials, ncols, &a.cy->orth[j]);
}

// ------------------------------------------------------------- x update

// x += Z y with y the solution of the small triangular system R y = g
// (LACE :721-744).  Every block solves it redundantly from R and g in L2
// (O(j^2) flops, shared memory), which costs less than one more launch.
constexpr int kPackMax = 64;  // cycles up to this length solve from shared memory
template <typename ZT>
__global__ void __launch_bounds__(kTPB) k_xupdate(int n, const ZT *__restrict__ Z, size_t ldz,
                                                  double *__restrict__ x, Cycle *cy,
                                                  const Control *ctrl) {
  const int ns = ctrl->nsteps;
  if (!ctrl->done || ns == 0) return;
  __shared__ double sy[kLdT];
  __shared__ double sR[kPackMax * (kPackMax + 1) / 2];
  const bool packed = ns <= kPackMax;
  if (packed) {
    // column jj of the upper triangle at offset jj*(jj+1)/2
    for (int jj = 0; jj < ns; ++jj)
      for (int i = threadIdx.x; i <= jj; i += kTPB) sR[jj * (jj + 1) / 2 + i] = cy->R[i + jj * kLdT];
  }
  for (int k = threadIdx.x; k < ns; k += kTPB) sy[k] = cy->g[k];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int jj = ns - 1; jj >= 0; --jj) {
      const double rjj = packed ? sR[jj * (jj + 1) / 2 + jj] : cy->R[jj + jj * kLdT];
      const double yj = sy[jj] / rjj;
      sy[jj] = yj;
      for (int i = 0; i < jj; ++i)
        sy[i] = fma(-(packed ? sR[jj * (jj + 1) / 2 + i] : cy->R[i + jj * kLdT]), yj, sy[i]);
    }
    if (blockIdx.x == 0)
      for (int k = 0; k < ns; ++k) cy->yls[k] = sy[k];
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s0 = x[i], s1 = 0.0, s2 = 0.0, s3 = 0.0;  // LACE :735-744
    int k = 0;
    for (; k + 4 <= ns; k += 4) {
      s0 = fma(to_f64(Z[(size_t)k * ldz + i]), sy[k], s0);
      s1 = fma(to_f64(Z[(size_t)(k + 1) * ldz + i]), sy[k + 1], s1);
      s2 = fma(to_f64(Z[(size_t)(k + 2) * ldz + i]), sy[k + 2], s2);
      s3 = fma(to_f64(Z[(size_t)(k + 3) * ldz + i]), sy[k + 3], s3);
    }
    for (; k < ns; ++k) s0 = fma(to_f64(Z[(size_t)k * ldz + i]), sy[k], s0);
    x[i] = (s0 + s1) + (s2 + s3);
  }
}

// ------------------------------------------------------------ launchers


__global__ void k_sell_values(size_t count, const int *__restrict__ map, const double *__restrict__ src,
                              double *__restrict__ dst, float2 *__restrict__ pair) {
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < count; q += (size_t)gridDim.x * blockDim.x) {
    const int e = map[q];
    const double v = e >= 0 ? src[e] : 0.0;
    dst[q] = v;
    pair[q] = df_split(v);
  }
}

void launch_sell_values(cudaStream_t s, size_t count, const int *map, const double *src, double *dst,
                        float2 *pair) {
  if (count == 0) return;
  const int grid = (int)std::min<size_t>((size_t)num_sms() * 8, (count + 255) / 256);
  k_sell_values<<<grid, 256, 0, s>>>(count, map, src, dst, pair);
}


void launch_cycle_residual(cudaStream_t s, const ArnoldiArgs &a, const double *b, const double *x, bool mgs) {
  OpView op = opview(a);
  const int g = mgs ? 1 : 0;
  switch (a.bs ? 8 : (a.lanes <= 8 ? 1 : a.lanes)) {
    case 1: k_cycle_residual<1><<<a.grid, kTPB, 0, s>>>(a.n, op, b, x, a.w, a.partials, a.cy, a.ctrl, g, a.m); break;
    case 4: k_cycle_residual<4><<<a.grid, kTPB, 0, s>>>(a.n, op, b, x, a.w, a.partials, a.cy, a.ctrl, g, a.m); break;
    case 16: k_cycle_residual<16><<<a.grid, kTPB, 0, s>>>(a.n, op, b, x, a.w, a.partials, a.cy, a.ctrl, g, a.m); break;
    case 32: k_cycle_residual<32><<<a.grid, kTPB, 0, s>>>(a.n, op, b, x, a.w, a.partials, a.cy, a.ctrl, g, a.m); break;
    default: k_cycle_residual<8><<<a.grid, kTPB, 0, s>>>(a.n, op, b, x, a.w, a.partials, a.cy, a.ctrl, g, a.m); break;
  }
}


void launch_cycle_init(cudaStream_t s, const ArnoldiArgs &a) {
  const Prefill pf = prefill_for(a, 0);
  if (a.q_f32)
    k_cycle_init<float><<<rowgrid(a.n), kTPB, 0, s>>>(a.n, a.w, a.V, a.Vf, a.Vlo, (float *)a.q, a.cy, a.ctrl, pf);
  else
    k_cycle_init<double><<<rowgrid(a.n), kTPB, 0, s>>>(a.n, a.w, a.V, nullptr, nullptr, (double *)a.q, a.cy, a.ctrl,
                                                       pf);
}


// dot-product slots per warp for j+1 basis columns
static int slots_for(int jp1) {
  const int need = (jp1 + 7) / 8;
  return need <= 2 ? 2 : (need <= 4 ? 4 : (need <= 8 ? 8 : kSlots));
}

template <typename ZT, int NS>
static void passA_ns(cudaStream_t s, const ArnoldiArgs &a, int j) {
  OpView op = opview(a);
  const ZT *z = (const ZT *)a.Z + (size_t)j * a.ldz;
  switch (a.bs ? 8 : (a.lanes <= 8 ? 1 : a.lanes)) {
    case 1: {
      static const int g = wave_grid(k_passA<1, ZT, NS>, a.grid);
      k_passA<1, ZT, NS><<<g, kTPB, 0, s>>>(a.n, op, z, a.w, a.V, a.ldv, j + 1, a.partials, a.cy, a.ctrl);
      break;
    }
    case 16: k_passA<16, ZT, NS><<<a.grid, kTPB, 0, s>>>(a.n, op, z, a.w, a.V, a.ldv, j + 1, a.partials, a.cy, a.ctrl); break;
    case 32: k_passA<32, ZT, NS><<<a.grid, kTPB, 0, s>>>(a.n, op, z, a.w, a.V, a.ldv, j + 1, a.partials, a.cy, a.ctrl); break;
    default: k_passA<8, ZT, NS><<<a.grid, kTPB, 0, s>>>(a.n, op, z, a.w, a.V, a.ldv, j + 1, a.partials, a.cy, a.ctrl); break;
  }
}

template <typename ZT>
static void passA_t(cudaStream_t s, const ArnoldiArgs &a, int j) {
  switch (slots_for(j + 1)) {
    case 2: passA_ns<ZT, 2>(s, a, j); break;
    case 4: passA_ns<ZT, 4>(s, a, j); break;
    case 8: passA_ns<ZT, 8>(s, a, j); break;
    default: passA_ns<ZT, kSlots>(s, a, j); break;
  }
}

void launch_passA(cudaStream_t s, const ArnoldiArgs &a, int j) {
  if (a.z_f32) passA_t<float>(s, a, j);
  else passA_t<double>(s, a, j);
}

template <int NS>
static void passB_ns(cudaStream_t s, const ArnoldiArgs &a, int j) {
  static const int g = wave_grid(k_passB<NS>, a.grid);
  k_passB<NS><<<g, kTPB, 0, s>>>(a.n, a.V, a.ldv, j, a.m, a.w, a.partials, a.cy, a.ctrl);
}

void launch_passB(cudaStream_t s, const ArnoldiArgs &a, int j) {
  switch (slots_for(j + 1)) {
    case 2: passB_ns<2>(s, a, j); break;
    case 4: passB_ns<4>(s, a, j); break;
    case 8: passB_ns<8>(s, a, j); break;
    default: passB_ns<kSlots>(s, a, j); break;
  }
}

void launch_passC(cudaStream_t s, const ArnoldiArgs &a, int j) {
  const Prefill pf = prefill_for(a, j + 1);  // for the next step's solves
  if (a.q_f32) {
    static const int g = wave_grid(k_passC<float>, num_sms() * 8);
    k_passC<float><<<std::min(g, rowgrid(a.n)), kTPB, 0, s>>>(a.n, a.V, a.Vf, a.Vlo, a.ldv, j, a.w, (float *)a.q,
                                                                a.cy, a.ctrl, pf);
  } else {
    static const int g = wave_grid(k_passC<double>, num_sms() * 8);
    k_passC<double><<<std::min(g, rowgrid(a.n)), kTPB, 0, s>>>(a.n, a.V, nullptr, nullptr, a.ldv, j, a.w,
                                                                  (double *)a.q, a.cy, a.ctrl, pf);
  }
}

template <typename ZT, typename QT>
static int hh_step_t(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t, void *mark_z) {
  // one block per SM when the kernel fits there with the largest shared
  // memory (0: it does not); set once, thread-safely
  static const int G = [] {
    int per_sm = 0;
    if (cudaFuncSetAttribute(k_hh_step<ZT, QT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kHHSmemMax) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hh_step<ZT, QT>, kHHTPB, kHHSmemMax) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      return 0;
    }
    return num_sms();
  }();
  if (G == 0) return 1;
  HHStep p;
  p.n = a.n;
  p.rb = ((a.n + G - 1) / G + 31) / 32 * 32;
  if ((size_t)p.rb * 8 > (size_t)kHHSmemMax || (size_t)G * kLdT * 2 > (size_t)a.grid * kLdT) return 1;
  p.op = opview(a);
  p.z = (const char *)a.Z + (size_t)j * a.ldz * sizeof(ZT);
  p.V = a.V;
  p.Vf = a.Vf;
  p.ldv = a.ldv;
  p.q = a.q;
  p.partials = a.partials;
  p.cy = a.cy;
  p.ctrl = a.ctrl;
  p.m = a.m;
  p.pf = prefill_for(a, j + 1);
  if (mark_t && p.pf.t) {
    p.pf.t = mark_t;
    p.pf.z = mark_z;
  }
  void *args[] = {&p, &j};
  if (cudaLaunchCooperativeKernel((const void *)k_hh_step<ZT, QT>, dim3(G), dim3(kHHTPB), args,
                                  (size_t)p.rb * 8, s) != cudaSuccess) {
    cudaGetLastError();
    return 2;
  }
  return 0;
}

static int hh_step_df(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t, void *mark_z) {
  static const int G = [] {
    int per_sm = 0;
    if (cudaFuncSetAttribute(k_hh_step_df, cudaFuncAttributeMaxDynamicSharedMemorySize, kHHSmemMax) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_hh_step_df, kHHTPB, kHHSmemMax) != cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      return 0;
    }
    return num_sms();
  }();
  if (G == 0) return 1;
  HHStepDF pd;
  HHStep &p = pd.base;
  p.n = a.n;
  p.rb = ((a.n + G - 1) / G + 31) / 32 * 32;
  // two phases of 2 kLdT fold values per block, then the carried partials,
  // in the partials buffer
  if ((size_t)p.rb * 8 > (size_t)kHHSmemMax || (size_t)G * kLdT * 5 > (size_t)a.grid * kLdT) return 1;
  p.op = opview(a);
  p.z = (const char *)a.Z + (size_t)j * a.ldz * sizeof(float);
  p.V = a.V;
  p.Vf = a.Vf;
  p.ldv = a.ldv;
  p.q = a.q;
  p.partials = a.partials;
  p.cy = a.cy;
  p.ctrl = a.ctrl;
  p.m = a.m;
  p.pf = prefill_for(a, j + 1);
  if (mark_t && p.pf.t) {
    p.pf.t = mark_t;
    p.pf.z = mark_z;
  }
  pd.Vlo = a.Vlo;
  pd.carry = a.partials + (size_t)4 * kLdT * G;
  pd.sell_pair = a.sell_pair;
  void *args[] = {&pd, &j};
  if (cudaLaunchCooperativeKernel((const void *)k_hh_step_df, dim3(G), dim3(kHHTPB), args, (size_t)p.rb * 8, s) !=
      cudaSuccess) {
    cudaGetLastError();
    return 2;
  }
  return 0;
}

int launch_hh_step(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t, void *mark_z) {
  if (a.bs || !a.sell_ptr) return 1;
  if (a.z_f32 && a.q_f32 && a.Vf && a.Vlo && a.sell_pair) return hh_step_df(s, a, j, mark_t, mark_z);
  if (a.z_f32 && a.q_f32 && a.Vf) return hh_step_t<float, float>(s, a, j, mark_t, mark_z);
  if (!a.z_f32 && !a.q_f32) return hh_step_t<double, double>(s, a, j, mark_t, mark_z);
  return 1;
}

void launch_xupdate(cudaStream_t s, const ArnoldiArgs &a, double *x) {
  if (a.z_f32)
    k_xupdate<float><<<rowgrid(a.n), kTPB, 0, s>>>(a.n, (const float *)a.Z, a.ldz, x, a.cy, a.ctrl);
  else
    k_xupdate<double><<<rowgrid(a.n), kTPB, 0, s>>>(a.n, (const double *)a.Z, a.ldz, x, a.cy, a.ctrl);
}

int num_sms() {
  // the first device's count, set once (thread-safe static initialisation)
  static const int sms = [] {
    int dev = 0, v = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
    return v > 0 ? v : 132;
  }();
  return sms;
}

}  // namespace lace
