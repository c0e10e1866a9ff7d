// FGMRES with modified Gram-Schmidt Arnoldi: LACE's data_fgmres_restart
// (src/fgmres_restart.cpp:63-532) and data_fgmres (src/fgmres.cpp:64-517).
//
// Modified Gram-Schmidt is sequential in the basis index: the coefficient of
// v_k is taken from u after v_0..v_{k-1} were removed, so step j needs j+2
// grid-wide sums one after another.  Two forms of the step after the solves:
//   k_mgs_step (default): one cooperative kernel, one block per SM keeping
//     its rows of u in shared memory; each sum is a block sum, a grid barrier
//     and a fold every block performs in the same order; the second pass
//     (LACE :336-360) and the rotations run in the same kernel;
//   one kernel per sum (BCSR operators, u too large for shared memory), each
//     fusing the previous subtraction with the next dot product in one pass
//     over u, the second pass in a conditional graph node that the first
//     pass's norm kernel switches on.
// The scalars (coefficients, Brown/Hindmarsh test, Givens rotations,
// convergence) stay in device memory, so a cycle runs from a CUDA graph
// without host round trips, and every kernel returns at once once
// Control::done is set.
#include <float.h>
#include <math.h>

#include "krylov_tile.cuh"

namespace lace {

// two block sums at once (a, b valid in thread 0)
__device__ __forceinline__ void block_sum2(double &a, double &b, double *scratch) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  a = warp_sum(a);
  b = warp_sum(b);
  __syncthreads();
  if (lane == 0) {
    scratch[wid] = a;
    scratch[kTPB / 32 + wid] = b;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double s0 = 0.0, s1 = 0.0;
    for (int w = 0; w < kTPB / 32; ++w) {
      s0 += scratch[w];
      s1 += scratch[kTPB / 32 + w];
    }
    a = s0;
    b = s1;
  }
}

// the last block's sum of partials[b * kLdT + k] over the blocks, in fixed
// order (valid in thread 0; every thread calls it)
__device__ __forceinline__ double fold_one(const double *partials, int k) {
  return block_fold(partials + k, kLdT, (int)gridDim.x);
}

// ------------------------------------------------------------ cycle start

// v_0 = r / ||r|| (:211-218), and the first step's solve outputs marked
// unsolved
__global__ void __launch_bounds__(kTPB) k_mgs_cycle_init(int n, const double *__restrict__ r,
                                                         double *__restrict__ V, const Cycle *cy,
                                                         const Control *ctrl, Prefill pf) {
  if (ctrl->done) return;
  const double inv = cy->hinv;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    V[i] = r[i] * inv;
    prefill_row(pf, i);
  }
}

// --------------------------------------------------------------- operator

// u = A z_j (:284-290), ||u|| (:291) and h_0 = v_0 . u, the first
// Gram-Schmidt coefficient (:305-313)
template <int LPR, typename ZT>
__global__ void __launch_bounds__(kTPB) k_mgs_operator(int n, OpView op, const ZT *__restrict__ z,
                                                       double *__restrict__ u, const double *__restrict__ v0,
                                                       double *partials, Cycle *cy, Control *ctrl) {
  if (ctrl->done) return;
  __shared__ double swb[2][kTPB];
  __shared__ double scratch[2 * kTPB / 32];
  int buf = 0;
  const int tr = (op.bs == 0) ? kTPB : (kTPB / op.bs) * op.bs;
  double nrm = 0.0, dot = 0.0;
  for (int base = blockIdx.x * tr; base < n; base += gridDim.x * tr, buf ^= 1) {
    double *sw = swb[buf];
    tile_apply<LPR, ZT>(op, n, base, tr, z, sw);
    __syncthreads();
    for (int t = threadIdx.x; t < tr; t += kTPB) {
      const int i = base + t;
      if (i < n) {
        const double ui = sw[t];
        u[i] = ui;
        nrm = fma(ui, ui, nrm);
        dot = fma(v0[i], ui, dot);
      }
    }
  }
  block_sum2(nrm, dot, scratch);
  if (threadIdx.x == 0) {
    partials[(size_t)blockIdx.x * kLdT] = nrm;
    partials[(size_t)blockIdx.x * kLdT + 1] = dot;
  }
  if (!arrive_last(&ctrl->block_count[1])) return;
  const double snrm = fold_one(partials, 0), sdot = fold_one(partials, 1);
  if (threadIdx.x == 0) {
    cy->normav = sqrt(snrm);
    cy->h[0] = sdot;
  }
}

// ------------------------------------------------------------------ sweep

// u -= c_{k-1} v_{k-1} (k > 0), then the dot product v_k . u; pass 0:
// h_k = it (:305-328); pass 1, the second Gram-Schmidt pass: hr_k = it and
// h_k += it (:339-359).  Row pairs per thread, 16-byte loads.
__global__ void __launch_bounds__(kTPB) k_mgs_sweep(int n, const double *__restrict__ V, size_t ldv, int k,
                                                    double *__restrict__ u, int pass, double *partials,
                                                    Cycle *cy, Control *ctrl) {
  if (ctrl->done || (pass && !cy->reorth)) return;
  __shared__ double scratch[kTPB / 32];
  const double c = k > 0 ? (pass ? cy->hr[k - 1] : cy->h[k - 1]) : 0.0;
  const double *vp = V + (size_t)(k > 0 ? k - 1 : 0) * ldv;
  const double *vk = V + (size_t)k * ldv;
  double dot = 0.0;
  const int npair = n / 2;
  // a few row pairs per thread: unrolled so that their loads are in flight together
#pragma unroll 4
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += gridDim.x * blockDim.x) {
    const int i = 2 * p;
    double2 uu = *reinterpret_cast<const double2 *>(u + i);
    if (k > 0) {
      const double2 a = __ldg(reinterpret_cast<const double2 *>(vp + i));
      uu.x = fma(-c, a.x, uu.x);
      uu.y = fma(-c, a.y, uu.y);
      *reinterpret_cast<double2 *>(u + i) = uu;
    }
    const double2 b = __ldg(reinterpret_cast<const double2 *>(vk + i));
    dot = fma(b.x, uu.x, dot);
    dot = fma(b.y, uu.y, dot);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int i = n - 1;
    double ui = u[i];
    if (k > 0) {
      ui = fma(-c, vp[i], ui);
      u[i] = ui;
    }
    dot = fma(vk[i], ui, dot);
  }
  const double tot = block_sum(dot, scratch);
  if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kLdT] = tot;
  if (!arrive_last(&ctrl->block_count[2])) return;
  const double s = fold_one(partials, 0);
  if (threadIdx.x == 0) {
    if (pass) {
      cy->hr[k] = s;
      cy->h[k] += s;
    } else {
      cy->h[k] = s;
    }
  }
}

// ------------------------------------------------------------------- norm

// rotations and the convergence test of step j (:362-459), thread 0 of the
// last block; h_{j+1} is in cy->h[j+1]
__device__ void mgs_finish(int j, int m, int restarted, Cycle *cy, Control *ctrl) {
  const double hj1 = cy->h[j + 1];
  // happy breakdown (:363; fgmres.cpp:341): v_{j+1} stays zero
  const double brk = restarted ? 0.0 : DBL_EPSILON;
  cy->hinv = fabs(hj1) > brk ? 1.0 / hj1 : 0.0;
  double *R = cy->R + (size_t)j * kLdT;
  for (int k = 0; k <= j + 1; ++k) R[k] = cy->h[k];
  for (int k = 0; k < j; ++k) {  // :406-415
    const double delta = R[k];
    R[k] = cy->cs[k] * delta - cy->sn[k] * R[k + 1];
    R[k + 1] = cy->sn[k] * delta + cy->cs[k] * R[k + 1];
  }
  const double gamma = sqrt(R[j] * R[j] + R[j + 1] * R[j + 1]);  // :417-420
  if (gamma > 0.0) {                                               // :421-432
    const double c = R[j] / gamma, s = -R[j + 1] / gamma;
    cy->cs[j] = c;
    cy->sn[j] = s;
    R[j] = c * R[j] - s * R[j + 1];
    R[j + 1] = 0.0;
    const double delta = cy->g[j];
    cy->g[j] = c * delta - s * cy->g[j + 1];
    cy->g[j + 1] = s * delta + c * cy->g[j + 1];
  }
  const double gj1 = cy->g[j + 1];
  const double resid = fabs(gj1);
  cy->hist[j] = resid;
  ctrl->resid = resid;
  const bool conv = resid < ctrl->rtol_abs;
  const bool finite = isfinite(gj1);
  // :459 (fgmres.cpp:440 also stops on a non-finite residual; so does the
  // restarted variant here rather than running every remaining direction on
  // NaN values)
  if (conv || j == m - 1 || !finite) {
    ctrl->nsteps = j + 1;
    ctrl->converged = conv ? 1 : 0;
    if (!finite) ctrl->status |= kStatusBreakdown;
    ctrl->done = 1;
  }
}

// u -= c_j v_j, h_{j+1} = ||u|| (:329-333).  Pass 0: the Brown/Hindmarsh
// test (:336-338) decides the second pass (cond set to 1, the rotations
// wait for it); otherwise, and after pass 1 (:360), the rotations and the
// convergence test.
__global__ void __launch_bounds__(kTPB) k_mgs_norm(int n, const double *__restrict__ V, size_t ldv, int j,
                                                   double *__restrict__ u, int pass, int m, int restarted,
                                                   int reorth, cudaGraphConditionalHandle cond, int has_cond,
                                                   double *partials, Cycle *cy, Control *ctrl) {
  if (ctrl->done || (pass && !cy->reorth)) return;
  __shared__ double scratch[kTPB / 32];
  const double c = pass ? cy->hr[j] : cy->h[j];
  const double *vj = V + (size_t)j * ldv;
  double nrm = 0.0;
  const int npair = n / 2;
#pragma unroll 4
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += gridDim.x * blockDim.x) {
    const int i = 2 * p;
    double2 uu = *reinterpret_cast<const double2 *>(u + i);
    const double2 a = __ldg(reinterpret_cast<const double2 *>(vj + i));
    uu.x = fma(-c, a.x, uu.x);
    uu.y = fma(-c, a.y, uu.y);
    *reinterpret_cast<double2 *>(u + i) = uu;
    nrm = fma(uu.x, uu.x, nrm);
    nrm = fma(uu.y, uu.y, nrm);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int i = n - 1;
    const double ui = fma(-c, vj[i], u[i]);
    u[i] = ui;
    nrm = fma(ui, ui, nrm);
  }
  const double tot = block_sum(nrm, scratch);
  if (threadIdx.x == 0) partials[(size_t)blockIdx.x * kLdT] = tot;
  if (!arrive_last(&ctrl->block_count[2])) return;
  const double s = fold_one(partials, 0);
  if (threadIdx.x != 0) return;
  const double hn = sqrt(s);
  cy->h[j + 1] = hn;
  if (!pass) {
    const double normav = cy->normav;
    const double hr = (normav + 0.001 * hn) - normav;
    const int again = ((reorth == 0 && hr <= 4.9406564584124654e-324) || reorth == 2) ? 1 : 0;
    cy->reorth = again;
    cy->nreorth += again;
    if (has_cond) cudaGraphSetConditional(cond, again);
    if (again) return;
  }
  mgs_finish(j, m, restarted, cy, ctrl);
}

// ------------------------------------------------------------------- next

// v_{j+1} = u / h_{j+1} (zero after a breakdown, :363-378), and the next
// step's solve outputs marked unsolved
__global__ void __launch_bounds__(kTPB) k_mgs_next(int n, double *__restrict__ vn, const double *__restrict__ u,
                                                   const Cycle *cy, const Control *ctrl, Prefill pf) {
  if (ctrl->done) return;
  const double inv = cy->hinv;
  const int npair = n / 2;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npair; p += gridDim.x * blockDim.x) {
    const int i = 2 * p;
    const double2 uu = *reinterpret_cast<const double2 *>(u + i);
    *reinterpret_cast<double2 *>(vn + i) = make_double2(inv == 0.0 ? 0.0 : uu.x * inv, inv == 0.0 ? 0.0 : uu.y * inv);
    prefill_row(pf, i);
    prefill_row(pf, i + 1);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) {
    const int i = n - 1;
    vn[i] = inv == 0.0 ? 0.0 : u[i] * inv;
    prefill_row(pf, i);
  }
}

// --------------------------------------------------------------- x update

// the least-squares solve as LACE writes it (:461-469: a_i = g_i / R_ii,
// then a_i -= R_ij a_j / R_ii for j = ns-1..1, i < j), redundantly in every
// block, then x += sum_j z_j a_j: column by column (restarted, :472-481)
// or summed first and added once (fgmres.cpp:453-474)
template <typename ZT>
__global__ void __launch_bounds__(kTPB) k_mgs_xupdate(int n, const ZT *__restrict__ Z, size_t ldz,
                                                      double *__restrict__ x, Cycle *cy, const Control *ctrl,
                                                      int restarted) {
  const int ns = ctrl->nsteps;
  if (!ctrl->done || ns == 0) return;
  __shared__ double sa[kLdT];
  if (threadIdx.x == 0) {
    const double *R = cy->R;
    for (int i = 0; i < ns; ++i) sa[i] = cy->g[i] / R[i + (size_t)i * kLdT];
    for (int j = ns - 1; j > 0; --j)
      for (int i = j - 1; i >= 0; --i)
        sa[i] = sa[i] - R[i + (size_t)j * kLdT] * sa[j] / R[i + (size_t)i * kLdT];
    if (blockIdx.x == 0)
      for (int k = 0; k < ns; ++k) cy->yls[k] = sa[k];
  }
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (restarted) {
      double s = x[i];
      for (int k = 0; k < ns; ++k) s = fma(to_f64(Z[(size_t)k * ldz + i]), sa[k], s);
      x[i] = s;
    } else {
      double s = 0.0;
      for (int k = 0; k < ns; ++k) s = fma(to_f64(Z[(size_t)k * ldz + i]), sa[k], s);
      x[i] = x[i] + s;
    }
  }
}

// ------------------------------------------ one persistent kernel per step

// The whole Arnoldi step after the solves (operator, both Gram-Schmidt
// passes, rotations, the next basis vector) in one cooperative launch of
// one block per SM: block b keeps rows [b*RB, (b+1)*RB) of u in shared
// memory, and each Gram-Schmidt sum is a block sum, a grid barrier and a
// fold of the blocks' partial sums that every block performs in the same
// order, so every block holds the same coefficient.  u never leaves the SM;
// a sum costs one barrier instead of a kernel boundary.
constexpr int kStepTPB = 1024;
constexpr int kStepSmemMax = 200 * 1024;  // rows of u per block: at most 25,600 (plus 16 KB static)

// v[q] summed over the grid, the same value in every block.  FP64 adds are
// this part's scarce resource, so both reductions stage the values in
// shared memory and let few warps add them (a butterfly in every warp would
// cost five FP64 adds per warp): the block's threads' values are summed by
// four warps (one per SM sub-partition) and the four results in order; after
// the barrier one warp folds the grid's partial sums.  Fixed orders: every
// block computes the same value.  partials: 4 x gridDim.x doubles, two
// phases so that a block may run ahead into the next sum while others still
// fold this one.  sbuf: NV x blockDim.x doubles; sred: 8 * NV + NV doubles.
template <int NV>
__device__ __forceinline__ bool grid_sum(double (&v)[NV], double *partials, int &phase, Control *ctrl,
                                         double *sbuf, double *sred) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int T = blockDim.x, G = gridDim.x;
#pragma unroll
  for (int q = 0; q < NV; ++q) sbuf[q * T + threadIdx.x] = v[q];
  __syncthreads();
  if (wid < 4) {
    const int quarter = T >> 2;
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double t = 0.0;
      for (int k = wid * quarter + lane; k < (wid + 1) * quarter; k += 32) t += sbuf[q * T + k];
      t = warp_sum(t);
      if (lane == 0) sred[q * 8 + wid] = t;
    }
  }
  __syncthreads();
  if (threadIdx.x < NV)
    partials[(size_t)(phase * 2 + threadIdx.x) * G + blockIdx.x] =
        ((sred[threadIdx.x * 8] + sred[threadIdx.x * 8 + 1]) + sred[threadIdx.x * 8 + 2]) + sred[threadIdx.x * 8 + 3];
  if (!grid_barrier(ctrl)) return false;
  if (wid == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double t = 0.0;
      for (int b = lane; b < G; b += 32) t += __ldcg(partials + (size_t)(phase * 2 + q) * G + b);
      t = warp_sum(t);
      if (lane == 0) sred[8 * NV + q] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = sred[8 * NV + q];
  __syncthreads();
  phase ^= 1;
  return true;
}

struct MgsStep {
  int n, rb;  // rows; rows of u per block (a multiple of 32)
  OpView op;  // sliced ELL
  const void *z;
  double *V;
  size_t ldv;
  double *partials;
  Cycle *cy;
  Control *ctrl;
  int m, restarted, reorth;
  Prefill pf;
};

template <typename ZT>
__global__ void __launch_bounds__(kStepTPB, 1) k_mgs_step(MgsStep a, int j) {
  if (a.ctrl->done) return;
  extern __shared__ double su[];
  __shared__ double sbuf[2 * kStepTPB];
  __shared__ double sred[8 * 2 + 2];
  __shared__ double sh[kLdT + 1];
  const int r0 = blockIdx.x * a.rb, r1 = min(a.n, r0 + a.rb);
  const int T = blockDim.x;
  const ZT *z = (const ZT *)a.z;
  int phase = 0;
  // u = A z_j for this block's rows (a warp per 32-row slice), ||u||^2, v_0 . u
  double acc[2] = {0.0, 0.0};
  {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = T >> 5;
    for (int sl = (r0 >> 5) + wid; 32 * sl < r1; sl += nw) {
      const int i = 32 * sl + lane;
      double s = 0.0;
      if (i < r1) {
        const int len = a.op.row[i + 1] - a.op.row[i];
        const int *cp = a.op.sell_col + a.op.sell_ptr[sl] + lane;
        const double *vp = a.op.sell_val + (cp - a.op.sell_col);
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
        su[i - r0] = s;
        acc[0] = fma(s, s, acc[0]);
        acc[1] = fma(a.V[i], s, acc[1]);
      }
    }
  }
  if (!grid_sum<2>(acc, a.partials, phase, a.ctrl, sbuf, sred)) return;
  const double normav = sqrt(acc[0]);
  if (threadIdx.x == 0) sh[0] = acc[1];
  __syncthreads();
  // Gram-Schmidt passes: sums k = 1..j+1 (the last one the norm); pass 1
  // (the second pass) only when the Brown/Hindmarsh test asks
  double hn = 0.0;
  int again = 0;
  // the vector loops walk row pairs (16-byte loads, four pairs per thread in
  // flight: one 8-byte load per thread would keep too few bytes in flight to
  // stream from HBM); an odd last row is thread 0's
  const int p0 = r0 >> 1, p1 = r1 >> 1;
  const bool tail = (r1 & 1) && r1 > r0 && threadIdx.x == 0;
  double2 *su2 = reinterpret_cast<double2 *>(su);
  for (int pass = 0; pass < 2; ++pass) {
    double c = sh[0];
    if (pass) {
      // hr_0 = v_0 . u before any subtraction of the second pass
      double d[1] = {0.0};
      const double2 *v2 = reinterpret_cast<const double2 *>(a.V);
#pragma unroll 4
      for (int p = p0 + threadIdx.x; p < p1; p += T) {
        const double2 v = __ldg(v2 + p), u = su2[p - p0];
        d[0] = fma(v.x, u.x, d[0]);
        d[0] = fma(v.y, u.y, d[0]);
      }
      if (tail) d[0] = fma(a.V[r1 - 1], su[r1 - 1 - r0], d[0]);
      if (!grid_sum<1>(d, a.partials, phase, a.ctrl, sbuf, sred)) return;
      c = d[0];
      if (threadIdx.x == 0) sh[0] += c;
    }
    for (int k = 1; k <= j + 1; ++k) {
      const double *vp = a.V + (size_t)(k - 1) * a.ldv;
      const double *vk = a.V + (size_t)k * a.ldv;
      const double2 *vp2 = reinterpret_cast<const double2 *>(vp);
      const double2 *vk2 = reinterpret_cast<const double2 *>(vk);
      double d[1] = {0.0};
      if (k <= j) {
#pragma unroll 4
        for (int p = p0 + threadIdx.x; p < p1; p += T) {
          const double2 v = __ldg(vp2 + p), w = __ldg(vk2 + p);
          double2 u = su2[p - p0];
          u.x = fma(-c, v.x, u.x);
          u.y = fma(-c, v.y, u.y);
          su2[p - p0] = u;
          d[0] = fma(w.x, u.x, d[0]);
          d[0] = fma(w.y, u.y, d[0]);
        }
        if (tail) {
          const double ui = fma(-c, vp[r1 - 1], su[r1 - 1 - r0]);
          su[r1 - 1 - r0] = ui;
          d[0] = fma(vk[r1 - 1], ui, d[0]);
        }
      } else {
#pragma unroll 4
        for (int p = p0 + threadIdx.x; p < p1; p += T) {
          const double2 v = __ldg(vp2 + p);
          double2 u = su2[p - p0];
          u.x = fma(-c, v.x, u.x);
          u.y = fma(-c, v.y, u.y);
          su2[p - p0] = u;
          d[0] = fma(u.x, u.x, d[0]);
          d[0] = fma(u.y, u.y, d[0]);
        }
        if (tail) {
          const double ui = fma(-c, vp[r1 - 1], su[r1 - 1 - r0]);
          su[r1 - 1 - r0] = ui;
          d[0] = fma(ui, ui, d[0]);
        }
      }
      if (!grid_sum<1>(d, a.partials, phase, a.ctrl, sbuf, sred)) return;
      if (k <= j) {
        c = d[0];
        if (threadIdx.x == 0) sh[k] = pass ? sh[k] + c : c;
      } else {
        hn = sqrt(d[0]);
      }
      __syncthreads();
    }
    if (pass) break;
    const double hr = (normav + 0.001 * hn) - normav;  // :336-338
    again = ((a.reorth == 0 && hr <= 4.9406564584124654e-324) || a.reorth == 2) ? 1 : 0;
    if (!again) break;
  }
  // block 0: the column, the rotations and the convergence test
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    Cycle *cy = a.cy;
    for (int k = 0; k <= j; ++k) cy->h[k] = sh[k];
    cy->h[j + 1] = hn;
    cy->normav = normav;
    cy->reorth = again;
    cy->nreorth += again;
    mgs_finish(j, a.m, a.restarted, cy, a.ctrl);
  }
  // v_{j+1} = u / h_{j+1} (zero after a breakdown), the next solves' outputs marked
  const double brk = a.restarted ? 0.0 : DBL_EPSILON;
  const double inv = fabs(hn) > brk ? 1.0 / hn : 0.0;
  double *vn = a.V + (size_t)(j + 1) * a.ldv;
  double2 *vn2 = reinterpret_cast<double2 *>(vn);
#pragma unroll 4
  for (int p = p0 + threadIdx.x; p < p1; p += T) {
    const double2 u = su2[p - p0];
    vn2[p] = inv == 0.0 ? make_double2(0.0, 0.0) : make_double2(u.x * inv, u.y * inv);
    prefill_row(a.pf, 2 * p);
    prefill_row(a.pf, 2 * p + 1);
  }
  if (tail) {
    vn[r1 - 1] = inv == 0.0 ? 0.0 : su[r1 - 1 - r0] * inv;
    prefill_row(a.pf, r1 - 1);
  }
}

// -------------------------------------------------------------- launchers

template <typename ZT>
static int mgs_step_t(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t, void *mark_z) {
  // one block per SM when the kernel fits there with the largest shared
  // memory (0: it does not); set once, thread-safely
  static const int G = [] {
    int per_sm = 0;
    if (cudaFuncSetAttribute(k_mgs_step<ZT>, cudaFuncAttributeMaxDynamicSharedMemorySize, kStepSmemMax) !=
            cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_mgs_step<ZT>, kStepTPB, kStepSmemMax) !=
            cudaSuccess ||
        per_sm < 1) {
      cudaGetLastError();
      return 0;
    }
    return num_sms();
  }();
  if (G == 0) return 1;
  MgsStep p;
  p.n = a.n;
  p.rb = ((a.n + G - 1) / G + 31) / 32 * 32;
  if ((size_t)p.rb * 8 > (size_t)kStepSmemMax) return 1;
  p.op = opview(a);
  p.z = (const char *)a.Z + (size_t)j * a.ldz * sizeof(ZT);
  p.V = a.V;
  p.ldv = a.ldv;
  p.partials = a.partials;
  p.cy = a.cy;
  p.ctrl = a.ctrl;
  p.m = a.m;
  p.restarted = a.mgs_restarted;
  p.reorth = a.mgs_reorth;
  p.pf = prefill_for(a, j + 1);
  if (mark_t && p.pf.t) {
    p.pf.t = mark_t;
    p.pf.z = mark_z;
  }
  void *args[] = {&p, &j};
  if (cudaLaunchCooperativeKernel((const void *)k_mgs_step<ZT>, dim3(G), dim3(kStepTPB), args,
                                  (size_t)p.rb * 8, s) != cudaSuccess) {
    cudaGetLastError();
    return 2;
  }
  return 0;
}

int launch_mgs_step(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t, void *mark_z) {
  if (a.bs || !a.sell_ptr) return 1;
  return a.z_f32 ? mgs_step_t<float>(s, a, j, mark_t, mark_z) : mgs_step_t<double>(s, a, j, mark_t, mark_z);
}

void launch_mgs_cycle_init(cudaStream_t s, const ArnoldiArgs &a) {
  k_mgs_cycle_init<<<rowgrid(a.n), kTPB, 0, s>>>(a.n, a.w, a.V, a.cy, a.ctrl, prefill_for(a, 0));
}

template <int LPR, typename ZT>
static void mgs_operator_t(cudaStream_t s, const ArnoldiArgs &a, const ZT *z) {
  static const int g = wave_grid(k_mgs_operator<LPR, ZT>, a.grid);
  k_mgs_operator<LPR, ZT><<<g, kTPB, 0, s>>>(a.n, opview(a), z, a.w, a.V, a.partials, a.cy, a.ctrl);
}

template <typename ZT>
static void mgs_operator_z(cudaStream_t s, const ArnoldiArgs &a, int j) {
  const ZT *z = (const ZT *)a.Z + (size_t)j * a.ldz;
  switch (a.bs ? 8 : (a.lanes <= 8 ? 1 : a.lanes)) {
    case 1: mgs_operator_t<1, ZT>(s, a, z); break;
    case 16: mgs_operator_t<16, ZT>(s, a, z); break;
    case 32: mgs_operator_t<32, ZT>(s, a, z); break;
    default: mgs_operator_t<8, ZT>(s, a, z); break;
  }
}

void launch_mgs_operator(cudaStream_t s, const ArnoldiArgs &a, int j) {
  if (a.z_f32) mgs_operator_z<float>(s, a, j);
  else mgs_operator_z<double>(s, a, j);
}

void launch_mgs_sweep(cudaStream_t s, const ArnoldiArgs &a, int j, int k, int pass) {
  (void)j;  // the sweep depends on k only
  static const int g = wave_grid(k_mgs_sweep, a.grid);
  k_mgs_sweep<<<std::min(g, rowgrid(a.n)), kTPB, 0, s>>>(a.n, a.V, a.ldv, k, a.w, pass, a.partials, a.cy,
                                                          a.ctrl);
}

void launch_mgs_norm(cudaStream_t s, const ArnoldiArgs &a, int j, int pass, unsigned long long cond) {
  static const int g = wave_grid(k_mgs_norm, a.grid);
  k_mgs_norm<<<std::min(g, rowgrid(a.n)), kTPB, 0, s>>>(a.n, a.V, a.ldv, j, a.w, pass, a.m, a.mgs_restarted,
                                                         a.mgs_reorth, (cudaGraphConditionalHandle)cond,
                                                         cond != 0, a.partials, a.cy, a.ctrl);
}

void launch_mgs_next(cudaStream_t s, const ArnoldiArgs &a, int j) {
  static const int g = wave_grid(k_mgs_next, num_sms() * 8);
  k_mgs_next<<<std::min(g, rowgrid(a.n)), kTPB, 0, s>>>(a.n, a.V + (size_t)(j + 1) * a.ldv, a.w, a.cy, a.ctrl,
                                                         prefill_for(a, j + 1));
}

void launch_mgs_xupdate(cudaStream_t s, const ArnoldiArgs &a, double *x) {
  if (a.z_f32)
    k_mgs_xupdate<float><<<rowgrid(a.n), kTPB, 0, s>>>(a.n, (const float *)a.Z, a.ldz, x, a.cy, a.ctrl,
                                                        a.mgs_restarted);
  else
    k_mgs_xupdate<double><<<rowgrid(a.n), kTPB, 0, s>>>(a.n, (const double *)a.Z, a.ldz, x, a.cy, a.ctrl,
                                                         a.mgs_restarted);
}

}  // namespace lace
