// Batched solves as one persistent launch: every CTA takes systems from a
// queue (largest first) and carries each through ParILU(0) and FGMRES-
// Householder for all of its right-hand sides (four in lockstep) on its own,
// with CTA barriers only - no grid barrier, no wait on another CTA.
//
// Per system (its rows and entries are a contiguous range of the block-
// diagonal operator the batch uploads):
//   * the synchronous ParILU sweeps in A's order from the A-order records
//     (the same per-entry formula as parilu.cu's k_parilu_sweep_ao,
//     src/parilu_v0_3.cpp:62-108 in synchronous form), factor values in A's
//     order, double-buffered between CTA barriers;
//   * M^-1 q as two level-scheduled triangular solves read straight from the
//     A-order factor values (L: the entries left of the diagonal, unit
//     diagonal; U: the diagonal and right of it), levels built on the host,
//     one CTA barrier per level, the four right-hand sides in one pass;
//   * FGMRES-Householder per (system, rhs) in LACE's arithmetic
//     (src/fgmres_householder_restart.cpp: reflectors, compact-WY T, Givens
//     rotations, the least-squares update), the basis and Z in a per-CTA
//     workspace, the small matrices in shared memory and a per-CTA slice of
//     global memory.
// A (system, rhs) process is the one a lone solve of that pair runs: the
// pairs of a CTA only share the operator and factor reads and the barriers.
#include <algorithm>
#include <cmath>

#include "context.h"
#include "krylov_tile.cuh"

namespace lace {

constexpr int kPBThreads = 512;
constexpr int kPBRhs = 4;            // right-hand sides in lockstep
constexpr int kPBMaxLd = kBatchMaxM + 2;  // the small matrices' largest leading dimension
constexpr int kPBMaxW = kBatchMaxW;       // off-diagonal entries a triangle's row holds at most

template <typename T>
__device__ __forceinline__ double pb_f64(T v) {
  return (double)v;
}
template <>
__device__ __forceinline__ double pb_f64<float>(float v) {
  return to_f64(v);
}

// eight FP64 sums over the warp, reduce-scatter: afterwards lane l holds the
// total of value ((l >> 2) & 7) in v[0] (9 additions a lane, not 40)
__device__ __forceinline__ double warp_sum8(double (&a)[8]) {
  const int lane = threadIdx.x & 31;
  {
    const bool hi = lane & 16;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const double send = hi ? a[c] : a[c + 4];
      const double got = __shfl_xor_sync(0xffffffffu, send, 16);
      a[c] = (hi ? a[c + 4] : a[c]) + got;
    }
  }
  {
    const bool hi = lane & 8;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const double send = hi ? a[c] : a[c + 2];
      const double got = __shfl_xor_sync(0xffffffffu, send, 8);
      a[c] = (hi ? a[c + 2] : a[c]) + got;
    }
  }
  {
    const bool hi = lane & 4;
    const double send = hi ? a[0] : a[1];
    const double got = __shfl_xor_sync(0xffffffffu, send, 4);
    a[0] = (hi ? a[1] : a[0]) + got;
  }
  a[0] += __shfl_xor_sync(0xffffffffu, a[0], 2);
  a[0] += __shfl_xor_sync(0xffffffffu, a[0], 1);
  return a[0];
}
// which of the eight values lane l holds after warp_sum8: bit 2 of the
// index from lane bit 4, bit 1 from lane bit 3, bit 0 from lane bit 2
__device__ __forceinline__ int warp_sum8_slot(int lane) {
  return (((lane >> 4) & 1) << 2) | (((lane >> 3) & 1) << 1) | ((lane >> 2) & 1);
}

struct PBatch {
  int nsys, nrhs, m, ld, restart_max, sweeps, tol_type;
  double rtol;
  int njobs;
  const int *jsys, *jrhs, *jnr;      // jobs: system, first rhs, rhs count (largest systems first)
  const int *n, *roff, *lsys, *usys;  // rows, first row, first L / U level of each system
  const int *Arow, *Acol;
  const double *Aval;
  const int *pptr, *dpos, *diag;    // A-order sweep records
  const int2 *pairs;
  void *F;                          // per CTA: two buffers of factor values in A's order (FT), fstride each
  const int *lptr, *lrows, *uptr, *urows;  // levels: row ranges and rows
  int w;                            // record width (off-diagonals per row, <= kPBMaxW)
  const int *cL, *fL, *cU, *fU, *dU;  // level-ordered records: local columns (-1: none), A positions
  void *vrec;                       // per CTA: the records' values, L then U then U's diagonal (FT)
  const double *b;
  double *x;
  int N;                            // rows of all systems (vector stride between rhs)
  size_t nmax, fstride;             // workspace rows per vector; entries per factor buffer
  double *V, *W, *Tm, *Rm;          // per CTA: kPBRhs x (m+1) x nmax, kPBRhs x nmax, kPBRhs x ld^2 (two)
  void *Z, *Q, *Tt;                 // per CTA: kPBRhs x m x nmax, kPBRhs x nmax (two), FT
  int *next;                        // queue head
  int *iters, *conv;                // per (system, rhs), system-major
};

// out[k] (k < ncols) = sum over rows i >= lo of V[k][i] w[i] (one right-hand
// side): eight columns at a time, rows over the CTA's threads, reduce-scatter
// in the warp, warps summed in a fixed order
__device__ void pb_dots(const double *V, size_t nmax, int ncols, int n, int lo, const double *w, double *out,
                        double *sred) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int k0 = 0; k0 < ncols; k0 += 8) {
    double a[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    for (int i = lo + (int)threadIdx.x; i < n; i += blockDim.x) {
      const double wi = w[i];
#pragma unroll
      for (int c = 0; c < 8; ++c)
        if (k0 + c < ncols) a[c] = fma(V[(size_t)(k0 + c) * nmax + i], wi, a[c]);
    }
    const double v = warp_sum8(a);
    if ((lane & 3) == 0) sred[wid * 8 + warp_sum8_slot(lane)] = v;
    __syncthreads();
    if ((int)threadIdx.x < 8 && k0 + (int)threadIdx.x < ncols) {
      double t = 0.0;
      for (int w2 = 0; w2 < nw; ++w2) t += sred[w2 * 8 + threadIdx.x];
      out[k0 + threadIdx.x] = t;
    }
    __syncthreads();
  }
}

template <typename FT>
__global__ void __launch_bounds__(kPBThreads, 1) k_batch_persist(PBatch P) {
  const int tid = threadIdx.x, T = blockDim.x, lane = tid & 31, wid = tid >> 5;
  const int m = P.m, ld = P.ld;
  __shared__ int s_job;
  __shared__ double sred[(kPBThreads / 32) * 8];
  __shared__ double sg[kPBRhs][kPBMaxLd], scs[kPBRhs][kPBMaxLd], ssn[kPBRhs][kPBMaxLd];
  __shared__ double sc[kPBRhs][kPBMaxLd], ss[kPBRhs][kPBMaxLd], sd[kPBRhs][kPBMaxLd], srho[kPBRhs][kPBMaxLd];
  __shared__ double s_dd[kPBRhs], s_ia[kPBRhs], s_rtol[kPBRhs];
  __shared__ int s_live[kPBRhs], s_step[kPBRhs], s_conv[kPBRhs], s_iters[kPBRhs], s_first[kPBRhs];
  // this CTA's workspace
  const size_t nmax = P.nmax;
  double *V0 = P.V + (size_t)blockIdx.x * kPBRhs * (m + 1) * nmax;
  double *W0 = P.W + (size_t)blockIdx.x * kPBRhs * nmax;
  double *Tm0 = P.Tm + (size_t)blockIdx.x * kPBRhs * ld * ld;
  double *Rm0 = P.Rm + (size_t)blockIdx.x * kPBRhs * ld * ld;
  FT *Z0 = (FT *)P.Z + (size_t)blockIdx.x * kPBRhs * m * nmax;
  FT *Q0 = (FT *)P.Q + (size_t)blockIdx.x * kPBRhs * nmax;
  FT *Tt0 = (FT *)P.Tt + (size_t)blockIdx.x * kPBRhs * nmax;
  FT *Fcta = (FT *)P.F + (size_t)blockIdx.x * 2 * P.fstride;
  const int W = P.w;
  FT *vL0 = (FT *)P.vrec + (size_t)blockIdx.x * (2 * W + 1) * nmax;
  FT *vU0 = vL0 + (size_t)W * nmax, *vD0 = vU0 + (size_t)W * nmax;
  for (;;) {
    if (tid == 0) s_job = atomicAdd(P.next, 1);
    __syncthreads();
    const int job = s_job;
    __syncthreads();
    if (job >= P.njobs) break;
    const int sys = P.jsys[job];
    const int n = P.n[sys], r0 = P.roff[sys];
    const int e0 = P.Arow[r0], e1 = P.Arow[r0 + n];
    // ---- ParILU(0) of the system into this CTA's buffers (indexed from e0):
    // F = A, then the synchronous sweeps
    FT *Fa = Fcta - e0, *Fb = Fcta + P.fstride - e0;
    for (int p = e0 + tid; p < e1; p += T) Fa[p] = (FT)P.Aval[p];
    __syncthreads();
    for (int sw = 0; sw < P.sweeps; ++sw) {
      for (int p = e0 + tid; p < e1; p += T) {
        FT s = (FT)P.Aval[p];
        for (int q = P.pptr[p]; q < P.pptr[p + 1]; ++q) {
          const int2 pr = P.pairs[q];
          s = fma(-Fa[pr.x], Fa[pr.y], s);
        }
        const int d = P.dpos[p];
        Fb[p] = d >= 0 ? s / Fa[d] : s;
      }
      __syncthreads();
      FT *t = Fa;
      Fa = Fb;
      Fb = t;
    }
    const FT *F = Fa;
    // the factor values into the level-ordered records of the two triangles
    const int kbL = P.lptr[P.lsys[sys]], kbU = P.uptr[P.usys[sys]];
    for (int t = tid; t < n * W; t += T) {
      const int fl = P.fL[(size_t)kbL * W + t], fu = P.fU[(size_t)kbU * W + t];
      vL0[t] = fl >= 0 ? F[fl] : (FT)0;
      vU0[t] = fu >= 0 ? F[fu] : (FT)0;
    }
    for (int t = tid; t < n; t += T) vD0[t] = F[P.dU[kbU + t]];
    __syncthreads();
    // ---- FGMRES-Householder for the job's right-hand sides, in lockstep
    {
      const int rg = P.jrhs[job];
      const int nr = P.jnr[job];
      if (tid < kPBRhs) {
        s_conv[tid] = tid < nr ? 0 : 1;
        s_iters[tid] = 0;
        s_first[tid] = 1;
        s_step[tid] = 0;
        s_live[tid] = 0;
      }
      __syncthreads();
      for (int cyc = 0; cyc < P.restart_max; ++cyc) {
        // r = b - A x into W, per right-hand side still running
        for (int c = 0; c < nr; ++c) {
          if (s_conv[c]) continue;  // uniform
          const double *b = P.b + (size_t)(rg + c) * P.N + r0;
          const double *x = P.x + (size_t)(rg + c) * P.N + r0;
          double *w = W0 + (size_t)c * nmax;
          for (int i = tid; i < n; i += T) {
            double s = b[i];
            for (int p = P.Arow[r0 + i]; p < P.Arow[r0 + i + 1]; ++p) s = fma(-P.Aval[p], x[P.Acol[p] - r0], s);
            w[i] = s;
          }
        }
        __syncthreads();
        for (int c = 0; c < nr; ++c) {
          if (s_conv[c]) continue;
          double *w = W0 + (size_t)c * nmax;
          pb_dots(w, 0, 1, n, 0, w, &ss[c][0], sred);  // ||r||^2
        }
        if (tid < nr && !s_conv[tid]) {
          const int c = tid;
          const double *w = W0 + (size_t)c * nmax;
          const double rn2 = ss[c][0], rnorm = sqrt(rn2);
          if (s_first[c]) {
            s_rtol[c] = P.tol_type == 1 ? P.rtol * rnorm : P.rtol;
            s_first[c] = 0;
          }
          s_step[c] = 0;
          if (!(rnorm >= s_rtol[c])) {
            s_conv[c] = 1;
            s_live[c] = 0;
          } else {
            const double w0 = w[0];
            const double dd = mysgn(w0) * rnorm;
            const double alpha = sqrt(2.0 * (rn2 + fabs(w0) * rnorm));
            s_dd[c] = dd;
            s_ia[c] = alpha > 0.0 ? 1.0 / alpha : 0.0;
            sg[c][0] = -dd;
            Tm0[(size_t)c * ld * ld] = 2.0;
            s_live[c] = 1;
          }
        }
        if (tid >= nr && tid < kPBRhs) s_live[tid] = 0;
        __syncthreads();
        // v_0 = (r + dd e_0) / alpha, q_0 = -r / dd
        for (int c = 0; c < nr; ++c) {
          if (!s_live[c]) continue;
          const double *w = W0 + (size_t)c * nmax;
          double *v = V0 + (size_t)c * (m + 1) * nmax;
          FT *q = Q0 + (size_t)c * nmax;
          const double dd = s_dd[c], ia = s_ia[c];
          for (int i = tid; i < n; i += T) {
            v[i] = (i == 0 ? w[i] + dd : w[i]) * ia;
            q[i] = (FT)(-w[i] / dd);
          }
        }
        __syncthreads();
        for (int j = 0; j < m; ++j) {
          bool any = false;
          for (int c = 0; c < nr; ++c) any = any || s_live[c];
          if (!any) break;
          const int jp1 = j + 1;
          // ---- z_j = U^-1 L^-1 q_j, level by level, all live rhs per pass: a
          // row's record (columns, values, right-hand side) is loaded for the
          // next level before the barrier, so a level waits for one load
          // (the solved values it reads)
          {
            bool live[kPBRhs];
#pragma unroll
            for (int c = 0; c < kPBRhs; ++c) live[c] = c < nr && s_live[c];
            for (int pass = 0; pass < 2; ++pass) {
              const bool lower = pass == 0;
              const int *lp = lower ? P.lptr : P.uptr;
              const int *lr = lower ? P.lrows : P.urows;
              const int *cw = lower ? P.cL : P.cU;
              const FT *vw = lower ? vL0 : vU0;
              const int kb0 = lower ? kbL : kbU;
              const int l0 = lower ? P.lsys[sys] : P.usys[sys], l1 = lower ? P.lsys[sys + 1] : P.usys[sys + 1];
              FT *out[kPBRhs];
              const FT *in[kPBRhs];
#pragma unroll
              for (int c = 0; c < kPBRhs; ++c) {
                out[c] = lower ? Tt0 + (size_t)c * nmax : Z0 + ((size_t)c * m + j) * nmax;
                in[c] = lower ? Q0 + (size_t)c * nmax : Tt0 + (size_t)c * nmax;
              }
              // one row's record
              int ri = -1, rc[kPBMaxW];
              FT rv[kPBMaxW], rq[kPBRhs], rd = (FT)1;
              auto load = [&](int k) {
                ri = k >= 0 ? lr[k] - r0 : -1;
#pragma unroll
                for (int w = 0; w < kPBMaxW; ++w) {
                  rc[w] = (k >= 0 && w < W) ? cw[(size_t)k * W + w] : -1;
                  rv[w] = (k >= 0 && w < W) ? vw[(size_t)(k - kb0) * W + w] : (FT)0;
                }
#pragma unroll
                for (int c = 0; c < kPBRhs; ++c) rq[c] = (k >= 0 && live[c]) ? in[c][ri] : (FT)0;
                if (!lower && k >= 0) rd = vD0[k - kb0];
              };
              auto solve = [&]() {
#pragma unroll
                for (int c = 0; c < kPBRhs; ++c) {
                  if (!live[c]) continue;
                  FT acc = rq[c];
#pragma unroll
                  for (int w = 0; w < kPBMaxW; ++w)
                    if (rc[w] >= 0) acc = fma(-rv[w], out[c][rc[w]], acc);
                  out[c][ri] = lower ? acc : acc / rd;
                }
              };
              int lv = l0, kb = lp[lv], ke = lp[lv + 1];
              load(kb + tid < ke ? kb + tid : -1);
              while (lv < l1) {
                if (ri >= 0) solve();
                for (int k = kb + tid + T; k < ke; k += T) {  // levels wider than the CTA
                  load(k);
                  solve();
                }
                ++lv;
                if (lv < l1) {
                  kb = lp[lv];
                  ke = lp[lv + 1];
                  load(kb + tid < ke ? kb + tid : -1);
                }
                __syncthreads();
              }
            }
          }
          // ---- w = A z_j
          for (int c = 0; c < nr; ++c) {
            if (!s_live[c]) continue;
            const FT *zv = Z0 + ((size_t)c * m + j) * nmax;
            double *w = W0 + (size_t)c * nmax;
            for (int i = tid; i < n; i += T) {
              double s = 0.0;
              for (int p = P.Arow[r0 + i]; p < P.Arow[r0 + i + 1]; ++p)
                s = fma(P.Aval[p], pb_f64(zv[P.Acol[p] - r0]), s);
              w[i] = s;
            }
          }
          __syncthreads();
          // ---- s = V^T w, y = T^T s, w -= V y
          for (int c = 0; c < nr; ++c)
            if (s_live[c]) pb_dots(V0 + (size_t)c * (m + 1) * nmax, nmax, jp1, n, 0, W0 + (size_t)c * nmax, &ss[c][0], sred);
          for (int c = wid; c < nr; c += (T >> 5)) {  // a warp per rhs
            if (!s_live[c]) continue;
            const double *Tc = Tm0 + (size_t)c * ld * ld;
            for (int k = lane; k < jp1; k += 32) {
              double y = 0.0;
              for (int l = 0; l <= k; ++l) y = fma(Tc[l + k * ld], ss[c][l], y);
              sd[c][k] = y;
            }
          }
          __syncthreads();
          for (int c = 0; c < nr; ++c) {
            if (!s_live[c]) continue;
            const double *v = V0 + (size_t)c * (m + 1) * nmax;
            double *w = W0 + (size_t)c * nmax;
            for (int i = tid; i < n; i += T) {
              double s = w[i];
              for (int k = 0; k < jp1; ++k) s = fma(-v[(size_t)k * nmax + i], sd[c][k], s);
              w[i] = s;
            }
          }
          __syncthreads();
          // ---- V^T w over rows > j, ||w_{j+1:}||^2
          for (int c = 0; c < nr; ++c) {
            if (!s_live[c]) continue;
            double *w = W0 + (size_t)c * nmax;
            pb_dots(V0 + (size_t)c * (m + 1) * nmax, nmax, jp1, n, jp1, w, &ss[c][0], sred);
            pb_dots(w, 0, 1, n, jp1, w, &ss[c][jp1], sred);
          }
          // ---- the new reflector, T's column, c = T_{j+1} rho, Givens (a warp per rhs)
          for (int c = wid; c < nr; c += (T >> 5)) {
            if (!s_live[c]) continue;
            const double *v = V0 + (size_t)c * (m + 1) * nmax;
            const double *w = W0 + (size_t)c * nmax;
            double *Tc = Tm0 + (size_t)c * ld * ld;
            const double nrm2 = jp1 < n ? ss[c][jp1] : 0.0;
            const double wn = sqrt(nrm2);
            const double wj1 = jp1 < n ? w[jp1] : 0.0;
            const double dd = mysgn(wj1) * wn;
            const double alpha = sqrt(2.0 * (nrm2 + fabs(wj1) * wn));
            const double ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
            for (int k = lane; k < jp1; k += 32) {
              const double vk = jp1 < n ? v[(size_t)k * nmax + jp1] : 0.0;
              sd[c][k] = (ss[c][k] + dd * vk) * ia;
              srho[c][k] = vk;
            }
            if (lane == 0) srho[c][jp1] = (wj1 + dd) * ia;
            __syncwarp();
            for (int k = lane; k < jp1; k += 32) {
              double t = 0.0;
              for (int l = k; l < jp1; ++l) t = fma(Tc[k + l * ld], sd[c][l], t);
              Tc[k + jp1 * ld] = -2.0 * t;
            }
            for (int k = jp1 + lane; k < ld; k += 32) Tc[k + jp1 * ld] = k == jp1 ? 2.0 : 0.0;
            __syncwarp();
            for (int k = lane; k <= jp1; k += 32) {
              double t = 0.0;
              for (int l = k; l <= jp1; ++l) t = fma(Tc[k + l * ld], srho[c][l], t);
              sc[c][k] = t;
            }
            if (lane == 0) {
              s_dd[c] = dd;
              s_ia[c] = ia;
              double *Rj = Rm0 + (size_t)c * ld * ld + (size_t)j * ld;
              for (int k = 0; k <= j; ++k) Rj[k] = w[k];
              for (int k = 0; k < j; ++k) {
                const double a0 = Rj[k], a1 = Rj[k + 1];
                Rj[k + 1] = -ssn[c][k] * a0 + scs[c][k] * a1;
                Rj[k] = scs[c][k] * a0 + ssn[c][k] * a1;
              }
              double cg, sn;
              givens_rot(Rj[j], -dd, 4.9406564584124654e-324, &cg, &sn);
              scs[c][j] = cg;
              ssn[c][j] = sn;
              Rj[j] = cg * Rj[j] - sn * dd;
              const double gj = sg[c][j];
              sg[c][jp1] = -sn * gj;
              sg[c][j] = cg * gj;
              const double resid = fabs(sg[c][jp1]);
              s_step[c] = jp1;
              if (resid < s_rtol[c] || j == m - 1 || !(resid == resid)) {
                s_live[c] = 0;
                if (resid < s_rtol[c]) s_conv[c] = 1;
              }
            }
          }
          __syncthreads();
          // ---- v_{j+1} and q_{j+1} = e_{j+1} - V_{j+1} c, for the rhs that go on
          for (int c = 0; c < nr; ++c) {
            if (!s_live[c] || jp1 >= m) continue;
            double *v = V0 + (size_t)c * (m + 1) * nmax;
            const double *w = W0 + (size_t)c * nmax;
            FT *q = Q0 + (size_t)c * nmax;
            const double dd = s_dd[c], ia = s_ia[c];
            for (int i = tid; i < n; i += T) {
              const double vi = i > j ? (i == jp1 ? w[i] + dd : w[i]) * ia : 0.0;
              v[(size_t)jp1 * nmax + i] = vi;
              double acc = (i == jp1 ? 1.0 : 0.0) - vi * sc[c][jp1];
              for (int k = 0; k < jp1; ++k) acc = fma(-v[(size_t)k * nmax + i], sc[c][k], acc);
              q[i] = (FT)acc;
            }
          }
          __syncthreads();
        }
        // ---- least squares R y = g and x += Z y, per rhs that ran this cycle
        for (int c = wid; c < nr; c += (T >> 5)) {
          const int ns = s_step[c];
          if (ns == 0 || lane != 0) continue;
          const double *R = Rm0 + (size_t)c * ld * ld;
          double *y = &sd[c][0];
          for (int i = 0; i < ns; ++i) y[i] = sg[c][i] / R[i + i * ld];
          for (int jj = ns - 1; jj > 0; --jj)
            for (int i = jj - 1; i >= 0; --i) y[i] = y[i] - R[i + jj * ld] * y[jj] / R[i + i * ld];
        }
        __syncthreads();
        for (int c = 0; c < nr; ++c) {
          const int ns = s_step[c];
          if (ns == 0) continue;
          double *x = P.x + (size_t)(rg + c) * P.N + r0;
          for (int i = tid; i < n; i += T) {
            double s = x[i];
            for (int k = 0; k < ns; ++k) s = fma(pb_f64(Z0[((size_t)c * m + k) * nmax + i]), sd[c][k], s);
            x[i] = s;
          }
        }
        __syncthreads();
        if (tid < nr) {
          s_iters[tid] += s_step[tid];
          s_step[tid] = 0;
        }
        __syncthreads();
        bool all = true;
        for (int c = 0; c < nr; ++c) all = all && s_conv[c];
        if (all) break;
      }
      if (tid < nr) {
        P.iters[sys * P.nrhs + rg + tid] = s_iters[tid];
        P.conv[sys * P.nrhs + rg + tid] = s_conv[tid];
      }
      __syncthreads();
    }
  }
}

int launch_batch_persist(cudaStream_t s, const PBatchHost &h) {
  PBatch P;
  P.nsys = h.nsys;
  P.nrhs = h.nrhs;
  P.m = h.m;
  P.ld = h.m + 2;
  P.restart_max = h.restart_max;
  P.sweeps = h.sweeps;
  P.tol_type = 1;
  P.rtol = h.rtol;
  P.njobs = h.njobs;
  P.jsys = h.jsys;
  P.jrhs = h.jrhs;
  P.jnr = h.jnr;
  P.n = h.n;
  P.roff = h.roff;
  P.lsys = h.lsys;
  P.usys = h.usys;
  P.Arow = h.Arow;
  P.Acol = h.Acol;
  P.Aval = h.Aval;
  P.pptr = h.pptr;
  P.dpos = h.dpos;
  P.diag = h.diag;
  P.pairs = h.pairs;
  P.F = h.F;
  P.fstride = h.fstride;
  P.lptr = h.lptr;
  P.w = h.w;
  P.cL = h.cL;
  P.fL = h.fL;
  P.cU = h.cU;
  P.fU = h.fU;
  P.dU = h.dU;
  P.vrec = h.vrec;
  P.lrows = h.lrows;
  P.uptr = h.uptr;
  P.urows = h.urows;
  P.b = h.b;
  P.x = h.x;
  P.N = h.N;
  P.nmax = h.nmax;
  P.V = h.V;
  P.W = h.W;
  P.Tm = h.Tm;
  P.Rm = h.Rm;
  P.Z = h.Z;
  P.Q = h.Q;
  P.Tt = h.Tt;
  P.next = h.next;
  P.iters = h.iters;
  P.conv = h.conv;
  if (h.f32)
    k_batch_persist<float><<<h.grid, kPBThreads, 0, s>>>(P);
  else
    k_batch_persist<double><<<h.grid, kPBThreads, 0, s>>>(P);
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

int batch_persist_threads() { return kPBThreads; }
int batch_persist_rhs() { return kPBRhs; }

}  // namespace lace
