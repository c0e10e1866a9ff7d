// Batched solves (lace_gpu_batch_*): many independent systems, several
// right-hand sides each, advanced together.
//
// The systems are assembled into one block-diagonal matrix S (no coupling
// entries), so one ParILU sweep, one SpMV and one block-scheduled triangular
// solve serve all systems at once (the solve takes every right-hand side in
// the same launch, blockIdx.y = rhs).  Vectors are rhs-major: vector r of the
// batch is v[r*N + row_off[s] + i].  Every (system, rhs) pair is a segment
// with its own FGMRES-Householder process (reflectors, compact-WY T, Givens,
// convergence to its own relative tolerance): the Arnoldi passes run over row
// tiles that never straddle a segment, write per-tile partial sums, and one
// warp per segment folds them (deterministic order) and does the segment's
// scalar work.  A converged segment's tiles are skipped.  One cycle of
// search_max steps is captured once in a CUDA graph and replayed per restart.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"

namespace lace {


constexpr int kBT = 256;      // rows per tile, threads per block
constexpr int kBMaxM = 64;    // largest search_max of the batched solver
constexpr int kBSlots = (kBMaxM + 2 + 7) / 8;

struct Seg {  // per-segment arrays, ld = m + 2
  double *T, *R, *g, *cs, *sn, *y, *c, *yls, *hist;
  double *dd, *ia, *dd0, *ia0, *rnorm, *rtol_abs;
  int *done, *conv, *nsteps, *first;
};

struct Tiles {
  const int *seg;    // tile -> segment
  const int *voff;   // tile -> first row in the rhs-major vectors
  const int *mrow;   // tile -> first matrix row of S
  const int *len;    // tile -> rows
  const int *lrow0;  // tile -> first local row (inside its segment)
  const int *seg_t0, *seg_nt;  // segment -> first tile, tile count
  int ntiles, nseg;
};

struct Mat {
  const int *row, *col;
  const double *val;
};

__device__ __forceinline__ double row_dot(const Mat &A, int mr, const double *z, int zoff) {
  double s = 0.0;
  for (int p = A.row[mr]; p < A.row[mr + 1]; ++p) s = fma(A.val[p], z[zoff + A.col[p]], s);
  return s;
}
__device__ __forceinline__ double row_dot(const Mat &A, int mr, const float *z, int zoff) {
  double s = 0.0;
  for (int p = A.row[mr]; p < A.row[mr + 1]; ++p) s = fma(A.val[p], (double)z[zoff + A.col[p]], s);
  return s;
}

// ------------------------------------------------------------ residual
__global__ void __launch_bounds__(kBT) k_bres(Tiles T, Mat A, int N, const double *b, const double *x,
                                              double *r, double *part, Seg S) {
  __shared__ double red[kBT / 32];
  for (int t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int sg = T.seg[t];
    if (S.conv[sg]) continue;  // block-uniform
    const int k = threadIdx.x;
    double nr = 0.0;
    if (k < T.len[t]) {
      const int gi = T.voff[t] + k, mr = T.mrow[t] + k;
      const int zoff = gi - mr;  // start of this rhs's vector
      const double ri = b[gi] - row_dot(A, mr, x, zoff);
      r[gi] = ri;
      nr = ri * ri;
    }
    nr = warp_sum(nr);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nr;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int w = 0; w < kBT / 32; ++w) s += red[w];
      part[(size_t)t * (kBMaxM + 2)] = s;
    }
    __syncthreads();
  }
}

// one warp per segment: ||r||, first reflector scalars, convergence test
__global__ void k_bstart(Tiles T, int ld, const double *r, const double *part, Seg S, double rtol, int tol_type) {
  const int sg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sg >= T.nseg) return;
  if (S.conv[sg]) return;
  double s = 0.0;
  for (int q = lane; q < T.seg_nt[sg]; q += 32) s += part[(size_t)(T.seg_t0[sg] + q) * (kBMaxM + 2)];
  s = warp_sum(s);
  if (lane != 0) return;
  const double rnorm = sqrt(s);
  S.rnorm[sg] = rnorm;
  if (S.first[sg]) {
    S.rtol_abs[sg] = tol_type == 1 ? rtol * rnorm : rtol;
    S.first[sg] = 0;
  }
  S.nsteps[sg] = 0;
  if (!(rnorm >= S.rtol_abs[sg])) {
    S.done[sg] = 1;
    S.conv[sg] = 1;
    return;
  }
  const double r0 = r[T.voff[T.seg_t0[sg]]];
  const double dd = mysgn(r0) * rnorm;
  const double alpha = sqrt(2.0 * (s + fabs(r0) * rnorm));
  S.dd0[sg] = dd;
  S.ia0[sg] = alpha > 0.0 ? 1.0 / alpha : 0.0;
  S.g[(size_t)sg * ld] = -dd;
  S.T[(size_t)sg * ld * ld] = 2.0;
  S.done[sg] = 0;
}

__global__ void __launch_bounds__(kBT) k_binit(Tiles T, const double *r, double *V, double *q, Seg S) {
  for (int t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int sg = T.seg[t];
    if (S.done[sg]) continue;
    const int k = threadIdx.x;
    if (k >= T.len[t]) continue;
    const int gi = T.voff[t] + k;
    const double ri = r[gi];
    const double dd = S.dd0[sg];
    V[gi] = (T.lrow0[t] + k == 0 ? ri + dd : ri) * S.ia0[sg];
    q[gi] = -ri / dd;
  }
}

// tile dots: acc[slot] += V[kk][gi] * sw[k] for kk = slot*8 + warp < ncols,
// rows k of the tile with local row >= lo
__device__ __forceinline__ void btile_dots(const double *V, size_t ldv, int ncols, int voff, int len,
                                           int lrow0, int lo, const double *sw, double (&acc)[kBSlots]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = lane; k < len; k += 32) {
    if (lrow0 + k < lo) continue;
    const double wi = sw[k];
#pragma unroll
    for (int sl = 0; sl < kBSlots; ++sl) {
      const int kk = sl * 8 + wid;
      if (kk < ncols) acc[sl] = fma(V[(size_t)kk * ldv + voff + k], wi, acc[sl]);
    }
  }
}

__device__ __forceinline__ void bflush(double (&acc)[kBSlots], int ncols, double *dst) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int sl = 0; sl < kBSlots; ++sl) {
    if (sl * 8 >= ncols) break;
    const double v = warp_sum(acc[sl]);
    const int kk = sl * 8 + wid;
    if (lane == 0 && kk < ncols) dst[kk] = v;
    acc[sl] = 0.0;
  }
}

// pass A: w = A z_j and per-tile V^T w
template <typename ZT>
__global__ void __launch_bounds__(kBT) k_bpassA(Tiles T, Mat A, const ZT *z, double *w, const double *V,
                                                size_t ldv, int j, double *part, Seg S) {
  __shared__ double sw[kBT];
  double acc[kBSlots];
#pragma unroll
  for (int sl = 0; sl < kBSlots; ++sl) acc[sl] = 0.0;
  for (int t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int sg = T.seg[t];
    if (S.done[sg]) continue;
    const int k = threadIdx.x, len = T.len[t];
    if (k < len) {
      const int gi = T.voff[t] + k, mr = T.mrow[t] + k;
      const double wi = row_dot(A, mr, z, gi - mr);
      w[gi] = wi;
      sw[k] = wi;
    }
    __syncthreads();
    btile_dots(V, ldv, j + 1, T.voff[t], len, T.lrow0[t], 0, sw, acc);
    bflush(acc, j + 1, part + (size_t)t * (kBMaxM + 2));
    __syncthreads();
  }
}

// warp per segment: s = sum of tile partials, y = T^T s
__global__ void k_breduceA(Tiles T, int ld, int j, const double *part, Seg S) {
  const int sg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sg >= T.nseg || S.done[sg]) return;
  double sk[kBMaxM + 2];
  for (int k = 0; k <= j; ++k) {
    double s = 0.0;
    for (int q = lane; q < T.seg_nt[sg]; q += 32) s += part[(size_t)(T.seg_t0[sg] + q) * (kBMaxM + 2) + k];
    sk[k] = warp_sum(s);
  }
  const double *Tm = S.T + (size_t)sg * ld * ld;
  for (int k = lane; k <= j; k += 32) {
    double y = 0.0;
    for (int l = 0; l <= k; ++l) y = fma(Tm[l + k * ld], sk[l], y);
    S.y[(size_t)sg * ld + k] = y;
  }
}

// pass B: w <- w - V y; per tile V^T w over local rows > j, ||w_{j+1:}||^2
__global__ void __launch_bounds__(kBT) k_bpassB(Tiles T, const double *V, size_t ldv, int ld, int j, double *w,
                                                double *part, Seg S) {
  __shared__ double sw[kBT];
  __shared__ double red[kBT / 32];
  double acc[kBSlots];
#pragma unroll
  for (int sl = 0; sl < kBSlots; ++sl) acc[sl] = 0.0;
  for (int t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int sg = T.seg[t];
    if (S.done[sg]) continue;
    const int k = threadIdx.x, len = T.len[t];
    const double *y = S.y + (size_t)sg * ld;
    double nr = 0.0;
    if (k < len) {
      const int gi = T.voff[t] + k;
      double s = w[gi];
      for (int kk = 0; kk <= j; ++kk) s = fma(-V[(size_t)kk * ldv + gi], y[kk], s);
      w[gi] = s;
      sw[k] = s;
      if (T.lrow0[t] + k > j) nr = s * s;
    }
    __syncthreads();
    btile_dots(V, ldv, j + 1, T.voff[t], len, T.lrow0[t], j + 1, sw, acc);
    double *dst = part + (size_t)t * (kBMaxM + 2);
    bflush(acc, j + 1, dst);
    nr = warp_sum(nr);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nr;
    __syncthreads();
    if (threadIdx.x == 0) {
      double s = 0.0;
      for (int q = 0; q < kBT / 32; ++q) s += red[q];
      dst[j + 1] = s;
    }
    __syncthreads();
  }
}

// warp per segment: new reflector, T column, Givens, least squares
__global__ void k_breduceB(Tiles T, int ld, int j, int m, const double *V, size_t ldv, const double *w,
                           const double *part, Seg S, int seglen_only) {
  const int sg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (sg >= T.nseg || S.done[sg]) return;
  (void)seglen_only;
  const int jp1 = j + 1;
  double sd[kBMaxM + 2];
  for (int k = 0; k <= jp1; ++k) {
    double s = 0.0;
    for (int q = lane; q < T.seg_nt[sg]; q += 32) s += part[(size_t)(T.seg_t0[sg] + q) * (kBMaxM + 2) + k];
    sd[k] = warp_sum(s);
  }
  if (lane != 0) return;
  const int t0 = T.seg_t0[sg];
  const int voff = T.voff[t0];
  int nloc = 0;
  for (int q = 0; q < T.seg_nt[sg]; ++q) nloc += T.len[t0 + q];
  const double nrm2 = jp1 < nloc ? sd[jp1] : 0.0;
  const double wn = sqrt(nrm2);
  const double wj1 = jp1 < nloc ? w[voff + jp1] : 0.0;
  const double dd = mysgn(wj1) * wn;
  const double alpha = sqrt(2.0 * (nrm2 + fabs(wj1) * wn));
  const double ia = alpha > 0.0 ? 1.0 / alpha : 0.0;
  S.dd[sg] = dd;
  S.ia[sg] = ia;
  double *Tm = S.T + (size_t)sg * ld * ld;
  double dv[kBMaxM + 2], rho[kBMaxM + 2];
  for (int k = 0; k < jp1; ++k) {
    const double vk = jp1 < nloc ? V[(size_t)k * ldv + voff + jp1] : 0.0;
    dv[k] = (sd[k] + dd * vk) * ia;
    rho[k] = vk;
  }
  rho[jp1] = (wj1 + dd) * ia;
  for (int k = 0; k < jp1; ++k) {
    double t = 0.0;
    for (int l = k; l < jp1; ++l) t = fma(Tm[k + l * ld], dv[l], t);
    Tm[k + jp1 * ld] = -2.0 * t;
  }
  Tm[jp1 + jp1 * ld] = 2.0;
  for (int k = jp1 + 1; k < ld; ++k) Tm[k + jp1 * ld] = 0.0;
  double *cvec = S.c + (size_t)sg * ld;
  for (int k = 0; k <= jp1; ++k) {
    double t = 0.0;
    for (int l = k; l <= jp1; ++l) t = fma(Tm[k + l * ld], rho[l], t);
    cvec[k] = t;
  }
  double *R = S.R + (size_t)sg * ld * ld;
  double *Rj = R + (size_t)j * ld;
  double *g = S.g + (size_t)sg * ld, *cs = S.cs + (size_t)sg * ld, *sn = S.sn + (size_t)sg * ld;
  for (int k = 0; k <= j; ++k) Rj[k] = w[voff + k];
  for (int k = 0; k < j; ++k) {
    const double a0 = Rj[k], a1 = Rj[k + 1];
    Rj[k + 1] = -sn[k] * a0 + cs[k] * a1;
    Rj[k] = cs[k] * a0 + sn[k] * a1;
  }
  double c, s;
  {
    const double a = Rj[j], bb = -dd;  // src/givens.cpp:46-67
    if (fabs(bb) <= 4.9406564584124654e-324) {
      c = 1.0;
      s = 0.0;
    } else if (fabs(bb) > fabs(a)) {
      const double tt = a / bb;
      s = 1.0 / sqrt(1.0 + tt * tt);
      c = tt * s;
    } else {
      const double tt = bb / a;
      c = 1.0 / sqrt(1.0 + tt * tt);
      s = tt * c;
    }
  }
  cs[j] = c;
  sn[j] = s;
  Rj[j] = c * Rj[j] - s * dd;
  g[jp1] = -s * g[j];
  g[j] = c * g[j];
  const double resid = fabs(g[jp1]);
  S.hist[(size_t)sg * ld + j] = resid;
  const bool conv = resid < S.rtol_abs[sg];
  if (conv || j == m - 1 || !(resid == resid)) {
    double *y = S.yls + (size_t)sg * ld;
    for (int i = 0; i <= j; ++i) y[i] = g[i] / R[i + i * ld];
    for (int jj = j; jj > 0; --jj)
      for (int i = jj - 1; i >= 0; --i) y[i] = y[i] - R[i + jj * ld] * y[jj] / R[i + i * ld];
    S.nsteps[sg] = jp1;
    S.conv[sg] = conv ? 1 : 0;
    S.done[sg] = 1;
  }
}

__global__ void __launch_bounds__(kBT) k_bpassC(Tiles T, double *V, size_t ldv, int ld, int j, const double *w,
                                                double *q, Seg S) {
  for (int t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int sg = T.seg[t];
    if (S.done[sg]) continue;
    const int k = threadIdx.x;
    if (k >= T.len[t]) continue;
    const int gi = T.voff[t] + k, li = T.lrow0[t] + k;
    const int jp1 = j + 1;
    const double *cv = S.c + (size_t)sg * ld;
    const double v = (li > j) ? (li == jp1 ? w[gi] + S.dd[sg] : w[gi]) * S.ia[sg] : 0.0;
    V[(size_t)jp1 * ldv + gi] = v;
    double acc = (li == jp1 ? 1.0 : 0.0) - v * cv[jp1];
    for (int kk = 0; kk < jp1; ++kk) acc = fma(-V[(size_t)kk * ldv + gi], cv[kk], acc);
    q[gi] = acc;
  }
}

template <typename ZT>
__global__ void __launch_bounds__(kBT) k_bxupdate(Tiles T, const ZT *Z, size_t ldz, int ld, double *x, Seg S) {
  for (int t = blockIdx.x; t < T.ntiles; t += gridDim.x) {
    const int sg = T.seg[t];
    const int ns = S.nsteps[sg];
    if (ns == 0) continue;
    const int k = threadIdx.x;
    if (k >= T.len[t]) continue;
    const int gi = T.voff[t] + k;
    const double *y = S.yls + (size_t)sg * ld;
    double s = x[gi];
    for (int kk = 0; kk < ns; ++kk) s = fma((double)Z[(size_t)kk * ldz + gi], y[kk], s);
    x[gi] = s;
  }
}

// reset "done" for segments that still need work (new cycle)
__global__ void k_brearm(int nseg, Seg S) {
  const int sg = blockIdx.x * blockDim.x + threadIdx.x;
  if (sg < nseg) {
    S.done[sg] = S.conv[sg];
    S.nsteps[sg] = 0;
  }
}

}  // namespace lace

using namespace lace;

struct lace_gpu_batch {
  lace_gpu_ctx *ctx = nullptr;
  int nsys = 0, nrhs = 0, N = 0, nseg = 0, m = 0;
  std::vector<int> n, row_off;
  lace::DBuf Srow, Scol, Sval;
  lace::DBuf tseg, tvoff, tmrow, tlen, tlrow0, st0, snt;
  int ntiles = 0;
  lace::DBuf segbuf, V, Z, w, q, t, part, tick[2];
  size_t ldv = 0;
  int ld = 0;
  lace::Seg S{};
  lace::Tiles T{};
  cudaGraphExec_t graph = nullptr;
  int graph_m = 0;
  ~lace_gpu_batch() {
    if (graph) cudaGraphExecDestroy(graph);
  }
};

extern "C" int lace_gpu_batch_create(lace_gpu_batch **out, lace_gpu_ctx *ctx, int nsys, const int *n,
                                     const int *row_off, const int *nnz_off, const int *row, const int *col,
                                     const double *val, int nrhs) {
  if (!out || !ctx || !n || !row_off || !nnz_off || !row || !col || !val) return set_err(DEV_ERR_INVALID_PTR);
  if (nsys < 1 || nrhs < 1 || nrhs > 64) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(ctx->device);
  auto *B = new lace_gpu_batch();
  B->ctx = ctx;
  B->nsys = nsys;
  B->nrhs = nrhs;
  B->n.assign(n, n + nsys);
  B->row_off.assign(row_off, row_off + nsys);
  // block-diagonal S: system s occupies rows row_off[s] .. row_off[s]+n[s]
  int N = 0;
  for (int s = 0; s < nsys; ++s) {
    if (row_off[s] != N || n[s] < 1) {
      delete B;
      return set_err(DEV_ERR_ILLEGAL_VALUE);
    }
    N += n[s];
  }
  B->N = N;
  std::vector<int> Sr(N + 1, 0);
  long long nnz = 0;
  for (int s = 0; s < nsys; ++s) nnz += row[row_off[s] + s + n[s]] - row[row_off[s] + s];
  std::vector<int> Sc(nnz);
  std::vector<double> Sv(nnz);
  long long p = 0;
  for (int s = 0; s < nsys; ++s) {
    // system s's row pointers are local, stored at row[row_off[s] + s .. + n[s]]
    const int *rp = row + row_off[s] + s;
    for (int i = 0; i < n[s]; ++i) {
      for (int e = rp[i]; e < rp[i + 1]; ++e) {
        Sc[p] = col[nnz_off[s] + e] + row_off[s];
        Sv[p] = val[nnz_off[s] + e];
        ++p;
      }
      Sr[row_off[s] + i + 1] = (int)p;
    }
  }
  int rc = lace_gpu_upload_csr_host(ctx, N, (int)nnz, Sr.data(), Sc.data(), Sv.data());
  if (rc) {
    delete B;
    return rc;
  }
  // tiles: segments (system, rhs) split in tiles of <= kBT rows
  std::vector<int> tseg, tvoff, tmrow, tlen, tlrow0, st0, snt;
  for (int r = 0; r < nrhs; ++r)
    for (int s = 0; s < nsys; ++s) {
      const int sg = r * nsys + s;
      st0.push_back((int)tseg.size());
      int cnt = 0;
      for (int i0 = 0; i0 < n[s]; i0 += kBT) {
        tseg.push_back(sg);
        tvoff.push_back(r * N + row_off[s] + i0);
        tmrow.push_back(row_off[s] + i0);
        tlen.push_back(std::min(kBT, n[s] - i0));
        tlrow0.push_back(i0);
        ++cnt;
      }
      snt.push_back(cnt);
    }
  B->nseg = nsys * nrhs;
  B->ntiles = (int)tseg.size();
  cudaStream_t st = ctx->stream;
  if (B->tseg.upload(tseg.data(), 4 * tseg.size(), st) || B->tvoff.upload(tvoff.data(), 4 * tvoff.size(), st) ||
      B->tmrow.upload(tmrow.data(), 4 * tmrow.size(), st) || B->tlen.upload(tlen.data(), 4 * tlen.size(), st) ||
      B->tlrow0.upload(tlrow0.data(), 4 * tlrow0.size(), st) || B->st0.upload(st0.data(), 4 * st0.size(), st) ||
      B->snt.upload(snt.data(), 4 * snt.size(), st)) {
    delete B;
    return set_err(DEV_ERR_DEVICE_ALLOC);
  }
  lace::Tiles &T = B->T;
  T.seg = (const int *)B->tseg.p;
  T.voff = (const int *)B->tvoff.p;
  T.mrow = (const int *)B->tmrow.p;
  T.len = (const int *)B->tlen.p;
  T.lrow0 = (const int *)B->tlrow0.p;
  T.seg_t0 = (const int *)B->st0.p;
  T.seg_nt = (const int *)B->snt.p;
  T.ntiles = B->ntiles;
  T.nseg = B->nseg;
  if (cudaStreamSynchronize(st) != cudaSuccess) {
    delete B;
    return set_err(DEV_ERR_UNKNOWN);
  }
  *out = B;
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_batch_destroy(lace_gpu_batch *B) {
  if (B) {
    cudaSetDevice(B->ctx->device);
    cudaStreamSynchronize(B->ctx->stream);
  }
  delete B;
  return DEV_SUCCESS;
}

static int batch_workspace(lace_gpu_batch *B, int m) {
  if (m == B->m && B->V.p) return 0;
  const int ld = m + 2;
  const size_t NN = (size_t)B->N * B->nrhs;
  B->ldv = (NN + 31) / 32 * 32;
  const bool zf32 = B->ctx->vtype() != VType::F64;
  int rc = 0;
  rc |= B->V.ensure(8 * B->ldv * (m + 1));
  rc |= B->Z.ensure((zf32 ? 4 : 8) * B->ldv * m);
  rc |= B->w.ensure(8 * B->ldv);
  rc |= B->q.ensure(8 * B->ldv);
  rc |= B->t.ensure(8 * B->ldv);
  rc |= B->part.ensure(8 * (size_t)B->ntiles * (kBMaxM + 2));
  const size_t ns = B->nseg;
  const size_t dbl = ns * (2 * (size_t)ld * ld + 7 * (size_t)ld + 6);
  rc |= B->segbuf.ensure(8 * dbl + 4 * 4 * ns);
  for (int k = 0; k < 2; ++k) {
    rc |= B->tick[k].ensure(4 * (size_t)(B->nrhs + 1));
  }
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  for (int k = 0; k < 2; ++k) {
    cudaMemsetAsync(B->tick[k].p, 0, B->tick[k].bytes, B->ctx->stream);
  }
  double *d = (double *)B->segbuf.p;
  lace::Seg &S = B->S;
  S.T = d; d += ns * ld * ld;
  S.R = d; d += ns * ld * ld;
  S.g = d; d += ns * ld;
  S.cs = d; d += ns * ld;
  S.sn = d; d += ns * ld;
  S.y = d; d += ns * ld;
  S.c = d; d += ns * ld;
  S.yls = d; d += ns * ld;
  S.hist = d; d += ns * ld;
  S.dd = d; d += ns;
  S.ia = d; d += ns;
  S.dd0 = d; d += ns;
  S.ia0 = d; d += ns;
  S.rnorm = d; d += ns;
  S.rtol_abs = d; d += ns;
  int *ip = (int *)d;
  S.done = ip; ip += ns;
  S.conv = ip; ip += ns;
  S.nsteps = ip; ip += ns;
  S.first = ip;
  B->m = m;
  B->ld = ld;
  if (B->graph) {
    cudaGraphExecDestroy(B->graph);
    B->graph = nullptr;
  }
  return 0;
}

static int batch_cycle_body(lace_gpu_batch *B, int m) {
  lace_gpu_ctx *c = B->ctx;
  cudaStream_t s = c->stream;
  const VType vt = c->vtype();
  const int f32 = vt != VType::F64;
  const int grid = std::min(B->ntiles, num_sms() * 8);
  const int sgrid = (B->nseg * 32 + 255) / 256;
  lace::Mat A{(const int *)c->Arow.p, (const int *)c->Acol.p, (const double *)c->Aval.p};
  const size_t ldz = B->ldv;
  for (int j = 0; j < m; ++j) {
    void *zj = (char *)B->Z.p + (size_t)j * ldz * (f32 ? 4 : 8);
    TriDev tl = c->tri(0), tu = c->tri(1);
    launch_sptrsv_blk_multi(s, c->plans[0].dev, tl.val, vt, B->q.p, 0, B->t.p, f32, B->N, B->nrhs,
                            (int *)B->tick[0].p, &c->ctrl()->status, nullptr);
    launch_sptrsv_blk_multi(s, c->plans[1].dev, tu.val, vt, B->t.p, f32, zj, f32, B->N, B->nrhs,
                            (int *)B->tick[1].p, &c->ctrl()->status, nullptr);
    if (f32)
      k_bpassA<float><<<grid, kBT, 0, s>>>(B->T, A, (const float *)zj, (double *)B->w.p, (const double *)B->V.p,
                                          B->ldv, j, (double *)B->part.p, B->S);
    else
      k_bpassA<double><<<grid, kBT, 0, s>>>(B->T, A, (const double *)zj, (double *)B->w.p,
                                           (const double *)B->V.p, B->ldv, j, (double *)B->part.p, B->S);
    k_breduceA<<<sgrid, 256, 0, s>>>(B->T, B->ld, j, (const double *)B->part.p, B->S);
    k_bpassB<<<grid, kBT, 0, s>>>(B->T, (const double *)B->V.p, B->ldv, B->ld, j, (double *)B->w.p,
                                  (double *)B->part.p, B->S);
    k_breduceB<<<sgrid, 256, 0, s>>>(B->T, B->ld, j, m, (const double *)B->V.p, B->ldv, (const double *)B->w.p,
                                     (const double *)B->part.p, B->S, 0);
    k_bpassC<<<grid, kBT, 0, s>>>(B->T, (double *)B->V.p, B->ldv, B->ld, j, (const double *)B->w.p,
                                  (double *)B->q.p, B->S);
  }
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

extern "C" int lace_gpu_batch_solve(lace_gpu_batch *B, int sweeps, int search_max, int restart_max, double rtol,
                                    const double *b, double *x, int *iters_out) {
  if (!B || !b || !x) return set_err(DEV_ERR_INVALID_PTR);
  if (search_max < 1 || search_max > kBMaxM) return set_err(DEV_ERR_NOT_SUPPORTED);
  lace_gpu_ctx *c = B->ctx;
  cudaSetDevice(c->device);
  if (c->opt.trsv_mode != LACE_TRSV_SYNCFREE) return set_err(DEV_ERR_NOT_SUPPORTED);
  int rc = c->parilu(sweeps, nullptr, nullptr, false, nullptr);
  if (!rc) rc = c->ensure_vectors();
  if (!rc) rc = c->autotune_trsv();
  if (!rc) rc = c->ensure_plan(0);
  if (!rc) rc = c->ensure_plan(1);
  if (!rc) rc = batch_workspace(B, search_max);
  if (rc) return set_err(rc);
  cudaStream_t s = c->stream;
  const int grid = std::min(B->ntiles, num_sms() * 8);
  const int sgrid = (B->nseg * 32 + 255) / 256;
  lace::Mat A{(const int *)c->Arow.p, (const int *)c->Acol.p, (const double *)c->Aval.p};
  // fresh per-segment state
  cudaMemsetAsync(B->S.done, 0, 4 * (size_t)B->nseg, s);
  cudaMemsetAsync(B->S.conv, 0, 4 * (size_t)B->nseg, s);
  std::vector<int> ones(B->nseg, 1);
  cudaMemcpyAsync(B->S.first, ones.data(), 4 * ones.size(), cudaMemcpyHostToDevice, s);
  std::vector<int> total(B->nseg, 0), conv(B->nseg), ns(B->nseg);
  for (int restart = 0; restart < restart_max; ++restart) {
    k_brearm<<<(B->nseg + 255) / 256, 256, 0, s>>>(B->nseg, B->S);
    k_bres<<<grid, kBT, 0, s>>>(B->T, A, B->N, b, x, (double *)B->w.p, (double *)B->part.p, B->S);
    k_bstart<<<sgrid, 256, 0, s>>>(B->T, B->ld, (const double *)B->w.p, (const double *)B->part.p, B->S, rtol, 1);
    k_binit<<<grid, kBT, 0, s>>>(B->T, (const double *)B->w.p, (double *)B->V.p, (double *)B->q.p, B->S);
    if (c->opt.use_graph) {
      if (!B->graph || B->graph_m != search_max) {
        if (B->graph) cudaGraphExecDestroy(B->graph);
        cudaGraph_t g;
        if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
        rc = batch_cycle_body(B, search_max);
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (rc || ce != cudaSuccess) return set_err(rc ? rc : DEV_ERR_UNKNOWN);
        ce = cudaGraphInstantiate(&B->graph, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
        B->graph_m = search_max;
      }
      if (cudaGraphLaunch(B->graph, s) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
    } else {
      rc = batch_cycle_body(B, search_max);
      if (rc) return set_err(rc);
    }
    if (c->vtype() != VType::F64)
      k_bxupdate<float><<<grid, kBT, 0, s>>>(B->T, (const float *)B->Z.p, B->ldv, B->ld, x, B->S);
    else
      k_bxupdate<double><<<grid, kBT, 0, s>>>(B->T, (const double *)B->Z.p, B->ldv, B->ld, x, B->S);
    cudaMemcpyAsync(conv.data(), B->S.conv, 4 * (size_t)B->nseg, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(ns.data(), B->S.nsteps, 4 * (size_t)B->nseg, cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
    bool all = true;
    for (int k = 0; k < B->nseg; ++k) {
      total[k] += ns[k];
      all = all && conv[k];
    }
    if (c->h_status() & kStatusSpinTimeout) return set_err(DEV_ERR_INTERNAL_LIMIT);
    if (all) break;
  }
  if (iters_out) {
    // per (system, rhs) in system-major order
    for (int sy = 0; sy < B->nsys; ++sy)
      for (int r = 0; r < B->nrhs; ++r) iters_out[sy * B->nrhs + r] = total[r * B->nsys + sy];
  }
  bool all = true;
  for (int k = 0; k < B->nseg; ++k) all = all && conv[k];
  return all ? DEV_SUCCESS : DEV_NOTCONVERGED;
}
