// ParILU(0) sweeps on the GPU.
//
// LACE's sweep (src/parilu_v0_3.cpp:67-103, and the one-block GPU copy in
// src/parilu_v0_3_gpu.cpp:17-105) updates L and U in place from every thread,
// an asynchronous iteration.  Here every sweep is synchronous (Jacobi): it
// reads the previous iterate (Lold/Uold) and writes the next (Lnew/Unew), so a
// sweep is deterministic and the step sum is a reduction without races.
// Per nonzero (i,j) of A:
//     s = a_ij - sum_{k < min(i,j)} l_ik u_kj      (merge of L row i, U col j)
//     l_ij = s / u_jj  (i > j)      u_ij = s  (i <= j)
// L is CSRL (unit diagonal last in each row), U is CSCU (diagonal last in
// each column).  One thread per row of A: the row's L entries are reused for
// all of its nonzeros, and the target position of an entry is found by the
// same merge walk (no position map is stored).
#include <algorithm>

#include "internal.h"

namespace lace {

constexpr int kPTPB = 256;

static int sweep_grid_pub(int rows) {
  int g = (rows + kPTPB - 1) / kPTPB;
  int cap = num_sms() * 8;
  return g < 1 ? 1 : (g > cap ? cap : g);
}

__device__ __forceinline__ double block_sum_p(double v) {
  __shared__ double scratch[kPTPB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < kPTPB / 32; ++w) t += scratch[w];
  return t;
}

// last block folds the per-block partials (deterministic order) into *out
__device__ __forceinline__ void finish_sum(double local, double *partials, int *counter,
                                           double *out) {
  double t = block_sum_p(local);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
  if (!arrive_last(counter)) return;
  const double s = block_fold(partials, 1, (int)gridDim.x);
  if (threadIdx.x == 0) *out = s;
}

template <typename FT, typename CT>
__global__ void __launch_bounds__(kPTPB) k_parilu_sweep(
    int n, const int *__restrict__ Arow, const int *__restrict__ Acol,
    const double *__restrict__ Aval, const int *__restrict__ Lrow, const int *__restrict__ Lcol,
    const FT *__restrict__ Lold, FT *__restrict__ Lnew, const int *__restrict__ Ucp,
    const int *__restrict__ Uri, const FT *__restrict__ Uold, FT *__restrict__ Unew,
    double *partials, int *counter, double *step) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int lb = Lrow[i], le = Lrow[i + 1];
    int lpos = lb;  // L entries of row i appear in the order of A's strict-lower entries
    for (int p = Arow[i]; p < Arow[i + 1]; ++p) {
      const int j = Acol[p];
      const int kmax = i < j ? i : j;
      CT s = (CT)Aval[p];
      int il = lb, iu = Ucp[j];
      const int ue = Ucp[j + 1];
      while (il < le && iu < ue) {
        const int jl = Lcol[il], ju = Uri[iu];
        if (jl >= kmax || ju >= kmax) break;
        if (jl == ju) {
          s = fma(-cvt<CT>(Lold[il]), cvt<CT>(Uold[iu]), s);
          ++il;
          ++iu;
        } else if (jl < ju) {
          ++il;
        } else {
          ++iu;
        }
      }
      if (i > j) {
        const CT nv = s / cvt<CT>(Uold[ue - 1]);
        while (Lcol[lpos] != j) ++lpos;
        const double d = to_f64(nv) - fval(Lold[lpos]);  // exact conversions on the integer pipes
        acc = fma(d, d, acc);
        Lnew[lpos] = cvt<FT>(nv);
        ++lpos;
      } else {
        while (Uri[iu] != i) ++iu;
        const double d = to_f64(s) - fval(Uold[iu]);
        acc = fma(d, d, acc);
        Unew[iu] = cvt<FT>(s);
      }
    }
  }
  finish_sum(acc, partials, counter, step);
}

// sum over S(A) of (sum_{k<=min(i,j)} l_ik u_kj - a_ij)^2
template <typename FT, typename CT>
__global__ void __launch_bounds__(kPTPB) k_ilu_residual(
    int n, const int *__restrict__ Arow, const int *__restrict__ Acol,
    const double *__restrict__ Aval, const int *__restrict__ Lrow, const int *__restrict__ Lcol,
    const FT *__restrict__ L, const int *__restrict__ Ucp, const int *__restrict__ Uri,
    const FT *__restrict__ U, double *partials, int *counter, double *out) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int lb = Lrow[i], le = Lrow[i + 1];
    for (int p = Arow[i]; p < Arow[i + 1]; ++p) {
      const int j = Acol[p];
      double t = 0.0;
      int il = lb, iu = Ucp[j];
      const int ue = Ucp[j + 1];
      while (il < le && iu < ue) {
        const int jl = Lcol[il], ju = Uri[iu];
        if (jl == ju) {
          t = fma(fval(L[il]), fval(U[iu]), t);
          ++il;
          ++iu;
        } else if (jl < ju) {
          ++il;
        } else {
          ++iu;
        }
      }
      const double d = t - Aval[p];
      acc = fma(d, d, acc);
    }
  }
  finish_sum(acc, partials, counter, out);
}

// ||LU||_F^2 and sum over S(A) of (LU)_ij^2, thread per row: row i of LU is
// sum_k l_ik U(k,:), so ||(LU)(i,:)||^2 = sum_{k,k'} l_ik l_ik' <U(k,:),U(k',:)>
// (sparse dots of U's CSR rows).  With the S(A) part of the ILU residual this
// gives LACE's full residual ||LU - A|| over pattern(LU) (control/norms.cpp:
// 389-398) without forming LU:  res^2 = sum_S (LU-A)^2 + ||LU||^2 - sum_S LU^2,
// S = the entries of A that the product's pattern holds (LACE skips the
// others, :380-388).  unit: L's diagonal entries count as 1 (a CSRL L with
// unit diagonal); otherwise L's values as stored (data_zilures_bcsr).
template <typename FT, typename CT>
__global__ void __launch_bounds__(kPTPB) k_lu_fro(
    int n, const int *__restrict__ Arow, const int *__restrict__ Acol, const double *__restrict__ Aval,
    const int *__restrict__ Lrow, const int *__restrict__ Lcol, const FT *__restrict__ L,
    const int *__restrict__ Urow, const int *__restrict__ Ucol, const FT *__restrict__ Ur,
    const int *__restrict__ Ucp, const int *__restrict__ Uri, const FT *__restrict__ Uc, double *partials,
    int *counter, double *out3, int unit) {
  double fro = 0.0, onS = 0.0, nl = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int lb = Lrow[i], le = Lrow[i + 1];
    for (int a = lb; a < le; ++a) {
      const int k = Lcol[a];
      const double lk = (unit && k == i) ? 1.0 : fval(L[a]);
      for (int b = a; b < le; ++b) {
        const int k2 = Lcol[b];
        const double lk2 = (unit && k2 == i) ? 1.0 : fval(L[b]);
        double dot = 0.0;
        int p = Urow[k], q = Urow[k2];
        const int pe = Urow[k + 1], qe = Urow[k2 + 1];
        while (p < pe && q < qe) {
          const int cp = Ucol[p], cq = Ucol[q];
          if (cp == cq) {
            dot = fma(fval(Ur[p]), fval(Ur[q]), dot);
            ++p;
            ++q;
          } else if (cp < cq) {
            ++p;
          } else {
            ++q;
          }
        }
        fro = fma((a == b ? 1.0 : 2.0) * lk * lk2, dot, fro);
      }
    }
    for (int p = Arow[i]; p < Arow[i + 1]; ++p) {
      const int j = Acol[p];
      double t = 0.0;
      bool hit = false;
      int il = lb, iu = Ucp[j];
      const int ue = Ucp[j + 1];
      while (il < le && iu < ue) {
        const int jl = Lcol[il], ju = Uri[iu];
        if (jl == ju) {
          t = fma((unit && jl == i) ? 1.0 : fval(L[il]), fval(Uc[iu]), t);
          hit = true;
          ++il;
          ++iu;
        } else if (jl < ju) {
          ++il;
        } else {
          ++iu;
        }
      }
      if (!hit) continue;  // (i, j) is not in the product's pattern
      onS = fma(t, t, onS);
      const double d = t - Aval[p];  // the nonlinear residual's entry, from the same product
      nl = fma(d, d, nl);
    }
  }
  // three sums: fold each through the deterministic last-block protocol
  double t1 = block_sum_p(fro);
  double t2 = block_sum_p(onS);
  double t3 = block_sum_p(nl);
  if (threadIdx.x == 0) {
    partials[3 * blockIdx.x] = t1;
    partials[3 * blockIdx.x + 1] = t2;
    partials[3 * blockIdx.x + 2] = t3;
  }
  if (!arrive_last(counter)) return;
  const double s1 = block_fold(partials, 3, (int)gridDim.x);
  const double s2 = block_fold(partials + 1, 3, (int)gridDim.x);
  const double s3 = block_fold(partials + 2, 3, (int)gridDim.x);
  if (threadIdx.x == 0) {
    out3[0] = s1;
    out3[1] = s2;
    out3[2] = s3;
  }
}

void launch_lu_fro(cudaStream_t s, const IluArgs &a, VType t, const int *Urow, const int *Ucol,
                   const void *L, const void *Ur, const void *Uc, double *out3, int unit) {
  const int grid = sweep_grid_pub(a.n);
  if (t == VType::F64)
    k_lu_fro<double, double><<<grid, kPTPB, 0, s>>>(a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const double *)L,
                                                    Urow, Ucol, (const double *)Ur, a.Ucp, a.Uri,
                                                    (const double *)Uc, a.partials, a.counter, out3, unit);
  else if (t == VType::F32)
    k_lu_fro<float, float><<<grid, kPTPB, 0, s>>>(a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const float *)L,
                                                  Urow, Ucol, (const float *)Ur, a.Ucp, a.Uri, (const float *)Uc,
                                                  a.partials, a.counter, out3, unit);
  else
    k_lu_fro<__nv_bfloat16, float><<<grid, kPTPB, 0, s>>>(
        a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const __nv_bfloat16 *)L, Urow, Ucol,
        (const __nv_bfloat16 *)Ur, a.Ucp, a.Uri, (const __nv_bfloat16 *)Uc, a.partials, a.counter, out3, unit);
}

// ---------------------------------------------------------------- BCSR
// Block sweep (src/parilu_v0_3_bcsr.cpp:129-249 in synchronous form):
//   S = A_ij - sum_{k<min} L_ik U_kj ;  L_ij = S inv(U_jj) (i > j), U_ij = S.
// One thread per (block, row-of-block): the bs threads of a block cooperate
// through shared memory for the S inv(U_jj) product.  U blocks (BCSC) are
// stored untransposed, as LACE keeps them (control/magma_zmtranspose.cpp:358-363).
template <typename FT, typename CT>
__device__ void blk_inverse(int bs, const CT *a, CT *inv) {
  // Gauss-Jordan without pivoting (LACE's data_inverse is LU without
  // pivoting, src/inverse.cpp:46); bs <= 8
  CT w[8][16];
  for (int r = 0; r < bs; ++r)
    for (int c = 0; c < 2 * bs; ++c) w[r][c] = (c < bs) ? a[r * bs + c] : (CT)(c - bs == r ? 1 : 0);
  for (int p = 0; p < bs; ++p) {
    CT rp = (CT)1 / w[p][p];
    for (int c = 0; c < 2 * bs; ++c) w[p][c] *= rp;
    for (int r = 0; r < bs; ++r) {
      if (r == p) continue;
      CT f = w[r][p];
      for (int c = 0; c < 2 * bs; ++c) w[r][c] -= f * w[p][c];
    }
  }
  for (int r = 0; r < bs; ++r)
    for (int c = 0; c < bs; ++c) inv[r * bs + c] = w[r][bs + c];
}

template <typename FT, typename CT>
__global__ void __launch_bounds__(kPTPB) k_bcsr_parilu_sweep(
    int nb, int bs, const int *__restrict__ Arow, const int *__restrict__ Acol,
    const double *__restrict__ Aval, const int *__restrict__ Lrow, const int *__restrict__ Lcol,
    const FT *__restrict__ Lold, FT *__restrict__ Lnew, const int *__restrict__ Ucp,
    const int *__restrict__ Uri, const FT *__restrict__ Uold, FT *__restrict__ Unew,
    double *partials, int *counter, double *step) {
  const int ld = bs * bs;
  double acc = 0.0;
  // one thread per block row of A
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nb; I += gridDim.x * blockDim.x) {
    const int lb = Lrow[I], le = Lrow[I + 1];
    int lpos = lb;
    for (int p = Arow[I]; p < Arow[I + 1]; ++p) {
      const int J = Acol[p];
      const int kmax = I < J ? I : J;
      CT S[64];
      for (int e = 0; e < ld; ++e) S[e] = (CT)Aval[(size_t)p * ld + e];
      int il = lb, iu = Ucp[J];
      const int ue = Ucp[J + 1];
      while (il < le && iu < ue) {
        const int jl = Lcol[il], ju = Uri[iu];
        if (jl >= kmax || ju >= kmax) break;
        if (jl == ju) {
          const FT *Lb = Lold + (size_t)il * ld;
          const FT *Ub = Uold + (size_t)iu * ld;
          for (int r = 0; r < bs; ++r)
            for (int c = 0; c < bs; ++c) {
              CT t = 0;
              for (int q = 0; q < bs; ++q) t = fma(cvt<CT>(Lb[r * bs + q]), cvt<CT>(Ub[q * bs + c]), t);
              S[r * bs + c] -= t;
            }
          ++il;
          ++iu;
        } else if (jl < ju) {
          ++il;
        } else {
          ++iu;
        }
      }
      if (I > J) {
        CT D[64], Di[64];
        const FT *Ud = Uold + (size_t)(ue - 1) * ld;
        for (int e = 0; e < ld; ++e) D[e] = cvt<CT>(Ud[e]);
        blk_inverse<FT, CT>(bs, D, Di);
        while (Lcol[lpos] != J) ++lpos;
        FT *Ln = Lnew + (size_t)lpos * ld;
        const FT *Lo = Lold + (size_t)lpos * ld;
        for (int r = 0; r < bs; ++r)
          for (int c = 0; c < bs; ++c) {
            CT t = 0;
            for (int q = 0; q < bs; ++q) t = fma(S[r * bs + q], Di[q * bs + c], t);
            const double d = (double)t - (double)cvt<CT>(Lo[r * bs + c]);
            acc = fma(d, d, acc);
            Ln[r * bs + c] = cvt<FT>(t);
          }
        ++lpos;
      } else {
        while (Uri[iu] != I) ++iu;
        FT *Un = Unew + (size_t)iu * ld;
        const FT *Uo = Uold + (size_t)iu * ld;
        for (int e = 0; e < ld; ++e) {
          const double d = (double)S[e] - (double)cvt<CT>(Uo[e]);
          acc = fma(d, d, acc);
          Un[e] = cvt<FT>(S[e]);
        }
      }
    }
  }
  finish_sum(acc, partials, counter, step);
}

template <typename FT, typename CT>
__global__ void __launch_bounds__(kPTPB) k_block_diag_inverse(int nb, int bs,
                                                              const int *__restrict__ Urow,
                                                              const FT *__restrict__ U,
                                                              FT *__restrict__ dinv, int *status) {
  const int ld = bs * bs;
  for (int I = blockIdx.x * blockDim.x + threadIdx.x; I < nb; I += gridDim.x * blockDim.x) {
    CT D[64], Di[64];
    const FT *Ud = U + (size_t)Urow[I] * ld;  // diagonal block first in its block row
    for (int e = 0; e < ld; ++e) D[e] = cvt<CT>(Ud[e]);
    blk_inverse<FT, CT>(bs, D, Di);
    bool bad = false;
    for (int e = 0; e < ld; ++e) {
      if (!(Di[e] == Di[e]) || isinf((double)Di[e])) bad = true;
      dinv[(size_t)I * ld + e] = cvt<FT>(Di[e]);
    }
    if (bad) atomicOr(status, kStatusBreakdown);
  }
}

// ------------------------------------------------------------ helpers

template <typename S, typename D>
__global__ void k_gather(int count, const int *__restrict__ perm, const S *__restrict__ src,
                         D *__restrict__ dst) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < count; p += gridDim.x * blockDim.x) {
    const int q = perm ? perm[p] : p;
    dst[p] = cvt<D>(src[q]);
  }
}

template <typename S>
static void gather_dst(cudaStream_t s, int count, const int *perm, const S *src, VType td, void *dst) {
  int grid = min((count + 255) / 256, num_sms() * 16);
  if (grid < 1) return;
  switch (td) {
    case VType::F64: k_gather<S, double><<<grid, 256, 0, s>>>(count, perm, src, (double *)dst); break;
    case VType::F32: k_gather<S, float><<<grid, 256, 0, s>>>(count, perm, src, (float *)dst); break;
    case VType::BF16: k_gather<S, __nv_bfloat16><<<grid, 256, 0, s>>>(count, perm, src, (__nv_bfloat16 *)dst); break;
  }
}

void launch_gather(cudaStream_t s, int count, const int *perm, VType ts, const void *src, VType td,
                   void *dst) {
  switch (ts) {
    case VType::F64: gather_dst<double>(s, count, perm, (const double *)src, td, dst); break;
    case VType::F32: gather_dst<float>(s, count, perm, (const float *)src, td, dst); break;
    case VType::BF16: gather_dst<__nv_bfloat16>(s, count, perm, (const __nv_bfloat16 *)src, td, dst); break;
  }
}

void launch_convert(cudaStream_t s, int count, VType ts, const void *src, VType td, void *dst) {
  launch_gather(s, count, nullptr, ts, src, td, dst);
}

static int sweep_grid(int rows) {
  int g = (rows + kPTPB - 1) / kPTPB;
  int cap = num_sms() * 8;
  return g < 1 ? 1 : (g > cap ? cap : g);
}

// ---------------------------------------------------------------- A order
// The synchronous sweep over A's entries in A's own order, on one array F of
// factor values in A's order (F[p] = l_ij for i > j, u_ij for i <= j; L's
// unit diagonal implicit).  The pattern's merges are done once on the host:
// for entry p = (i,j) the positions in A of the pairs (l_ik, u_kj) with
// k < min(i,j), in ascending k (pairs[pptr[p] .. pptr[p+1])), and for i > j
// the position of u_jj (dpos[p], -1 for i <= j).  A sweep is then a stream
// of A's values and the per-entry records, coalesced, thread per entry, with
// the few pair operands gathered from the previous F (on a 7-point stencil
// three pairs per row, all on the diagonal entry):
//     s = a_ij - sum_k l_ik u_kj          (ascending k, as the merge walk)
//     F_new[p] = i > j ? s / u_jj : s
// The step sum (F_new - F_old)^2 is accumulated per thread in the compute
// type and folded in FP64 across the grid.
// Each thread takes U entries a grid stride apart (coalesced across the
// warp): their independent loads first, then their pair records PU at a
// time with all the operands of a batch gathered together, then the
// arithmetic.  MINB: blocks per SM the register budget is set for.  On the
// 128^3 convection-diffusion system one entry per thread with three pairs
// per batch at full occupancy measured fastest (93 us against 113-151 us for
// two or four entries per thread at lower occupancy); the autotune keeps
// the choice per pattern.
template <typename FT, typename CT, int U, int PU, int MINB>
__global__ void __launch_bounds__(kPTPB, MINB) k_parilu_sweep_ao(int nnz, const double *__restrict__ Aval,
                                                                 const int *__restrict__ dpos,
                                                                 const int *__restrict__ pptr,
                                                                 const int2 *__restrict__ pairs,
                                                                 const FT *__restrict__ Fold, FT *__restrict__ Fnew,
                                                                 double *partials, int *counter, double *step) {
  CT acc = (CT)0;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x + threadIdx.x; base < nnz; base += U * stride) {
    CT sv[U], dv[U], fo[U];
    int b[U], cnt[U];
    bool isl[U];
    int most = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = base + u * stride;
      b[u] = 0;
      cnt[u] = 0;
      sv[u] = (CT)0;
      dv[u] = (CT)1;
      fo[u] = (CT)0;
      isl[u] = false;
      if (p < nnz) {
        sv[u] = (CT)__ldcs(Aval + p);
        b[u] = __ldcs(pptr + p);
        cnt[u] = __ldg(pptr + p + 1) - b[u];
        const int d = __ldcs(dpos + p);
        isl[u] = d >= 0;
        if (isl[u]) dv[u] = cvt<CT>(Fold[d]);
        fo[u] = cvt<CT>(Fold[p]);
      }
      most = max(most, cnt[u]);
    }
    for (int k0 = 0; k0 < most; k0 += PU) {
      int2 pr[U][PU];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < PU; ++j) pr[u][j] = k0 + j < cnt[u] ? __ldg(pairs + b[u] + k0 + j) : make_int2(-1, -1);
      CT lv[U][PU], uv[U][PU];
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < PU; ++j) {
          lv[u][j] = pr[u][j].x >= 0 ? cvt<CT>(Fold[pr[u][j].x]) : (CT)0;
          uv[u][j] = pr[u][j].x >= 0 ? cvt<CT>(Fold[pr[u][j].y]) : (CT)0;
        }
#pragma unroll
      for (int u = 0; u < U; ++u)
#pragma unroll
        for (int j = 0; j < PU; ++j)
          if (k0 + j < cnt[u]) sv[u] = fma(-lv[u][j], uv[u][j], sv[u]);
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = base + u * stride;
      if (p < nnz) {
        const CT nv = isl[u] ? sv[u] / dv[u] : sv[u];
        const CT df = nv - fo[u];
        acc = fma(df, df, acc);
        Fnew[p] = cvt<FT>(nv);
      }
    }
  }
  finish_sum((double)acc, partials, counter, step);
}

// dst[q] = map[q] >= 0 ? src[map[q]] : 1 (L's unit diagonal), same value type
template <typename T>
__global__ void k_factor_gather(int count, const int *__restrict__ map, const T *__restrict__ src,
                                T *__restrict__ dst) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < count; q += gridDim.x * blockDim.x) {
    const int m = map[q];
    dst[q] = m >= 0 ? src[m] : cvt<T>(1.0f);
  }
}

template <int U, int PU, int MINB>
static void sweep_ao_variant(cudaStream_t s, int nnz, VType t, const double *Aval, const int *dpos, const int *pptr,
                             const int2 *pairs, const void *Fold, void *Fnew, double *partials, int *counter,
                             double *step) {
  int grid = (nnz + kPTPB * U - 1) / (kPTPB * U);
  const int cap = num_sms() * MINB;
  grid = grid < 1 ? 1 : (grid > cap ? cap : grid);
  if (t == VType::F64)
    k_parilu_sweep_ao<double, double, U, PU, MINB><<<grid, kPTPB, 0, s>>>(
        nnz, Aval, dpos, pptr, pairs, (const double *)Fold, (double *)Fnew, partials, counter, step);
  else if (t == VType::F32)
    k_parilu_sweep_ao<float, float, U, PU, MINB><<<grid, kPTPB, 0, s>>>(
        nnz, Aval, dpos, pptr, pairs, (const float *)Fold, (float *)Fnew, partials, counter, step);
  else
    k_parilu_sweep_ao<__nv_bfloat16, float, U, PU, MINB><<<grid, kPTPB, 0, s>>>(
        nnz, Aval, dpos, pptr, pairs, (const __nv_bfloat16 *)Fold, (__nv_bfloat16 *)Fnew, partials, counter, step);
}

int parilu_sweep_variants() { return 4; }

void launch_parilu_sweep_ao(cudaStream_t s, int nnz, VType t, const double *Aval, const int *dpos,
                            const int *pptr, const int2 *pairs, const void *Fold, void *Fnew, double *partials,
                            int *counter, double *step, int variant) {
  switch (variant) {
    case 1: sweep_ao_variant<1, 2, 8>(s, nnz, t, Aval, dpos, pptr, pairs, Fold, Fnew, partials, counter, step); break;
    case 2: sweep_ao_variant<1, 4, 8>(s, nnz, t, Aval, dpos, pptr, pairs, Fold, Fnew, partials, counter, step); break;
    case 3: sweep_ao_variant<2, 3, 6>(s, nnz, t, Aval, dpos, pptr, pairs, Fold, Fnew, partials, counter, step); break;
    default: sweep_ao_variant<1, 3, 8>(s, nnz, t, Aval, dpos, pptr, pairs, Fold, Fnew, partials, counter, step); break;
  }
}

void launch_factor_gather(cudaStream_t s, int count, const int *map, VType t, const void *src, void *dst) {
  int grid = (count + 255) / 256;
  const int cap = num_sms() * 8;
  grid = grid < 1 ? 1 : (grid > cap ? cap : grid);
  if (t == VType::F64)
    k_factor_gather<double><<<grid, 256, 0, s>>>(count, map, (const double *)src, (double *)dst);
  else if (t == VType::F32)
    k_factor_gather<float><<<grid, 256, 0, s>>>(count, map, (const float *)src, (float *)dst);
  else
    k_factor_gather<__nv_bfloat16><<<grid, 256, 0, s>>>(count, map, (const __nv_bfloat16 *)src,
                                                        (__nv_bfloat16 *)dst);
}

// ------------------------------------------------------ BCSR, A order
// The block sweep in A's block order (block sizes up to 5: a block's BS*BS
// values on one warp's lanes, lane r*BS + c holding entry (r, c)), on the
// block analogue of F: F[p] = L_IJ (I > J) or U_IJ (I <= J) as a BS*BS
// row-major block, L's identity diagonal blocks implicit.  Per block, from
// the pair records of the scalar sweep (pattern-level):
//     S = A_IJ - sum_K L_IK U_KJ      (each product an FMA chain over q, then
//                                      subtracted, as the row-walking kernel)
//     F_new[p] = I > J ? S inv(U_JJ) : S
// inv(U_JJ) of the previous iterate comes from k_bcsr_diag_inverse_warp,
// once per sweep and block row, not once per L block.  A warp keeps two
// blocks in flight.
template <typename FT, typename CT, int BS>
__global__ void __launch_bounds__(kPTPB) k_bcsr_parilu_sweep_ao(int nnzb, const double *__restrict__ Aval,
                                                                const int *__restrict__ Acol,
                                                                const int *__restrict__ dpos,
                                                                const int *__restrict__ pptr,
                                                                const int2 *__restrict__ pairs,
                                                                const CT *__restrict__ Dinv,
                                                                const FT *__restrict__ Fold, FT *__restrict__ Fnew,
                                                                double *partials, int *counter, double *step) {
  constexpr int LD = BS * BS;
  constexpr int U = 2;
  const int lane = threadIdx.x & 31;
  const bool on = lane < LD;
  const int r = lane / BS, c = lane % BS;
  const int e = on ? lane : 0;
  CT acc = (CT)0;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  for (int base = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; base < nnzb; base += U * nw) {
    CT sv[U], fo[U], di[U];
    int b[U], cnt[U];
    bool isl[U];
    int most = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = base + u * nw;
      sv[u] = fo[u] = di[u] = (CT)0;
      b[u] = cnt[u] = 0;
      isl[u] = false;
      if (p < nnzb) {
        sv[u] = on ? (CT)__ldcs(Aval + (size_t)p * LD + e) : (CT)0;
        fo[u] = on ? cvt<CT>(Fold[(size_t)p * LD + e]) : (CT)0;
        b[u] = __ldg(pptr + p);
        cnt[u] = __ldg(pptr + p + 1) - b[u];
        isl[u] = __ldg(dpos + p) >= 0;
        if (isl[u]) di[u] = on ? Dinv[(size_t)__ldg(Acol + p) * LD + e] : (CT)0;
      }
      most = max(most, cnt[u]);
    }
    for (int k = 0; k < most; ++k) {
      CT lv[U], uv[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        lv[u] = uv[u] = (CT)0;
        if (k < cnt[u]) {
          const int2 pr = __ldg(pairs + b[u] + k);
          lv[u] = on ? cvt<CT>(Fold[(size_t)pr.x * LD + e]) : (CT)0;
          uv[u] = on ? cvt<CT>(Fold[(size_t)pr.y * LD + e]) : (CT)0;
        }
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        if (k < cnt[u]) {  // warp-uniform: the whole warp works on block u
          CT t = (CT)0;
#pragma unroll
          for (int q = 0; q < BS; ++q)
            t = fma(__shfl_sync(0xffffffffu, lv[u], r * BS + q), __shfl_sync(0xffffffffu, uv[u], q * BS + c), t);
          sv[u] -= t;
        }
      }
    }
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int p = base + u * nw;
      if (p >= nnzb) continue;  // warp-uniform
      CT nv = sv[u];
      if (isl[u]) {
        CT t = (CT)0;
#pragma unroll
        for (int q = 0; q < BS; ++q)
          t = fma(__shfl_sync(0xffffffffu, sv[u], r * BS + q), __shfl_sync(0xffffffffu, di[u], q * BS + c), t);
        nv = t;
      }
      if (on) {
        const CT df = nv - fo[u];
        acc = fma(df, df, acc);
        Fnew[(size_t)p * LD + e] = cvt<FT>(nv);
      }
    }
  }
  finish_sum((double)acc, partials, counter, step);
}

// inv of each block row's diagonal block of F, one block per warp: lane
// r*BS + c holds entry (r, c) of [D | I] in two registers, and each
// Gauss-Jordan step shares the pivot row and column by shuffles - the
// operations and their order are blk_inverse's.  A non-finite inverse sets
// the breakdown bit.
template <typename FT, typename CT, int BS>
__global__ void __launch_bounds__(kPTPB) k_bcsr_diag_inverse_warp(int nb, const int *__restrict__ diag,
                                                                  const FT *__restrict__ F, CT *__restrict__ Dinv,
                                                                  int *status) {
  constexpr int LD = BS * BS;
  const int lane = threadIdx.x & 31;
  const bool on = lane < LD;
  const int r = lane / BS, c = lane % BS;
  const int nw = (gridDim.x * blockDim.x) >> 5;
  bool bad = false;
  for (int I = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; I < nb; I += nw) {
    CT wl = on ? cvt<CT>(F[(size_t)__ldg(diag + I) * LD + lane]) : (CT)0;  // D
    CT wr = (on && r == c) ? (CT)1 : (CT)0;                                 // I
#pragma unroll
    for (int p = 0; p < BS; ++p) {
      const CT rp = (CT)1 / __shfl_sync(0xffffffffu, wl, p * BS + p);
      if (r == p) {
        wl *= rp;
        wr *= rp;
      }
      const CT f = __shfl_sync(0xffffffffu, wl, (r * BS + p) & 31);  // w[r][p], untouched for r != p
      const CT pl = __shfl_sync(0xffffffffu, wl, p * BS + c), pr = __shfl_sync(0xffffffffu, wr, p * BS + c);
      if (r != p) {
        wl -= f * pl;
        wr -= f * pr;
      }
    }
    if (on) {
      if (!(wr == wr) || isinf((double)wr)) bad = true;
      Dinv[(size_t)I * LD + lane] = wr;
    }
  }
  if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(status, kStatusBreakdown);
}

// block values from F to BCSRL / BCSCU positions: dst block q = src block
// map[q], or the identity (L's diagonal blocks) for map[q] < 0
template <typename T>
__global__ void k_factor_gather_blk(int count, int bs, const int *__restrict__ map, const T *__restrict__ src,
                                    T *__restrict__ dst) {
  const int ld = bs * bs;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)count * ld;
       q += (long long)gridDim.x * blockDim.x) {
    const int blk = (int)(q / ld), e = (int)(q % ld);
    const int m = map[blk];
    dst[q] = m >= 0 ? src[(size_t)m * ld + e] : cvt<T>((e / bs == e % bs) ? 1.0f : 0.0f);
  }
}

// one resident wave of a warp-per-item block kernel (the sweep, or the
// diagonal inverses): as many warps as the SMs hold at once, at most one per
// item (the kernels stride over the rest); a grid of more blocks than stay
// resident runs a second, partial wave
template <typename FT, typename CT, int BSV, bool SWEEP>
static int resident_grid(int items) {
  static const int per_sm = [] {
    int b = 0;
    const cudaError_t e =
        SWEEP ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bcsr_parilu_sweep_ao<FT, CT, BSV>, kPTPB, 0)
              : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, k_bcsr_diag_inverse_warp<FT, CT, BSV>, kPTPB, 0);
    if (e != cudaSuccess || b < 1) {
      cudaGetLastError();
      b = 1;
    }
    return b;
  }();
  const int grid = (items + kPTPB / 32 - 1) / (kPTPB / 32);
  return std::max(1, std::min(grid, num_sms() * per_sm));
}

template <typename FT, typename CT>
static void bcsr_sweep_ao_bs(cudaStream_t s, int bs, int nnzb, const double *Aval, const int *Acol,
                             const int *dpos, const int *pptr, const int2 *pairs, const void *Dinv, const void *Fold,
                             void *Fnew, double *partials, int *counter, double *step) {
#define LACE_BSW(BSV)                                                                                   \
  k_bcsr_parilu_sweep_ao<FT, CT, BSV><<<resident_grid<FT, CT, BSV, true>(nnzb), kPTPB, 0, s>>>(          \
      nnzb, Aval, Acol, dpos, pptr, pairs, (const CT *)Dinv, (const FT *)Fold, (FT *)Fnew, partials, counter, step)
  switch (bs) {
    case 1: LACE_BSW(1); break;
    case 2: LACE_BSW(2); break;
    case 3: LACE_BSW(3); break;
    case 4: LACE_BSW(4); break;
    default: LACE_BSW(5); break;
  }
#undef LACE_BSW
}

template <typename FT, typename CT>
static void diag_inverse_warp_bs(cudaStream_t s, int nb, int bs, const int *diag, const void *F, void *Dinv,
                                 int *status) {
#define LACE_DIW(BSV)                                                                                 \
  k_bcsr_diag_inverse_warp<FT, CT, BSV><<<resident_grid<FT, CT, BSV, false>(nb), kPTPB, 0, s>>>(       \
      nb, diag, (const FT *)F, (CT *)Dinv, status)
  switch (bs) {
    case 1: LACE_DIW(1); break;
    case 2: LACE_DIW(2); break;
    case 3: LACE_DIW(3); break;
    case 4: LACE_DIW(4); break;
    default: LACE_DIW(5); break;
  }
#undef LACE_DIW
}

void launch_bcsr_parilu_sweep_ao(cudaStream_t s, int nnzb, int bs, VType t, const double *Aval, const int *Acol,
                                 const int *dpos, const int *pptr, const int2 *pairs, const void *Dinv,
                                 const void *Fold, void *Fnew, double *partials, int *counter, double *step) {
  if (t == VType::F64)
    bcsr_sweep_ao_bs<double, double>(s, bs, nnzb, Aval, Acol, dpos, pptr, pairs, Dinv, Fold, Fnew, partials, counter,
                                     step);
  else if (t == VType::F32)
    bcsr_sweep_ao_bs<float, float>(s, bs, nnzb, Aval, Acol, dpos, pptr, pairs, Dinv, Fold, Fnew, partials, counter,
                                   step);
  else
    bcsr_sweep_ao_bs<__nv_bfloat16, float>(s, bs, nnzb, Aval, Acol, dpos, pptr, pairs, Dinv, Fold, Fnew, partials,
                                           counter, step);
}

void launch_bcsr_diag_inverse_ao(cudaStream_t s, int nb, int bs, const int *diag, VType t, const void *F,
                                 void *Dinv, int *status) {
  if (t == VType::F64) diag_inverse_warp_bs<double, double>(s, nb, bs, diag, F, Dinv, status);
  else if (t == VType::F32) diag_inverse_warp_bs<float, float>(s, nb, bs, diag, F, Dinv, status);
  else diag_inverse_warp_bs<__nv_bfloat16, float>(s, nb, bs, diag, F, Dinv, status);
}

void launch_factor_gather_blk(cudaStream_t s, int count, int bs, const int *map, VType t, const void *src,
                              void *dst) {
  const long long tot = (long long)count * bs * bs;
  int grid = (int)std::min<long long>((tot + 255) / 256, (long long)num_sms() * 16);
  if (grid < 1) return;
  if (t == VType::F64)
    k_factor_gather_blk<double><<<grid, 256, 0, s>>>(count, bs, map, (const double *)src, (double *)dst);
  else if (t == VType::F32)
    k_factor_gather_blk<float><<<grid, 256, 0, s>>>(count, bs, map, (const float *)src, (float *)dst);
  else
    k_factor_gather_blk<__nv_bfloat16><<<grid, 256, 0, s>>>(count, bs, map, (const __nv_bfloat16 *)src,
                                                            (__nv_bfloat16 *)dst);
}

void launch_parilu_sweep(cudaStream_t s, const IluArgs &a, VType t, const void *Lold, void *Lnew,
                         const void *Uold, void *Unew, double *step) {
  if (a.bs > 0) {
    const int grid = sweep_grid(a.n);
    if (t == VType::F64)
      k_bcsr_parilu_sweep<double, double><<<grid, kPTPB, 0, s>>>(
          a.n, a.bs, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const double *)Lold, (double *)Lnew,
          a.Ucp, a.Uri, (const double *)Uold, (double *)Unew, a.partials, a.counter, step);
    else if (t == VType::F32)
      k_bcsr_parilu_sweep<float, float><<<grid, kPTPB, 0, s>>>(
          a.n, a.bs, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const float *)Lold, (float *)Lnew,
          a.Ucp, a.Uri, (const float *)Uold, (float *)Unew, a.partials, a.counter, step);
    else
      k_bcsr_parilu_sweep<__nv_bfloat16, float><<<grid, kPTPB, 0, s>>>(
          a.n, a.bs, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const __nv_bfloat16 *)Lold,
          (__nv_bfloat16 *)Lnew, a.Ucp, a.Uri, (const __nv_bfloat16 *)Uold, (__nv_bfloat16 *)Unew,
          a.partials, a.counter, step);
    return;
  }
  const int grid = sweep_grid(a.n);
  if (t == VType::F64)
    k_parilu_sweep<double, double><<<grid, kPTPB, 0, s>>>(
        a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const double *)Lold, (double *)Lnew, a.Ucp,
        a.Uri, (const double *)Uold, (double *)Unew, a.partials, a.counter, step);
  else if (t == VType::F32)
    k_parilu_sweep<float, float><<<grid, kPTPB, 0, s>>>(
        a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const float *)Lold, (float *)Lnew, a.Ucp,
        a.Uri, (const float *)Uold, (float *)Unew, a.partials, a.counter, step);
  else
    k_parilu_sweep<__nv_bfloat16, float><<<grid, kPTPB, 0, s>>>(
        a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const __nv_bfloat16 *)Lold,
        (__nv_bfloat16 *)Lnew, a.Ucp, a.Uri, (const __nv_bfloat16 *)Uold, (__nv_bfloat16 *)Unew,
        a.partials, a.counter, step);
}

void launch_ilu_residual(cudaStream_t s, const IluArgs &a, VType t, const void *L, const void *U,
                         double *out) {
  const int grid = sweep_grid(a.n);
  if (t == VType::F64)
    k_ilu_residual<double, double><<<grid, kPTPB, 0, s>>>(a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol,
                                                          (const double *)L, a.Ucp, a.Uri,
                                                          (const double *)U, a.partials, a.counter, out);
  else if (t == VType::F32)
    k_ilu_residual<float, float><<<grid, kPTPB, 0, s>>>(a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol,
                                                        (const float *)L, a.Ucp, a.Uri,
                                                        (const float *)U, a.partials, a.counter, out);
  else
    k_ilu_residual<__nv_bfloat16, float><<<grid, kPTPB, 0, s>>>(
        a.n, a.Arow, a.Acol, a.Aval, a.Lrow, a.Lcol, (const __nv_bfloat16 *)L, a.Ucp, a.Uri,
        (const __nv_bfloat16 *)U, a.partials, a.counter, out);
}

void launch_block_diag_inverse(cudaStream_t s, int nb, int bs, const int *Urow, VType t,
                               const void *Uval, void *dinv, int *status) {
  const int grid = sweep_grid(nb);
  if (t == VType::F64)
    k_block_diag_inverse<double, double><<<grid, kPTPB, 0, s>>>(nb, bs, Urow, (const double *)Uval,
                                                               (double *)dinv, status);
  else if (t == VType::F32)
    k_block_diag_inverse<float, float><<<grid, kPTPB, 0, s>>>(nb, bs, Urow, (const float *)Uval,
                                                             (float *)dinv, status);
  else
    k_block_diag_inverse<__nv_bfloat16, float><<<grid, kPTPB, 0, s>>>(
        nb, bs, Urow, (const __nv_bfloat16 *)Uval, (__nv_bfloat16 *)dinv, status);
}

}  // namespace lace
