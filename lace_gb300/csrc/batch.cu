// Batched solves (lace_gpu_batch_*): many independent systems, several
// right-hand sides each.
//
// lace_gpu_batch_create assembles the systems into one block-diagonal CSR
// operator on the batch's context (so the context's pattern analysis builds
// the A-order ParILU records for all of them at once) and, per system, the
// level sets of its two triangles.  lace_gpu_batch_solve then runs the whole
// solve - every system's ParILU sweeps and FGMRES-Householder for every
// (system, rhs) pair - as one persistent launch (batch_persist.cu), captured
// in a CUDA graph when the context's options ask for graphs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "context.h"

using namespace lace;

struct lace_gpu_batch {
  lace_gpu_ctx *ctx = nullptr;
  int nsys = 0, nrhs = 0, N = 0, nmax = 0;
  std::vector<int> n, row_off;
  DBuf dn, droff, lsys, lptr, lrows, usys, uptr, urows;  // per system and its levels
  DBuf cL, fL, cU, fU, dU;                               // level-ordered row records (columns, A positions)
  int w = 0;                                             // record width
  DBuf vrec;                                             // per CTA: the records' factor values
  DBuf jsys, jrhs, jnr;                                  // jobs: (system, first rhs, rhs count)
  int njobs = 0;
  size_t nnzmax = 0;                                     // the largest system's entries
  DBuf F;                                                // per CTA: factor values in A's order, twice
  DBuf V, W, Tm, Rm, Z, Q, Tt, ctl;                              // per-CTA workspace, queue and results
  int grid = 0, m = 0, f32 = -1;
};

namespace {

// levels of one triangle of system rows [r0, r0 + n) (global indices in
// the block-diagonal CSR): lower: a row's level is one more than the largest
// level of the columns left of it; upper: of the columns right of it.  Rows
// grouped by level in ascending order; ptr gets the level boundaries
// (relative to the concatenated rows), one entry per level start.
void levels(const std::vector<int> &row, const std::vector<int> &col, int r0, int n, bool lower,
            std::vector<int> &lev, std::vector<int> &ptr, std::vector<int> &rows) {
  int depth = 0;
  for (int k = 0; k < n; ++k) {
    const int i = lower ? r0 + k : r0 + n - 1 - k;
    int l = 0;
    for (int p = row[i]; p < row[i + 1]; ++p) {
      const int c = col[p];
      if (lower ? c < i : c > i) l = std::max(l, lev[c - r0] + 1);
    }
    lev[i - r0] = l;
    depth = std::max(depth, l + 1);
  }
  std::vector<int> cnt(depth + 1, 0);
  for (int k = 0; k < n; ++k) ++cnt[lev[k] + 1];
  for (int l = 0; l < depth; ++l) cnt[l + 1] += cnt[l];
  const int base = (int)rows.size();
  rows.resize(base + n);
  std::vector<int> fill(cnt.begin(), cnt.end() - 1);
  for (int k = 0; k < n; ++k) rows[base + fill[lev[k]]++] = r0 + k;  // ascending rows within a level
  for (int l = 0; l < depth; ++l) ptr.push_back(base + cnt[l]);
}

}  // namespace

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
    B->nmax = std::max(B->nmax, n[s]);
  }
  B->N = N;
  std::vector<int> Sr(N + 1, 0);
  long long nnz = 0;
  for (int s = 0; s < nsys; ++s) nnz += row[row_off[s] + s + n[s]] - row[row_off[s] + s];
  if (nnz > 0x7fffffffLL) {
    delete B;
    return set_err(DEV_ERR_NOT_SUPPORTED);
  }
  std::vector<int> Sc(nnz);
  std::vector<double> Sv(nnz);
  long long p = 0;
  for (int s = 0; s < nsys; ++s) {
    // system s's row pointers are local, stored at row[row_off[s] + s .. + n[s]]
    const int *rp = row + row_off[s] + s;
    for (int i = 0; i < n[s]; ++i) {
      for (int e = rp[i]; e < rp[i + 1]; ++e) {
        const int c = col[nnz_off[s] + e];
        if (c < 0 || c >= n[s]) {
          delete B;
          return set_err(DEV_ERR_ILLEGAL_VALUE);
        }
        Sc[p] = c + row_off[s];
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
  // per system: the triangles' levels; the queue order, largest first
  std::vector<int> lev(B->nmax), lsys(nsys + 1), usys(nsys + 1), lptr, lrows, uptr, urows;
  lrows.reserve(N);
  urows.reserve(N);
  for (int s = 0; s < nsys; ++s) {
    lsys[s] = (int)lptr.size();
    levels(Sr, Sc, row_off[s], n[s], true, lev, lptr, lrows);
    usys[s] = (int)uptr.size();
    levels(Sr, Sc, row_off[s], n[s], false, lev, uptr, urows);
  }
  lsys[nsys] = (int)lptr.size();
  usys[nsys] = (int)uptr.size();
  lptr.push_back(N);
  uptr.push_back(N);
  // level-ordered records of the two triangles: for the k-th row of the
  // level order, its off-diagonal entries' local columns and A positions
  // (W of them, -1 beyond the row's count) and, for U, its diagonal's position
  std::vector<int> dpos_row(N), sys_of(N);
  int W = 0;
  for (int s = 0; s < nsys; ++s)
    for (int i = row_off[s]; i < row_off[s] + n[s]; ++i) {
      sys_of[i] = s;
      int d = -1;
      for (int q = Sr[i]; q < Sr[i + 1]; ++q)
        if (Sc[q] == i) d = q;
      if (d < 0) {  // the upload checked this already
        delete B;
        return set_err(DEV_ERR_NOT_SUPPORTED);
      }
      dpos_row[i] = d;
      W = std::max(W, std::max(d - Sr[i], Sr[i + 1] - d - 1));
    }
  if (W > kBatchMaxW) {
    delete B;
    return set_err(DEV_ERR_NOT_SUPPORTED);
  }
  W = std::max(W, 1);
  B->w = W;
  std::vector<int> cLh((size_t)N * W, -1), fLh((size_t)N * W, -1), cUh((size_t)N * W, -1), fUh((size_t)N * W, -1),
      dUh(N);
  for (int k = 0; k < N; ++k) {
    const int gl = lrows[k], gu = urows[k];
    const int rl = row_off[sys_of[gl]], ru = row_off[sys_of[gu]];
    for (int q = Sr[gl], w = 0; q < dpos_row[gl]; ++q, ++w) {
      cLh[(size_t)k * W + w] = Sc[q] - rl;
      fLh[(size_t)k * W + w] = q;
    }
    for (int q = dpos_row[gu] + 1, w = 0; q < Sr[gu + 1]; ++q, ++w) {
      cUh[(size_t)k * W + w] = Sc[q] - ru;
      fUh[(size_t)k * W + w] = q;
    }
    dUh[k] = dpos_row[gu];
  }
  // jobs, largest systems first: a system of at least kSplitRows rows gives
  // each right-hand side its own job (its FGMRES processes run on different
  // SMs: the longest of them sets the launch's time), a smaller one takes its
  // right-hand sides in groups of up to four (the operator, factor and
  // level-barrier work shared)
  constexpr int kSplitRows = 16384;
  std::vector<int> order(nsys);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return n[a] > n[b]; });
  std::vector<int> jsys, jrhs, jnr;
  const int R = batch_persist_rhs();
  for (int s : order) {
    const int g = n[s] >= kSplitRows ? 1 : R;
    for (int r = 0; r < nrhs; r += g) {
      jsys.push_back(s);
      jrhs.push_back(r);
      jnr.push_back(std::min(g, nrhs - r));
    }
    B->nnzmax = std::max(B->nnzmax, (size_t)(Sr[row_off[s] + n[s]] - Sr[row_off[s]]));
  }
  B->njobs = (int)jsys.size();
  cudaStream_t st = ctx->stream;
  if (B->dn.upload(n, 4 * (size_t)nsys, st) || B->droff.upload(row_off, 4 * (size_t)nsys, st) ||
      B->jsys.upload(jsys.data(), 4 * jsys.size(), st) || B->jrhs.upload(jrhs.data(), 4 * jrhs.size(), st) ||
      B->jnr.upload(jnr.data(), 4 * jnr.size(), st) || B->lsys.upload(lsys.data(), 4 * lsys.size(), st) ||
      B->usys.upload(usys.data(), 4 * usys.size(), st) || B->lptr.upload(lptr.data(), 4 * lptr.size(), st) ||
      B->uptr.upload(uptr.data(), 4 * uptr.size(), st) || B->lrows.upload(lrows.data(), 4 * lrows.size(), st) ||
      B->urows.upload(urows.data(), 4 * urows.size(), st) || B->cL.upload(cLh.data(), 4 * cLh.size(), st) ||
      B->fL.upload(fLh.data(), 4 * fLh.size(), st) || B->cU.upload(cUh.data(), 4 * cUh.size(), st) ||
      B->fU.upload(fUh.data(), 4 * fUh.size(), st) || B->dU.upload(dUh.data(), 4 * dUh.size(), st)) {
    delete B;
    return set_err(DEV_ERR_DEVICE_ALLOC);
  }
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

// the per-CTA workspace for search_max m: one CTA per SM (the kernel's
// register budget), at most one per system
static int batch_workspace(lace_gpu_batch *B, int m, bool f32) {
  if (m == B->m && (int)f32 == B->f32 && B->V.p) return 0;
  const int R = batch_persist_rhs();
  B->grid = std::max(1, std::min(B->njobs, num_sms()));
  const size_t G = (size_t)B->grid, nmax = (size_t)B->nmax, ld = (size_t)m + 2;
  const size_t fb = f32 ? 4 : 8;
  int rc = 0;
  rc |= B->F.ensure(fb * G * 2 * (B->nnzmax + 4));
  rc |= B->vrec.ensure(fb * G * (2 * (size_t)B->w + 1) * nmax);
  rc |= B->V.ensure(8 * G * R * (m + 1) * nmax);
  rc |= B->W.ensure(8 * G * R * nmax);
  rc |= B->Tm.ensure(8 * G * R * ld * ld);
  rc |= B->Rm.ensure(8 * G * R * ld * ld);
  rc |= B->Z.ensure(fb * G * R * m * nmax);
  rc |= B->Q.ensure(fb * G * R * nmax);
  rc |= B->Tt.ensure(fb * G * R * nmax);
  rc |= B->ctl.ensure(4 * (1 + 2 * (size_t)B->nsys * B->nrhs));
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  B->m = m;
  B->f32 = f32;
  return 0;
}

extern "C" int lace_gpu_batch_solve(lace_gpu_batch *B, int sweeps, int search_max, int restart_max, double rtol,
                                    const double *b, double *x, int *iters_out) {
  if (!B || !b || !x) return set_err(DEV_ERR_INVALID_PTR);
  if (search_max < 1 || search_max > kBatchMaxM || sweeps < 0 || restart_max < 1)
    return set_err(DEV_ERR_NOT_SUPPORTED);
  lace_gpu_ctx *c = B->ctx;
  cudaSetDevice(c->device);
  if (c->opt.trsv_mode != LACE_TRSV_SYNCFREE) return set_err(DEV_ERR_NOT_SUPPORTED);
  if (!c->sweep_ao) return set_err(DEV_ERR_NOT_SUPPORTED);  // the A-order records
  const bool f32 = c->vtype() != VType::F64;
  int rc = batch_workspace(B, search_max, f32);
  if (rc) return set_err(rc);
  cudaStream_t s = c->stream;
  const size_t pairs = (size_t)B->nsys * B->nrhs;
  int *ctl = (int *)B->ctl.p;
  if (cudaMemsetAsync(ctl, 0, B->ctl.bytes, s) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
  PBatchHost h;
  h.nsys = B->nsys;
  h.nrhs = B->nrhs;
  h.m = search_max;
  h.restart_max = restart_max;
  h.sweeps = sweeps;
  h.N = B->N;
  h.grid = B->grid;
  h.f32 = f32 ? 1 : 0;
  h.rtol = rtol;
  h.njobs = B->njobs;
  h.jsys = (const int *)B->jsys.p;
  h.jrhs = (const int *)B->jrhs.p;
  h.jnr = (const int *)B->jnr.p;
  h.n = (const int *)B->dn.p;
  h.roff = (const int *)B->droff.p;
  h.lsys = (const int *)B->lsys.p;
  h.usys = (const int *)B->usys.p;
  h.Arow = (const int *)c->Arow.p;
  h.Acol = (const int *)c->Acol.p;
  h.Aval = (const double *)c->Aval.p;
  h.pptr = (const int *)c->sw_pptr.p;
  h.dpos = (const int *)c->sw_dpos.p;
  h.diag = (const int *)c->sw_diag.p;
  h.pairs = (const int2 *)c->sw_pairs.p;
  h.F = B->F.p;
  h.fstride = B->nnzmax + 4;
  h.lptr = (const int *)B->lptr.p;
  h.w = B->w;
  h.cL = (const int *)B->cL.p;
  h.fL = (const int *)B->fL.p;
  h.cU = (const int *)B->cU.p;
  h.fU = (const int *)B->fU.p;
  h.dU = (const int *)B->dU.p;
  h.vrec = B->vrec.p;
  h.lrows = (const int *)B->lrows.p;
  h.uptr = (const int *)B->uptr.p;
  h.urows = (const int *)B->urows.p;
  h.b = b;
  h.x = x;
  h.nmax = (size_t)B->nmax;
  h.V = (double *)B->V.p;
  h.W = (double *)B->W.p;
  h.Tm = (double *)B->Tm.p;
  h.Rm = (double *)B->Rm.p;
  h.Z = B->Z.p;
  h.Q = B->Q.p;
  h.Tt = B->Tt.p;
  h.next = ctl;
  h.iters = ctl + 1;
  h.conv = ctl + 1 + pairs;
  cudaGraphExec_t ge = nullptr;
  if (c->opt.use_graph) {
    // the one launch, captured and replayed as a graph
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
    rc = launch_batch_persist(s, h);
    const cudaError_t ce = cudaStreamEndCapture(s, &g);
    if (rc || ce != cudaSuccess) return set_err(rc ? rc : DEV_ERR_UNKNOWN);
    const cudaError_t ie = cudaGraphInstantiate(&ge, g, 0);
    cudaGraphDestroy(g);
    if (ie != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
    if (cudaGraphLaunch(ge, s) != cudaSuccess) {
      cudaGraphExecDestroy(ge);
      return set_err(DEV_ERR_UNKNOWN);
    }
  } else {
    rc = launch_batch_persist(s, h);
    if (rc) return set_err(rc);
  }
  std::vector<int> res(2 * pairs);
  const bool ok = cudaMemcpyAsync(res.data(), ctl + 1, 4 * res.size(), cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                  cudaStreamSynchronize(s) == cudaSuccess;
  if (ge) cudaGraphExecDestroy(ge);
  if (!ok) return set_err(DEV_ERR_UNKNOWN);
  bool all = true;
  for (size_t k = 0; k < pairs; ++k) {
    if (iters_out) iters_out[k] = res[k];
    all = all && res[pairs + k];
  }
  return all ? DEV_SUCCESS : DEV_NOTCONVERGED;
}
