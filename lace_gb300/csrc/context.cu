// GPU-resident context: device layout of the matrix, its factors and the
// Krylov workspace; the host drivers of ParILU, SpTRSV and FGMRES-Householder
// (the lace_gpu_* half of include/lace_gb300.h).
//
// HBM layout for one CSR system (n rows, nnz entries):
//   A      row[n+1] col[nnz] i32, val[nnz] f64
//   L      CSRL  (strict lower + unit diagonal last)  ptr/idx i32, 2 value buffers
//   U      CSCU  (column form, diagonal last) for the sweeps, 2 value buffers,
//          plus its CSR form (diagonal first) for the solves, with a position
//          map csr->csc (the CSR values are gathered after the sweeps)
//   L^T    CSR of L's transpose (adjoint solves), with a position map
//   per triangle: chunk kinds (u8), ready flags (i32), level lists (i32)
//   Krylov V[ldv x (m+1)] f64 column-major (ldv = n rounded up to 32, plus
//          32 so that columns are not a power of two bytes apart),
//          Z[ldv x m] f32 (mixed precision) or f64, w/q/t vectors
#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <thread>
#include <tuple>
#include <vector>

#include "context.h"
#include "hostpar.h"

namespace lace {

// pinned host scalars: the residual history of a cycle (up to kLdT), then
// single values at fixed slots
constexpr int kScalHost = 256;
constexpr int kScalCycleRnorm = 200;  // ||r|| at the start of the latest cycle
constexpr int kScalReorth = 201;      // the cycle's reorthogonalised steps (an int)

thread_local int g_last_error = 0;

int set_err(int code) {
  g_last_error = code;
  return code;
}

int cuda_code(cudaError_t e) {
  if (e == cudaSuccess) return DEV_SUCCESS;
  if (e == cudaErrorMemoryAllocation) return DEV_ERR_DEVICE_ALLOC;
  return DEV_ERR_UNKNOWN;
}

#define LCHK(expr)                                             \
  do {                                                         \
    cudaError_t e_ = (expr);                                   \
    if (e_ != cudaSuccess) return set_err(cuda_code(e_));      \
  } while (0)

// ------------------------------------------------------------ device buffers
void DBuf::free() {
  if (p) cudaFree(p);
  p = nullptr;
  bytes = 0;
}
// Injected allocation failure (lace_gpu_inject_alloc_failure): the number of
// device allocations still allowed to succeed; negative = no injection.
std::atomic<long long> g_alloc_budget{-1};

int DBuf::ensure(size_t b) {
  if (b <= bytes && p) return 0;
  free();
  if (b == 0) b = 16;
  if (g_alloc_budget.load() >= 0 && g_alloc_budget.fetch_sub(1) <= 0) {
    g_alloc_budget.store(0);
    p = nullptr;
    return DEV_ERR_DEVICE_ALLOC;
  }
  cudaError_t e = cudaMalloc(&p, b);
  if (e != cudaSuccess) {
    p = nullptr;
    cudaGetLastError();
    return DEV_ERR_DEVICE_ALLOC;
  }
  bytes = b;
  return 0;
}
int DBuf::upload(const void *h, size_t b, cudaStream_t s) {
  int rc = ensure(b);
  if (rc) return rc;
  if (b) {
    if (cudaMemcpyAsync(p, h, b, cudaMemcpyHostToDevice, s) != cudaSuccess) return DEV_ERR_UNKNOWN;
  }
  return 0;
}

static size_t vsize(VType t) { return t == VType::F64 ? 8 : (t == VType::F32 ? 4 : 2); }

// ---------------------------------------------------------- small kernels

// Lv[p] = 1 on the diagonal (map -1), A value otherwise, in value type T
template <typename T>
__global__ void k_init_from_A(int count, const int *__restrict__ map, const double *__restrict__ Aval,
                              int ld, T *__restrict__ out) {
  // ld > 1: block values (map indexes blocks), diagonal blocks = identity
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < (long long)count * ld;
       q += (long long)gridDim.x * blockDim.x) {
    const int p = (int)(q / ld), e = (int)(q % ld);
    const int src = map[p];
    double v;
    if (src >= 0) v = Aval[(size_t)src * ld + e];
    else {
      int bs = 1;
      while (bs * bs < ld) ++bs;
      v = (e / bs == e % bs) ? 1.0 : 0.0;
    }
    out[q] = cvt<T>(v);
  }
}

static void init_from_A(cudaStream_t s, int count, const int *map, const double *Aval, int ld,
                        VType t, void *out) {
  long long tot = (long long)count * ld;
  int grid = (int)std::min<long long>((tot + 255) / 256, (long long)num_sms() * 16);
  if (grid < 1) return;
  switch (t) {
    case VType::F64: k_init_from_A<double><<<grid, 256, 0, s>>>(count, map, Aval, ld, (double *)out); break;
    case VType::F32: k_init_from_A<float><<<grid, 256, 0, s>>>(count, map, Aval, ld, (float *)out); break;
    case VType::BF16: k_init_from_A<__nv_bfloat16><<<grid, 256, 0, s>>>(count, map, Aval, ld, (__nv_bfloat16 *)out); break;
  }
}

// *diff |= (a differs from b anywhere in count ints)
__global__ void k_pattern_diff(size_t count, const int *__restrict__ a, const int *__restrict__ b, int *diff) {
  bool d = false;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count; i += (size_t)gridDim.x * blockDim.x)
    d |= a[i] != b[i];
  if (__syncthreads_or(d) && threadIdx.x == 0) atomicOr(diff, 1);
}

// dLdA_ij = -lambda_i x_j on A's pattern (CSR order)
__global__ void k_grad_A(int n, const int *__restrict__ row, const int *__restrict__ col,
                         const double *__restrict__ lam, const double *__restrict__ x,
                         double *__restrict__ g) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const double li = lam[i];
    for (int p = row[i]; p < row[i + 1]; ++p) g[p] = -li * x[col[p]];
  }
}

// ------------------------------------------------------------- analysis

int validate_csr(int n, int nnz, const int *row, const int *col) {
  if (n < 0 || nnz < 0) return DEV_ERR_ILLEGAL_VALUE;
  if (row[0] != 0 || row[n] != nnz) return DEV_ERR_ILLEGAL_VALUE;
  // rows checked in parallel ranges; the first faulty row decides the code
  std::mutex mu;
  int bad_row = n, bad_code = 0;
  par_for((size_t)n, 65536, [&](size_t b, size_t e) {
    for (int i = (int)b; i < (int)e; ++i) {
      int code = 0;
      if (row[i + 1] < row[i]) {
        code = DEV_ERR_ILLEGAL_VALUE;
      } else {
        bool diag = false;
        for (int p = row[i]; p < row[i + 1] && !code; ++p) {
          if (col[p] < 0 || col[p] >= n) code = DEV_ERR_ILLEGAL_VALUE;
          else if (p > row[i] && col[p] <= col[p - 1]) code = DEV_ERR_NOT_SUPPORTED;  // unsorted / duplicate
          else if (col[p] == i) diag = true;
        }
        if (!code && !diag) code = DEV_ERR_NOT_SUPPORTED;  // ParILU needs every diagonal entry
      }
      if (code) {
        std::lock_guard<std::mutex> lk(mu);
        if (i < bad_row) {
          bad_row = i;
          bad_code = code;
        }
        return;
      }
    }
  });
  return bad_code;
}

void transpose_pattern(const Pattern &P, Pattern &T, std::vector<int> &t2p) {
  const int n = P.n;
  T.n = n;
  T.ptr.assign(n + 1, 0);
  for (int i : P.idx) T.ptr[i + 1]++;
  for (int i = 0; i < n; ++i) T.ptr[i + 1] += T.ptr[i];
  T.idx.resize(P.idx.size());
  t2p.resize(P.idx.size());
  std::vector<int> fill(T.ptr.begin(), T.ptr.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int p = P.ptr[i]; p < P.ptr[i + 1]; ++p) {
      const int q = fill[P.idx[p]]++;
      T.idx[q] = i;
      t2p[q] = p;
    }
}

int levels(const Pattern &T, bool lower, std::vector<int> &lptr, std::vector<int> &lrows) {
  const int n = T.n;
  std::vector<int> lev(n, 0);
  int nl = 0;
  for (int k = 0; k < n; ++k) {
    const int i = lower ? k : n - 1 - k;
    int l = 0;
    for (int p = T.ptr[i]; p < T.ptr[i + 1]; ++p) {
      const int j = T.idx[p];
      if (lower ? j < i : j > i) l = std::max(l, lev[j] + 1);
    }
    lev[i] = l;
    nl = std::max(nl, l + 1);
  }
  lptr.assign(nl + 1, 0);
  for (int i = 0; i < n; ++i) lptr[lev[i] + 1]++;
  for (int l = 0; l < nl; ++l) lptr[l + 1] += lptr[l];
  lrows.resize(n);
  std::vector<int> fill(lptr.begin(), lptr.end() - 1);
  for (int k = 0; k < n; ++k) {
    const int i = lower ? k : n - 1 - k;
    lrows[fill[lev[i]]++] = i;
  }
  return nl;
}

int build_blk_plan_host(const Pattern &T, bool lower, bool unit, int R, int cpb, HostPlan &hp) {
  if (cpb < 1 || cpb > kBlkMaxUnits) return DEV_ERR_ILLEGAL_VALUE;
  const int n = T.n;
  const int CS = 32 * R;
  const int nch = (n + CS - 1) / CS;
  const int nblk = (nch + cpb - 1) / cpb;
  std::vector<int> cblk(nch), lev(nch, 0);
  std::vector<uint8_t> kind(nch, 0);
  for (int p = 0; p < nch; ++p) cblk[lower ? p : nch - 1 - p] = p / cpb;
  std::vector<int> deps;
  for (int p = 0; p < nch; ++p) {
    const int c = lower ? p : nch - 1 - p;
    deps.clear();
    const int r0 = c * CS, r1 = std::min(n, r0 + CS);
    for (int i = r0; i < r1; ++i) {
      const int prev = lower ? i - 1 : i + 1;
      for (int e = T.ptr[i]; e < T.ptr[i + 1]; ++e) {
        const int j = T.idx[e];
        if (j == i || (lower ? j > i : j < i)) continue;
        const int cj = j / CS;
        if (cj == c) {
          if (j != prev) kind[c] = 1;
        } else {
          deps.push_back(cj);
        }
      }
    }
    // the level over all dependencies, in this block or an earlier one: the
    // step of the whole solve's wavefront at which the chunk can go
    int l = 0;
    for (int cj : deps) l = std::max(l, lev[cj] + 1);
    lev[c] = l;
  }
  // per block: chunks ordered by level (then by position).  A block that
  // straddles two stretches of the wavefront (the end of one plane of a
  // stencil and the start of the next) then has its warps take the chunks in
  // the order they become ready; an in-block dependency always has a lower
  // level, so the order stays topological.
  std::vector<int4> &blk = hp.blk, &urec = hp.urec;
  blk.assign(nblk, int4{});
  urec.clear();
  urec.reserve(nch);
  int max_units = 0;
  for (int b = 0; b < nblk; ++b) {
    const int p0 = b * cpb, p1 = std::min(nch, p0 + cpb);
    int lmin = INT_MAX, lmax = 0;
    for (int p = p0; p < p1; ++p) {
      lmin = std::min(lmin, lev[lower ? p : nch - 1 - p]);
      lmax = std::max(lmax, lev[lower ? p : nch - 1 - p]);
    }
    const int nl = lmax - lmin + 1;
    std::vector<int> cnt(nl + 1, 0);
    for (int p = p0; p < p1; ++p) cnt[lev[lower ? p : nch - 1 - p] - lmin + 1]++;
    for (int l = 0; l < nl; ++l) cnt[l + 1] += cnt[l];
    std::vector<int> order(p1 - p0);
    for (int p = p0; p < p1; ++p) {
      const int c = lower ? p : nch - 1 - p;
      order[cnt[lev[c] - lmin]++] = c;
    }
    const int u0 = (int)urec.size();
    for (int c : order) urec.push_back(make_int4(c, lev[c] | ((int)kind[c] << 30), 0, 0));
    blk[b] = make_int4(u0, (int)urec.size(), nl, (lower ? p0 : nch - p1) * CS);
    max_units = std::max(max_units, p1 - p0);
  }
  // the plan's own layout: per unit, where each row's dependencies are read
  // and which CSR entries give their values
  const int S = blk_slots(R);
  const size_t nu = urec.size();
  const size_t rs = nu * (size_t)R * 32;
  std::vector<int> &ucode = hp.ucode, &umap = hp.umap, &udiag = hp.udiag, &uprev = hp.uprev, &uflag = hp.uflag;
  ucode.assign(rs * S, -1);
  umap.assign(rs * S, -1);
  udiag.assign(rs, -1);
  uprev.assign(rs, -1);
  uflag.assign(nu * 32, 0);
  for (size_t u = 0; u < nu; ++u) {
    const int c = urec[u].x;
    const bool serial = kind[c] != 0;
    const int4 B = blk[cblk[c]];
    const int row0 = B.w, brows = (B.y - B.x) * CS;
    const int base = c * CS, cnt = std::min(CS, n - base);
    for (int lane = 0; lane < 32; ++lane)
      for (int r = 0; r < R; ++r) {
        const int pos = lane * R + r;
        if (pos >= cnt) continue;
        const int i = lower ? base + pos : base + cnt - 1 - pos;
        const int prev = lower ? i - 1 : i + 1;
        const size_t q = (u * R + r) * 32 + lane;
        int next = 0;
        for (int e = T.ptr[i]; e < T.ptr[i + 1]; ++e) {
          const int j = T.idx[e];
          if (j == i) {
            if (!unit) udiag[q] = e;
            continue;
          }
          if (lower ? j > i : j < i) continue;
          if (j / CS == c) {
            if (!serial && j == prev) uprev[q] = e;
            continue;
          }
          if (next < S) {
            const size_t qs = ((u * S + next) * R + r) * 32 + lane;
            const int slot = j - row0;
            ucode[qs] = (slot >= 0 && slot < brows) ? slot : -j - 2;
            umap[qs] = e;
          }
          ++next;
        }
        if (next > S) {  // solved from the CSR arrays
          uflag[u * 32 + lane] |= 1 << r;
          for (int t = 0; t < S; ++t) {
            const size_t qs = ((u * S + t) * R + r) * 32 + lane;
            ucode[qs] = -1;
            umap[qs] = -1;
          }
        }
      }
  }
  hp.n = n;
  hp.nch = nch;
  hp.R = R;
  hp.cpb = cpb;
  hp.lower = lower;
  hp.unit = unit;
  hp.max_units = max_units;
  return 0;
}

int upload_blk_plan(const HostPlan &hp, PlanBufs &pb, cudaStream_t s) {
  // a failed upload leaves no plan behind that points at freed buffers
  pb.valid = false;
  const int S = blk_slots(hp.R);
  const size_t nu = hp.urec.size(), rs = nu * (size_t)hp.R * 32;
  int rc = 0;
  rc |= pb.blk.upload(hp.blk.data(), sizeof(int4) * hp.blk.size(), s);
  rc |= pb.urec.upload(hp.urec.data(), sizeof(int4) * hp.urec.size(), s);
  rc |= pb.ucode.upload(hp.ucode.data(), 4 * hp.ucode.size(), s);
  rc |= pb.umap.upload(hp.umap.data(), 4 * hp.umap.size(), s);
  rc |= pb.udiag.upload(hp.udiag.data(), 4 * hp.udiag.size(), s);
  rc |= pb.uprev.upload(hp.uprev.data(), 4 * hp.uprev.size(), s);
  rc |= pb.uflag.upload(hp.uflag.data(), 4 * hp.uflag.size(), s);
  rc |= pb.uvs.ensure(8 * rs * S);
  rc |= pb.uaps.ensure(8 * rs);
  rc |= pb.urd.ensure(8 * rs);
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  // the caller's host vectors may go: wait for the uploads
  if (cudaStreamSynchronize(s) != cudaSuccess) return DEV_ERR_UNKNOWN;
  TriBlkPlan &d = pb.dev;
  d.n = hp.n;
  d.nchunks = hp.nch;
  d.nblocks = (int)hp.blk.size();
  d.nunits = (int)nu;
  d.R = hp.R;
  d.cpb = hp.cpb;
  d.lower = hp.lower ? 1 : 0;
  d.unit = hp.unit ? 1 : 0;
  d.blk = (const int4 *)pb.blk.p;
  d.urec = (const int4 *)pb.urec.p;
  d.max_units = hp.max_units;
  d.ucode = (const int *)pb.ucode.p;
  d.umap = (const int *)pb.umap.p;
  d.udiag = (const int *)pb.udiag.p;
  d.uprev = (const int *)pb.uprev.p;
  d.uflag = (const int *)pb.uflag.p;
  d.uvs = pb.uvs.p;
  d.uaps = pb.uaps.p;
  d.urd = pb.urd.p;
  pb.vals_version = -1;
  pb.valid = true;
  return 0;
}

// dst <- a device copy of src's plan (its buffers, shape and gathered values)
int copy_blk_plan(const PlanBufs &src, PlanBufs &dst, cudaStream_t s) {
  dst.valid = false;
  const DBuf *from[10] = {&src.blk, &src.urec, &src.ucode, &src.umap, &src.udiag,
                          &src.uprev, &src.uflag, &src.uvs, &src.uaps, &src.urd};
  DBuf *to[10] = {&dst.blk, &dst.urec, &dst.ucode, &dst.umap, &dst.udiag, &dst.uprev, &dst.uflag, &dst.uvs, &dst.uaps,
                  &dst.urd};
  for (int k = 0; k < 10; ++k) {
    if (to[k]->ensure(from[k]->bytes)) return DEV_ERR_DEVICE_ALLOC;
    if (from[k]->bytes &&
        cudaMemcpyAsync(to[k]->p, from[k]->p, from[k]->bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
      return DEV_ERR_UNKNOWN;
  }
  dst.dev = src.dev;
  TriBlkPlan &d = dst.dev;
  d.blk = (const int4 *)dst.blk.p;
  d.urec = (const int4 *)dst.urec.p;
  d.ucode = (const int *)dst.ucode.p;
  d.umap = (const int *)dst.umap.p;
  d.udiag = (const int *)dst.udiag.p;
  d.uprev = (const int *)dst.uprev.p;
  d.uflag = (const int *)dst.uflag.p;
  d.uvs = dst.uvs.p;
  d.uaps = dst.uaps.p;
  d.urd = dst.urd.p;
  dst.vals_version = src.vals_version;
  dst.vals_type = src.vals_type;
  dst.vals_src = src.vals_src;
  dst.valid = src.valid;
  return 0;
}

// exchange two plans (buffers move with the pointers into them)
void swap_blk_plans(PlanBufs &a, PlanBufs &b) {
  DBuf *x[10] = {&a.blk, &a.urec, &a.ucode, &a.umap, &a.udiag, &a.uprev, &a.uflag, &a.uvs, &a.uaps, &a.urd};
  DBuf *y[10] = {&b.blk, &b.urec, &b.ucode, &b.umap, &b.udiag, &b.uprev, &b.uflag, &b.uvs, &b.uaps, &b.urd};
  for (int k = 0; k < 10; ++k) {
    std::swap(x[k]->p, y[k]->p);
    std::swap(x[k]->bytes, y[k]->bytes);
  }
  std::swap(a.dev, b.dev);
  std::swap(a.valid, b.valid);
  std::swap(a.vals_version, b.vals_version);
  std::swap(a.vals_type, b.vals_type);
  std::swap(a.vals_src, b.vals_src);
}

int build_blk_plan(const Pattern &T, bool lower, bool unit, int R, int cpb, PlanBufs &pb, cudaStream_t s) {
  HostPlan hp;
  const int rc = build_blk_plan_host(T, lower, unit, R, cpb, hp);
  return rc ? rc : upload_blk_plan(hp, pb, s);
}

}  // namespace lace

using namespace lace;

// the block-scheduled plan of one triangle with the current schedule shape,
// its values gathered from the current factor values
int lace_gpu_ctx::ensure_plan(int which) {
  PlanBufs &pb = plans[which];
  TriDev t = tri(which);
  if (!(pb.valid && pb.dev.R == plan_R && pb.dev.cpb == plan_cpb)) {
    const Pattern *pats[4] = {&hL, &hU, &hUc, &hLt};
    const bool low[4] = {true, false, true, false};
    int rc;
    auto it = prebuilt.find(std::make_tuple(which, plan_R, plan_cpb));
    if (it != prebuilt.end()) {
      rc = upload_blk_plan(it->second, pb, stream);
      prebuilt.erase(it);  // uploaded: its host memory goes
    } else {
      rc = build_blk_plan(*pats[which], low[which], t.unit != 0, plan_R, plan_cpb, pb, stream);
    }
    if (rc) return rc;
  }
  pb.dev.row = t.row;
  pb.dev.col = t.col;
  pb.dev.warps = plan_warps;
  pb.dev.cl = plan_cl;
  const int per_sm = plan_warps == 1 ? 16 : (plan_warps <= 8 ? 4 : (plan_warps <= 16 ? 2 : 1));
  pb.dev.grid = std::min(pb.dev.nblocks, num_sms() * per_sm);
  if (pb.vals_version != fact_version || pb.vals_type != (int)vtype() || pb.vals_src != t.val) {
    launch_plan_values(stream, pb.dev, t.val, vtype());
    pb.vals_version = fact_version;
    pb.vals_type = (int)vtype();
    pb.vals_src = t.val;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

// ======================================================================
// context lifetime
// ======================================================================

extern "C" void lace_gpu_default_options(lace_gpu_options *o) {
  o->precision = LACE_PREC_FP64;
  o->trsv_mode = LACE_TRSV_SYNCFREE;
  o->jacobi_sweeps = 8;
  o->jacobi_tol = 0.0;
  o->use_graph = 1;
  o->spmv_lanes = 0;
  o->trsv_rows_per_lane = 0;
  o->monitor_orthog = 0;
  o->trsv_chunks_per_block = 0;
  o->trsv_warps = 0;
  o->trsv_cluster = 0;
}

extern "C" int lace_gpu_ctx_create(lace_gpu_ctx **out, int device, void *stream) {
  if (!out) return set_err(DEV_ERR_INVALID_PTR);
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_err(DEV_ERR_NOT_INITIALIZED);
  }
  if (device < 0 || device >= ndev) return set_err(DEV_ERR_ILLEGAL_VALUE);
  LCHK(cudaSetDevice(device));
  lace_gpu_ctx *c = new lace_gpu_ctx();
  c->device = device;
  c->verbose = getenv("LACE_GB300_VERBOSE") != nullptr;
  // LACE_GB300_MGS_STEP=0: the Gram-Schmidt step as separate kernels
  if (const char *e = getenv("LACE_GB300_MGS_STEP")) c->mgs_persistent = atoi(e) != 0;
  // LACE_GB300_HH_STEP=0: the Householder step as passes A, B, C
  if (const char *e = getenv("LACE_GB300_HH_STEP")) c->hh_persistent = atoi(e) != 0;
  lace_gpu_default_options(&c->opt);
  if (stream) {
    c->stream = (cudaStream_t)stream;
    c->own_stream = false;
  } else {
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete c;
      return set_err(DEV_ERR_UNKNOWN);
    }
    c->own_stream = true;
  }
  if (c->ctrl_buf.ensure(sizeof(Control) * 2) || c->cycle_buf.ensure(sizeof(Cycle)) ||
      c->scal_buf.ensure(64 * sizeof(double)) || c->cnt_buf.ensure(64 * sizeof(int))) {
    delete c;
    return set_err(DEV_ERR_DEVICE_ALLOC);
  }
  cudaMemsetAsync(c->ctrl_buf.p, 0, sizeof(Control) * 2, c->stream);
  cudaMemsetAsync(c->cycle_buf.p, 0, sizeof(Cycle), c->stream);
  cudaMemsetAsync(c->cnt_buf.p, 0, 64 * sizeof(int), c->stream);
  if (cudaMallocHost(&c->h_ctrl, sizeof(Control)) != cudaSuccess ||
      cudaMallocHost(&c->h_scal, kScalHost * sizeof(double)) != cudaSuccess) {
    delete c;
    return set_err(DEV_ERR_HOST_ALLOC);
  }
  if (cudaStreamSynchronize(c->stream) != cudaSuccess) {
    delete c;
    return set_err(DEV_ERR_UNKNOWN);
  }
  *out = c;
  return DEV_SUCCESS;
}

lace_gpu_ctx::~lace_gpu_ctx() {
  for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
  if (h_ctrl) cudaFreeHost(h_ctrl);
  if (h_scal) cudaFreeHost(h_scal);
  if (own_stream && stream) cudaStreamDestroy(stream);
  if (side) cudaStreamDestroy(side);
}

extern "C" int lace_gpu_ctx_destroy(lace_gpu_ctx *c) {
  if (!c) return DEV_SUCCESS;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  delete c;
  return DEV_SUCCESS;
}

extern "C" void *lace_gpu_stream(lace_gpu_ctx *c) { return c ? (void *)c->stream : nullptr; }

void lace_gpu_ctx::drop_graphs() {
  for (auto &kv : graphs) cudaGraphExecDestroy(kv.second);
  graphs.clear();
}

extern "C" int lace_gpu_set_options(lace_gpu_ctx *c, const lace_gpu_options *o) {
  if (!c || !o) return set_err(DEV_ERR_INVALID_PTR);
  if (o->precision < 0 || o->precision > 2 || o->trsv_mode < 0 || o->trsv_mode > 3)
    return set_err(DEV_ERR_ILLEGAL_VALUE);
  if (o->trsv_chunks_per_block < 0 || o->trsv_chunks_per_block > kBlkMaxUnits || o->trsv_warps < 0 ||
      o->trsv_warps > 16 ||
      !(o->trsv_cluster == 0 || o->trsv_cluster == 1 || o->trsv_cluster == 2 || o->trsv_cluster == 4 ||
        o->trsv_cluster == 8 || o->trsv_cluster == 16))
    return set_err(DEV_ERR_ILLEGAL_VALUE);
  const lace_gpu_options &p = c->opt;
  // the drop-in entry points set their options on every call: the same
  // options keep the captured cycle graphs and the tuned schedules
  if (o->precision == p.precision && o->trsv_mode == p.trsv_mode && o->jacobi_sweeps == p.jacobi_sweeps &&
      o->jacobi_tol == p.jacobi_tol && o->use_graph == p.use_graph && o->spmv_lanes == p.spmv_lanes &&
      o->trsv_rows_per_lane == p.trsv_rows_per_lane && o->monitor_orthog == p.monitor_orthog &&
      o->trsv_chunks_per_block == p.trsv_chunks_per_block && o->trsv_warps == p.trsv_warps &&
      o->trsv_cluster == p.trsv_cluster)
    return DEV_SUCCESS;
  const bool prec_changed = o->precision != p.precision;
  // a new schedule choice: tuned again before the next solve
  if (o->trsv_rows_per_lane != p.trsv_rows_per_lane || o->trsv_chunks_per_block != p.trsv_chunks_per_block ||
      o->trsv_warps != p.trsv_warps || o->trsv_cluster != p.trsv_cluster)
    c->trsv_tuned = false;
  c->opt = *o;
  c->drop_graphs();
  if (prec_changed) {
    c->factors_ready = false;
    c->trsv_tuned = false;  // the window and the best schedule depend on the value type
    c->bcsr_tuned = false;
  }
  if (o->trsv_rows_per_lane > 0) c->set_rows_per_lane(o->trsv_rows_per_lane);
  if (o->spmv_lanes > 0) c->lanes = o->spmv_lanes;
  return DEV_SUCCESS;
}

// ======================================================================
// upload + analysis
// ======================================================================

// wall time of setup phases, printed when the context is verbose
struct SetupClock {
  bool on;
  std::chrono::steady_clock::time_point t;
  explicit SetupClock(bool on_) : on(on_), t(std::chrono::steady_clock::now()) {}
  void mark(const char *what) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    printf("%% setup %-30s %8.2f ms\n", what, std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

int lace_gpu_ctx::analyse(int n_, const int *row, const int *col, int bs_) {
  SetupClock sc(verbose);
  n_blk = n_;
  bs = bs_;
  // L = strict lower + diagonal last (CSRL), U = diagonal + upper (CSRU):
  // counted per row, then filled, both over parallel row ranges
  Pattern L, Ur;
  L.n = Ur.n = n_;
  L.ptr.assign(n_ + 1, 0);
  Ur.ptr.assign(n_ + 1, 0);
  par_for((size_t)n_, 65536, [&](size_t b, size_t e) {
    for (int i = (int)b; i < (int)e; ++i) {
      int cl = 1, cu = 0;  // the unit diagonal of L
      for (int p = row[i]; p < row[i + 1]; ++p) {
        if (col[p] < i) ++cl;
        else ++cu;
      }
      L.ptr[i + 1] = cl;
      Ur.ptr[i + 1] = cu;
    }
  });
  for (int i = 0; i < n_; ++i) {
    L.ptr[i + 1] += L.ptr[i];
    Ur.ptr[i + 1] += Ur.ptr[i];
  }
  std::vector<int> l2a(L.ptr[n_]), ur2a(Ur.ptr[n_]);
  L.idx.resize(L.ptr[n_]);
  Ur.idx.resize(Ur.ptr[n_]);
  par_for((size_t)n_, 65536, [&](size_t b, size_t e) {
    for (int i = (int)b; i < (int)e; ++i) {
      int ql = L.ptr[i], qu = Ur.ptr[i];
      for (int p = row[i]; p < row[i + 1]; ++p) {
        const int j = col[p];
        if (j < i) {
          L.idx[ql] = j;
          l2a[ql++] = p;
        } else {
          Ur.idx[qu] = j;
          ur2a[qu++] = p;
        }
      }
      L.idx[ql] = i;
      l2a[ql] = -1;  // unit diagonal
    }
  });
  sc.mark("L/U split");
  int rc = analyse_factors(L, Ur);
  if (rc) return rc;
  std::vector<int> uc2a(hUc.idx.size());
  par_for(uc2a.size(), 1 << 20, [&](size_t b, size_t e) {
    for (size_t q = b; q < e; ++q) uc2a[q] = ur2a[uc2ur_h[q]];
  });
  rc |= map_l2a.upload(l2a.data(), 4 * l2a.size(), stream);
  rc |= map_uc2a.upload(uc2a.data(), 4 * uc2a.size(), stream);
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  sweep_ao = false;
  sweep_variant = -1;
  if (bs_ <= 5) {  // scalar entries, or blocks whose values fit one warp's lanes
    rc = build_sweep_records(row, col, L, Ur, l2a, ur2a, uc2a);
    if (rc) return rc;
    sc.mark("sweep records");
  }
  AT_ready = false;
  return 0;
}

// The A-order sweep's records (parilu.cu k_parilu_sweep_ao): for every entry
// p = (i,j) of A, the pairs (position of l_ik, position of u_kj) in A with
// k < min(i,j), ascending k (L row i merged with U column j), and for i > j
// the position of u_jj.  Counted per row, offset by one prefix sum and
// filled, over parallel row ranges.
int lace_gpu_ctx::build_sweep_records(const int *row, const int *col, const Pattern &L, const Pattern &Ur,
                                      const std::vector<int> &l2a, const std::vector<int> &ur2a,
                                      const std::vector<int> &uc2a) {
  const int nr = n_blk;
  const int nz = row[nr];
  std::vector<int> pptr((size_t)nz + 1, 0), dpos(std::max(1, nz), -1);
  auto walk = [&](int i, int p, int2 *out) {
    const int j = col[p];
    const int kmax = std::min(i, j);
    int il = L.ptr[i], ie = L.ptr[i + 1] - 1;  // strict lower part (the unit diagonal is last)
    int iu = hUc.ptr[j], ue = hUc.ptr[j + 1];
    int cnt = 0;
    while (il < ie && iu < ue) {
      const int kl = L.idx[il], ku = hUc.idx[iu];
      if (kl >= kmax || ku >= kmax) break;
      if (kl == ku) {
        if (out) out[cnt] = make_int2(l2a[il], uc2a[iu]);
        ++cnt;
        ++il;
        ++iu;
      } else if (kl < ku) {
        ++il;
      } else {
        ++iu;
      }
    }
    return cnt;
  };
  par_for((size_t)nr, 16384, [&](size_t b, size_t e) {
    for (int i = (int)b; i < (int)e; ++i)
      for (int p = row[i]; p < row[i + 1]; ++p) {
        pptr[p + 1] = walk(i, p, nullptr);
        if (col[p] < i) dpos[p] = ur2a[Ur.ptr[col[p]]];  // u_jj: first entry of U's row j
      }
  });
  for (int p = 0; p < nz; ++p) pptr[p + 1] += pptr[p];
  std::vector<int2> pairs(std::max(1, pptr[nz]));
  par_for((size_t)nr, 16384, [&](size_t b, size_t e) {
    for (int i = (int)b; i < (int)e; ++i)
      for (int p = row[i]; p < row[i + 1]; ++p) walk(i, p, pairs.data() + pptr[p]);
  });
  // the position in A of every (block) row's diagonal entry
  std::vector<int> diag(std::max(1, nr));
  for (int i = 0; i < nr; ++i) diag[i] = ur2a[Ur.ptr[i]];
  int rc = 0;
  rc |= sw_pptr.upload(pptr.data(), 4 * pptr.size(), stream);
  rc |= sw_pairs.upload(pairs.data(), sizeof(int2) * pairs.size(), stream);
  rc |= sw_dpos.upload(dpos.data(), 4 * dpos.size(), stream);
  rc |= sw_diag.upload(diag.data(), 4 * diag.size(), stream);
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  // the host arrays go when this returns
  if (cudaStreamSynchronize(stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  sweep_ao = true;
  return 0;
}

// factor patterns L (CSRL) and U (CSRU) -> CSC of U, L^T, maps, chunk kinds,
// level sets, ready flags
int lace_gpu_ctx::analyse_factors(const Pattern &L, const Pattern &Ur) {
  SetupClock sc(verbose);
  Pattern Uc, Lt;
  std::vector<int> lt2l;
  {  // the two transposes on two host threads
    std::thread tu([&] { transpose_pattern(Ur, Uc, uc2ur_h); });
    transpose_pattern(L, Lt, lt2l);
    tu.join();
  }
  sc.mark("transposes");
  std::vector<int> ur2uc(uc2ur_h.size());
  for (size_t q = 0; q < uc2ur_h.size(); ++q) ur2uc[uc2ur_h[q]] = (int)q;
  nnzL = (int)L.idx.size();
  nnzU = (int)Ur.idx.size();
  hL = L;
  hU = Ur;
  hUc = std::move(Uc);
  hLt = std::move(Lt);
  sc.mark("maps, pattern copies");
  map_ur2uc_el.free();
  for (auto &pb : plans) pb.valid = false;
  int rc = 0;
  rc |= Lrow.upload(L.ptr.data(), 4 * L.ptr.size(), stream);
  rc |= Lcol.upload(L.idx.data(), 4 * L.idx.size(), stream);
  rc |= Ucp.upload(hUc.ptr.data(), 4 * hUc.ptr.size(), stream);
  rc |= Uri.upload(hUc.idx.data(), 4 * hUc.idx.size(), stream);
  rc |= Urow.upload(Ur.ptr.data(), 4 * Ur.ptr.size(), stream);
  rc |= Ucol.upload(Ur.idx.data(), 4 * Ur.idx.size(), stream);
  rc |= Ltp.upload(hLt.ptr.data(), 4 * hLt.ptr.size(), stream);
  rc |= Lti.upload(hLt.idx.data(), 4 * hLt.idx.size(), stream);
  rc |= map_ur2uc.upload(ur2uc.data(), 4 * ur2uc.size(), stream);
  rc |= map_lt2l.upload(lt2l.data(), 4 * lt2l.size(), stream);
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  sc.mark("pattern uploads");
  // level sets of the four triangles (level-scheduled option, sweep caps),
  // one host thread each
  const Pattern *pats[4] = {&hL, &hU, &hUc, &hLt};
  const bool low[4] = {true, false, true, false};
  std::vector<int> lp[4], lr[4];
  {
    std::thread th[4];
    for (int t = 0; t < 4; ++t) th[t] = std::thread([&, t] { nlevels[t] = levels(*pats[t], low[t], lp[t], lr[t]); });
    for (auto &x : th) x.join();
  }
  for (int t = 0; t < 4; ++t) {
    rc |= lvl_ptr[t].upload(lp[t].data(), 4 * lp[t].size(), stream);
    rc |= lvl_rows[t].upload(lr[t].data(), 4 * lr[t].size(), stream);
    // ready flags of the BCSR solve: one per block row; zero = never set
    const int maxch = L.n + 1;
    rc |= ready[t].ensure(4 * (size_t)maxch);
    if (!rc) cudaMemsetAsync(ready[t].p, 0, 4 * (size_t)maxch, stream);
  }
  sc.mark("level sets");
  if (bs > 0) {
    // chunks of the BCSR solves: at most 64 block rows, in solve order, a
    // new chunk wherever a block row does not depend on the one solved just
    // before it (so a chunk is at most a grid line: the chain along the line
    // stays in one warp's registers)
    const int cap = 64;
    for (int t = 0; t < 2; ++t) {
      const Pattern &P = t == 0 ? hL : hU;
      const int nb = P.n;
      std::vector<int> first;
      int in_chunk = 0;
      for (int pos = 0; pos < nb; ++pos) {
        const int I = t == 0 ? pos : nb - 1 - pos;
        const int prev = t == 0 ? I - 1 : I + 1;
        bool dep = false;
        if (pos > 0)
          for (int q = P.ptr[I]; q < P.ptr[I + 1] && !dep; ++q) dep = P.idx[q] == prev;
        if (pos == 0 || !dep || in_chunk == cap) {
          first.push_back(pos);
          in_chunk = 0;
        }
        ++in_chunk;
      }
      first.push_back(nb);
      bnch[t] = (int)first.size() - 1;
      rc |= bch_first[t].upload(first.data(), 4 * first.size(), stream);
    }
    // the host vectors go when this returns
    if (!rc && cudaStreamSynchronize(stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  }
  // the epochs of the new ready arrays restart with the zeroed flags
  Control zero;
  memset(&zero, 0, sizeof(zero));
  cudaMemsetAsync(ctrl_buf.p, 0, sizeof(Control) * 2, stream);
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  factors_ready = false;
  trsv_tuned = false;
  bcsr_tuned = false;
  ws_m = 0;
  drop_graphs();
  return 0;
}

int lace_gpu_ctx::device_anorm() {
  const size_t ld = bs ? (size_t)bs * bs : 1;
  const size_t count = (size_t)nnzA * ld;
  double *partials = (double *)part_ensure();
  if (!partials) return DEV_ERR_DEVICE_ALLOC;
  launch_sumsq(stream, count, (const double *)Aval.p, partials, (int *)cnt_buf.p + 8, (double *)scal_buf.p + 8);
  if (cudaMemcpyAsync(h_scal + 8, (double *)scal_buf.p + 8, 8, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return DEV_ERR_UNKNOWN;
  anorm = std::sqrt(h_scal[8]);
  return 0;
}

// Whether the caller's host arrays h[k] (count[k] ints) equal the resident
// device arrays dev[k]: the host arrays go up (about 0.4 ms for A's pattern of
// the 128^3 system) and are compared on the GPU, instead of against host
// copies by the CPU.
int lace_gpu_ctx::same_on_device(int parts, const int *const *h, const int *const *dev, const size_t *count,
                                 bool *same) {
  size_t tot = 0;
  for (int k = 0; k < parts; ++k) tot += count[k];
  if (pat_stage.ensure(4 * tot + 16)) return DEV_ERR_DEVICE_ALLOC;
  int *flag = (int *)pat_stage.p, *stage = flag + 4;
  if (cudaMemsetAsync(flag, 0, 4, stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  size_t off = 0;
  for (int k = 0; k < parts; ++k) {
    if (count[k] && cudaMemcpyAsync(stage + off, h[k], 4 * count[k], cudaMemcpyHostToDevice, stream) != cudaSuccess)
      return DEV_ERR_UNKNOWN;
    const int grid = (int)std::max<size_t>(1, std::min<size_t>((size_t)num_sms() * 8, (count[k] + 255) / 256));
    if (count[k]) k_pattern_diff<<<grid, 256, 0, stream>>>(count[k], stage + off, dev[k], flag);
    off += count[k];
  }
  int f = 1;
  if (cudaMemcpyAsync(&f, flag, 4, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
      cudaStreamSynchronize(stream) != cudaSuccess)
    return DEV_ERR_UNKNOWN;
  *same = f == 0;
  return 0;
}

int lace_gpu_ctx::set_factors_csc_host(int nrows, const int *lrow, const int *lcol, const double *lval,
                                       const int *ucp, const int *uri, const double *ucval) {
  // rows (block rows for BCSR factors) and values per pattern entry
  const int nr = n_blk;
  const size_t ld = bs ? (size_t)bs * bs : 1;
  if (nrows != nr || (int)hL.ptr.size() != nr + 1 || (int)hUc.ptr.size() != nr + 1) return 1;
  if (lrow[nr] != nnzL || ucp[nr] != nnzU) return 1;
  {
    const int *h[4] = {lrow, ucp, lcol, uri};
    const int *d[4] = {(const int *)Lrow.p, (const int *)Ucp.p, (const int *)Lcol.p, (const int *)Uri.p};
    const size_t cnt[4] = {(size_t)nr + 1, (size_t)nr + 1, (size_t)nnzL, (size_t)nnzU};
    bool same = false;
    const int rc = same_on_device(4, h, d, cnt, &same);
    if (rc) return rc;
    if (!same) return 1;
  }
  int rc = alloc_factor_values();
  if (rc) return rc;
  const VType t = vtype();
  cur = 0;
  const size_t nl = (size_t)nnzL * ld, nu = (size_t)nnzU * ld;
  if (t == VType::F64) {
    if (cudaMemcpyAsync(Lv[0].p, lval, 8 * nl, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(Ucv[0].p, ucval, 8 * nu, cudaMemcpyHostToDevice, stream) != cudaSuccess)
      return DEV_ERR_UNKNOWN;
  } else {
    // FP64 values through a staging buffer the context keeps (no allocation
    // per call), converted on the GPU
    if (stage64.ensure(8 * (nl + nu))) return DEV_ERR_DEVICE_ALLOC;
    double *tl = (double *)stage64.p, *tu = tl + nl;
    if (cudaMemcpyAsync(tl, lval, 8 * nl, cudaMemcpyHostToDevice, stream) != cudaSuccess ||
        cudaMemcpyAsync(tu, ucval, 8 * nu, cudaMemcpyHostToDevice, stream) != cudaSuccess)
      return DEV_ERR_UNKNOWN;
    launch_convert(stream, (int)nl, VType::F64, tl, t, Lv[0].p);
    launch_convert(stream, (int)nu, VType::F64, tu, t, Ucv[0].p);
  }
  // U's CSR image and L^T (for BCSR: U's block-row image and the inverses
  // of the diagonal blocks), on the GPU
  rc = finish_factors();
  if (rc) return rc;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  return 0;
}

// caller-supplied factors (host, FP64): L CSRL, U CSR (diagonal first).  The
// factor analysis is redone only when the patterns differ from the current
// ones.  Values are stored in the context's precision.
int lace_gpu_ctx::set_factors_host(int nrows, const int *lrow, const int *lcol, const double *lval,
                                   const int *urow, const int *ucol, const double *uval) {
  if (bs) return DEV_ERR_NOT_SUPPORTED;
  Pattern L, Ur;
  L.n = Ur.n = nrows;
  L.ptr.assign(lrow, lrow + nrows + 1);
  L.idx.assign(lcol, lcol + lrow[nrows]);
  Ur.ptr.assign(urow, urow + nrows + 1);
  Ur.idx.assign(ucol, ucol + urow[nrows]);
  // structural requirements of the solves: L diagonal last, U diagonal first
  for (int i = 0; i < nrows; ++i) {
    if (L.ptr[i + 1] <= L.ptr[i] || L.idx[L.ptr[i + 1] - 1] != i) return DEV_ERR_NOT_SUPPORTED;
    if (Ur.ptr[i + 1] <= Ur.ptr[i] || Ur.idx[Ur.ptr[i]] != i) return DEV_ERR_NOT_SUPPORTED;
    for (int p = L.ptr[i]; p < L.ptr[i + 1] - 1; ++p)
      if (L.idx[p] >= i || (p > L.ptr[i] && L.idx[p] <= L.idx[p - 1])) return DEV_ERR_NOT_SUPPORTED;
    for (int p = Ur.ptr[i] + 1; p < Ur.ptr[i + 1]; ++p)
      if (Ur.idx[p] <= Ur.idx[p - 1] || Ur.idx[p] >= nrows) return DEV_ERR_NOT_SUPPORTED;
  }
  const bool same = (L.ptr == hL.ptr && L.idx == hL.idx && Ur.ptr == hU.ptr && Ur.idx == hU.idx);
  if (!same) {
    int rc = analyse_factors(L, Ur);
    if (rc) return rc;
  }
  int rc = alloc_factor_values();
  if (rc) return rc;
  const VType t = vtype();
  DBuf tl, tu;
  if (tl.upload(lval, 8 * (size_t)nnzL, stream) || tu.upload(uval, 8 * (size_t)nnzU, stream))
    return DEV_ERR_DEVICE_ALLOC;
  cur = 0;
  launch_convert(stream, nnzL, VType::F64, tl.p, t, Lv[0].p);
  launch_convert(stream, nnzU, VType::F64, tu.p, t, Urv.p);
  // CSC image of U and L^T from the CSR values
  std::vector<int> uc2ur = uc2ur_h;
  DBuf m;
  if (m.upload(uc2ur.data(), 4 * uc2ur.size(), stream)) return DEV_ERR_DEVICE_ALLOC;
  launch_gather(stream, nnzU, (const int *)m.p, VType::F64, tu.p, t, Ucv[0].p);
  launch_gather(stream, nnzL, (const int *)map_lt2l.p, VType::F64, tl.p, t, Ltv.p);
  factors_ready = true;
  ++fact_version;
  if (cudaStreamSynchronize(stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  return 0;
}

void lace_gpu_ctx::set_rows_per_lane(int R) {
  if (R != 1 && R != 2 && R != 4 && R != 8) R = 4;
  rows_per_lane = R;
  drop_graphs();
}

TriDev lace_gpu_ctx::tri(int which) const {
  // which: 0 L, 1 U, 2 U^T, 3 L^T
  TriDev t;
  t.n = bs ? n_blk * bs : n_blk;
  t.slot = which;
  t.ready = (int *)ready[which].p;
  t.rows_per_lane = rows_per_lane;
  t.nchunks = (n_blk + 32 * rows_per_lane - 1) / (32 * rows_per_lane);
  t.lvl_ptr = (const int *)lvl_ptr[which].p;
  t.lvl_rows = (const int *)lvl_rows[which].p;
  t.nlevels = nlevels[which];
  if (which < 2) {
    t.bchunk_first = (const int *)bch_first[which].p;
    t.bnch = bnch[which];
  }
  switch (which) {
    case 0: t.row = (const int *)Lrow.p; t.col = (const int *)Lcol.p; t.val = Lv[cur].p; t.lower = 1; t.unit = 1; t.nnz = nnzL; break;
    case 1: t.row = (const int *)Urow.p; t.col = (const int *)Ucol.p; t.val = Urv.p; t.lower = 0; t.unit = 0; t.nnz = nnzU; break;
    case 2: t.row = (const int *)Ucp.p; t.col = (const int *)Uri.p; t.val = Ucv[cur].p; t.lower = 1; t.unit = 0; t.nnz = nnzU; break;
    default: t.row = (const int *)Ltp.p; t.col = (const int *)Lti.p; t.val = Ltv.p; t.lower = 0; t.unit = 1; t.nnz = nnzL; break;
  }
  return t;
}

int lace_gpu_ctx::upload_common(int n_, int nnz_, const int *hrow, const int *hcol, int bs_) {
  int rc = analyse(n_, hrow, hcol, bs_);
  if (rc) return rc;
  n = bs_ ? n_ * bs_ : n_;
  nnzA = nnz_;
  // Frobenius norm of A (data_zfrobenius) - computed on upload from device values
  return 0;
}

// new values for the resident CSR or BCSR pattern (the caller has checked
// that the pattern is the same): the analysis, plans and maps are kept
int lace_gpu_ctx::upload_values_same_pattern(const double *val) {
  ++aval_version;
  const size_t ld = bs ? (size_t)bs * bs : 1;
  if (Aval.upload(val, 8 * (size_t)nnzA * ld, stream)) return DEV_ERR_DEVICE_ALLOC;
  factors_ready = false;
  const int rc = device_anorm();
  if (rc) return rc;
  AT_ready = false;
  return autotune_spmv();
}

extern "C" int lace_gpu_upload_csr_host(lace_gpu_ctx *c, int n, int nnz, const int *row,
                                        const int *col, const double *val) {
  if (!c || !row || (nnz > 0 && (!col || !val))) return set_err(DEV_ERR_INVALID_PTR);
  cudaSetDevice(c->device);
  // same pattern as the resident matrix: only the values travel (the
  // analysis - splits, maps, chunk kinds, level sets - is kept)
  bool same = c->bs == 0 && c->n_blk == n && c->nnzA == nnz && (int)c->hArow.size() == n + 1 && row[n] == nnz;
  if (same) {  // compared with the resident pattern on the GPU
    const int *h[2] = {row, col};
    const int *d[2] = {(const int *)c->Arow.p, (const int *)c->Acol.p};
    const size_t cnt[2] = {(size_t)n + 1, (size_t)nnz};
    const int rc = c->same_on_device(2, h, d, cnt, &same);
    if (rc) return set_err(rc);
  }
  if (same) {
    const int rc = c->upload_values_same_pattern(val);
    return rc ? set_err(rc) : DEV_SUCCESS;
  }
  int rc = validate_csr(n, nnz, row, col);
  if (rc) return set_err(rc);
  ++c->aval_version;
  {
    c->sell_valid = false;
    if (c->Arow.upload(row, 4 * (size_t)(n + 1), c->stream) ||
        c->Acol.upload(col, 4 * (size_t)nnz, c->stream) || c->Aval.upload(val, 8 * (size_t)nnz, c->stream))
      return set_err(DEV_ERR_DEVICE_ALLOC);
    SetupClock sc(c->verbose);
    rc = c->upload_common(n, nnz, row, col, 0);
    if (rc) return set_err(rc);
    sc.mark("analysis");
    c->hArow.assign(row, row + n + 1);
    c->hAcol.assign(col, col + nnz);
    sc.mark("host copy of the pattern");
  }
  c->factors_ready = false;
  rc = c->device_anorm();
  if (rc) return set_err(rc);
  c->AT_ready = false;
  SetupClock sc(c->verbose && !same);
  rc = c->autotune_spmv();
  sc.mark("SpMV autotune");
  return rc;
}

extern "C" int lace_gpu_upload_csr_device(lace_gpu_ctx *c, int n, int nnz, const int *row,
                                          const int *col, const double *val) {
  if (!c || !row || (nnz > 0 && (!col || !val))) return set_err(DEV_ERR_INVALID_PTR);
  cudaSetDevice(c->device);
  std::vector<int> hrow(n + 1), hcol(nnz);
  std::vector<double> hval(nnz);
  LCHK(cudaMemcpy(hrow.data(), row, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost));
  LCHK(cudaMemcpy(hcol.data(), col, 4 * (size_t)nnz, cudaMemcpyDeviceToHost));
  LCHK(cudaMemcpy(hval.data(), val, 8 * (size_t)nnz, cudaMemcpyDeviceToHost));
  return lace_gpu_upload_csr_host(c, n, nnz, hrow.data(), hcol.data(), hval.data());
}

extern "C" int lace_gpu_upload_bcsr_host(lace_gpu_ctx *c, int nb, int bs, int nblk, const int *row,
                                         const int *col, const double *val) {
  if (!c || !row || (nblk > 0 && (!col || !val))) return set_err(DEV_ERR_INVALID_PTR);
  if (bs < 1 || bs > 8) return set_err(DEV_ERR_NOT_SUPPORTED);
  cudaSetDevice(c->device);
  // same block pattern as the resident matrix: only the values travel
  bool same = c->bs == bs && c->n_blk == nb && c->nnzA == nblk && row[nb] == nblk;
  if (same) {  // compared with the resident pattern on the GPU
    const int *h[2] = {row, col};
    const int *d[2] = {(const int *)c->Arow.p, (const int *)c->Acol.p};
    const size_t cnt[2] = {(size_t)nb + 1, (size_t)nblk};
    const int rc = c->same_on_device(2, h, d, cnt, &same);
    if (rc) return set_err(rc);
  }
  if (same) {
    const int rc = c->upload_values_same_pattern(val);
    return rc ? set_err(rc) : DEV_SUCCESS;
  }
  int rc = validate_csr(nb, nblk, row, col);
  if (rc) return set_err(rc);
  const size_t ld = (size_t)bs * bs;
  ++c->aval_version;
  c->sell_valid = false;
  if (c->Arow.upload(row, 4 * (size_t)(nb + 1), c->stream) || c->Acol.upload(col, 4 * (size_t)nblk, c->stream) ||
      c->Aval.upload(val, 8 * (size_t)nblk * ld, c->stream))
    return set_err(DEV_ERR_DEVICE_ALLOC);
  rc = c->upload_common(nb, nblk, row, col, bs);
  if (rc) return set_err(rc);
  c->hArow.clear();
  c->hAcol.clear();
  double s = 0.0;
  for (size_t p = 0; p < (size_t)nblk * ld; ++p) s += val[p] * val[p];
  c->anorm = std::sqrt(s);
  c->AT_ready = false;
  if (c->opt.trsv_rows_per_lane <= 0) c->rows_per_lane = 1;  // BCSR chunks: block rows
  LCHK(cudaStreamSynchronize(c->stream));
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_update_values_device(lace_gpu_ctx *c, const double *val) {
  if (!c || !val) return set_err(DEV_ERR_INVALID_PTR);
  const size_t ld = c->bs ? (size_t)c->bs * c->bs : 1;
  LCHK(cudaMemcpyAsync(c->Aval.p, val, 8 * (size_t)c->nnzA * ld, cudaMemcpyDeviceToDevice, c->stream));
  ++c->aval_version;
  // ||A||_F on the device
  const int rc = c->device_anorm();
  if (rc) return set_err(rc);
  c->factors_ready = false;
  c->AT_ready = false;
  return DEV_SUCCESS;
}

void *lace_gpu_ctx::part_ensure() {
  const size_t need = sizeof(double) * (size_t)(num_sms() * 16 + 8) * kLdT;
  if (part_buf.ensure(need)) return nullptr;
  return part_buf.p;
}

int lace_gpu_ctx::autotune_spmv() {
  if (opt.spmv_lanes > 0) {
    lanes = opt.spmv_lanes;
    return DEV_SUCCESS;
  }
  if (bs) return DEV_SUCCESS;
  const double avg = n_blk ? (double)nnzA / n_blk : 1.0;
  // signature cache: rows, nnz, rounded average row length
  auto key = std::make_tuple(n_blk, nnzA);
  static std::map<std::tuple<int, int>, int> cache;
  auto it = cache.find(key);
  if (it != cache.end()) {
    lanes = it->second;
    return DEV_SUCCESS;
  }
  int cand[5] = {2, 4, 8, 16, 32};
  DBuf xb, yb;
  if (xb.ensure(8 * (size_t)n_blk) || yb.ensure(8 * (size_t)n_blk)) return set_err(DEV_ERR_DEVICE_ALLOC);
  cudaMemsetAsync(xb.p, 0, 8 * (size_t)n_blk, stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bestl = avg > 12 ? 16 : 8;
  for (int ci = 0; ci < 5; ++ci) {
    const int L = cand[ci];
    if (L > 4 * std::max(1.0, avg) && L > 4) continue;
    launch_spmv_f64x(stream, L, n_blk, (const int *)Arow.p, (const int *)Acol.p, (const double *)Aval.p,
                     (const double *)xb.p, 1.0, 0.0, (double *)yb.p);
    cudaEventRecord(e0, stream);
    for (int r = 0; r < 3; ++r)
      launch_spmv_f64x(stream, L, n_blk, (const int *)Arow.p, (const int *)Acol.p,
                       (const double *)Aval.p, (const double *)xb.p, 1.0, 0.0, (double *)yb.p);
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) {
      best = ms;
      bestl = L;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  lanes = bestl;
  cache[key] = bestl;
  return cudaGetLastError() == cudaSuccess ? DEV_SUCCESS : set_err(DEV_ERR_UNKNOWN);
}

// ======================================================================
// ParILU
// ======================================================================

VType lace_gpu_ctx::vtype() const {
  return opt.precision == LACE_PREC_FP64 ? VType::F64 : (opt.precision == LACE_PREC_FP32 ? VType::F32 : VType::BF16);
}

int lace_gpu_ctx::alloc_factor_values() {
  const VType t = vtype();
  const size_t ld = bs ? (size_t)bs * bs : 1;
  const size_t s = vsize(t);
  int rc = 0;
  for (int k = 0; k < 2; ++k) {
    rc |= Lv[k].ensure(s * nnzL * ld);
    rc |= Ucv[k].ensure(s * nnzU * ld);
  }
  rc |= Urv.ensure(s * nnzU * ld);
  rc |= Ltv.ensure(s * nnzL * ld);
  if (bs) rc |= dinv.ensure(s * (size_t)n_blk * ld);
  if (sweep_ao) {
    rc |= Fv[0].ensure(s * (size_t)nnzA * ld);
    rc |= Fv[1].ensure(s * (size_t)nnzA * ld);
    if (bs) rc |= sw_dinv.ensure((t == VType::F64 ? 8 : 4) * (size_t)n_blk * ld);
  }
  return rc ? DEV_ERR_DEVICE_ALLOC : 0;
}

IluArgs lace_gpu_ctx::ilu_args() {
  IluArgs a;
  a.n = n_blk;
  a.nnzA = nnzA;
  a.Arow = (const int *)Arow.p;
  a.Acol = (const int *)Acol.p;
  a.Aval = (const double *)Aval.p;
  a.Lrow = (const int *)Lrow.p;
  a.Lcol = (const int *)Lcol.p;
  a.Ucp = (const int *)Ucp.p;
  a.Uri = (const int *)Uri.p;
  a.bs = bs;
  a.partials = (double *)part_ensure();
  a.counter = (int *)cnt_buf.p;
  return a;
}

// values for the solves from the sweep buffers: U CSR (gather), L^T (gather),
// BCSR diagonal inverses
int lace_gpu_ctx::finish_factors() {
  const VType t = vtype();
  const int ld = bs ? bs * bs : 1;
  if (bs == 0) {
    launch_gather(stream, nnzU, (const int *)map_ur2uc.p, t, Ucv[cur].p, t, Urv.p);
    launch_gather(stream, nnzL, (const int *)map_lt2l.p, t, Lv[cur].p, t, Ltv.p);
  } else {
    // block values move as ld-element records: gather each component
    std::vector<int> dummy;
    // expand block maps into element maps once
    if (!map_ur2uc_el.p) {
      std::vector<int> m(hU.idx.size() * ld);
      std::vector<int> ur2uc(hU.idx.size());
      cudaMemcpy(ur2uc.data(), map_ur2uc.p, 4 * ur2uc.size(), cudaMemcpyDeviceToHost);
      for (size_t p = 0; p < ur2uc.size(); ++p)
        for (int e = 0; e < ld; ++e) m[p * ld + e] = ur2uc[p] * ld + e;
      if (map_ur2uc_el.upload(m.data(), 4 * m.size(), stream)) return DEV_ERR_DEVICE_ALLOC;
    }
    launch_gather(stream, nnzU * ld, (const int *)map_ur2uc_el.p, t, Ucv[cur].p, t, Urv.p);
    launch_block_diag_inverse(stream, n_blk, bs, (const int *)Urow.p, t, Urv.p, dinv.p,
                              &ctrl()->status);
  }
  factors_ready = true;
  ++fact_version;
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

int lace_gpu_ctx::init_factors() {
  int rc = alloc_factor_values();
  if (rc) return rc;
  const VType t = vtype();
  const int ld = bs ? bs * bs : 1;
  for (int k = 0; k < 2; ++k) {
    init_from_A(stream, nnzL, (const int *)map_l2a.p, (const double *)Aval.p, ld, t, Lv[k].p);
    init_from_A(stream, nnzU, (const int *)map_uc2a.p, (const double *)Aval.p, ld, t, Ucv[k].p);
  }
  cur = 0;
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

// the CSR sweep's launch shape that runs fastest on this pattern (each
// candidate sweeps from the initial guess in Fold into Fnew, which the real
// sweep then overwrites)
int lace_gpu_ctx::autotune_sweep(const IluArgs &a, const void *Fold, void *Fnew) {
  const VType t = vtype();
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int pick = 0;
  double *dstep = (double *)scal_buf.p + 32;
  for (int v = 0; v < parilu_sweep_variants(); ++v) {
    float ms = 0.f;
    for (int rep = 0; rep < 3; ++rep) {
      cudaEventRecord(e0, stream);
      launch_parilu_sweep_ao(stream, nnzA, t, (const double *)Aval.p, (const int *)sw_dpos.p, (const int *)sw_pptr.p,
                             (const int2 *)sw_pairs.p, Fold, Fnew, a.partials, a.counter, dstep, v);
      cudaEventRecord(e1, stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return DEV_ERR_UNKNOWN;
      }
      float tt = 0.f;
      cudaEventElapsedTime(&tt, e0, e1);
      if (rep > 0) ms += tt;
    }
    if (verbose) printf("%% parilu sweep autotune: variant %d: %.1f us\n", v, ms * 500.f);
    if (ms < best) {
      best = ms;
      pick = v;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  sweep_variant = pick;
  return 0;
}

int lace_gpu_ctx::parilu(int sweeps, double *step_out, double *nonlin_out, bool sync_each,
                         std::vector<double> *steps, double stop_below, int min_sweeps, bool reuse_init) {
  if (!n_blk) return DEV_ERR_NOT_INITIALIZED;
  // the status bits describe this factorisation only (an earlier solve may
  // have left its own)
  if (cudaMemsetAsync(&ctrl()->status, 0, 4, stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  // the sweeps run on the A-order values F from A itself (the A-initial
  // guess), and L and U are gathered from F after them
  const bool ao = sweep_ao && sweeps > 0;
  const int ldb = bs ? bs * bs : 1;
  int rc = ao ? alloc_factor_values() : (reuse_init && factors_ready ? 0 : init_factors());
  if (rc) return rc;
  IluArgs a = ilu_args();
  if (!a.partials) return DEV_ERR_DEVICE_ALLOC;
  const VType t = vtype();
  int fc = 0;
  if (ao) launch_convert(stream, nnzA * ldb, VType::F64, Aval.p, t, Fv[0].p);
  double *dstep = (double *)scal_buf.p;  // [0..] per sweep
  for (int s = 0; s < sweeps; ++s) {
    if (ao && bs) {
      launch_bcsr_diag_inverse_ao(stream, n_blk, bs, (const int *)sw_diag.p, t, Fv[fc].p, sw_dinv.p,
                                  &ctrl()->status);
      launch_bcsr_parilu_sweep_ao(stream, nnzA, bs, t, (const double *)Aval.p, (const int *)Acol.p,
                                  (const int *)sw_dpos.p, (const int *)sw_pptr.p, (const int2 *)sw_pairs.p,
                                  sw_dinv.p, Fv[fc].p, Fv[1 - fc].p, a.partials, a.counter, dstep + (s % 32));
      fc = 1 - fc;
    } else if (ao) {
      if (sweep_variant < 0) {
        rc = autotune_sweep(a, Fv[fc].p, Fv[1 - fc].p);
        if (rc) return rc;
      }
      launch_parilu_sweep_ao(stream, nnzA, t, (const double *)Aval.p, (const int *)sw_dpos.p,
                             (const int *)sw_pptr.p, (const int2 *)sw_pairs.p, Fv[fc].p, Fv[1 - fc].p, a.partials,
                             a.counter, dstep + (s % 32), sweep_variant);
      fc = 1 - fc;
    } else {
      launch_parilu_sweep(stream, a, t, Lv[cur].p, Lv[1 - cur].p, Ucv[cur].p, Ucv[1 - cur].p,
                          dstep + (s % 32));
      cur = 1 - cur;
    }
    if (sync_each || s % 32 == 31 || s == sweeps - 1) {
      // entries of this batch not yet read: one when reading every sweep
      const int first = sync_each ? s % 32 : (s / 32) * 32 % 32;
      const int cnt = s % 32 + 1 - first;
      LCHK(cudaMemcpyAsync(h_scal, dstep + first, 8 * cnt, cudaMemcpyDeviceToHost, stream));
      LCHK(cudaStreamSynchronize(stream));
      if (steps)
        for (int k = 0; k < cnt; ++k) steps->push_back(h_scal[k] / anorm);
      if (step_out) *step_out = h_scal[cnt - 1] / anorm;
      if (sync_each && s + 1 >= min_sweeps && !(h_scal[cnt - 1] / anorm > stop_below)) break;
    }
  }
  if (ao && bs) {
    cur = 0;
    launch_factor_gather_blk(stream, nnzL, bs, (const int *)map_l2a.p, t, Fv[fc].p, Lv[0].p);
    launch_factor_gather_blk(stream, nnzU, bs, (const int *)map_uc2a.p, t, Fv[fc].p, Ucv[0].p);
  } else if (ao) {
    cur = 0;
    launch_factor_gather(stream, nnzL, (const int *)map_l2a.p, t, Fv[fc].p, Lv[0].p);
    launch_factor_gather(stream, nnzU, (const int *)map_uc2a.p, t, Fv[fc].p, Ucv[0].p);
  }
  rc = finish_factors();
  if (rc) return rc;
  if (nonlin_out) {
    if (bs) {
      *nonlin_out = NAN;  // block residual is not formed on the GPU
    } else {
      launch_ilu_residual(stream, a, t, Lv[cur].p, Ucv[cur].p, (double *)scal_buf.p + 40);
      LCHK(cudaMemcpyAsync(h_scal + 40, (double *)scal_buf.p + 40, 8, cudaMemcpyDeviceToHost, stream));
      LCHK(cudaStreamSynchronize(stream));
      *nonlin_out = std::sqrt(h_scal[40]) / anorm;
    }
  }
  LCHK(cudaStreamSynchronize(stream));
  if (h_status() & kStatusBreakdown) return DEV_ERR_BADPRECOND;
  return DEV_SUCCESS;
}

// LACE's data_zilures pair for the current factors (CSR only): res over
// pattern(LU) and nonlinres over S(A), both un-normalised
int lace_gpu_ctx::ilu_residuals(double *res, double *nonlin) {
  if (bs || !factors_ready) return DEV_ERR_NOT_SUPPORTED;
  IluArgs a = ilu_args();
  const VType t = vtype();
  // one kernel: ||LU||^2, sum over S(A) of (LU)_ij^2 and of (LU - A)_ij^2
  double *d = (double *)scal_buf.p + 42;
  launch_lu_fro(stream, a, t, (const int *)Urow.p, (const int *)Ucol.p, Lv[cur].p, Urv.p, Ucv[cur].p, d, 1);
  LCHK(cudaMemcpyAsync(h_scal + 42, d, 3 * 8, cudaMemcpyDeviceToHost, stream));
  LCHK(cudaStreamSynchronize(stream));
  const double fro = h_scal[42], onS = h_scal[43], nl2 = h_scal[44];
  if (nonlin) *nonlin = std::sqrt(nl2);
  if (res) *res = std::sqrt(std::max(0.0, nl2 + fro - onS));
  return 0;
}

int lace_gpu_ctx::h_status() {
  int st = 0;
  cudaMemcpy(&st, &ctrl()->status, 4, cudaMemcpyDeviceToHost);
  return st;
}

extern "C" int lace_gpu_parilu0(lace_gpu_ctx *c, int sweeps, double *step_out, double *nonlin_out) {
  if (!c) return set_err(DEV_ERR_INVALID_PTR);
  if (sweeps < 0) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(c->device);
  double step = 0.0;
  int rc = c->parilu(sweeps, &step, nonlin_out, false, nullptr);
  if (step_out) *step_out = step;
  if (rc) return set_err(rc);
  // a zero or non-finite pivot makes the factors non-finite (LACE's drop-in
  // only logs it as a non-finite step; this call reports it)
  if (sweeps > 0 && !std::isfinite(step)) return set_err(DEV_ERR_BADPRECOND);
  return DEV_SUCCESS;
}

// ======================================================================
// SpMV / SpTRSV
// ======================================================================

extern "C" int lace_gpu_spmv(lace_gpu_ctx *c, double alpha, const double *x, double beta, double *y) {
  if (!c || !x || !y) return set_err(DEV_ERR_INVALID_PTR);
  if (!c->n_blk) return set_err(DEV_ERR_NOT_INITIALIZED);
  if (c->bs) {
    launch_bcsr_spmv(c->stream, c->n_blk, c->bs, (const int *)c->Arow.p, (const int *)c->Acol.p,
                     (const double *)c->Aval.p, x, alpha, beta, y);
  } else if (c->opt.spmv_lanes <= 0 && c->ensure_sell() == 0 && c->sell_valid) {
    // the sliced-ELL copy the Arnoldi operator uses (built on the first call)
    launch_sell_spmv(c->stream, c->n_blk, (const int *)c->Arow.p, (const int *)c->sell_ptr.p,
                     (const int *)c->sell_col.p, (const double *)c->sell_val.p, x, alpha, beta, y);
  } else
    launch_spmv_f64x(c->stream, c->lanes, c->n_blk, (const int *)c->Arow.p, (const int *)c->Acol.p,
                     (const double *)c->Aval.p, x, alpha, beta, y);
  LCHK(cudaGetLastError());
  return DEV_SUCCESS;
}

// one triangle solve with the configured mode; in/out typed
bool lace_gpu_ctx::syncfree_blocks() const {
  return bs == 0 && opt.trsv_mode != LACE_TRSV_LEVELS && opt.trsv_mode != LACE_TRSV_JACOBI &&
         opt.trsv_mode != LACE_TRSV_NONE;
}

int lace_gpu_ctx::solve_tri(int which, const void *b, int in_f32, void *x, int out_f32,
                            bool honor_done, void *tmp, bool prefilled) {
  TriDev t = tri(which);
  const VType vt = vtype();
  Control *cb = ctrl();
  switch (opt.trsv_mode) {
    case LACE_TRSV_LEVELS:
      if (bs) return DEV_ERR_NOT_SUPPORTED;
      launch_sptrsv_levels(stream, t, vt, b, in_f32, x, out_f32, cb, honor_done);
      break;
    case LACE_TRSV_JACOBI: {
      if (bs) return DEV_ERR_NOT_SUPPORTED;
      // sweeps from y = 0 (LACE starts from a zeroed vector); ping-pong so
      // that the last sweep lands in x
      const int k = std::max(1, opt.jacobi_sweeps);
      void *bufs[2] = {tmp, x};
      int w = (k % 2 == 1) ? 1 : 0;  // first write target so that sweep k-1 writes x
      const void *yold = nullptr;
      for (int s = 0; s < k; ++s) {
        launch_jacobi_sweep(stream, t, vt, b, in_f32, yold, bufs[w], out_f32, cb, honor_done);
        yold = bufs[w];
        w = 1 - w;
      }
      break;
    }
    case LACE_TRSV_NONE:
      launch_convert(stream, n, in_f32 ? VType::F32 : VType::F64, b, out_f32 ? VType::F32 : VType::F64, x);
      break;
    default:
      if (bs) {
        if (b == x) {  // the solve fills x before it reads b
          cudaMemcpyAsync(tmp, b, (size_t)n * (in_f32 ? 4 : 8), cudaMemcpyDeviceToDevice, stream);
          b = tmp;
        }
        launch_bcsr_sptrsv(stream, t, bs, vt, which == 1 ? dinv.p : nullptr, b, in_f32, x, out_f32, cb,
                           bcsr_grid, honor_done);
      } else {
        int rc = ensure_plan(which);
        if (rc) return rc;
        if (b == x) {  // the solve fills x before it reads b
          cudaMemcpyAsync(tmp, b, (size_t)n * (in_f32 ? 4 : 8), cudaMemcpyDeviceToDevice, stream);
          b = tmp;
        }
        launch_sptrsv_blk(stream, plans[which].dev, t.val, vt, b, in_f32, x, out_f32, cb, which, honor_done,
                          prefilled && b != x);
      }
  }
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

int lace_gpu_ctx::ensure_vectors() {
  const size_t ldv_ = ((size_t)n + 31) / 32 * 32;
  int rc = 0;
  rc |= vec_w.ensure(8 * ldv_);
  rc |= vec_q.ensure(8 * ldv_);
  rc |= vec_t.ensure(8 * ldv_);
  rc |= vec_t2.ensure(8 * ldv_);
  rc |= vec_r.ensure(8 * ldv_);
  return rc ? DEV_ERR_DEVICE_ALLOC : 0;
}

// BCSR solves: the grid (resident blocks per SM) that solves the pair
// fastest, timed as the cycle runs it
int lace_gpu_ctx::autotune_bcsr_trsv() {
  if (bcsr_tuned) return 0;
  int rc = ensure_vectors();
  if (rc) return rc;
  const int f32 = vtype() != VType::F64;
  cudaMemsetAsync(vec_q.p, 0, 8 * (size_t)n, stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int best_grid = num_sms() * 8;
  for (int per_sm : {2, 4, 8}) {
    bcsr_grid = num_sms() * per_sm;
    float ms = 0.f;
    for (int rep = 0; rep < 3 && !rc; ++rep) {
      cudaEventRecord(e0, stream);
      rc = solve_tri(0, vec_q.p, 0, vec_t.p, f32, false, vec_t2.p);
      if (!rc) rc = solve_tri(1, vec_t.p, f32, vec_r.p, f32, false, vec_t2.p);
      cudaEventRecord(e1, stream);
      if (cudaEventSynchronize(e1) != cudaSuccess) rc = DEV_ERR_UNKNOWN;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0) ms += t;  // the first rep warms up
    }
    if (rc) break;
    if (verbose) printf("%% bcsr trsv autotune: %d blocks/SM: %.3f ms per pair\n", per_sm, ms / 2);
    if (ms < best) {
      best = ms;
      best_grid = bcsr_grid;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  bcsr_grid = best_grid;
  if (rc) return rc;
  if (h_status() & kStatusSpinTimeout) return DEV_ERR_INTERNAL_LIMIT;
  bcsr_tuned = true;
  return 0;
}

int lace_gpu_ctx::autotune_trsv() {
  if (bs && opt.trsv_mode == LACE_TRSV_SYNCFREE) return autotune_bcsr_trsv();
  if (bs || opt.trsv_mode != LACE_TRSV_SYNCFREE) return 0;
  if (trsv_tuned) return 0;
  int rc = ensure_vectors();
  if (rc) return rc;
  const bool f32 = vtype() != VType::F64;
  cudaMemsetAsync(vec_q.p, 0, 8 * (size_t)n, stream);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bR = 4, bC = 1, bW = 1, bL = 1;
  // schedule shapes: (rows per lane, chunks per block, warps per CTA, CTAs
  // per cluster); a block of one chunk on one warp is the warp-level
  // sync-free solve; in a cluster, consecutive blocks pass their rows on in
  // distributed shared memory
  struct Cand {
    int R, cpb, w, cl;
    int fam = 0, grp = 0;  // shape family, and the group whose plans are built together
  };
  // blocks up to the shared-memory window (160 KB of solved rows: 40960 rows
  // in FP32, 20480 in FP64) keep every in-block dependency on chip; a block
  // holds at most 1024 chunks (its unit records are staged in shared memory)
  std::vector<Cand> cands = {{4, 1, 1, 1},    {1, 1, 1, 1},    {4, 32, 8, 1},   {1, 64, 8, 1},
                             {1, 128, 16, 1},  {1, 256, 16, 1},  {1, 512, 16, 1}, {1, 1024, 16, 1},
                             {2, 256, 16, 1},  {4, 64, 16, 1},   {4, 128, 16, 1}, {4, 256, 16, 1},
                             {1, 256, 16, 2},  {1, 256, 16, 4},  {1, 384, 16, 4}, {1, 512, 16, 4},
                             {1, 512, 16, 8},  {2, 256, 16, 4}};
  if (opt.trsv_chunks_per_block > 0) {
    cands = {{opt.trsv_rows_per_lane > 0 ? opt.trsv_rows_per_lane : 1, opt.trsv_chunks_per_block,
              opt.trsv_warps > 0 ? opt.trsv_warps : 16, opt.trsv_cluster > 0 ? opt.trsv_cluster : 1}};
  } else if (opt.trsv_rows_per_lane > 0) {
    std::vector<Cand> keep;
    for (auto c : cands)
      if (c.R == 4) keep.push_back({opt.trsv_rows_per_lane, c.cpb, c.w, c.cl});
    cands = keep;
  }
  const int nch_min = (n + 31) / 32;
  // one block would hold everything
  cands.erase(std::remove_if(cands.begin(), cands.end(),
                             [&](const Cand &c) { return c.cpb > 1 && c.cpb * 32 * c.R > 2 * n && cands.size() > 1; }),
              cands.end());
  // Families of shapes: one row per lane in multi-chunk blocks (tried in
  // full), two rows, four rows, and one chunk per block.  The other families
  // are tried through one representative first; their other shapes, whose
  // times stay within about 15 % of one another, are built and timed only if
  // the representative comes within 1.5x of the best so far.
  auto family = [](const Cand &c) { return c.cpb == 1 ? 3 : (c.R == 1 ? 0 : (c.R == 2 ? 1 : 2)); };
  const Cand reps[4] = {{1, 0, 0, 0}, {2, 256, 16, 1}, {4, 128, 16, 1}, {1, 1, 1, 1}};
  for (int f = 1; f < 4; ++f) {
    bool have_rep = false;
    for (auto &c : cands)
      have_rep |= family(c) == f && c.R == reps[f].R && c.cpb == reps[f].cpb && c.w == reps[f].w && c.cl == reps[f].cl;
    bool first = !have_rep;
    for (auto &c : cands)
      if (family(c) == f) {
        const bool is_rep = have_rep ? (c.R == reps[f].R && c.cpb == reps[f].cpb && c.w == reps[f].w &&
                                        c.cl == reps[f].cl)
                                     : first;
        first = false;
        c.grp = is_rep ? 2 * f - 1 : 2 * f;
      }
  }
  for (auto &c : cands) c.fam = family(c);
  float rep_ms[4] = {0.f, 0.f, 0.f, 0.f};
  PlanBufs kept[2];  // the fastest candidate's plans so far
  // The host halves of the candidates' plans (L and U) are built in parallel
  // ahead of their turn, a group at a time, in batches of about 4 GB of host
  // memory.
  const size_t plan_bytes = (size_t)n * 48 + ((size_t)1 << 20);
  const size_t batch = std::max<size_t>(2, std::min<size_t>(24, ((size_t)4 << 30) / plan_bytes));
  // groups in order; in a group, candidates of one plan shape next to each
  // other: the plan is built once
  std::stable_sort(cands.begin(), cands.end(), [](const Cand &a, const Cand &b) {
    return a.grp != b.grp ? a.grp < b.grp : (a.R != b.R ? a.R < b.R : a.cpb < b.cpb);
  });
  auto have = [&](int w, int R, int cpb) {
    return prebuilt.count(std::make_tuple(w, R, cpb)) || (plans[w].valid && plans[w].dev.R == R && plans[w].dev.cpb == cpb);
  };
  auto prebuild_from = [&](size_t first) {
    // the shapes tried in any case (the first family and every other
    // family's first shape) are built together; the rest of a family when
    // its turn comes
    auto eager = [](const Cand &c) { return c.grp == 0 || c.grp % 2 == 1; };
    std::vector<std::tuple<int, int, int>> keys;
    for (size_t c = first; c < cands.size() && keys.size() < batch; ++c) {
      if (eager(cands[first]) ? !eager(cands[c]) : cands[c].grp != cands[first].grp) continue;
      for (int w = 0; w < 2; ++w) {
        const auto k = std::make_tuple(w, cands[c].R, cands[c].cpb);
        if (!have(w, cands[c].R, cands[c].cpb) && std::find(keys.begin(), keys.end(), k) == keys.end())
          keys.push_back(k);
      }
    }
    std::vector<HostPlan *> out;
    for (auto &k : keys) out.push_back(&prebuilt[k]);  // map nodes stay put
    const Pattern *pats[2] = {&hL, &hU};
    std::vector<int> err(keys.size(), 0);
    std::vector<std::thread> th;
    for (size_t i = 0; i < keys.size(); ++i)
      th.emplace_back([&, i] {
        const int w = std::get<0>(keys[i]);
        err[i] = build_blk_plan_host(*pats[w], w == 0, w == 0, std::get<1>(keys[i]), std::get<2>(keys[i]), *out[i]);
      });
    for (auto &x : th) x.join();
    for (int e : err)
      if (e) return e;
    return 0;
  };
  for (size_t ci = 0; ci < cands.size(); ++ci) {
    Cand cd = cands[ci];
    if (cd.grp > 0 && cd.grp % 2 == 0 && rep_ms[cd.fam] > 1.5f * best) {
      if (verbose)
        printf("trsv autotune R=%d cpb=%d warps=%d cluster=%d: skipped (its family's first shape %.3f ms per pair)\n",
               cd.R, cd.cpb, cd.w, cd.cl, rep_ms[cd.fam] / 2);
      continue;
    }
    if (!have(0, cd.R, cd.cpb) || !have(1, cd.R, cd.cpb))
      if ((rc = prebuild_from(ci))) return rc;
    plan_R = cd.R;
    plan_cpb = cd.cpb;
    plan_warps = cd.w;
    plan_cl = cd.cl;
    if ((rc = ensure_plan(0)) || (rc = ensure_plan(1))) return rc;
    if (cd.cl > 1 && !(sptrsv_cluster_supported(plans[0].dev, vtype()) &&
                       sptrsv_cluster_supported(plans[1].dev, vtype()))) {
      if (cands.size() > 1) continue;
      plan_cl = cd.cl = 1;  // a pinned schedule runs without the cluster
      if ((rc = ensure_plan(0)) || (rc = ensure_plan(1))) return rc;
    }
    // the pair as the Arnoldi cycle runs it: q, intermediate and z all in
    // the factor precision's vector type
    solve_tri(0, vec_q.p, f32, vec_t.p, f32, false, vec_t2.p);
    solve_tri(1, vec_t.p, f32, vec_t2.p, f32, false, vec_r.p);
    cudaEventRecord(e0, stream);
    for (int r = 0; r < 2; ++r) {
      solve_tri(0, vec_q.p, f32, vec_t.p, f32, false, vec_t2.p);
      solve_tri(1, vec_t.p, f32, vec_t2.p, f32, false, vec_r.p);
    }
    cudaEventRecord(e1, stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    // a shape whose solves gave up waiting is not a candidate
    const int st = h_status();
    if (st & kStatusSpinTimeout) {
      cudaMemsetAsync(&ctrl()->status, 0, 4, stream);
      ms = 1e30f;
    }
    if (verbose)
      printf("trsv autotune R=%d cpb=%d warps=%d cluster=%d: %.3f ms per pair%s\n", cd.R, cd.cpb, cd.w, cd.cl,
             ms / 2, (st & kStatusSpinTimeout) ? " (wait timed out)" : "");
    if (cd.grp % 2 == 1) rep_ms[cd.fam] = ms;
    if (ms < best) {
      // the leader's plans kept on the device, so that they need no rebuild
      // when later candidates have loaded theirs
      if ((rc = copy_blk_plan(plans[0], kept[0], stream)) || (rc = copy_blk_plan(plans[1], kept[1], stream))) return rc;
      best = ms;
      bR = cd.R;
      bC = cd.cpb;
      bW = cd.w;
      bL = cd.cl;
    }
  }
  (void)nch_min;
  for (int w = 0; w < 2; ++w)
    if (kept[w].valid && !(plans[w].valid && plans[w].dev.R == bR && plans[w].dev.cpb == bC))
      swap_blk_plans(plans[w], kept[w]);
  if (cudaStreamSynchronize(stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
  prebuilt.clear();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  plan_R = bR;
  plan_cpb = bC;
  plan_warps = bW;
  plan_cl = bL;
  rows_per_lane = bR;
  trsv_tuned = true;
  cudaMemsetAsync(&ctrl()->status, 0, 4, stream);
  drop_graphs();
  if (best >= 1e30f) return DEV_ERR_INTERNAL_LIMIT;  // no shape finished its solves
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

extern "C" int lace_gpu_sptrsv(lace_gpu_ctx *c, int which, const double *b, double *x) {
  if (!c || !b || !x) return set_err(DEV_ERR_INVALID_PTR);
  if (which < 0 || which > 3) return set_err(DEV_ERR_ILLEGAL_VALUE);
  if (!c->factors_ready) return set_err(DEV_ERR_NOT_INITIALIZED);
  if (c->bs && which > 1) return set_err(DEV_ERR_NOT_SUPPORTED);
  cudaSetDevice(c->device);
  int rc = c->ensure_vectors();
  if (!rc) rc = c->autotune_trsv();
  if (rc) return set_err(rc);
  cudaMemsetAsync(&c->ctrl()->status, 0, 4, c->stream);
  const bool f32 = c->vtype() != VType::F64;
  if (f32) {
    rc = c->solve_tri(which, b, 0, c->vec_t.p, 1, false, c->vec_t2.p);
    if (!rc) launch_convert(c->stream, c->n, VType::F32, c->vec_t.p, VType::F64, x);
  } else {
    rc = c->solve_tri(which, b, 0, x, 0, false, c->vec_t2.p);
  }
  if (rc) return set_err(rc);
  LCHK(cudaStreamSynchronize(c->stream));
  int st = c->h_status();
  if (st & kStatusSpinTimeout) return set_err(DEV_ERR_INTERNAL_LIMIT);
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_precond_enqueue(lace_gpu_ctx *c, const void *q, void *z) {
  if (!c || !q || !z) return set_err(DEV_ERR_INVALID_PTR);
  if (!c->factors_ready || !c->trsv_tuned) return set_err(DEV_ERR_NOT_INITIALIZED);
  cudaSetDevice(c->device);
  const int f32 = c->vtype() != VType::F64;
  int rc = c->solve_tri(0, q, f32, c->vec_t.p, f32, false, c->vec_t2.p);
  if (!rc) rc = c->solve_tri(1, c->vec_t.p, f32, z, f32, false, c->vec_t2.p);
  return rc ? set_err(rc) : DEV_SUCCESS;
}

extern "C" int lace_gpu_get_trsv_schedule(lace_gpu_ctx *c, int *out) {
  if (!c || !out) return set_err(DEV_ERR_INVALID_PTR);
  if (!c->trsv_tuned) return set_err(DEV_ERR_NOT_INITIALIZED);
  out[0] = c->plan_R;
  out[1] = c->plan_cpb;
  out[2] = c->plan_warps;
  out[3] = c->plan_cl;
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_apply_precond(lace_gpu_ctx *c, const double *q, double *z) {
  if (!c || !q || !z) return set_err(DEV_ERR_INVALID_PTR);
  if (!c->factors_ready) return set_err(DEV_ERR_NOT_INITIALIZED);
  cudaSetDevice(c->device);
  int rc = c->ensure_vectors();
  if (!rc) rc = c->autotune_trsv();
  if (rc) return set_err(rc);
  cudaMemsetAsync(&c->ctrl()->status, 0, 4, c->stream);
  const int f32 = c->vtype() != VType::F64;
  rc = c->solve_tri(0, q, 0, c->vec_t.p, f32, false, c->vec_t2.p);
  if (!rc) {
    if (f32) {
      rc = c->solve_tri(1, c->vec_t.p, 1, c->vec_r.p, 1, false, c->vec_t2.p);
      launch_convert(c->stream, c->n, VType::F32, c->vec_r.p, VType::F64, z);
    } else {
      rc = c->solve_tri(1, c->vec_t.p, 0, z, 0, false, c->vec_t2.p);
    }
  }
  if (rc) return set_err(rc);
  LCHK(cudaStreamSynchronize(c->stream));
  if (c->h_status() & kStatusSpinTimeout) return set_err(DEV_ERR_INTERNAL_LIMIT);
  return DEV_SUCCESS;
}

// ======================================================================
// FGMRES-Householder
// ======================================================================

int lace_gpu_ctx::ensure_krylov(int m, bool monitor) {
  int rc = ensure_vectors();
  if (rc) return rc;
  const bool zf32 = vtype() != VType::F64;
  // columns a power of two bytes apart would put one row's entries of every
  // column on the same memory channels
  ldv = ((size_t)n + 31) / 32 * 32 + 32;
  const size_t vbytes = 8 * ldv * (size_t)(m + 1), zbytes = (zf32 ? 4 : 8) * ldv * (size_t)m;
  const size_t vfbytes = zf32 ? 2 * 4 * ldv * (size_t)(m + 1) : 0;  // Vf, then Vlo
  if (m > ws_m || zf32 != ws_zf32 || Vb.bytes < vbytes || Zb.bytes < zbytes || Vfb.bytes < vfbytes) {
    drop_graphs();
    rc |= Vb.ensure(vbytes);
    rc |= Zb.ensure(zbytes);
    if (zf32) rc |= Vfb.ensure(vfbytes);
    if (rc) return DEV_ERR_DEVICE_ALLOC;
    ws_m = m;
    ws_zf32 = zf32;
  }
  if (monitor && Qmon.bytes < 8 * ldv * (size_t)(m + 1)) {
    drop_graphs();
    if (Qmon.ensure(8 * ldv * (size_t)(m + 1))) return DEV_ERR_DEVICE_ALLOC;
  }
  if (!part_ensure()) return DEV_ERR_DEVICE_ALLOC;
  return 0;
}

// A in sliced ELL (slices of 32 rows; within a slice, entry t of all rows
// together), built from the host copy of the pattern; values gathered from
// the resident CSR values whenever they change
int lace_gpu_ctx::ensure_sell() {
  if (bs || (int)hArow.size() != n + 1) return 0;  // CSR uploads only
  if (!sell_valid) {
    // slice widths, their offsets, then the slices, over parallel ranges
    const int nsl = (n + 31) / 32;
    std::vector<int> ptr(nsl + 1, 0);
    par_for((size_t)nsl, 8192, [&](size_t b, size_t e) {
      for (int s = (int)b; s < (int)e; ++s) {
        int w = 0;
        for (int i = 32 * s; i < std::min(n, 32 * s + 32); ++i) w = std::max(w, hArow[i + 1] - hArow[i]);
        ptr[s + 1] = 32 * w;
      }
    });
    for (int s = 0; s < nsl; ++s) ptr[s + 1] += ptr[s];
    std::vector<int> col(std::max(1, ptr[nsl])), map(std::max(1, ptr[nsl]), -1);
    par_for((size_t)nsl, 8192, [&](size_t b, size_t e) {
      for (int s = (int)b; s < (int)e; ++s)
        for (int l = 0; l < 32; ++l) {
          const int i = 32 * s + l;
          const int w = (ptr[s + 1] - ptr[s]) / 32;
          for (int t = 0; t < w; ++t) {
            const int q = ptr[s] + 32 * t + l;
            const bool in = i < n && t < hArow[i + 1] - hArow[i];
            col[q] = in ? hAcol[hArow[i] + t] : 0;
            map[q] = in ? hArow[i] + t : -1;
          }
        }
    });
    int rc = 0;
    rc |= sell_ptr.upload(ptr.data(), 4 * ptr.size(), stream);
    rc |= sell_col.upload(col.data(), 4 * col.size(), stream);
    rc |= sell_map.upload(map.data(), 4 * map.size(), stream);
    rc |= sell_val.ensure(8 * col.size());
    rc |= sell_pair.ensure(8 * col.size());
    if (rc) return DEV_ERR_DEVICE_ALLOC;
    if (cudaStreamSynchronize(stream) != cudaSuccess) return DEV_ERR_UNKNOWN;
    sell_slots = (size_t)ptr[nsl];
    sell_valid = true;
    sell_version = -1;
    drop_graphs();
  }
  if (sell_version != aval_version) {
    launch_sell_values(stream, sell_slots, (const int *)sell_map.p, (const double *)Aval.p,
                       (double *)sell_val.p, (float2 *)sell_pair.p);
    sell_version = aval_version;
  }
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

int lace_gpu_ctx::ensure_AT() {
  if (AT_ready) return 0;
  if (bs) return DEV_ERR_NOT_SUPPORTED;
  Pattern A, T;
  A.n = n_blk;
  A.ptr.resize(n_blk + 1);
  A.idx.resize(nnzA);
  cudaMemcpy(A.ptr.data(), Arow.p, 4 * (size_t)(n_blk + 1), cudaMemcpyDeviceToHost);
  cudaMemcpy(A.idx.data(), Acol.p, 4 * (size_t)nnzA, cudaMemcpyDeviceToHost);
  std::vector<int> t2a;
  transpose_pattern(A, T, t2a);
  int rc = 0;
  rc |= ATrow.upload(T.ptr.data(), 4 * T.ptr.size(), stream);
  rc |= ATcol.upload(T.idx.data(), 4 * T.idx.size(), stream);
  rc |= map_at2a.upload(t2a.data(), 4 * t2a.size(), stream);
  rc |= ATval.ensure(8 * (size_t)nnzA);
  if (rc) return DEV_ERR_DEVICE_ALLOC;
  launch_gather(stream, nnzA, (const int *)map_at2a.p, VType::F64, Aval.p, VType::F64, ATval.p);
  AT_ready = true;
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

ArnoldiArgs lace_gpu_ctx::arnoldi_args(int m, bool adjoint) {
  ArnoldiArgs a;
  a.n = n;
  a.bs = bs;
  if (adjoint) {
    a.row = (const int *)ATrow.p;
    a.col = (const int *)ATcol.p;
    a.val = (const double *)ATval.p;
  } else {
    a.row = (const int *)Arow.p;
    a.col = (const int *)Acol.p;
    a.val = (const double *)Aval.p;
    if (sell_valid && !bs) {
      a.sell_ptr = (const int *)sell_ptr.p;
      a.sell_col = (const int *)sell_col.p;
      a.sell_val = (const double *)sell_val.p;
      a.sell_pair = (const float2 *)sell_pair.p;
    }
  }
  a.lanes = lanes;
  a.V = (double *)Vb.p;
  a.ldv = ldv;
  a.Vf = vtype() != VType::F64 ? (float *)Vfb.p : nullptr;
  a.Vlo = a.Vf ? a.Vf + ldv * (size_t)(m + 1) : nullptr;
  a.Z = Zb.p;
  a.ldz = ldv;
  a.z_f32 = ws_zf32 ? 1 : 0;
  a.w = (double *)vec_w.p;
  a.q = vec_q.p;
  a.q_f32 = vtype() != VType::F64 ? 1 : 0;
  a.partials = (double *)part_buf.p;
  a.grid = num_sms() * 8;
  a.cy = (Cycle *)cycle_buf.p;
  a.ctrl = ctrl();
  a.m = m;
  a.prefill = syncfree_blocks() ? 1 : 0;
  a.fill_t = vec_t.p;
  a.fill_t_f32 = vtype() != VType::F64 ? 1 : 0;
  return a;
}

// the search-direction loop of one cycle (LACE :311-759), all on the device
int lace_gpu_ctx::enqueue_cycle_body(const ArnoldiArgs &a, int m, bool adjoint, bool capturing) {
  const int t1 = adjoint ? 2 : 0, t2 = adjoint ? 3 : 1;
  const int tf32 = vtype() != VType::F64;  // the intermediate vector of the two solves
  for (int j = 0; j < m; ++j) {
    void *zj = (char *)a.Z + (size_t)j * a.ldz * (a.z_f32 ? 4 : 8);
    // both outputs were marked unsolved by the kernel before (a.prefill)
    int rc = solve_tri(t1, a.q, a.q_f32, vec_t.p, tf32, true, vec_t2.p, a.prefill != 0);
    if (!rc) rc = solve_tri(t2, vec_t.p, tf32, zj, a.z_f32, true, vec_t2.p, a.prefill != 0);
    if (rc) return rc;
    // passes A, B and C as one cooperative kernel where it applies
    const int st = hh_persistent ? launch_hh_step(stream, a, j) : 1;
    if (st == 2) {
      hh_persistent = false;
      if (verbose) printf("%% cooperative launch refused: the Householder step runs as three passes\n");
      if (capturing) return DEV_ERR_NOT_SUPPORTED;
    }
    if (st != 0) {
      launch_passA(stream, a, j);
      launch_passB(stream, a, j);
      launch_passC(stream, a, j);
    }
    if (opt.monitor_orthog && Qmon.p) {
      // q_{j+1} into the monitor basis, then ||I - Q^T Q|| over q_0..q_j
      launch_convert(stream, n, a.q_f32 ? VType::F32 : VType::F64, a.q, VType::F64,
                     (double *)Qmon.p + (size_t)(j + 1) * ldv);
      launch_orthog_monitor(stream, a, j, (double *)Qmon.p, ldv);
    }
  }
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

// the modified Gram-Schmidt search-direction loop of one cycle
// (src/fgmres_restart.cpp:227-494), all on the device
int lace_gpu_ctx::enqueue_mgs_body(const ArnoldiArgs &a, int m, bool capturing) {
  const int tf32 = vtype() != VType::F64;
  // LACE's test reorthogonalises for reorth 0 (when needed) and 2 (always)
  const bool second = a.mgs_reorth == 0 || a.mgs_reorth == 2;
  for (int j = 0; j < m; ++j) {
    void *zj = (char *)a.Z + (size_t)j * a.ldz * (a.z_f32 ? 4 : 8);
    const double *vj = a.V + (size_t)j * a.ldv;
    // z_j = U^{-1} L^{-1} v_j (:239-270); outputs marked unsolved before
    int rc = solve_tri(0, vj, 0, vec_t.p, tf32, true, vec_t2.p, a.prefill != 0);
    if (!rc) rc = solve_tri(1, vec_t.p, tf32, zj, a.z_f32, true, vec_t2.p, a.prefill != 0);
    if (rc) return rc;
    // the whole step as one cooperative kernel where it applies
    const int st = mgs_persistent ? launch_mgs_step(stream, a, j) : 1;
    if (st == 2) {
      // the cooperative launch was refused: inside a capture that ends the
      // capture, so start it again without; otherwise carry on without
      mgs_persistent = false;
      if (verbose) printf("%% cooperative launch refused: the Gram-Schmidt step runs as separate kernels\n");
      if (capturing) return DEV_ERR_NOT_SUPPORTED;
    } else if (st == 0) {
      if (opt.monitor_orthog) launch_orthog_monitor(stream, a, j, a.V, a.ldv);
      continue;
    }
    launch_mgs_operator(stream, a, j);
    for (int k = 1; k <= j; ++k) launch_mgs_sweep(stream, a, j, k, 0);
    if (second && capturing && cond_nodes) {
      // the second pass in a conditional node that the norm kernel sets
      cudaStreamCaptureStatus st;
      cudaGraph_t g = nullptr;
      if (cudaStreamGetCaptureInfo(stream, &st, nullptr, &g) != cudaSuccess || st != cudaStreamCaptureStatusActive)
        return DEV_ERR_UNKNOWN;
      cudaGraphConditionalHandle h;
      if (cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault) != cudaSuccess) {
        cond_nodes = false;
        return DEV_ERR_NOT_SUPPORTED;
      }
      launch_mgs_norm(stream, a, j, 0, (unsigned long long)h);
      const cudaGraphNode_t *deps = nullptr;
      size_t ndeps = 0;
      if (cudaStreamGetCaptureInfo(stream, &st, nullptr, &g, &deps, nullptr, &ndeps) != cudaSuccess)
        return DEV_ERR_UNKNOWN;
      cudaGraphNodeParams p = {};
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = h;
      p.conditional.type = cudaGraphCondTypeIf;
      p.conditional.size = 1;
      cudaGraphNode_t node;
      cond_nodes = false;  // until the node is in place
      if (cudaGraphAddNode(&node, g, deps, nullptr, ndeps, &p) != cudaSuccess) return DEV_ERR_NOT_SUPPORTED;
      cudaGraph_t body = p.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(side, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal) !=
          cudaSuccess)
        return DEV_ERR_NOT_SUPPORTED;
      for (int k = 0; k <= j; ++k) launch_mgs_sweep(side, a, j, k, 1);
      launch_mgs_norm(side, a, j, 1, 0);
      cudaGraph_t captured = body;
      const cudaError_t ce = cudaStreamEndCapture(side, &captured);
      if (ce != cudaSuccess || cudaGetLastError() != cudaSuccess) return DEV_ERR_NOT_SUPPORTED;
      cond_nodes = true;
      if (cudaStreamUpdateCaptureDependencies(stream, &node, nullptr, 1, cudaStreamSetCaptureDependencies) !=
          cudaSuccess)
        return DEV_ERR_UNKNOWN;
    } else {
      launch_mgs_norm(stream, a, j, 0, 0);
      if (second) {  // launched always; returns at once unless the test asked for it
        for (int k = 0; k <= j; ++k) launch_mgs_sweep(stream, a, j, k, 1);
        launch_mgs_norm(stream, a, j, 1, 0);
      }
    }
    launch_mgs_next(stream, a, j);
    if (opt.monitor_orthog) launch_orthog_monitor(stream, a, j, a.V, a.ldv);  // v_0..v_j (:380-387)
  }
  return cudaGetLastError() == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

int lace_gpu_ctx::fgmres(const double *b, double *x, int m, int restart_max, int tol_type,
                         double rtol, bool adjoint, data_d_gmres_log *log, int *total_iters,
                         std::vector<double> *hist, int method, int restarted, int reorth) {
  if (m < 1) return DEV_ERR_NOT_SUPPORTED;
  // LACE's own tests ask for up to 2000 directions per cycle where a handful
  // converge: the device cycle holds kMaxM, and a longer one runs its first
  // kMaxM directions and reports DEV_ERR_NOT_SUPPORTED only if it needs more
  const bool capped = m > kMaxM;
  if (capped) m = kMaxM;
  last_m = m;
  const bool mgs = method == 1;
  if (mgs && adjoint) return DEV_ERR_NOT_SUPPORTED;
  if (mgs && !restarted) restart_max = std::min(restart_max, 1);
  if (!factors_ready && opt.trsv_mode != LACE_TRSV_NONE) return DEV_ERR_NOT_INITIALIZED;
  SetupClock sc(verbose);
  int rc = ensure_krylov(m, opt.monitor_orthog != 0);
  sc.mark("Krylov workspace");
  if (!rc) rc = autotune_trsv();
  sc.mark("SpTRSV autotune");
  if (!rc && adjoint) rc = ensure_AT();
  if (!rc && !adjoint) rc = ensure_sell();
  sc.mark("operator (A^T or sliced ELL)");
  // solve plans are built on the host: before any graph capture
  if (!rc && !bs && opt.trsv_mode == LACE_TRSV_SYNCFREE) {
    rc = ensure_plan(adjoint ? 2 : 0);
    if (!rc) rc = ensure_plan(adjoint ? 3 : 1);
  }
  if (!rc && cudaStreamSynchronize(stream) != cudaSuccess) rc = DEV_ERR_UNKNOWN;
  if (rc) return rc;
  sc.mark("solve plans");
  if (mgs && !side && cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess)
    return DEV_ERR_UNKNOWN;
  ArnoldiArgs a = arnoldi_args(m, adjoint);
  a.mgs_restarted = restarted ? 1 : 0;
  a.mgs_reorth = reorth;
  Cycle *cy = a.cy;
  // tolerance set-up scalars
  {
    struct {
      int tol_type, first;
      double rtol;
    } hs = {tol_type, 1, rtol};
    LCHK(cudaMemcpyAsync(&cy->tol_type, &hs.tol_type, 4, cudaMemcpyHostToDevice, stream));
    LCHK(cudaMemcpyAsync(&cy->first_cycle, &hs.first, 4, cudaMemcpyHostToDevice, stream));
    LCHK(cudaMemcpyAsync(&cy->rtol, &hs.rtol, 8, cudaMemcpyHostToDevice, stream));
    int zero = 0;
    LCHK(cudaMemcpyAsync(&a.ctrl->status, &zero, 4, cudaMemcpyHostToDevice, stream));
    // grid-barrier arrivals of the one-kernel Gram-Schmidt step (left
    // non-zero only by a step that gave up a wait)
    LCHK(cudaMemsetAsync(&a.ctrl->block_count[3], 0, 4, stream));
  }
  const auto key = std::make_tuple(m, adjoint ? 1 : 0, opt.trsv_mode, rows_per_lane,
                                   opt.jacobi_sweeps, (int)vtype(), opt.monitor_orthog, lanes, method,
                                   mgs ? (restarted ? 1 : 0) : 0, mgs ? reorth : 0);
  int total = 0;
  bool converged = false;
  int last_cycle = 0, last_steps = 0;
  last_reorth = 0;
  last_orth.clear();
  double rnorm0 = 0.0, final_res = 0.0;
  for (int restart = 0; restart < restart_max; ++restart) {
    launch_cycle_residual(stream, a, b, x, mgs);
    if (mgs) {
      launch_mgs_cycle_init(stream, a);
    } else {
      launch_cycle_init(stream, a);
      if (opt.monitor_orthog && Qmon.p)
        launch_convert(stream, n, a.q_f32 ? VType::F32 : VType::F64, a.q, VType::F64, Qmon.p);
    }
    if (opt.use_graph) {
      auto it = graphs.find(key);
      if (it == graphs.end()) {
        SetupClock gc(verbose);
        cudaGraphExec_t ge = nullptr;
        for (int attempt = 0; attempt < 3 && !ge; ++attempt) {
          cudaGraph_t g;
          LCHK(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
          rc = mgs ? enqueue_mgs_body(a, m, true) : enqueue_cycle_body(a, m, adjoint, true);
          cudaError_t ce = cudaStreamEndCapture(stream, &g);
          if (rc == DEV_ERR_NOT_SUPPORTED && attempt < 2) {
            // a refused cooperative launch or conditional node (the flag
            // that chose it is cleared): capture again without it
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            cudaGetLastError();
            if (verbose && !cond_nodes) printf("%% conditional graph nodes unavailable: the second Gram-Schmidt pass launches always\n");
            rc = 0;
            continue;
          }
          if (rc) {
            if (ce == cudaSuccess) cudaGraphDestroy(g);
            return rc;
          }
          LCHK(ce);
          gc.mark("cycle graph capture");
          ce = cudaGraphInstantiate(&ge, g, 0);
          cudaGraphDestroy(g);
          LCHK(ce);
          gc.mark("cycle graph instantiation");
        }
        if (!ge) return DEV_ERR_UNKNOWN;
        it = graphs.emplace(key, ge).first;
      }
      LCHK(cudaGraphLaunch(it->second, stream));
    } else {
      rc = mgs ? enqueue_mgs_body(a, m, false) : enqueue_cycle_body(a, m, adjoint, false);
      if (rc) return rc;
    }
    if (mgs) launch_mgs_xupdate(stream, a, x);
    else launch_xupdate(stream, a, x);
    LCHK(cudaMemcpyAsync(h_ctrl, a.ctrl, sizeof(Control), cudaMemcpyDeviceToHost, stream));
    LCHK(cudaMemcpyAsync(h_scal, cy->hist, 8 * (size_t)m, cudaMemcpyDeviceToHost, stream));
    if (mgs) {
      LCHK(cudaMemcpyAsync(h_scal + kScalCycleRnorm, &cy->rnorm, 8, cudaMemcpyDeviceToHost, stream));
      LCHK(cudaMemcpyAsync(h_scal + kScalReorth, &cy->nreorth, 4, cudaMemcpyDeviceToHost, stream));
    }
    LCHK(cudaStreamSynchronize(stream));
    if (restart == 0) sc.mark("first cycle");
    const Control &hc = *h_ctrl;
    if (restart == 0) rnorm0 = hc.rnorm0;
    // LACE's Gram-Schmidt FGMRES logs the residual at the start of every
    // cycle (src/fgmres_restart.cpp:221-223), the Householder one the first
    if (mgs && !(hc.converged && hc.nsteps == 0)) {
      rnorm0 = h_scal[kScalCycleRnorm];
      int nr = 0;
      memcpy(&nr, h_scal + kScalReorth, 4);
      last_reorth += nr;
    }
    if (hc.status & kStatusSpinTimeout) return DEV_ERR_INTERNAL_LIMIT;
    const int ns = hc.nsteps;
    if (capped && ns == m && !hc.converged && !(hc.status & kStatusBreakdown)) return DEV_ERR_NOT_SUPPORTED;
    if (hist)
      for (int k = 0; k < ns; ++k) hist->push_back(h_scal[k]);
    if (opt.monitor_orthog) {
      std::vector<double> oh(ns);
      if (ns > 0) LCHK(cudaMemcpy(oh.data(), cy->orth, 8 * (size_t)ns, cudaMemcpyDeviceToHost));
      last_orth.insert(last_orth.end(), oh.begin(), oh.end());
      if (verbose)
        for (int k = 0; k < ns; ++k)
          printf("%s_gpu_ortherr(%d) = %.16e;\n", mgs ? "FGMRES" : "FGMRES_Householders", total + k + 1, oh[k]);
    }
    total += ns;
    if (ns > 0) {
      last_cycle = restart;
      last_steps = ns;
      final_res = h_scal[ns - 1];
    }
    if (hc.converged) {
      converged = true;
      if (ns == 0) final_res = 0.0;
      break;
    }
    if (hc.status & kStatusBreakdown) break;
    if (ns == 0) break;
    int zero = 0;
    LCHK(cudaMemcpyAsync(&cy->first_cycle, &zero, 4, cudaMemcpyHostToDevice, stream));
  }
  if (log) {
    log->restarts = last_cycle;
    log->search_directions = last_steps;
    log->initial_residual = rnorm0;
    log->final_residual = final_res;
  }
  if (total_iters) *total_iters = total;
  return converged ? DEV_SUCCESS : DEV_NOTCONVERGED;
}

extern "C" int lace_gpu_fgmres_householder(lace_gpu_ctx *c, const double *b, double *x,
                                           const data_d_gmres_param *par, data_d_gmres_log *log,
                                           int *total_iters) {
  if (!c || !b || !x || !par) return set_err(DEV_ERR_INVALID_PTR);
  cudaSetDevice(c->device);
  auto t0 = std::chrono::steady_clock::now();
  int rc = c->fgmres(b, x, par->search_max, par->restart_max, par->tol_type, par->rtol, false, log,
                     total_iters, &c->last_hist);
  if (log)
    log->solve_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc != DEV_SUCCESS && rc != DEV_NOTCONVERGED) return set_err(rc);
  return rc;
}

extern "C" int lace_gpu_fgmres_mgs(lace_gpu_ctx *c, const double *b, double *x, const data_d_gmres_param *par,
                                   int restarted, data_d_gmres_log *log, int *total_iters) {
  if (!c || !b || !x || !par) return set_err(DEV_ERR_INVALID_PTR);
  cudaSetDevice(c->device);
  auto t0 = std::chrono::steady_clock::now();
  int rc = c->fgmres(b, x, par->search_max, restarted ? par->restart_max : 1, par->tol_type, par->rtol, false,
                     log, total_iters, &c->last_hist, 1, restarted ? 1 : 0, par->reorth);
  if (log)
    log->solve_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rc != DEV_SUCCESS && rc != DEV_NOTCONVERGED) return set_err(rc);
  return rc;
}

extern "C" int lace_gpu_get_solve_stats(lace_gpu_ctx *c, int *out) {
  if (!c || !out) return set_err(DEV_ERR_INVALID_PTR);
  out[0] = c->last_reorth;
  out[1] = c->cond_nodes ? 1 : 0;
  out[2] = c->mgs_persistent ? 1 : 0;
  out[3] = c->hh_persistent ? 1 : 0;
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_time_arnoldi_step(lace_gpu_ctx *c, int method, int j, int reps, double *seconds) {
  if (!c || !seconds) return set_err(DEV_ERR_INVALID_PTR);
  if (reps < 1 || j < 0 || j + 2 > c->last_m || !c->Vb.p) return set_err(DEV_ERR_ILLEGAL_VALUE);
  cudaSetDevice(c->device);
  ArnoldiArgs a = c->arnoldi_args(c->last_m, false);
  a.mgs_restarted = 1;
  a.mgs_reorth = 0;
  // the replays must neither stop nor skip: no convergence (tolerance 0),
  // not done, barrier arrivals cleared
  const double zero = 0.0;
  LCHK(cudaMemcpyAsync(&a.ctrl->rtol_abs, &zero, 8, cudaMemcpyHostToDevice, c->stream));
  LCHK(cudaMemsetAsync(&a.ctrl->done, 0, 4, c->stream));
  LCHK(cudaMemsetAsync(&a.ctrl->status, 0, 4, c->stream));
  LCHK(cudaMemsetAsync(&a.ctrl->block_count[3], 0, 4, c->stream));
  // the unsolved marks go to two scratch vectors (same element types, same
  // traffic), so that the basis and Z stay as the solve left them
  void *mt = c->vec_t2.p, *mz = c->vec_r.p;
  auto launch = [&]() {
    return method == 1 ? launch_mgs_step(c->stream, a, j, mt, mz) : launch_hh_step(c->stream, a, j, mt, mz);
  };
  if (launch() != 0) return set_err(DEV_ERR_NOT_SUPPORTED);
  cudaEvent_t e0, e1;
  LCHK(cudaEventCreate(&e0));
  LCHK(cudaEventCreate(&e1));
  cudaEventRecord(e0, c->stream);
  for (int r = 0; r < reps; ++r) launch();
  cudaEventRecord(e1, c->stream);
  const cudaError_t ce = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  LCHK(ce);
  const int st = c->h_status();
  // the replays' own status (their drifting rotations may even report a
  // breakdown) must not reach the next operation
  LCHK(cudaMemsetAsync(&a.ctrl->status, 0, 4, c->stream));
  LCHK(cudaMemsetAsync(&a.ctrl->done, 0, 4, c->stream));
  if (st & kStatusSpinTimeout) return set_err(DEV_ERR_INTERNAL_LIMIT);
  *seconds = ms * 1e-3 / reps;
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_solve_backward(lace_gpu_ctx *c, const double *x, const double *dLdx,
                                       const data_d_gmres_param *par, double *dLdb, double *dLdA,
                                       int *total_iters) {
  if (!c || !x || !dLdx || !par) return set_err(DEV_ERR_INVALID_PTR);
  if (c->bs) return set_err(DEV_ERR_NOT_SUPPORTED);
  cudaSetDevice(c->device);
  int rc = c->ensure_vectors();
  if (rc) return set_err(rc);
  // lambda = A^{-T} dL/dx, initial guess 0
  double *lam = dLdb;
  DBuf tmp;
  if (!lam) {
    if (tmp.ensure(8 * (size_t)c->n)) return set_err(DEV_ERR_DEVICE_ALLOC);
    lam = (double *)tmp.p;
  }
  cudaMemsetAsync(lam, 0, 8 * (size_t)c->n, c->stream);
  // transposed factor values L^T follow the current L
  rc = c->fgmres(dLdx, lam, par->search_max, par->restart_max, par->tol_type, par->rtol, true,
                 nullptr, total_iters, nullptr);
  if (rc != DEV_SUCCESS && rc != DEV_NOTCONVERGED) return set_err(rc);
  if (dLdA) {
    int grid = std::min((c->n + 255) / 256, num_sms() * 8);
    k_grad_A<<<grid, 256, 0, c->stream>>>(c->n, (const int *)c->Arow.p, (const int *)c->Acol.p, lam, x,
                                          dLdA);
  }
  LCHK(cudaStreamSynchronize(c->stream));
  return rc;
}

extern "C" int lace_gpu_last_error(void) { return g_last_error; }

extern "C" void lace_gpu_inject_alloc_failure(int after) {
  g_alloc_budget.store(after < 0 ? -1 : (long long)after);
}

extern "C" const char *lace_gpu_error_string(int code) {
  switch (code) {
    case DEV_SUCCESS: return "success";
    case DEV_ERR_NOT_INITIALIZED: return "not initialized (no GPU, no matrix, or no factors)";
    case DEV_ERR_NOT_SUPPORTED: return "not supported (format, unsorted/missing diagonal, size limit)";
    case DEV_ERR_ILLEGAL_VALUE: return "illegal value";
    case DEV_ERR_INTERNAL_LIMIT: return "a bounded device wait gave up (dependency never satisfied)";
    case DEV_ERR_DEVICE_ALLOC: return "device allocation failed";
    case DEV_ERR_HOST_ALLOC: return "host allocation failed";
    case DEV_ERR_INVALID_PTR: return "invalid pointer";
    case DEV_ERR_BADPRECOND: return "breakdown in the preconditioner (zero or non-finite pivot)";
    case DEV_NOTCONVERGED: return "not converged";
    default: return "CUDA or unknown error";
  }
}
