// Drop-in entry points with LACE's names and signatures (the first half of
// include/lace_gb300.h).  Each call uploads the caller's host containers,
// runs on the GPU through a process-wide context and writes the results back
// into the same containers, allocating output arrays the way LACE does
// (64-byte aligned, released with free() by data_zmfree).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <mutex>
#include <thread>
#include <vector>

#include "context.h"
#include "hostpar.h"

using namespace lace;

namespace {

std::mutex g_mu;
lace_gpu_ctx *g_ctx = nullptr;
lace_gpu_options g_dopt;
bool g_dopt_set = false;

// options the drop-in entry points run with (precision of the factors and
// solves, SpTRSV mode, graphs); LACE's own calls carry no such knobs
lace_gpu_options dropin_opts() {
  if (!g_dopt_set) {
    lace_gpu_default_options(&g_dopt);
    g_dopt_set = true;
  }
  return g_dopt;
}

int default_ctx(lace_gpu_ctx **out) {
  if (!g_ctx) {
    int dev = 0;
    if (const char *e = getenv("LACE_GB300_DEVICE")) dev = atoi(e);
    int rc = lace_gpu_ctx_create(&g_ctx, dev, nullptr);
    if (rc) return rc;
    g_ctx->verbose = getenv("LACE_GB300_VERBOSE") != nullptr;
  }
  cudaSetDevice(g_ctx->device);
  *out = g_ctx;
  return 0;
}

// wall time of the phases of a drop-in call, printed when the context is verbose
struct PhaseClock {
  bool on;
  const char *what;
  std::chrono::steady_clock::time_point t0, t;
  PhaseClock(bool on_, const char *what_) : on(on_), what(what_) { t0 = t = std::chrono::steady_clock::now(); }
  void mark(const char *phase) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    printf("%% %s %-28s %8.2f ms (%8.2f ms)\n", what, phase,
           std::chrono::duration<double, std::milli>(now - t).count(),
           std::chrono::duration<double, std::milli>(now - t0).count());
    t = now;
  }
};

template <typename T>
T *lace_alloc(size_t count) {
  // LACE_CALLOC (include/dense_types.h:430-449): posix_memalign(64), zeroed
  void *p = nullptr;
  size_t bytes = count * sizeof(T);
  size_t padded = (bytes / 64 + 1) * 64;
  if (posix_memalign(&p, 64, padded) != 0) return nullptr;
  memset(p, 0, padded);
  return (T *)p;
}

// the same allocation for `count` elements the caller writes at once: only
// the padding past them is zeroed here
template <typename T>
T *lace_alloc_filled(size_t count) {
  void *p = nullptr;
  size_t bytes = count * sizeof(T);
  size_t padded = (bytes / 64 + 1) * 64;
  if (posix_memalign(&p, 64, padded) != 0) return nullptr;
  memset((char *)p + bytes, 0, padded - bytes);
  return (T *)p;
}

// data_zmconvert frees these members of the output container first
// (control/magma_zmconverter.cpp:221-248)
void release_members(data_d_matrix *B) {
  free(B->val);
  free(B->col);
  free(B->row);
  free(B->rowidx);
  free(B->list);
  free(B->blockinfo);
  free(B->diag);
  B->val = nullptr;
  B->col = nullptr;
  B->row = nullptr;
  B->rowidx = nullptr;
  B->list = nullptr;
  B->blockinfo = nullptr;
  B->diag = nullptr;
}

bool is_csr(data_storage_t s) {
  return s == Magma_CSR || s == Magma_CUCSR || s == Magma_CSRL || s == Magma_CSRU;
}

// An output container from the factor pattern, in two steps: the host part
// (allocation, the pattern, the values' pages mapped) needs nothing from the
// GPU and can run while it works; the FP64 values on the device then go
// straight into the container's array.
// one piece of the output containers' bulk fill: a copy of src, or zeros
struct FillPiece {
  char *dst;
  const char *src;
  size_t bytes;
};

// the pieces as one byte range cut evenly over the host threads
void fill_pieces(const std::vector<FillPiece> &pc) {
  size_t total = 0;
  for (const FillPiece &p : pc) total += p.bytes;
  const int nt = host_threads(total);
  par_run(nt, [&](int t) {
    const size_t b = total * t / nt, e = total * (t + 1) / nt;
    size_t base = 0;
    for (const FillPiece &p : pc) {
      const size_t s = std::max(b, base), f = std::min(e, base + p.bytes);
      if (s < f) {
        if (p.src) memcpy(p.dst + (s - base), p.src + (s - base), f - s);
        else memset(p.dst + (s - base), 0, f - s);
      }
      base += p.bytes;
    }
  });
}

// the container's fields and arrays; its bulk fill appended to `pieces`
int prepare_csr_out(data_d_matrix *B, data_storage_t st, data_uplo_t fill, int n, const std::vector<int> &ptr,
                    const std::vector<int> &idx, int blocksize, std::vector<FillPiece> &pieces) {
  release_members(B);
  const int ld = blocksize > 0 ? blocksize * blocksize : 1;
  const size_t nval = idx.size() * ld;
  B->storage_type = st;
  B->major = MagmaRowMajor;
  B->fill_mode = fill;
  B->num_rows = n;
  B->num_cols = n;
  B->row = lace_alloc_filled<int>(ptr.size());
  B->col = lace_alloc_filled<int>(idx.size());
  B->val = lace_alloc_filled<double>(nval);
  if (!B->row || !B->col || !B->val) return DEV_ERR_HOST_ALLOC;
  // the values' pages mapped by host threads now, so that the copy into them
  // runs at full speed (faults taken inside it cost several times more)
  pieces.push_back({(char *)B->val, nullptr, 8 * nval});
  pieces.push_back({(char *)B->row, (const char *)ptr.data(), 4 * ptr.size()});
  pieces.push_back({(char *)B->col, (const char *)idx.data(), 4 * idx.size()});
  if (blocksize > 0) {
    B->blocksize = blocksize;
    B->ldblock = ld;
    B->numblocks = (int)idx.size();
    B->nnz = (int)nval;
  } else {
    B->nnz = (int)idx.size();
  }
  B->true_nnz = B->nnz;
  return 0;
}

// The output containers' host part for L (CSRL) and U (CSCU) of the
// context's factor patterns, on a host thread (spreading the bulk fill of
// both over the host pool), running while the GPU works.
struct OutPrep {
  std::thread th;
  int rcl = 0, rcu = 0;
  double ms = 0.0;
  std::chrono::steady_clock::time_point t0;
  bool started = false;
  void start(data_d_matrix *L, data_d_matrix *U, const lace_gpu_ctx *c, bool bcsr, int n, int blocksize) {
    L->diagorder_type = Magma_UNITY;
    U->diagorder_type = Magma_VALUE;
    t0 = std::chrono::steady_clock::now();
    th = std::thread([this, L, U, c, bcsr, n, blocksize] {
      std::vector<FillPiece> pieces;
      rcl = prepare_csr_out(L, bcsr ? Magma_BCSR : Magma_CSRL, MagmaLower, n, c->hL.ptr, c->hL.idx, blocksize,
                            pieces);
      rcu = prepare_csr_out(U, bcsr ? Magma_BCSCU : Magma_CSCU, MagmaUpper, n, c->hUc.ptr, c->hUc.idx, blocksize,
                            pieces);
      if (!rcl && !rcu) fill_pieces(pieces);
    });
    started = true;
  }
  int join() {
    if (th.joinable()) th.join();
    if (started) ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    started = false;
    return rcl ? rcl : rcu;
  }
  ~OutPrep() { join(); }
};

// the values (nval FP64 on the device) into a prepared container; enqueued
int finish_csr_out(data_d_matrix *B, const void *dval, size_t nval, cudaStream_t s) {
  return cudaMemcpyAsync(B->val, dval, 8 * nval, cudaMemcpyDeviceToHost, s) == cudaSuccess ? 0 : DEV_ERR_UNKNOWN;
}

// mode 0: data_PariLU_v0_3 stop rule (step <= reduction*Ares, <= 20 sweeps,
// src/parilu_v0_3.cpp:43-62); mode 1: prescribed sweeps (log->maxSweeps, step
// > 4 eps, src/parilu_v0_3_prescribedSweeps.cpp:62)
void parilu_dropin(data_d_matrix *A, data_d_matrix *L, data_d_matrix *U, dataType reduction,
                   data_d_preconditioner_log *log, int mode) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto fail = [&](int code) {
    set_err(code);
    if (log) log->sweeps = -1;
  };
  if (!A || !L || !U || !log) return fail(DEV_ERR_INVALID_PTR);
  lace_gpu_ctx *c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return fail(rc);
  lace_gpu_options o = dropin_opts();
  lace_gpu_set_options(c, &o);
  PhaseClock pc(c->verbose, "parilu");
  const bool bcsr = A->storage_type == Magma_BCSR;
  const int n = A->num_rows;
  OutPrep prep;
  // The common case, the pattern the context already holds: checked first
  // (on the GPU), so that the output containers can be prepared from the
  // start, while A's values go up and the GPU sweeps.
  bool known = false;
  const int nblk_in = bcsr ? (A->numblocks > 0 ? A->numblocks : A->row[n]) : A->row[n];
  if (((!bcsr && is_csr(A->storage_type) && c->bs == 0 && (int)c->hArow.size() == n + 1) ||
       (bcsr && c->bs == A->blocksize && A->row[n] == nblk_in)) &&
      c->n_blk == n && c->nnzA == nblk_in && (int)c->hL.ptr.size() == n + 1 &&
      c->hL.idx.size() == (size_t)c->nnzL) {
    const int *h[2] = {A->row, A->col};
    const int *d[2] = {(const int *)c->Arow.p, (const int *)c->Acol.p};
    const size_t cnt[2] = {(size_t)n + 1, (size_t)nblk_in};
    rc = c->same_on_device(2, h, d, cnt, &known);
    if (rc) return fail(rc);
  }
  if (known) {
    prep.start(L, U, c, bcsr, n, bcsr ? A->blocksize : 0);
    rc = c->upload_values_same_pattern(A->val);
  } else if (bcsr) {
    const int bs = A->blocksize;
    const int nblk = A->numblocks > 0 ? A->numblocks : A->row[n];
    rc = lace_gpu_upload_bcsr_host(c, n, bs, nblk, A->row, A->col, A->val);
  } else if (is_csr(A->storage_type)) {
    rc = lace_gpu_upload_csr_host(c, n, A->row[n], A->row, A->col, A->val);
  } else {
    rc = DEV_ERR_NOT_SUPPORTED;
  }
  if (rc) return fail(rc);
  pc.mark("upload A");
  // residuals of the A-initial guess (src/parilu_v0_3.cpp:30-34), on the GPU
  double ares = 0.0, nonlin0 = NAN;
  if (!bcsr) {
    rc = c->parilu(0, nullptr, nullptr, true, nullptr);
    if (!rc) rc = c->ilu_residuals(&ares, &nonlin0);
    if (rc) return fail(rc);
  }
  double tol;
  int maxs;
  if (bcsr) {  // src/parilu_v0_3_bcsr.cpp:61,118: un-normalised step <= reduction
    tol = reduction / c->anorm;
    maxs = 100;
  } else if (mode == 0) {
    tol = reduction * ares;
    // LACE caps its asynchronous sweeps at 20 (:45).  A synchronous sweep
    // needs up to (dependency depth of L and U) sweeps to reach the same
    // fixed point, so the cap is raised to that depth where it is larger.
    maxs = std::max(20, c->nlevels[0] + c->nlevels[1] + 2);
  } else {
    tol = std::numeric_limits<double>::epsilon() * 4.0;
    maxs = log->maxSweeps;
  }
  // A synchronous sweep can take a small step while still away from the fixed
  // point (LACE's in-place sweep reaches it in one pass in its one-thread
  // order).  When the dependency depth is small, run at least depth+1 sweeps:
  // the synchronous iteration is then exact, like LACE's.
  const int depth = c->nlevels[0] + c->nlevels[1];
  const int min_sweeps = (mode == 0 && !bcsr && depth + 1 <= 64) ? std::min(depth + 1, maxs) : 0;
  std::vector<double> steps;
  double step = 0.0;
  // a new pattern: the output containers are prepared while the GPU sweeps
  if (!known) prep.start(L, U, c, bcsr, n, bcsr ? A->blocksize : 0);
  auto t0 = std::chrono::steady_clock::now();
  // the sweeps start from the initial guess the residuals above were taken
  // of (no second initialisation); like LACE, no residual after them
  rc = c->parilu(maxs, &step, nullptr, true, &steps, tol, min_sweeps, !bcsr);
  const double gen = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  const int prep_rc = prep.join();
  if (rc) return fail(rc);
  if (prep_rc) return fail(prep_rc);
  if (c->verbose) printf("%% parilu (output containers prepared in %.2f ms)\n", prep.ms);
  pc.mark("residuals + sweeps");
  // L values (CSRL order) and U values (CSCU order) as FP64, copied straight
  // into the output containers
  const int ld = bcsr ? A->blocksize * A->blocksize : 1;
  const size_t nl = (size_t)c->nnzL * ld, nu = (size_t)c->nnzU * ld;
  const void *dl = c->Lv[c->cur].p, *du = c->Ucv[c->cur].p;
  if (c->vtype() != VType::F64) {
    // FP32 / BF16 factors travel back as LACE's FP64 values, through the
    // context's staging buffer (no allocation per call)
    if (c->stage64.ensure(8 * (nl + nu))) return fail(DEV_ERR_DEVICE_ALLOC);
    double *tl = (double *)c->stage64.p, *tu = tl + nl;
    launch_convert(c->stream, (int)nl, c->vtype(), dl, VType::F64, tl);
    launch_convert(c->stream, (int)nu, c->vtype(), du, VType::F64, tu);
    dl = tl;
    du = tu;
  }
  if (cudaGetLastError() != cudaSuccess) return fail(DEV_ERR_UNKNOWN);
  rc = finish_csr_out(L, dl, nl, c->stream);
  if (!rc) rc = finish_csr_out(U, du, nu, c->stream);
  if (!rc && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = DEV_ERR_UNKNOWN;
  if (rc) return fail(rc);
  U->major = MagmaColMajor;
  pc.mark("fill L, U");
  log->sweeps = (int)steps.size();
  log->tol = tol;
  log->finalStep = steps.empty() ? 0.0 : steps.back();
  log->A_Frobenius = c->anorm;
  log->precond_generation_time = gen;
  log->initial_residual = ares;
  log->initial_nonlinear_residual = nonlin0;
  log->omp_num_threads = num_sms();
  set_err(0);
}

int upload_vec(DBuf &d, const double *h, int n, cudaStream_t s) { return d.upload(h, 8 * (size_t)n, s); }

}  // namespace

extern "C" void data_PariLU_v0_3(data_d_matrix *A, data_d_matrix *L, data_d_matrix *U, dataType reduction,
                                 data_d_preconditioner_log *log) {
  parilu_dropin(A, L, U, reduction, log, 0);
}

extern "C" void data_PariLU_v0_3_prescribedSweeps(data_d_matrix *A, data_d_matrix *L, data_d_matrix *U,
                                                  dataType reduction, data_d_preconditioner_log *log) {
  parilu_dropin(A, L, U, reduction, log, 1);
}

extern "C" void data_PariLU_v0_3_gpu(data_d_matrix *A, data_d_matrix *L, data_d_matrix *U,
                                     dataType reduction, data_d_preconditioner_log *log, int nthreads) {
  (void)nthreads;
  parilu_dropin(A, L, U, reduction, log, 0);
}

extern "C" void data_PariLU_v0_3_gpu_prescribedSweeps(data_d_matrix *A, data_d_matrix *L,
                                                      data_d_matrix *U, dataType reduction,
                                                      data_d_preconditioner_log *log) {
  parilu_dropin(A, L, U, reduction, log, 1);
}

extern "C" int data_parcsrtrsv(const data_uplo_t uplo, const data_storage_t storage,
                               const data_diagorder_t diag, const int num_rows, const dataType *Aval,
                               const int *row, const int *col, const dataType *rhsval, dataType *yval,
                               const dataType tol, int *iter) {
  // storage / fill checks of src/trisolve.cpp:262-345
  bool lower;
  if (storage == Magma_CSRL && uplo == MagmaLower && diag != Magma_NODIAG) lower = true;
  else if (storage == Magma_CSRL || uplo == MagmaLower) return -1;
  else if (storage == Magma_CSRU && uplo == MagmaUpper && diag != Magma_NODIAG) lower = false;
  else if (storage == Magma_CSRU || uplo == MagmaUpper) return -1;
  else return 0;
  if (!iter) return set_err(DEV_ERR_INVALID_PTR);
  *iter = 0;
  if (num_rows <= 0) return 0;
  if (!Aval || !row || !col || !rhsval || !yval) return set_err(DEV_ERR_INVALID_PTR);
  std::lock_guard<std::mutex> lk(g_mu);
  lace_gpu_ctx *c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return set_err(rc);
  const int n = num_rows;
  const int nnz = row[n];
  if (nnz < 0) return set_err(DEV_ERR_ILLEGAL_VALUE);
  DBuf drow, dcol, dval, drhs, dy, da;
  if (drow.upload(row, 4 * (size_t)(n + 1), c->stream) || dcol.upload(col, 4 * (size_t)nnz, c->stream) ||
      dval.upload(Aval, 8 * (size_t)nnz, c->stream) || upload_vec(drhs, rhsval, n, c->stream) ||
      upload_vec(dy, yval, n, c->stream) || da.ensure(8 * (size_t)n))
    return set_err(DEV_ERR_DEVICE_ALLOC);
  PartrsvScratch sc;
  sc.a = (double *)da.p;
  sc.partials = (double *)c->part_ensure();
  if (!sc.partials) return set_err(DEV_ERR_DEVICE_ALLOC);
  sc.counters = (int *)c->cnt_buf.p + 16;
  sc.steps = (double *)c->scal_buf.p + 48;
  sc.h_steps = c->h_scal + 48;
  sc.h_status = (int *)(c->h_scal + 50);
  rc = partrsv_solve(c->stream, lower, n, (const int *)drow.p, (const int *)dcol.p, (const double *)dval.p,
                     (const double *)drhs.p, (double *)dy.p, tol, iter, sc);
  if (rc) return set_err(rc);
  if (cudaMemcpy(yval, dy.p, 8 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess) return set_err(DEV_ERR_UNKNOWN);
  return 0;
}

extern "C" int lace_gpu_get_orthog_history(lace_gpu_ctx *c, double *out, int capacity, int *count) {
  if (!count || (capacity > 0 && !out)) return set_err(DEV_ERR_INVALID_PTR);
  std::unique_lock<std::mutex> lk(g_mu, std::defer_lock);
  if (!c) {  // the LACE-named calls' context
    lk.lock();
    int rc = default_ctx(&c);
    if (rc) return set_err(rc);
  }
  const int nh = (int)c->last_orth.size();
  *count = nh;
  for (int k = 0; k < nh && k < capacity; ++k) out[k] = c->last_orth[k];
  return DEV_SUCCESS;
}

extern "C" int data_z_spmv(dataType alpha, data_d_matrix *A, data_d_matrix *x, dataType beta,
                           data_d_matrix *y) {
  if (!A || !x || !y) return set_err(DEV_ERR_INVALID_PTR);
  const bool bcsr = A->storage_type == Magma_BCSR;
  const int bs = bcsr ? A->blocksize : 1;
  const int ncols = bcsr ? A->num_cols * bs : A->num_cols;
  if (!(ncols == x->num_rows && x->num_cols == 1)) return DEV_ERR_NOT_SUPPORTED;  // blas/zspmv.cpp:71-75
  if (!bcsr && !is_csr(A->storage_type)) return DEV_ERR_NOT_SUPPORTED;         // :65-68
  std::lock_guard<std::mutex> lk(g_mu);
  lace_gpu_ctx *c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return set_err(rc);
  const int nr = A->num_rows;
  const int nnz = A->row[nr];
  const int ld = bcsr ? bs * bs : 1;
  const int nout = bcsr ? nr * bs : nr;
  DBuf drow, dcol, dval, dx, dy;
  if (drow.upload(A->row, 4 * (size_t)(nr + 1), c->stream) || dcol.upload(A->col, 4 * (size_t)nnz, c->stream) ||
      dval.upload(A->val, 8 * (size_t)nnz * ld, c->stream) || upload_vec(dx, x->val, ncols, c->stream) ||
      (beta != 0.0 ? upload_vec(dy, y->val, nout, c->stream) : dy.ensure(8 * (size_t)nout)))
    return set_err(DEV_ERR_DEVICE_ALLOC);
  if (bcsr)
    launch_bcsr_spmv(c->stream, nr, bs, (const int *)drow.p, (const int *)dcol.p, (const double *)dval.p,
                     (const double *)dx.p, alpha, beta, (double *)dy.p);
  else {
    const double avg = nr ? (double)nnz / nr : 1.0;
    const int lanes = avg > 24 ? 32 : (avg > 12 ? 16 : (avg > 6 ? 8 : 4));
    launch_spmv_f64x(c->stream, lanes, nr, (const int *)drow.p, (const int *)dcol.p, (const double *)dval.p,
                     (const double *)dx.p, alpha, beta, (double *)dy.p);
  }
  if (cudaMemcpyAsync(y->val, dy.p, 8 * (size_t)nout, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return set_err(DEV_ERR_UNKNOWN);
  return DEV_SUCCESS;
}

namespace {

// U as CSR with the diagonal first: CSRU as given, or the transpose of CSCU
void u_as_csr(const data_d_matrix *U, std::vector<int> &ptr, std::vector<int> &idx,
              std::vector<double> &val) {
  const int n = U->num_rows;
  const int nnz = U->row[n];
  if (U->storage_type == Magma_CSCU || U->storage_type == Magma_CSC) {
    Pattern P, T;
    P.n = n;
    P.ptr.assign(U->row, U->row + n + 1);
    P.idx.assign(U->col, U->col + nnz);
    std::vector<int> t2p;
    transpose_pattern(P, T, t2p);
    ptr = T.ptr;
    idx = T.idx;
    val.resize(nnz);
    for (int q = 0; q < nnz; ++q) val[q] = U->val[t2p[q]];
  } else {
    ptr.assign(U->row, U->row + n + 1);
    idx.assign(U->col, U->col + nnz);
    val.assign(U->val, U->val + nnz);
  }
}

// method 0: FGMRES-Householder; 1: FGMRES with modified Gram-Schmidt
// (restarted: data_fgmres_restart, else data_fgmres)
int fgmres_dropin(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0, data_d_matrix *L,
                  data_d_matrix *U, data_d_gmres_param *par, data_d_gmres_log *log, int restart_max,
                  int method, int restarted) {
  if (!A || !b || !x0 || !par || !log) return set_err(DEV_ERR_INVALID_PTR);
  // CSR, as LACE; a BCSR operator (with the BCSR / BCSC factors
  // data_PariLU_v0_3 returns for it) is this library's extension: LACE's
  // data_z_spmv and solves take CSR only
  const bool bcsr = A->storage_type == Magma_BCSR;
  if (!is_csr(A->storage_type) && !bcsr) return set_err(DEV_ERR_NOT_SUPPORTED);
  std::lock_guard<std::mutex> lk(g_mu);
  auto t0 = std::chrono::steady_clock::now();
  lace_gpu_ctx *c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return set_err(rc);
  lace_gpu_options o = dropin_opts();
  o.monitor_orthog = par->monitorOrthog == 1;
  // choice 1 (data_parcsrtrsv with tol 1.0, fgmres_householder_restart.cpp:
  // 333-344) sweeps in LACE's order, where the first sweep is the exact
  // substitution and the second changes nothing: its preconditioned vector is
  // the exact solve's, which the sync-free solves give (choice 0)
  const int choice = par->user_csrtrsv_choice;
  if (choice == 2) o.trsv_mode = LACE_TRSV_NONE;
  else if (o.trsv_mode != LACE_TRSV_LEVELS) o.trsv_mode = LACE_TRSV_SYNCFREE;
  lace_gpu_set_options(c, &o);
  PhaseClock pc(c->verbose, "fgmres");
  // rows of the pattern (block rows for BCSR) and of the vectors
  const int nr = A->num_rows;
  const int n = bcsr ? nr * A->blocksize : nr;
  if (bcsr)
    rc = lace_gpu_upload_bcsr_host(c, nr, A->blocksize, A->numblocks > 0 ? A->numblocks : A->row[nr], A->row, A->col,
                                   A->val);
  else
    rc = lace_gpu_upload_csr_host(c, nr, A->row[nr], A->row, A->col, A->val);
  if (rc) return set_err(rc);
  pc.mark("upload A");
  if (choice != 2) {
    if (!L || !U) return set_err(DEV_ERR_INVALID_PTR);
    // factors as ParILU returned them (U in CSC, or BCSC for a BCSR operator;
    // the context's own patterns): values go up as they are; CSR factors in
    // other layouts are converted on the host
    rc = 1;
    if (bcsr) {
      if (L->storage_type == Magma_BCSR && U->storage_type == Magma_BCSCU && L->num_rows == nr &&
          U->num_rows == nr && L->blocksize == A->blocksize && U->blocksize == A->blocksize)
        rc = c->set_factors_csc_host(nr, L->row, L->col, L->val, U->row, U->col, U->val);
      if (rc == 1) return set_err(DEV_ERR_NOT_SUPPORTED);
    } else if ((U->storage_type == Magma_CSCU || U->storage_type == Magma_CSC) && L->num_rows == n &&
               U->num_rows == n) {
      rc = c->set_factors_csc_host(n, L->row, L->col, L->val, U->row, U->col, U->val);
    }
    if (rc == 1) {
      std::vector<int> up, ui;
      std::vector<double> uv;
      u_as_csr(U, up, ui, uv);
      pc.mark("U as CSR");
      rc = c->set_factors_host(n, L->row, L->col, L->val, up.data(), ui.data(), uv.data());
    }
    if (rc) return set_err(rc);
    pc.mark("set factors");
  }
  // b and x0 in buffers the context keeps (no allocation per call)
  if (upload_vec(c->dropin_b, b->val, n, c->stream) || upload_vec(c->dropin_x, x0->val, n, c->stream))
    return set_err(DEV_ERR_DEVICE_ALLOC);
  int total = 0;
  rc = c->fgmres((const double *)c->dropin_b.p, (double *)c->dropin_x.p, par->search_max, restart_max,
                 par->tol_type, par->rtol, false, log, &total, nullptr, method, restarted, par->reorth);
  if (rc != DEV_SUCCESS && rc != DEV_NOTCONVERGED) return set_err(rc);
  pc.mark("b, x0 + solve");
  if (cudaMemcpy(x0->val, c->dropin_x.p, 8 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
    return set_err(DEV_ERR_UNKNOWN);
  pc.mark("download x");
  log->solve_time = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (c->verbose)
    printf("gmres_search_directions = %d;\ngmres_total_search_directions = %d;\n", log->search_directions,
           total);
  return rc;
}

}  // namespace

extern "C" int data_fgmres_householder_restart(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0,
                                               data_d_matrix *L, data_d_matrix *U,
                                               data_d_gmres_param *gmres_par, data_d_gmres_log *gmres_log) {
  return fgmres_dropin(A, b, x0, L, U, gmres_par, gmres_log, gmres_par ? gmres_par->restart_max : 0, 0, 1);
}

extern "C" int data_fgmres_householder(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0,
                                       data_d_matrix *L, data_d_matrix *U, data_d_gmres_param *gmres_par,
                                       data_d_gmres_log *gmres_log) {
  return fgmres_dropin(A, b, x0, L, U, gmres_par, gmres_log, 1, 0, 1);
}

extern "C" int data_fgmres_restart(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0, data_d_matrix *L,
                                   data_d_matrix *U, data_d_gmres_param *gmres_par, data_d_gmres_log *gmres_log) {
  return fgmres_dropin(A, b, x0, L, U, gmres_par, gmres_log, gmres_par ? gmres_par->restart_max : 0, 1, 1);
}

extern "C" int data_fgmres(data_d_matrix *A, data_d_matrix *b, data_d_matrix *x0, data_d_matrix *L,
                           data_d_matrix *U, data_d_gmres_param *gmres_par, data_d_gmres_log *gmres_log) {
  return fgmres_dropin(A, b, x0, L, U, gmres_par, gmres_log, 1, 1, 0);
}

// LACE's ILU residual pair (control/norms.cpp:301-405): res = ||A - LU||_F
// over the product's pattern (fill included) and nonlinres over the entries
// of A it holds, without forming LU.  L: CSRL with its unit diagonal stored
// (L.row[1] == 1), or strictly lower (L.row[1] == 0: the unit diagonal is
// implied, :327-349), as LACE tells them apart; U: CSRU or CSCU.  *LU is not
// formed: the caller's matrix is left as passed (LACE's callers only free it).
extern "C" int data_zilures(data_d_matrix A, data_d_matrix L, data_d_matrix U, data_d_matrix *LU,
                            dataType *res, dataType *nonlinres) {
  (void)LU;
  if (!res || !nonlinres) return set_err(DEV_ERR_INVALID_PTR);
  if (!is_csr(A.storage_type) || !L.row || !U.row) return set_err(DEV_ERR_NOT_SUPPORTED);
  const int n = A.num_rows;
  if (L.num_rows != n || U.num_rows != n || n < 1) return set_err(DEV_ERR_ILLEGAL_VALUE);
  std::vector<int> lp, li;
  std::vector<double> lv;
  if (L.row[1] == 1) {
    lp.assign(L.row, L.row + n + 1);
    li.assign(L.col, L.col + L.row[n]);
    lv.assign(L.val, L.val + L.row[n]);
  } else if (L.row[1] == 0) {  // strictly lower: the unit diagonal appended to each row
    lp.assign(n + 1, 0);
    for (int i = 0; i < n; ++i) {
      for (int p = L.row[i]; p < L.row[i + 1]; ++p) {
        li.push_back(L.col[p]);
        lv.push_back(L.val[p]);
      }
      li.push_back(i);
      lv.push_back(1.0);
      lp[i + 1] = (int)li.size();
    }
  } else {
    return set_err(DEV_ERR_NOT_SUPPORTED);  // LACE: "L neither lower nor strictly lower triangular"
  }
  std::lock_guard<std::mutex> lk(g_mu);
  lace_gpu_ctx *c = nullptr;
  int rc = default_ctx(&c);
  if (rc) return set_err(rc);
  lace_gpu_options o;
  lace_gpu_default_options(&o);
  lace_gpu_set_options(c, &o);
  rc = lace_gpu_upload_csr_host(c, n, A.row[n], A.row, A.col, A.val);
  if (rc) return set_err(rc);
  std::vector<int> up, ui;
  std::vector<double> uv;
  u_as_csr(&U, up, ui, uv);
  rc = c->set_factors_host(n, lp.data(), li.data(), lv.data(), up.data(), ui.data(), uv.data());
  if (!rc) rc = c->ilu_residuals(res, nonlinres);
  return rc ? set_err(rc) : DEV_SUCCESS;
}

namespace {

// a BCSR matrix (block rows nb, blocks bs x bs stored row-major) as scalar
// CSR holding every entry of every block, rows sorted by column (LACE's
// BCSR -> CSR conversion through mkl_dcsrbsr, control/magma_zmconverter.cpp:
// 802-836)
int bcsr_expand(const data_d_matrix &B, int nb, int bs, std::vector<int> &ptr, std::vector<int> &idx,
                std::vector<double> &val) {
  if (!B.row || !B.col || !B.val || B.row[0] != 0) return DEV_ERR_ILLEGAL_VALUE;
  const int ld = bs * bs;
  for (int I = 0; I < nb; ++I)
    if (B.row[I + 1] < B.row[I]) return DEV_ERR_ILLEGAL_VALUE;
  for (int p = 0; p < B.row[nb]; ++p)
    if (B.col[p] < 0 || B.col[p] >= nb) return DEV_ERR_ILLEGAL_VALUE;
  const int n = nb * bs;
  ptr.assign(n + 1, 0);
  for (int I = 0; I < nb; ++I)
    for (int r = 0; r < bs; ++r) ptr[I * bs + r + 1] = (B.row[I + 1] - B.row[I]) * bs;
  for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  idx.resize(ptr[n]);
  val.resize(ptr[n]);
  std::vector<std::pair<int, double>> row;
  for (int I = 0; I < nb; ++I)
    for (int r = 0; r < bs; ++r) {
      row.clear();
      for (int p = B.row[I]; p < B.row[I + 1]; ++p)
        for (int c = 0; c < bs; ++c) row.emplace_back(B.col[p] * bs + c, B.val[(size_t)p * ld + r * bs + c]);
      std::stable_sort(row.begin(), row.end(),
                       [](const std::pair<int, double> &x, const std::pair<int, double> &y) { return x.first < y.first; });
      int q = ptr[I * bs + r];
      for (const auto &e : row) {
        idx[q] = e.first;
        val[q++] = e.second;
      }
    }
  return 0;
}

}  // namespace

// data_zilures_bcsr (control/norms.cpp:409-468): L and U are read as BCSR
// (block rows L.num_rows, blocks L.blocksize^2, row-major) and expanded to
// scalar CSR with every block entry, their product measured against A
// (scalar CSR, num_rows = blocks x blocksize) as data_zilures does, L's
// values as stored.  LACE converts both factors with the BCSR reader
// whatever their storage tag, so a BCSCU U is read as its block transpose
// there and here alike.  *LU is not formed.
extern "C" int data_zilures_bcsr(data_d_matrix A, data_d_matrix L, data_d_matrix U, data_d_matrix *LU,
                                 dataType *res, dataType *nonlinres) {
  (void)LU;
  if (!res || !nonlinres) return set_err(DEV_ERR_INVALID_PTR);
  if (!is_csr(A.storage_type) || !A.row) return set_err(DEV_ERR_NOT_SUPPORTED);
  const int bs = L.blocksize, nb = L.num_rows;
  if (bs <= 0 || U.blocksize != bs || U.num_rows != nb || nb < 1) return set_err(DEV_ERR_NOT_SUPPORTED);
  const int n = nb * bs;
  if (A.num_rows != n) return set_err(DEV_ERR_ILLEGAL_VALUE);
  std::vector<int> lp, li, up, ui;
  std::vector<double> lv, uv;
  int rc = bcsr_expand(L, nb, bs, lp, li, lv);
  if (!rc) rc = bcsr_expand(U, nb, bs, up, ui, uv);
  if (rc) return set_err(rc);
  for (int p = 0; p < A.row[n]; ++p)
    if (A.col[p] < 0 || A.col[p] >= n) return set_err(DEV_ERR_ILLEGAL_VALUE);
  // U's CSC image for the entries of A
  Pattern P, Tp;
  P.n = n;
  P.ptr = up;
  P.idx = ui;
  std::vector<int> t2p;
  transpose_pattern(P, Tp, t2p);
  std::vector<double> ucv(t2p.size());
  for (size_t q = 0; q < t2p.size(); ++q) ucv[q] = uv[t2p[q]];
  std::lock_guard<std::mutex> lk(g_mu);
  lace_gpu_ctx *c = nullptr;
  rc = default_ctx(&c);
  if (rc) return set_err(rc);
  DBuf dAr, dAc, dAv, dLr, dLc, dLv, dUr, dUc, dUv, dCp, dCi, dCv;
  const cudaStream_t s = c->stream;
  if (dAr.upload(A.row, 4 * (size_t)(n + 1), s) || dAc.upload(A.col, 4 * (size_t)A.row[n] + 4, s) ||
      dAv.upload(A.val, 8 * (size_t)A.row[n] + 8, s) || dLr.upload(lp.data(), 4 * lp.size(), s) ||
      dLc.upload(li.data(), 4 * li.size() + 4, s) || dLv.upload(lv.data(), 8 * lv.size() + 8, s) ||
      dUr.upload(up.data(), 4 * up.size(), s) || dUc.upload(ui.data(), 4 * ui.size() + 4, s) ||
      dUv.upload(uv.data(), 8 * uv.size() + 8, s) || dCp.upload(Tp.ptr.data(), 4 * Tp.ptr.size(), s) ||
      dCi.upload(Tp.idx.data(), 4 * Tp.idx.size() + 4, s) || dCv.upload(ucv.data(), 8 * ucv.size() + 8, s))
    return set_err(DEV_ERR_DEVICE_ALLOC);
  IluArgs a = c->ilu_args();
  a.n = n;
  a.nnzA = A.row[n];
  a.Arow = (const int *)dAr.p;
  a.Acol = (const int *)dAc.p;
  a.Aval = (const double *)dAv.p;
  a.Lrow = (const int *)dLr.p;
  a.Lcol = (const int *)dLc.p;
  a.Ucp = (const int *)dCp.p;
  a.Uri = (const int *)dCi.p;
  a.bs = 0;
  if (!a.partials) return set_err(DEV_ERR_DEVICE_ALLOC);
  double *d = (double *)c->scal_buf.p + 42;
  launch_lu_fro(s, a, VType::F64, (const int *)dUr.p, (const int *)dUc.p, dLv.p, dUv.p, dCv.p, d, 0);
  if (cudaMemcpyAsync(c->h_scal + 42, d, 3 * 8, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return set_err(DEV_ERR_UNKNOWN);
  const double fro = c->h_scal[42], onS = c->h_scal[43], nl2 = c->h_scal[44];
  *nonlinres = std::sqrt(nl2);
  *res = std::sqrt(std::max(0.0, nl2 + fro - onS));
  return DEV_SUCCESS;
}

extern "C" int lace_gpu_dropin_set_options(const lace_gpu_options *opt) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!opt) {
    lace_gpu_default_options(&g_dopt);
  } else {
    if (opt->precision < 0 || opt->precision > 2 || opt->trsv_mode < 0 || opt->trsv_mode > 3)
      return set_err(DEV_ERR_ILLEGAL_VALUE);
    g_dopt = *opt;
  }
  g_dopt_set = true;
  return DEV_SUCCESS;
}

// ABI self-description: sizes and member offsets of LACE's structs
extern "C" int lace_gpu_abi_layout(int *out, int cap) {
  const int v[] = {
      (int)sizeof(data_d_matrix),
      (int)offsetof(data_d_matrix, num_rows),
      (int)offsetof(data_d_matrix, nnz),
      (int)offsetof(data_d_matrix, val),
      (int)offsetof(data_d_matrix, diag),
      (int)offsetof(data_d_matrix, row),
      (int)offsetof(data_d_matrix, rowidx),
      (int)offsetof(data_d_matrix, col),
      (int)offsetof(data_d_matrix, list),
      (int)offsetof(data_d_matrix, blockinfo),
      (int)offsetof(data_d_matrix, blocksize),
      (int)offsetof(data_d_matrix, ldblock),
      (int)offsetof(data_d_matrix, numblocks),
      (int)offsetof(data_d_matrix, major),
      (int)offsetof(data_d_matrix, ld),
      (int)offsetof(data_d_matrix, pad_cols),
      (int)sizeof(data_d_preconditioner_log),
      (int)offsetof(data_d_preconditioner_log, tol),
      (int)offsetof(data_d_preconditioner_log, omp_num_threads),
      (int)sizeof(data_d_gmres_log),
      (int)offsetof(data_d_gmres_log, solve_time),
      (int)offsetof(data_d_gmres_log, original_residual),
      (int)sizeof(data_d_gmres_param),
      (int)offsetof(data_d_gmres_param, rtol),
      (int)offsetof(data_d_gmres_param, restart_max),
      (int)offsetof(data_d_gmres_param, parilu_reduction),
      (int)offsetof(data_d_gmres_param, reorder),
  };
  const int nv = (int)(sizeof(v) / sizeof(v[0]));
  for (int i = 0; i < nv && i < cap; ++i) out[i] = v[i];
  return nv;
}
