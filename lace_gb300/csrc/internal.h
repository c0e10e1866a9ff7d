// Internal interfaces between the lace_gb300 translation units: device data
// structures shared by kernels and the host-side launchers that
// context.cu calls.  Not part of the public C ABI (include/lace_gb300.h).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace lace {

// Largest restart length (search_max) the device FGMRES supports.
constexpr int kMaxM = 128;
constexpr int kLdT = kMaxM + 2;  // leading dimension of the small matrices

// Device-resident scalar state of one FGMRES cycle.  The small matrices
// are column-major with leading dimension kLdT.
struct Cycle {
  double T[kLdT * kLdT];  // compact-WY factor: P_0...P_j = I - V T V^T
  double R[kLdT * kLdT];  // Givens-rotated Hessenberg (upper triangular)
  double g[kLdT];         // rotated right-hand side of the LS problem
  double cs[kLdT], sn[kLdT];
  double y[kLdT];         // T^T (V^T w) of pass A
  double c[kLdT];         // T_{j+1} rho of pass B, consumed by pass C
  double yls[kLdT];       // least-squares solution at the end of a cycle
  double hist[kLdT];      // |g_{j+1}| per search direction of the cycle
  double orth[kLdT];      // ||I - Q^T Q||_inf per direction (when monitored)
  double dd;              // sign(w_{j+1}) ||w_{j+1:}||   (H(j+1,j) = -dd)
  double inv_alpha;       // 1 / ||w_{j+1:} + dd e_{j+1}||
  double dd0, inv_alpha0; // first reflector of the cycle
  double rnorm;           // ||b - A x|| at the start of the cycle
  int tol_type;
  int first_cycle;
  double rtol;
  // modified Gram-Schmidt Arnoldi (data_fgmres_restart / data_fgmres):
  // column j of the Hessenberg matrix before the rotations, the second
  // pass's coefficients, ||A z_j||, 1/h_{j+1,j} (0 after a breakdown) and
  // whether this step reorthogonalises
  double h[kLdT];
  double hr[kLdT];
  double normav;
  double hinv;
  int reorth;
  int nreorth;  // steps of the cycle that reorthogonalised
  // rows 0..j+1 of w after the step's update, published by the blocks that
  // own them (the one-kernel Householder step)
  double wtop[kLdT];
  // the Gram matrix V^T V of the reflectors (column-major, diagonal 1): its
  // column j+1 is V^T v_{j+1}, which step j forms for T anyway; the
  // double-float one-kernel step takes V^T w over rows > j from it
  double G[kLdT * kLdT];
};

// Handles for the two triangles of one solve direction.
struct TriDev {
  int n = 0;
  int nnz = 0;
  const int *row = nullptr;
  const int *col = nullptr;
  const void *val = nullptr;  // double / float / bf16 per precision
  int lower = 1;
  int unit = 0;
  int rows_per_lane = 4;
  int nchunks = 0;
  int *ready = nullptr;
  int slot = 0;  // index into Control::trsv_epoch / tickets
  // level-scheduled option
  const int *lvl_ptr = nullptr;
  const int *lvl_rows = nullptr;
  int nlevels = 0;
  // BCSR solves: chunks of block rows in solve order (first position of each
  // chunk, bnch + 1 entries)
  const int *bchunk_first = nullptr;
  int bnch = 0;
};

enum class VType { F64 = 0, F32 = 1, BF16 = 2 };

// ---------------------------------------------------------------- SpMV
// y = alpha*A*x + beta*y (x double or float), lanes per row in {1,2,4,8,16,32}
void launch_spmv_f64x(cudaStream_t s, int lanes, int n, const int *row, const int *col,
                      const double *val, const double *x, double alpha, double beta, double *y);
void launch_spmv_f32x(cudaStream_t s, int lanes, int n, const int *row, const int *col,
                      const double *val, const float *x, double alpha, double beta, double *y);
void launch_bcsr_spmv(cudaStream_t s, int nb, int bs, const int *row, const int *col,
                      const double *val, const double *x, double alpha, double beta, double *y);
// the same on A's sliced-ELL copy (row: A's CSR row pointers, for the row lengths)
void launch_sell_spmv(cudaStream_t s, int n, const int *row, const int *sell_ptr, const int *sell_col,
                      const double *sell_val, const double *x, double alpha, double beta, double *y);

// ---------------------------------------------------- FGMRES-Householder
struct ArnoldiArgs {
  int n = 0;
  // operator: CSR (bs == 0) or BCSR (bs > 0)
  int bs = 0;
  const int *row = nullptr, *col = nullptr;
  const double *val = nullptr;
  int lanes = 8;
  // the same operator in sliced ELL (slices of 32 rows, entry t of the
  // slice's rows stored together: index sell_ptr[s] + 32 t + lane); null when
  // absent
  const int *sell_ptr = nullptr, *sell_col = nullptr;
  const double *sell_val = nullptr;
  const float2 *sell_pair = nullptr;  // sell_val as (hi, lo) pairs
  double *V = nullptr;   // reflectors, n x (m+1) column-major
  size_t ldv = 0;
  // the reflectors again in FP32 (rounded toward zero, same leading
  // dimension), when the next Krylov vector q is FP32: pass C forms q from
  // them, reading half the bytes; null otherwise
  float *Vf = nullptr;
  // with Vf: the remainder v - Vf, also in FP32 (same leading dimension), so
  // that (Vf, Vlo) hold each reflector entry to about 48 bits and the
  // one-kernel step forms its products on the FP32 unit; null otherwise
  float *Vlo = nullptr;
  void *Z = nullptr;     // preconditioned vectors, n x m (float or double)
  size_t ldz = 0;
  int z_f32 = 0;
  double *w = nullptr;   // work vector (A z, later the transformed column)
  void *q = nullptr;     // next Krylov vector (float when q_f32, else double)
  int q_f32 = 0;
  double *partials = nullptr;  // grid-reduction scratch
  int grid = 0;          // blocks of the reducing kernels
  Cycle *cy = nullptr;
  Control *ctrl = nullptr;
  int m = 0;
  // The step's two sync-free solves poll their outputs until the unsolved
  // pattern is gone; with prefill set, the kernel before them (the cycle's
  // first vector, else pass C of the previous step) writes the pattern into
  // the L solve's output (fill_t) and the next column of Z as it goes, and the
  // solves launch without their own fill.
  int prefill = 0;
  void *fill_t = nullptr;
  int fill_t_f32 = 0;
  // modified Gram-Schmidt variant: restarted (data_fgmres_restart: happy
  // breakdown below 0, the x update column by column) or one cycle
  // (data_fgmres: breakdown below DBL_EPSILON, x += sum_j z_j y_j);
  // reorth 0 Brown/Hindmarsh test, 1 never, 2 always
  int mgs_restarted = 1;
  int mgs_reorth = 0;
};

// mgs: set up the Gram-Schmidt cycle (g = ||r|| e_0, rotations cleared)
// instead of the first reflector
void launch_cycle_residual(cudaStream_t s, const ArnoldiArgs &a, const double *b, const double *x,
                           bool mgs = false);
void launch_cycle_init(cudaStream_t s, const ArnoldiArgs &a);
void launch_passA(cudaStream_t s, const ArnoldiArgs &a, int j);
void launch_passB(cudaStream_t s, const ArnoldiArgs &a, int j);
void launch_passC(cudaStream_t s, const ArnoldiArgs &a, int j);
void launch_orthog_monitor(cudaStream_t s, const ArnoldiArgs &a, int j, double *Q, size_t ldq);
void launch_xupdate(cudaStream_t s, const ArnoldiArgs &a, double *x);
// passes A, B and C of step j as one cooperative kernel with w in shared
// memory; returns 1 when it does not apply (BCSR, no sliced ELL, w too large
// for shared memory), 2 when the cooperative launch failed, 0 on success
// mark_t/mark_z (both or neither): where the unsolved marks go instead of
// the next step's solve outputs (a measurement's replays must keep Z intact)
int launch_hh_step(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t = nullptr, void *mark_z = nullptr);

// ------------------------------------ FGMRES, modified Gram-Schmidt Arnoldi
// (src/fgmres_restart.cpp, src/fgmres.cpp).  Basis v_j in a.V, the
// preconditioned vectors z_j in a.Z, u in a.w.  Step j: the two solves
// z_j = M^{-1} v_j, then
//   operator : u = A z_j, ||u||, h_0 = v_0 . u
//   sweep k  : u -= c_{k-1} v_{k-1}, then v_k . u          (k = 1..j)
//   norm     : u -= c_j v_j, h_{j+1} = ||u||; the Brown/Hindmarsh test, and
//              (no second pass) the rotations and the convergence test
//   [second pass when the test asks: sweep k = 0..j and norm again]
//   next     : v_{j+1} = u / h_{j+1}
// c_k is h_k in the first pass, the second pass's own coefficient in it.
// cond: a conditional-node handle set to 1 when the step reorthogonalises
// (0: none; the second-pass kernels also check Cycle::reorth).
void launch_mgs_cycle_init(cudaStream_t s, const ArnoldiArgs &a);
void launch_mgs_operator(cudaStream_t s, const ArnoldiArgs &a, int j);
void launch_mgs_sweep(cudaStream_t s, const ArnoldiArgs &a, int j, int k, int pass);
void launch_mgs_norm(cudaStream_t s, const ArnoldiArgs &a, int j, int pass, unsigned long long cond);
void launch_mgs_next(cudaStream_t s, const ArnoldiArgs &a, int j);
void launch_mgs_xupdate(cudaStream_t s, const ArnoldiArgs &a, double *x);
// the whole step after the solves (operator, both passes, rotations, next
// vector) as one cooperative kernel with u in shared memory; returns 1 when
// it does not apply (BCSR, no sliced ELL, u too large for shared memory),
// 2 when the cooperative launch failed, 0 on success
int launch_mgs_step(cudaStream_t s, const ArnoldiArgs &a, int j, void *mark_t = nullptr, void *mark_z = nullptr);

// ------------------------------------------------------------ ParILU
struct IluArgs {
  int n = 0, nnzA = 0;
  const int *Arow = nullptr, *Acol = nullptr;
  const double *Aval = nullptr;
  const int *Lrow = nullptr, *Lcol = nullptr;   // CSRL
  const int *Ucp = nullptr, *Uri = nullptr;     // CSCU
  int bs = 0;                                   // BCSR block size (0: CSR)
  double *partials = nullptr;
  int *counter = nullptr;
  int grid = 0;
};
// one synchronous sweep old -> new; writes sum (new-old)^2 to *step (device)
void launch_parilu_sweep(cudaStream_t s, const IluArgs &a, VType t, const void *Lold, void *Lnew,
                         const void *Uold, void *Unew, double *step);
// one synchronous sweep over A's entries in A's order on F (factor values in
// A's order), from the host-built pair records (parilu.cu); *step as above
// variant: the kernel's entries and pairs in flight per thread and its
// register budget (0 .. parilu_sweep_variants() - 1), chosen by the autotune
void launch_parilu_sweep_ao(cudaStream_t s, int nnz, VType t, const double *Aval, const int *dpos,
                            const int *pptr, const int2 *pairs, const void *Fold, void *Fnew, double *partials,
                            int *counter, double *step, int variant);
int parilu_sweep_variants();
// dst[q] = map[q] >= 0 ? src[map[q]] : 1, value type t
void launch_factor_gather(cudaStream_t s, int count, const int *map, VType t, const void *src, void *dst);
// the block sweep in A's block order (bs <= 5), Dinv: the block inverses of
// U's diagonal blocks of Fold in the compute type (float for FP32 / BF16)
void launch_bcsr_parilu_sweep_ao(cudaStream_t s, int nnzb, int bs, VType t, const double *Aval, const int *Acol,
                                 const int *dpos, const int *pptr, const int2 *pairs, const void *Dinv,
                                 const void *Fold, void *Fnew, double *partials, int *counter, double *step);
// Dinv[I] = inv(F[diag[I]]) per block row (bs <= 5, compute type), breakdown
// bit on a non-finite inverse
void launch_bcsr_diag_inverse_ao(cudaStream_t s, int nb, int bs, const int *diag, VType t, const void *F,
                                 void *Dinv, int *status);
// block gather: dst block q = src block map[q], identity for map[q] < 0
void launch_factor_gather_blk(cudaStream_t s, int count, int bs, const int *map, VType t, const void *src,
                              void *dst);
// ||(A - LU)|_S||_F^2 to *out (device)
void launch_ilu_residual(cudaStream_t s, const IluArgs &a, VType t, const void *L, const void *U,
                         double *out);
// out3 = {||LU||_F^2, sum over S of (LU)_ij^2, sum over S of (LU - A)_ij^2}
// with S the entries of A the product's pattern holds; Urow/Ucol/Ur: U in
// CSR, a.Ucp/a.Uri + Uc: U in CSC (same values); unit: L's diagonal counts
// as 1
void launch_lu_fro(cudaStream_t s, const IluArgs &a, VType t, const int *Urow, const int *Ucol,
                   const void *L, const void *Ur, const void *Uc, double *out3, int unit);
// the sliced-ELL values of the operator: dst[q] = map[q] >= 0 ? src[map[q]] : 0
// batched solves as one persistent launch (batch_persist.cu): systems from a
// queue, largest first, each carried by one CTA through ParILU and
// FGMRES-Householder for all its right-hand sides
constexpr int kBatchMaxM = 64;  // largest search_max of the batched solver
constexpr int kBatchMaxW = 4;   // off-diagonal entries per row of a triangle the batched solver takes
struct PBatchHost {
  int nsys = 0, nrhs = 0, m = 0, restart_max = 0, sweeps = 0, N = 0, grid = 0, f32 = 1;
  double rtol = 0.0;
  int njobs = 0;
  const int *jsys = nullptr, *jrhs = nullptr, *jnr = nullptr;  // jobs: system, first rhs, rhs count
  const int *n = nullptr, *roff = nullptr, *lsys = nullptr, *usys = nullptr;
  const int *Arow = nullptr, *Acol = nullptr;
  const double *Aval = nullptr;
  const int *pptr = nullptr, *dpos = nullptr, *diag = nullptr;
  const int2 *pairs = nullptr;
  void *F = nullptr;  // per CTA two factor buffers of fstride entries
  size_t fstride = 0;
  const int *lptr = nullptr, *lrows = nullptr, *uptr = nullptr, *urows = nullptr;
  int w = 0;
  const int *cL = nullptr, *fL = nullptr, *cU = nullptr, *fU = nullptr, *dU = nullptr;
  void *vrec = nullptr;
  const double *b = nullptr;
  double *x = nullptr;
  size_t nmax = 0;
  double *V = nullptr, *W = nullptr, *Tm = nullptr, *Rm = nullptr;
  void *Z = nullptr, *Q = nullptr, *Tt = nullptr;
  int *next = nullptr, *iters = nullptr, *conv = nullptr;
};
int launch_batch_persist(cudaStream_t s, const PBatchHost &h);
int batch_persist_threads();
int batch_persist_rhs();
void launch_sell_values(cudaStream_t s, size_t count, const int *map, const double *src, double *dst,
                        float2 *pair);
// gather: dst[p] = src[perm[p]] with type conversion
void launch_gather(cudaStream_t s, int count, const int *perm, VType ts, const void *src, VType td,
                   void *dst);
// convert / copy an array between value types
void launch_convert(cudaStream_t s, int count, VType ts, const void *src, VType td, void *dst);
// BCSR: inverse of each diagonal block of U (row form: diagonal block first
// in each block row) into dinv (nb * bs*bs), value type t
void launch_block_diag_inverse(cudaStream_t s, int nb, int bs, const int *Urow, VType t,
                               const void *Uval, void *dinv, int *status);

// ------------------------------------------------------------ SpTRSV
// x = T^{-1} b for one triangle; b/x typed by in_f32/out_f32 (else double).
// compute precision follows the factor value type (double for F64, float
// otherwise).  ctrl may be null (stand-alone call).
// Block-scheduled sync-free solve plan of one triangle (device arrays; see
// sptrsv_blk.cu).  Built on the host by build_blk_plan (context.cu).
// most chunks a block of a plan may hold
constexpr int kBlkMaxUnits = 1024;
// dependencies outside its chunk a row keeps in the plan's own layout (rows
// with more are solved from the CSR arrays)
__host__ __device__ constexpr int blk_slots(int R) { return R == 1 ? 4 : (R == 2 ? 3 : 2); }
struct TriBlkPlan {
  int n = 0, nchunks = 0, nblocks = 0, nunits = 0;
  int R = 4, cpb = 1, warps = 1, grid = 1;
  int unit = 0, lower = 1;
  const int *row = nullptr, *col = nullptr;
  // per block (solve order): {first unit, end unit, levels spanned, lowest row}
  const int4 *blk = nullptr;
  // per unit (blocks in solve order, a block's chunks by level):
  // {chunk, level | serial << 30, 0, 0}
  const int4 *urec = nullptr;
  int max_units = 0;  // most chunks in one block
  int cl = 1;         // CTAs per thread-block cluster (consecutive blocks pass rows on in shared memory)
  // The plan's own layout of the solve, coalesced per warp.  Per unit u,
  // slot t < S, row r < R, lane l: index ((u*S + t)*R + r)*32 + l for the
  // slot arrays, (u*R + r)*32 + l for the per-row ones.
  //   ucode: where the dependency is read: >= 0 row (code) of the block's
  //          window, <= -2 row -(code+2) of the output, -1 none
  //   umap, udiag, uprev: CSR entry of the dependency, the diagonal (-1 for a
  //          unit diagonal) and the previous row of a scan chunk (or -1)
  //   uflag: per unit and lane, bit r: row r has more than S dependencies
  //          (its slots are empty; it is solved from the CSR arrays)
  //   uvs, uaps, urd: values in the compute type, gathered from the factor
  //          values: a_ij / a_ii, -a_{i,prev} / a_ii and 1 / a_ii
  const int *ucode = nullptr, *umap = nullptr, *udiag = nullptr, *uprev = nullptr, *uflag = nullptr;
  void *uvs = nullptr, *uaps = nullptr, *urd = nullptr;
};
// 1 when the plan's cluster shape can be launched on this device with the
// value type's window (some cluster of it fits)
int sptrsv_cluster_supported(const TriBlkPlan &pl, VType vt);
// gather the plan's values (uvs, uaps, urd) from the triangle's values
void launch_plan_values(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt);
// x must not overlap b (x is filled with the unsolved pattern first)
// prefilled: x already holds the unsolved pattern (no fill launched)
void launch_sptrsv_blk(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                       int in_f32, void *x, int out_f32, Control *ctrl, int slot, bool honor_done,
                       bool prefilled = false);
void launch_sptrsv_blk_multi(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                             int in_f32, void *x, int out_f32, size_t vstride, int nrhs, int *tickets, int *status,
                             const int *done_flag, bool prefilled = false);

// honor_done: return at once when ctrl->done is set (inside an Arnoldi cycle)
void launch_sptrsv_levels(cudaStream_t s, const TriDev &t, VType vt, const void *b, int in_f32,
                          void *x, int out_f32, Control *ctrl, bool honor_done);
// one synchronous Jacobi sweep y_new = D^{-1}(b - (T - D) y_old); step partial sums
void launch_jacobi_sweep(cudaStream_t s, const TriDev &t, VType vt, const void *b, int in_f32,
                         const void *yold, void *ynew, int y_f32, Control *ctrl, bool honor_done);
// ParCSRTRSV in LACE's sweep order (partrsv.cu).  Scratch: a (n doubles),
// partials (partrsv_partials_needed() doubles), counters (4 ints), steps (2
// doubles) on the device; h_steps (2 doubles) and h_status (1 int) on the host
struct PartrsvScratch {
  double *a = nullptr;
  double *partials = nullptr;
  int *counters = nullptr;
  double *steps = nullptr;
  double *h_steps = nullptr;
  int *h_status = nullptr;
};
int partrsv_partials_needed();
// one sweep in LACE's order: rows before row i in the sweep are read from
// ynew (waiting until written), the others from yold; ynew must hold the
// unsolved pattern and *ticket 0; guard (may be null): run only while
// *guard > tol and finite; a wait gives up after max_polls polls (0: kMaxSpins)
void launch_partrsv_sweep(cudaStream_t s, bool lower, int n, const int *row, const int *col, const double *val,
                          const double *rhs, const double *yold, double *ynew, int *ticket, int *status,
                          const double *guard, double tol, int max_polls);
// data_parcsrtrsv's loop on device arrays: y is the start vector in and the
// iterate out; returns 0 or a DEV_ERR_* code
int partrsv_solve(cudaStream_t s, bool lower, int n, const int *row, const int *col, const double *val,
                  const double *rhs, double *y, double tol, int *iter, const PartrsvScratch &sc);
// block (BCSR) triangular solves: lower with identity diagonal blocks, or
// upper applying the inverted diagonal blocks dinv
void launch_bcsr_sptrsv(cudaStream_t s, const TriDev &t, int bs, VType vt, const void *dinv,
                        const void *b, int in_f32, void *x, int out_f32, Control *ctrl,
                        int grid_hint, bool honor_done);

// *out = sum (a_i - b_i)^2 (typed by f32), deterministic grid reduction
// sum of squares of count FP64 values into *out (partials: grid-sized scratch)
void launch_sumsq(cudaStream_t s, size_t count, const double *a, double *partials, int *counter, double *out);
void launch_sqdiff(cudaStream_t s, int n, const void *a, const void *b, int f32, double *partials,
                   int *counter, double *out);

int num_sms();

}  // namespace lace
