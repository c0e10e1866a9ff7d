// Host-side state of a lace_gpu_ctx (see context.cu for the HBM layout).
#pragma once

#include <map>
#include <tuple>
#include <vector>

#include "../../include/lace_gb300.h"
#include "internal.h"

namespace lace {

struct DBuf {
  void *p = nullptr;
  size_t bytes = 0;
  DBuf() = default;
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  ~DBuf() { free(); }
  void free();
  int ensure(size_t b);
  int upload(const void *h, size_t b, cudaStream_t s);
};

struct Pattern {
  int n = 0;
  std::vector<int> ptr, idx;
};

// device arrays of one triangle's block-scheduled solve plan
struct PlanBufs {
  DBuf blk, urec, ucode, umap, udiag, uprev, uflag, uvs, uaps, urd;
  TriBlkPlan dev;
  bool valid = false;
  // the factor values the plan's values were gathered from
  int vals_version = -1;
  int vals_type = -1;
  const void *vals_src = nullptr;
};

// host part of a plan (what build_blk_plan_host fills, upload_blk_plan sends)
struct HostPlan {
  int n = 0, nch = 0, R = 1, cpb = 1, max_units = 0;
  bool lower = true, unit = false;
  std::vector<int4> blk, urec;
  std::vector<int> ucode, umap, udiag, uprev, uflag;
};

// host construction of a plan: chunks of 32*R rows, blocks of cpb chunks (in
// solve order), chunks of a block in wavefront-level order, cross-block
// requirements; then its upload
int build_blk_plan_host(const Pattern &T, bool lower, bool unit, int R, int cpb, HostPlan &hp);
int upload_blk_plan(const HostPlan &hp, PlanBufs &pb, cudaStream_t s);
int build_blk_plan(const Pattern &T, bool lower, bool unit, int R, int cpb, PlanBufs &pb, cudaStream_t s);

extern thread_local int g_last_error;
int set_err(int code);
int cuda_code(cudaError_t e);
int validate_csr(int n, int nnz, const int *row, const int *col);
void transpose_pattern(const Pattern &P, Pattern &T, std::vector<int> &t2p);

}  // namespace lace

struct lace_gpu_ctx {
  using DBuf = lace::DBuf;
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  lace_gpu_options opt{};
  bool verbose = false;

  // matrix (CSR: bs == 0; BCSR: n_blk block rows of bs x bs blocks)
  int n = 0;       // scalar rows
  int n_blk = 0;   // rows of the (block) pattern
  int bs = 0;
  int nnzA = 0;    // entries (blocks) of A
  double anorm = 0.0;
  DBuf Arow, Acol, Aval;
  std::vector<int> hArow, hAcol;  // host copy of the resident CSR pattern
  int aval_version = 0;  // bumped whenever A's values change
  // A in sliced ELL for the Arnoldi operator (CSR only): slice offsets, columns,
  // source CSR entry of each slot (-1: padding) and the gathered values
  DBuf sell_ptr, sell_col, sell_map, sell_val, sell_pair;
  size_t sell_slots = 0;
  bool sell_valid = false;
  int sell_version = -1;
  int ensure_sell();
  // A^T for the adjoint
  bool AT_ready = false;
  DBuf ATrow, ATcol, ATval, map_at2a;

  // factor patterns and maps
  int nnzL = 0, nnzU = 0;
  lace::Pattern hL, hU, hUc, hLt;
  DBuf Lrow, Lcol, Ucp, Uri, Urow, Ucol, Ltp, Lti;
  DBuf map_l2a, map_uc2a, map_ur2uc, map_lt2l, map_ur2uc_el;
  // factor values (value type from opt.precision)
  DBuf Lv[2], Ucv[2], Urv, Ltv, dinv;
  // CSR sweeps: the factor values in A's order (ping-pong) and the sweep's
  // per-entry records (pair ranges, pairs of A positions, u_jj position)
  DBuf Fv[2], sw_pptr, sw_pairs, sw_dpos, sw_diag, sw_dinv;
  bool sweep_ao = false;
  int sweep_variant = -1;  // the CSR sweep's launch shape (autotuned)
  int autotune_sweep(const lace::IluArgs &a, const void *Fold, void *Fnew);
  int cur = 0;
  bool factors_ready = false;
  int fact_version = 0;  // bumped whenever the factor values change

  // SpTRSV per triangle (0 L, 1 U, 2 U^T, 3 L^T)
  DBuf ready[4];
  // BCSR solves of L and U: chunk tables (see sptrsv.cu k_bcsr_sptrsv)
  DBuf bch_first[2];
  int bnch[2] = {0, 0};
  int bcsr_grid = 0;  // blocks of the BCSR solves (autotuned; 0: the launcher's default)
  bool bcsr_tuned = false;
  int autotune_bcsr_trsv();
  DBuf lvl_ptr[4], lvl_rows[4];
  int nlevels[4] = {0, 0, 0, 0};
  int rows_per_lane = 4;
  bool trsv_tuned = false;
  lace::PlanBufs plans[4];
  int plan_R = 4, plan_cpb = 1, plan_warps = 1, plan_cl = 1;  // autotuned schedule shape
  int ensure_plan(int which);
  // host plans the autotune built in parallel, keyed (triangle, R, chunks per block)
  std::map<std::tuple<int, int, int>, lace::HostPlan> prebuilt;
  int lanes = 8;

  // Krylov workspace
  int ws_m = 0;
  bool ws_zf32 = false;
  size_t ldv = 0;
  DBuf Vb, Vfb, Zb, Qmon, vec_w, vec_q, vec_t, vec_t2, vec_r;
  DBuf part_buf;
  DBuf ctrl_buf, cycle_buf, scal_buf, cnt_buf;
  DBuf stage64;           // FP64 factor values on their way to FP32/BF16
  DBuf dropin_b, dropin_x;  // right-hand side and solution of the drop-in FGMRES
  lace::Control *h_ctrl = nullptr;
  double *h_scal = nullptr;
  std::map<std::tuple<int, int, int, int, int, int, int, int, int, int, int>, cudaGraphExec_t> graphs;
  // second stream: the body of the conditional Gram-Schmidt second pass is
  // captured on it
  cudaStream_t side = nullptr;
  bool cond_nodes = true;  // conditional graph nodes available (else the second pass launches always)
  bool mgs_persistent = true;  // the one-kernel Gram-Schmidt step (cooperative launch) available
  bool hh_persistent = true;   // the one-kernel Householder step (cooperative launch) available
  int last_reorth = 0;     // directions of the last Gram-Schmidt solve that reorthogonalised
  int last_m = 0;          // search directions per cycle of the last FGMRES solve
  std::vector<double> last_hist;
  std::vector<double> last_orth;  // ||I - Q^T Q||_inf per direction of the last solve (monitor on)

  ~lace_gpu_ctx();
  lace::Control *ctrl() const { return (lace::Control *)ctrl_buf.p; }
  void drop_graphs();
  int analyse(int n_, const int *row, const int *col, int bs_);
  int analyse_factors(const lace::Pattern &L, const lace::Pattern &Ur);
  int build_sweep_records(const int *row, const int *col, const lace::Pattern &L, const lace::Pattern &Ur,
                          const std::vector<int> &l2a, const std::vector<int> &ur2a, const std::vector<int> &uc2a);
  int set_factors_host(int nrows, const int *lrow, const int *lcol, const double *lval,
                       const int *urow, const int *ucol, const double *uval);
  // the same from U in CSC order (diagonal last in each column), when L's and
  // U's patterns are the context's own (as ParILU returned them): the values
  // are uploaded as they are and U's CSR image is gathered on the GPU.
  // Returns 1 (nothing done) when the patterns differ.
  int set_factors_csc_host(int nrows, const int *lrow, const int *lcol, const double *lval,
                           const int *ucp, const int *uri, const double *ucval);
  // ||A||_F from the resident values, on the GPU
  int device_anorm();
  DBuf pat_stage;  // a caller's pattern on its way to be compared with the resident one
  int same_on_device(int parts, const int *const *h, const int *const *dev, const size_t *count, bool *same);
  std::vector<int> uc2ur_h;  // CSC position of U -> CSR position
  int upload_common(int n_, int nnz_, const int *row, const int *col, int bs_);
  int upload_values_same_pattern(const double *val);
  void set_rows_per_lane(int R);
  lace::TriDev tri(int which) const;
  lace::VType vtype() const;
  void *part_ensure();
  int autotune_spmv();
  int autotune_trsv();
  int alloc_factor_values();
  lace::IluArgs ilu_args();
  int init_factors();
  int finish_factors();
  // up to `sweeps` sweeps; with sync_each, stops once the normalised step is
  // <= stop_below (LACE's stopping tests); steps receives every sweep's step
  // reuse_init: the factors already hold the initial guess (no re-initialisation)
  int parilu(int sweeps, double *step_out, double *nonlin_out, bool sync_each,
             std::vector<double> *steps, double stop_below = -1.0, int min_sweeps = 0,
             bool reuse_init = false);
  int h_status();
  int ilu_residuals(double *res, double *nonlin);
  // prefilled: x already holds the unsolved pattern (sync-free block solves)
  int solve_tri(int which, const void *b, int in_f32, void *x, int out_f32, bool honor_done,
                void *tmp, bool prefilled = false);
  bool syncfree_blocks() const;  // the solves are the block-scheduled sync-free ones
  int ensure_vectors();
  int ensure_krylov(int m, bool monitor);
  int ensure_AT();
  lace::ArnoldiArgs arnoldi_args(int m, bool adjoint);
  int enqueue_cycle_body(const lace::ArnoldiArgs &a, int m, bool adjoint, bool capturing);
  // the modified Gram-Schmidt cycle; capturing: inside a stream capture (the
  // second pass goes into conditional nodes when cond_nodes)
  int enqueue_mgs_body(const lace::ArnoldiArgs &a, int m, bool capturing);
  // method 0: Householder (fgmres_householder_restart.cpp); 1: modified
  // Gram-Schmidt, restarted (fgmres_restart.cpp) or one cycle (fgmres.cpp)
  // with reorth as LACE's gmres_par->reorth
  int fgmres(const double *b, double *x, int m, int restart_max, int tol_type, double rtol,
             bool adjoint, data_d_gmres_log *log, int *total_iters, std::vector<double> *hist,
             int method = 0, int restarted = 1, int reorth = 0);
};
