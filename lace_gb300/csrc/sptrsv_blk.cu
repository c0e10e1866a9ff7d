// Block-scheduled sync-free SpTRSV.
//
// The rows of one triangle are cut into chunks of 32*R consecutive rows (one
// warp each, lane l the R rows l*R.. in solve order; "scan" chunks whose only
// in-chunk dependency is the previous row are solved with a warp-wide affine
// scan, others position by position).  Consecutive chunks (in solve order)
// form blocks; one CTA owns a block at a time, taken by atomic ticket in solve
// order, so every block a CTA waits on is held by a CTA that is running.
//
// A solved value is its own ready flag.  Before the solve the output vector
// is filled with an "unsolved" bit pattern (all ones, a NaN that arithmetic
// does not produce; a solved value with those bits is stored as a quiet NaN),
// and a CTA keeps its block's rows in a shared-memory window filled the same
// way.  A row waits for a dependency by reading it until the pattern is gone:
// from the window when the dependency is in the same block, from L2
// otherwise.  There are no per-level barriers: warps take the block's chunks
// round robin in level order (a chunk's level is one more than the highest
// level of its dependencies, in any block: its step in the wavefront of the
// whole solve), so the lowest unsolved chunk can always proceed, and a block
// that holds parts of two stretches of the wavefront takes its chunks in the
// order they become ready.
//
// The plan holds the solve in its own layout, coalesced per warp: for each
// chunk, row and dependency slot where the dependency is read (window slot or
// row of the output) and, gathered from the factor values whenever they
// change, the entry scaled by the reciprocal of the diagonal (rows with more
// dependencies than slots are solved from the CSR arrays).  A warp loads the
// next chunk's data while it solves the current one, so what is left on the
// dependency chain is reading the dependencies, one fused multiply-add per
// entry, the scan, and the stores.
//
// For a lexicographic 7-point stencil with R = 4 (a chunk = one x-line) and
// blocks of whole planes, every x-line is one scan, the j- and k-direction
// dependencies inside a block are shared-memory reads, and only a block's
// first plane reads rows of another CTA.
#include <algorithm>

#include <cooperative_groups.h>

#include "internal.h"

namespace lace {

template <typename T>
__device__ __forceinline__ void st_out(void *x, int out_f32, int i, T v) {
  if (out_f32) ((volatile float *)x)[i] = (float)v;
  else ((volatile double *)x)[i] = (double)v;
}

// shared memory a CTA may use for its block's solved rows; a CTA of a
// cluster also holds the previous block's rows
constexpr int kSptrsvSmemMax = 160 * 1024;
constexpr size_t kSptrsvClusterSmemMax = 200 * 1024;

__device__ __forceinline__ bool is_unsolved(float v) { return __float_as_uint(v) == 0xffffffffu; }
__device__ __forceinline__ bool is_unsolved(double v) { return __double_as_longlong(v) == -1ll; }
template <typename CT>
__device__ __forceinline__ CT unsolved_value();
template <>
__device__ __forceinline__ float unsolved_value<float>() { return __uint_as_float(0xffffffffu); }
template <>
__device__ __forceinline__ double unsolved_value<double>() { return __longlong_as_double(-1ll); }
// a solved value never carries the pattern
template <typename CT>
__device__ __forceinline__ CT as_solved(CT v) {
  return is_unsolved(v) ? (CT)NAN : v;
}

__device__ __forceinline__ float rcp_rn(float d) { return __frcp_rn(d); }
__device__ __forceinline__ double rcp_rn(double d) { return __drcp_rn(d); }

// Read a dependency: from the window (code >= 0) or from the output (code
// <= -2, through L2).  *ok is cleared when it is not solved yet.
template <typename CT>
__device__ __forceinline__ CT read_dep(const CT *xs, const void *x, int f32, int code, bool &ok) {
  CT v;
  if (code >= 0) {
    v = ((const volatile CT *)xs)[code];
    ok &= !is_unsolved(v);
  } else if (f32) {
    const float f = ((const volatile float *)x)[-code - 2];
    ok &= !is_unsolved(f);
    v = (CT)f;
  } else {
    const double dv = ((const volatile double *)x)[-code - 2];
    ok &= !is_unsolved(dv);
    v = (CT)dv;
  }
  return v;
}

struct BlkPlanDev {
  int n, nblocks;
  const int *row, *col;
  const void *val;  // CSR values (rows solved from the CSR arrays, serial chunks)
  const int4 *blk;  // {first unit, end unit, levels spanned, lowest row}
  const int4 *urec; // {chunk, level | serial << 30, 0, 0}
  const int *ucode, *uflag;
  const void *uvs, *uaps, *urd;
  int win;  // rows of a block kept in shared memory (0: none), plus a spare slot
};

// The rows of the previous block of a thread-block cluster, which the CTA
// that solves them writes into this CTA's shared memory (the halo, from slot
// base on), and where this CTA writes its own rows for the next one.
template <typename CT>
struct Halo {
  int prev_row0;       // lowest row of the previous block
  unsigned prev_rows;  // its rows (0: no previous block in the cluster)
  unsigned base;       // first halo slot in shared memory
  CT *remote;          // the next CTA's shared memory (nullptr: none)
};

// One chunk's solve data, loaded by its warp ahead of its turn, and the
// record of the chunk this register set takes next (loaded one turn early, so
// that the right-hand-side loads need not wait for it).
template <typename CT, int R, int S>
struct Unit {
  int k;  // index in the block's unit list; -1: none
  int4 rec, nrec;
  int code[R][S];
  CT vs[R][S];
  CT aps[R], rd[R];
  unsigned long long braw[R];  // b_i: FP64 bits, or FP32 bits in the low word
  int flag;
};

// take chunk k (its record is d.nrec) and load the record of chunk k + step
template <typename CT, int R, int S, bool LOWER>
__device__ __forceinline__ void unit_load(Unit<CT, R, S> &d, int k, int step, int nunits, int ubase,
                                          const BlkPlanDev &P, const void *b, int in_f32, int lane) {
  constexpr int CS = 32 * R;
  d.k = k < nunits ? k : -1;
  if (d.k < 0) return;
  d.rec = d.nrec;
  if (k + step < nunits) d.nrec = P.urec[(size_t)ubase + k + step];
  const size_t u = (size_t)ubase + k;
  const CT *uvs = (const CT *)P.uvs, *uaps = (const CT *)P.uaps, *urd = (const CT *)P.urd;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const size_t q = (u * R + r) * 32 + lane;
    d.aps[r] = uaps[q];
    d.rd[r] = urd[q];
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const size_t qs = ((u * S + t) * R + r) * 32 + lane;
      d.code[r][t] = P.ucode[qs];
      d.vs[r][t] = uvs[qs];
    }
  }
  d.flag = P.uflag[u * 32 + lane];
  const int base = d.rec.x * CS, cnt = min(CS, P.n - base);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int pos = lane * R + r;
    d.braw[r] = 0;
    if (pos < cnt) {
      const int i = LOWER ? base + pos : base + cnt - 1 - pos;
      if (in_f32) d.braw[r] = ((const unsigned *)b)[i];
      else d.braw[r] = ((const unsigned long long *)b)[i];
    }
  }
}

// Phase A of a chunk's wait: rows outside the window, read through L2 (OT:
// the output's type).  Branch free over the slots - a slot without such a
// dependency reads an always-solved zero in this CTA's shared memory - so
// that the lanes' loads of one pass go out together.  Rows solved from the
// CSR arrays are read after.
// A far dependency (code <= -2) in the previous block of the cluster is read
// from the halo instead.
template <bool HALO, typename CT>
__device__ __forceinline__ bool in_halo(int code, const Halo<CT> &h) {
  return HALO && code <= -2 && (unsigned)(-code - 2 - h.prev_row0) < h.prev_rows;
}

template <typename CT, typename VT, typename OT, int R, int S, bool LOWER, bool HALO>
__device__ __forceinline__ void far_wait(const Unit<CT, R, S> &d, const BlkPlanDev &P, const CT *xs, const void *x,
                                         int row0, unsigned brows, unsigned win, int lane, const int *rows, int c,
                                         CT *Bv, const double *s_zero, int *status, const Halo<CT> &h) {
  constexpr int CS = 32 * R;
  const VT *val = (const VT *)P.val;
  const OT *zero = (const OT *)s_zero;
  const OT *src[R][S];
  CT w[R][S], acc0[R];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    acc0[r] = Bv[r];
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const int code = d.code[r][t];
      const bool glob = (code <= -2 && !in_halo<HALO>(code, h)) || code >= (int)win;
      src[r][t] = glob ? (const OT *)x + (code <= -2 ? -code - 2 : row0 + code) : zero;
      w[r][t] = glob ? d.vs[r][t] : (CT)0;
    }
  }
  for (int spins = 0;; ++spins) {
    bool ok = true;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      CT acc = acc0[r];
#pragma unroll
      for (int t = 0; t < S; ++t) {
        const OT v = *(const volatile OT *)src[r][t];
        ok &= !is_unsolved(v);
        acc -= w[r][t] * (CT)v;
      }
      if ((d.flag >> r) & 1) {
        const int i = rows[r];
        for (int e = P.row[i]; e < P.row[i + 1]; ++e) {
          const int jc = P.col[e];
          if (jc == i || (LOWER ? (jc > i) : (jc < i)) || jc / CS == c) continue;
          const unsigned slot = (unsigned)(jc - row0);
          const int code = (slot < brows && slot < win) ? (int)slot : -jc - 2;
          acc -= cvt<CT>(val[e]) * d.rd[r] * read_dep<CT>(xs, x, sizeof(OT) == 4, code, ok);
        }
      }
      Bv[r] = acc;
    }
    if (__all_sync(0xffffffffu, ok)) break;
    if (spins > kMaxSpins || ((spins & 1023) == 1023 && (*(const volatile int *)status & kStatusSpinTimeout))) {
      if (lane == 0) atomicOr(status, kStatusSpinTimeout);  // the solve is reported as failed
      break;
    }
    if (spins > 32) __nanosleep(32);
  }
}

template <typename CT, typename VT, int R, int S, bool LOWER, bool HALO>
__device__ __forceinline__ void unit_solve(const Unit<CT, R, S> &d, const BlkPlanDev &P, CT *xs, void *x,
                                           int in_f32, int out_f32, int row0, unsigned brows, unsigned win,
                                           int lane, const double *s_zero, int *status, const Halo<CT> &h) {
  constexpr int CS = 32 * R;
  const VT *val = (const VT *)P.val;
  const int c = d.rec.x;
  const bool serial = (d.rec.y >> 30) != 0;
  const int base = c * CS;
  const int cnt = min(CS, P.n - base);
  CT A[R], Bv[R], X[R];
  int rows[R];
  bool far = false;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int pos = lane * R + r;
    rows[r] = pos < cnt ? (LOWER ? base + pos : base + cnt - 1 - pos) : -1;
    A[r] = serial ? (CT)0 : d.aps[r];
    const CT bb = in_f32 ? (CT)__uint_as_float((unsigned)d.braw[r]) : (CT)__longlong_as_double((long long)d.braw[r]);
    Bv[r] = rows[r] >= 0 ? bb * d.rd[r] : (CT)0;
    X[r] = (CT)0;
    far |= (d.flag >> r) & 1;
#pragma unroll
    for (int t = 0; t < S; ++t)
      far |= (d.code[r][t] <= -2 && !in_halo<HALO>(d.code[r][t], h)) || d.code[r][t] >= (int)win;
  }
  // The scan's multipliers depend on the factor values only, so they are
  // formed before the wait: m[k] is the product of A over the rows of the
  // 2^k lanes before this lane's partial, and after the wait a round of the
  // scan is one shuffle and one multiply-add.
  CT m[5];
  if (!serial) {
    CT ca = (CT)1;
#pragma unroll
    for (int r = 0; r < R; ++r) ca = A[r] * ca;
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int o = 1 << k;
      const CT pa = __shfl_up_sync(0xffffffffu, ca, o);
      m[k] = ca;
      if (lane >= o) ca = ca * pa;
    }
  }
  // Wait for the chunk's dependencies with the whole warp in lock step
  // (lanes spinning on different branches of a diverged warp would wait for
  // the scheduler to switch between them): each pass reads all of a phase's
  // dependencies and forms the sums, and the warp leaves when every lane saw
  // them solved.  Phase A: rows outside the window (other blocks) and rows
  // solved from the CSR arrays, read through L2; they are usually solved
  // before the warp gets here.  Phase B: rows of the window (and of the halo),
  // branch free - an entry that is neither reads the always-solved spare slot
  // with weight 0.
  if (__any_sync(0xffffffffu, far)) {
    if (out_f32)
      far_wait<CT, VT, float, R, S, LOWER, HALO>(d, P, xs, x, row0, brows, win, lane, rows, c, Bv, s_zero, status, h);
    else
      far_wait<CT, VT, double, R, S, LOWER, HALO>(d, P, xs, x, row0, brows, win, lane, rows, c, Bv, s_zero, status, h);
  }
  // the slots read in phase B (window, halo, or the spare slot with weight 0)
  int idx[R][S];
  CT wv[R][S];
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const int code = d.code[r][t];
      const bool in = (unsigned)code < win;
      idx[r][t] = in ? code : (int)win;
      wv[r][t] = in ? d.vs[r][t] : (CT)0;
      if (in_halo<HALO>(code, h)) {
        idx[r][t] = (int)h.base + (-code - 2 - h.prev_row0);
        wv[r][t] = d.vs[r][t];
      }
    }
  CT v[R][S];
  for (int spins = 0;; ++spins) {
    bool ok = true;
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int t = 0; t < S; ++t) {
        v[r][t] = ((const volatile CT *)xs)[idx[r][t]];
        ok &= !is_unsolved(v[r][t]);
      }
    if (__all_sync(0xffffffffu, ok)) break;
    if (spins > kMaxSpins || ((spins & 1023) == 1023 && (*(const volatile int *)status & kStatusSpinTimeout))) {
      if (lane == 0) atomicOr(status, kStatusSpinTimeout);
      break;
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int t = 0; t < S; ++t) Bv[r] -= wv[r][t] * v[r][t];
  if (!serial) {
    // x_p = A_p x_{p-1} + B_p along the chunk: a warp-wide affine scan
    // (inclusive over the lanes' partials)
    CT cb = (CT)0;
#pragma unroll
    for (int r = 0; r < R; ++r) cb = A[r] * cb + Bv[r];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const CT pb = __shfl_up_sync(0xffffffffu, cb, 1 << k);
      if (lane >= (1 << k)) cb = m[k] * pb + cb;
    }
    if (R == 1) {
      X[0] = cb;
    } else {
      // the lane's rows from the partial before it
      CT xin = __shfl_up_sync(0xffffffffu, cb, 1);
      if (lane == 0) xin = (CT)0;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        xin = A[r] * xin + Bv[r];
        X[r] = xin;
      }
    }
  } else {
    // position by position: the owner's value is final, the later rows of
    // the chunk subtract it (entries from the CSR arrays)
    int e0[R], e1[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      e0[r] = rows[r] >= 0 ? P.row[rows[r]] : 0;
      e1[r] = rows[r] >= 0 ? P.row[rows[r] + 1] : 0;
    }
    for (int p = 0; p < cnt; ++p) {
      const int owner = p / R, rr = p % R;
      CT xp = (CT)0;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (lane == owner && r == rr) xp = Bv[r];
      xp = __shfl_sync(0xffffffffu, xp, owner);
      const int rowp = LOWER ? base + p : base + cnt - 1 - p;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int pos = lane * R + r;
        if (pos == p) X[r] = xp;
        if (pos > p && pos < cnt)
          for (int e = e0[r]; e < e1[r]; ++e)
            if (P.col[e] == rowp) Bv[r] -= cvt<CT>(val[e]) * d.rd[r] * xp;
      }
    }
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (rows[r] >= 0) {
      const CT v = as_solved(X[r]);
      const unsigned slot = (unsigned)(rows[r] - row0);
      if (slot < win) ((volatile CT *)xs)[slot] = v;
      if (HALO && h.remote != nullptr) ((volatile CT *)h.remote)[h.base + slot] = v;  // the next CTA's halo
      st_out<CT>(x, out_f32, rows[r], v);
    }
}

// The chunks of one block: a warp's chunks are k = warp, warp + nw, ...; two
// register sets take turns, so a chunk's data is loaded while the chunk
// before it is solved.
template <typename CT, typename VT, int R, bool LOWER, bool HALO>
__device__ __forceinline__ void solve_block(const BlkPlanDev &P, const int4 &B, CT *xs, const void *b, int in_f32,
                                            void *x, int out_f32, int warp, int nw, int lane, const double *s_zero,
                                            int *status, const Halo<CT> &h) {
  constexpr int CS = 32 * R;
  constexpr int S = blk_slots(R);
  const int nunits = B.y - B.x, row0 = B.w;
  const unsigned brows = (unsigned)(nunits * CS);
  const unsigned win = min(brows, (unsigned)P.win);
  Unit<CT, R, S> d0, d1;
  if (warp < nunits) d0.nrec = P.urec[B.x + warp];
  if (warp + nw < nunits) d1.nrec = P.urec[B.x + warp + nw];
  unit_load<CT, R, S, LOWER>(d0, warp, 2 * nw, nunits, B.x, P, b, in_f32, lane);
  unit_load<CT, R, S, LOWER>(d1, warp + nw, 2 * nw, nunits, B.x, P, b, in_f32, lane);
  while (d0.k >= 0) {
    unit_solve<CT, VT, R, S, LOWER, HALO>(d0, P, xs, x, in_f32, out_f32, row0, brows, win, lane, s_zero, status, h);
    unit_load<CT, R, S, LOWER>(d0, d0.k + 2 * nw, 2 * nw, nunits, B.x, P, b, in_f32, lane);
    if (d1.k < 0) break;
    unit_solve<CT, VT, R, S, LOWER, HALO>(d1, P, xs, x, in_f32, out_f32, row0, brows, win, lane, s_zero, status, h);
    unit_load<CT, R, S, LOWER>(d1, d1.k + 2 * nw, 2 * nw, nunits, B.x, P, b, in_f32, lane);
  }
}

// the CTA that leaves last re-arms the tickets
__device__ __forceinline__ void rearm_tickets(int *tickets) {
  if (threadIdx.x == 0) {
    const int nrhs = gridDim.y;
    const int e = atomicAdd(&tickets[nrhs], 1);
    if (e == (int)(gridDim.x * gridDim.y) - 1) {
      for (int r = 0; r <= nrhs; ++r) tickets[r] = 0;
      __threadfence();
    }
  }
}

// blockIdx.y selects one of several right-hand sides (vectors vstride
// elements apart, each filled with the unsolved pattern beforehand); each has
// its own ticket counter tickets[rhs]; tickets[gridDim.y] counts exiting CTAs.
template <typename CT, typename VT, int R, bool LOWER>
__global__ void __launch_bounds__(512, 1) k_sptrsv_blk(BlkPlanDev P, const void *b_, int in_f32, void *x_,
                                                    int out_f32, size_t vstride, int *tickets,
                                                    const int *done_flag, int *status) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  constexpr int CS = 32 * R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT *xs = reinterpret_cast<CT *>(smem_raw);
  __shared__ int s_blk;
  __shared__ double s_zero;  // always solved: read by dependency slots that read nothing
  if (threadIdx.x == 0) s_zero = 0.0;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int rhs = blockIdx.y;
  const void *b = (const char *)b_ + (size_t)rhs * vstride * (in_f32 ? 4 : 8);
  void *x = (char *)x_ + (size_t)rhs * vstride * (out_f32 ? 4 : 8);
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) s_blk = atomicAdd(&tickets[rhs], 1);
    __syncthreads();
    const int bk = s_blk;
    if (bk >= P.nblocks) break;
    const int4 B = P.blk[bk];
    const unsigned brows = (unsigned)((B.y - B.x) * CS);
    const unsigned win = min(brows, (unsigned)P.win);
    for (unsigned s = threadIdx.x; s < win; s += blockDim.x) xs[s] = unsolved_value<CT>();
    if (threadIdx.x == 0) xs[win] = (CT)0;  // the spare slot: always solved
    __syncthreads();
    solve_block<CT, VT, R, LOWER, false>(P, B, xs, b, in_f32, x, out_f32, warp, nw, lane, &s_zero, status,
                                         Halo<CT>{0, 0u, 0u, nullptr});
  }
  rearm_tickets(tickets);
}

// The thread-block cluster variant.  A cluster of C CTAs takes C consecutive
// blocks with one ticket (rank r the r-th), and every CTA but the last in the
// cluster writes each row it solves into the next CTA's halo through
// distributed shared memory, so the block after it reads the rows it depends
// on there instead of through L2.  Shared memory: the window (P.win rows and
// the spare slot), then the halo (P.win rows).  Cluster barriers separate
// the groups: a CTA fills its window and halo with the unsolved pattern only
// after every CTA of the cluster finished the previous group, and starts
// solving only after every CTA of the cluster filled its own.  Rank 0 hands
// the ticket to every CTA's own shared memory before the barrier, so that no
// CTA touches another's shared memory after the last barrier (a CTA may then
// leave).  A rank waits only for blocks before its own, which earlier ranks
// and clusters holding earlier tickets solve, so every wait ends.
template <typename CT, typename VT, int R, bool LOWER>
__global__ void __launch_bounds__(512, 1) k_sptrsv_cl(BlkPlanDev P, const void *b_, int in_f32, void *x_,
                                                   int out_f32, size_t vstride, int *tickets,
                                                   const int *done_flag, int *status) {
  // the same flag for every CTA: the whole cluster returns or none does
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  constexpr int CS = 32 * R;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT *xs = reinterpret_cast<CT *>(smem_raw);
  __shared__ int s_grp;
  __shared__ double s_zero;
  if (threadIdx.x == 0) s_zero = 0.0;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int rhs = blockIdx.y;
  const int rank = (int)cl.block_rank(), csize = (int)cl.num_blocks();
  const void *b = (const char *)b_ + (size_t)rhs * vstride * (in_f32 ? 4 : 8);
  void *x = (char *)x_ + (size_t)rhs * vstride * (out_f32 ? 4 : 8);
  const unsigned hbase = (unsigned)P.win + 1;
  CT *next_xs = rank + 1 < csize ? cl.map_shared_rank(xs, rank + 1) : nullptr;
  cl.sync();  // every CTA of the cluster runs before one writes to another
  while (true) {
    if (rank == 0 && threadIdx.x == 0) {
      const int g = atomicAdd(&tickets[rhs], 1);
      for (int r = 0; r < csize; ++r) *(volatile int *)cl.map_shared_rank(&s_grp, r) = g;
    }
    cl.sync();  // the ticket is out; every CTA is done with the previous group
    const int grp = *(const volatile int *)&s_grp;
    if (grp * csize >= P.nblocks) break;  // the same for the whole cluster
    const int bk = grp * csize + rank;
    const bool active = bk < P.nblocks;
    int4 B = make_int4(0, 0, 0, 0);
    Halo<CT> h{0, 0u, hbase, nullptr};
    if (active) {
      B = P.blk[bk];
      const unsigned brows = (unsigned)((B.y - B.x) * CS);
      const unsigned win = min(brows, (unsigned)P.win);
      for (unsigned s = threadIdx.x; s < win; s += blockDim.x) xs[s] = unsolved_value<CT>();
      if (threadIdx.x == 0) xs[win] = (CT)0;  // the spare slot: always solved
      if (rank > 0) {
        const int4 Bp = P.blk[bk - 1];
        h.prev_row0 = Bp.w;
        h.prev_rows = (unsigned)((Bp.y - Bp.x) * CS);
        for (unsigned s = threadIdx.x; s < h.prev_rows; s += blockDim.x) xs[hbase + s] = unsolved_value<CT>();
      }
      if (rank + 1 < csize && bk + 1 < P.nblocks) h.remote = next_xs;
    }
    cl.sync();  // every halo is filled before any CTA writes into one
    if (active)
      solve_block<CT, VT, R, LOWER, true>(P, B, xs, b, in_f32, x, out_f32, warp, nw, lane, &s_zero, status, h);
  }
  rearm_tickets(tickets);
}

// the plan's values from the triangle's values: per row slot q, 1/a_ii (1 for
// a unit diagonal), -a_{i,prev}/a_ii, and a_ij/a_ii per dependency slot
template <typename VT, typename CT>
__global__ void k_plan_values(size_t rs, int R, int S, const int *umap, const int *udiag, const int *uprev,
                              const VT *val, CT *uvs, CT *uaps, CT *urd) {
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t per = (size_t)R * 32;
  for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < rs; q += stride) {
    const int dg = udiag[q], pv = uprev[q];
    const CT rd = dg >= 0 ? (CT)1 / cvt<CT>(val[dg]) : (CT)1;
    urd[q] = rd;
    uaps[q] = pv >= 0 ? -cvt<CT>(val[pv]) * rd : (CT)0;
    const size_t u = q / per, w = q % per;
    for (int t = 0; t < S; ++t) {
      const size_t qs = (u * S + t) * per + w;
      const int e = umap[qs];
      uvs[qs] = e >= 0 ? cvt<CT>(val[e]) * rd : (CT)0;
    }
  }
}

void launch_plan_values(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt) {
  const size_t rs = (size_t)pl.nunits * pl.R * 32;
  const int S = blk_slots(pl.R);
  const int grid = (int)std::max<size_t>(1, std::min<size_t>((size_t)num_sms() * 8, (rs + 255) / 256));
  switch (vt) {
    case VType::F64:
      k_plan_values<double, double><<<grid, 256, 0, s>>>(rs, pl.R, S, pl.umap, pl.udiag, pl.uprev,
                                                         (const double *)val, (double *)pl.uvs,
                                                         (double *)pl.uaps, (double *)pl.urd);
      break;
    case VType::F32:
      k_plan_values<float, float><<<grid, 256, 0, s>>>(rs, pl.R, S, pl.umap, pl.udiag, pl.uprev,
                                                       (const float *)val, (float *)pl.uvs, (float *)pl.uaps,
                                                       (float *)pl.urd);
      break;
    case VType::BF16:
      k_plan_values<__nv_bfloat16, float><<<grid, 256, 0, s>>>(rs, pl.R, S, pl.umap, pl.udiag, pl.uprev,
                                                               (const __nv_bfloat16 *)val, (float *)pl.uvs,
                                                               (float *)pl.uaps, (float *)pl.urd);
      break;
  }
}

// fill nrhs vectors (vstride elements apart) of n elements with the unsolved pattern
__global__ void k_fill_unsolved(void *x, int f32, int n, size_t vstride, int nrhs, const int *done_flag) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  const size_t esz = f32 ? 4 : 8;
  const size_t stride = (size_t)gridDim.x * blockDim.x;
  const size_t t0 = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  for (int r = 0; r < nrhs; ++r) {
    unsigned char *v = (unsigned char *)x + (size_t)r * vstride * esz;
    const size_t bytes = (size_t)n * esz;
    // 16-byte stores over the aligned middle, single bytes at the ends
    const size_t head = (16 - ((uintptr_t)v & 15)) & 15;
    const size_t h = head < bytes ? head : bytes;
    const size_t nvec = (bytes - h) / 16;
    for (size_t k = t0; k < nvec; k += stride) reinterpret_cast<uint4 *>(v + h)[k] = make_uint4(~0u, ~0u, ~0u, ~0u);
    for (size_t k = t0; k < h; k += stride) v[k] = 0xff;
    for (size_t k = h + nvec * 16 + t0; k < bytes; k += stride) v[k] = 0xff;
  }
}

struct BlkArgs {
  const void *b;
  int in_f32;
  void *x;
  int out_f32;
  size_t vstride;
  int nrhs;
  int *tickets, *status;
  const int *dfl;
  int max_units, lower;
  int cl;  // CTAs per thread-block cluster (1: the plain kernel)
};

template <typename CT, typename VT, int R, bool LOWER>
static cudaError_t cl_launch(cudaStream_t s, const BlkPlanDev &P, int warps, int grid, const BlkArgs &a,
                             bool query_only, int *clusters) {
  auto fn = k_sptrsv_cl<CT, VT, R, LOWER>;
  const size_t sm = (2 * (size_t)P.win + 1) * sizeof(CT);
  if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  // clusters of 16 (one 128x128 plane per CTA: 8 clusters cover 128 planes) are
  // beyond the portable size of 8
  if (a.cl > 8) cudaFuncSetAttribute(fn, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid, a.nrhs);
  cfg.blockDim = dim3(32 * warps);
  cfg.dynamicSmemBytes = sm;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeClusterDimension;
  at[0].val.clusterDim.x = (unsigned)a.cl;
  at[0].val.clusterDim.y = 1;
  at[0].val.clusterDim.z = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  if (query_only) return cudaOccupancyMaxActiveClusters(clusters, fn, &cfg);
  return cudaLaunchKernelEx(&cfg, fn, P, a.b, a.in_f32, a.x, a.out_f32, a.vstride, a.tickets, a.dfl, a.status);
}

template <typename CT, typename VT, int R>
static cudaError_t cl_launch_l(cudaStream_t s, const BlkPlanDev &P, int warps, int grid, const BlkArgs &a,
                               bool query_only, int *clusters) {
  return a.lower ? cl_launch<CT, VT, R, true>(s, P, warps, grid, a, query_only, clusters)
                 : cl_launch<CT, VT, R, false>(s, P, warps, grid, a, query_only, clusters);
}

template <typename CT, typename VT, int R>
static void blk_launch(cudaStream_t s, const BlkPlanDev &P, int warps, int grid, const BlkArgs &a) {
  if (R <= 4 && a.cl > 1) {
    cl_launch_l<CT, VT, (R <= 4 ? R : 4)>(s, P, warps, grid, a, false, nullptr);
    return;
  }
  dim3 g(grid, a.nrhs);
  const size_t sm = ((size_t)P.win + 1) * sizeof(CT);
  if (a.lower) {
    auto fn = k_sptrsv_blk<CT, VT, R, true>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    fn<<<g, 32 * warps, sm, s>>>(P, a.b, a.in_f32, a.x, a.out_f32, a.vstride, a.tickets, a.dfl, a.status);
  } else {
    auto fn = k_sptrsv_blk<CT, VT, R, false>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    fn<<<g, 32 * warps, sm, s>>>(P, a.b, a.in_f32, a.x, a.out_f32, a.vstride, a.tickets, a.dfl, a.status);
  }
}

template <typename CT, typename VT>
static void blk_launch_r(cudaStream_t s, int R, const BlkPlanDev &P, int warps, int grid, const BlkArgs &a) {
  switch (R) {
    case 1: blk_launch<CT, VT, 1>(s, P, warps, grid, a); break;
    case 2: blk_launch<CT, VT, 2>(s, P, warps, grid, a); break;
    case 8: blk_launch<CT, VT, 8>(s, P, warps, grid, a); break;
    default: blk_launch<CT, VT, 4>(s, P, warps, grid, a); break;
  }
}

static BlkPlanDev plan_dev(const TriBlkPlan &pl, const void *val) {
  BlkPlanDev P;
  P.n = pl.n;
  P.nblocks = pl.nblocks;
  P.row = pl.row;
  P.col = pl.col;
  P.val = val;
  P.blk = pl.blk;
  P.urec = pl.urec;
  P.ucode = pl.ucode;
  P.uflag = pl.uflag;
  P.uvs = pl.uvs;
  P.uaps = pl.uaps;
  P.urd = pl.urd;
  P.win = 0;
  return P;
}

// shared memory of a block's window; the cluster variant needs twice that
// (window and halo) and a window that holds the whole block
static int window_rows(const TriBlkPlan &pl, VType vt) {
  const size_t rows = (size_t)pl.cpb * 32 * pl.R;
  const size_t esz = vt == VType::F64 ? 8 : 4;
  return rows * esz <= (size_t)kSptrsvSmemMax ? (int)rows : 0;
}

static int cluster_size(const TriBlkPlan &pl, VType vt) {
  if (pl.cl <= 1 || pl.R > 4) return 1;
  const size_t esz = vt == VType::F64 ? 8 : 4;
  const int win = window_rows(pl, vt);
  if (win == 0 || (2 * (size_t)win + 1) * esz > kSptrsvClusterSmemMax) return 1;
  return pl.cl;
}

int sptrsv_cluster_supported(const TriBlkPlan &pl, VType vt) {
  if (cluster_size(pl, vt) <= 1) return 0;
  BlkPlanDev P = plan_dev(pl, nullptr);
  P.win = window_rows(pl, vt);
  BlkArgs a{nullptr, 0, nullptr, 0, 0, 1, nullptr, nullptr, nullptr, pl.max_units, pl.lower, pl.cl};
  int clusters = 0;
  cudaError_t e = cudaSuccess;
  switch (vt) {
    case VType::F64:
      e = pl.R == 1 ? cl_launch_l<double, double, 1>(0, P, pl.warps, pl.cl, a, true, &clusters)
                    : (pl.R == 2 ? cl_launch_l<double, double, 2>(0, P, pl.warps, pl.cl, a, true, &clusters)
                                 : cl_launch_l<double, double, 4>(0, P, pl.warps, pl.cl, a, true, &clusters));
      break;
    default:
      e = pl.R == 1 ? cl_launch_l<float, float, 1>(0, P, pl.warps, pl.cl, a, true, &clusters)
                    : (pl.R == 2 ? cl_launch_l<float, float, 2>(0, P, pl.warps, pl.cl, a, true, &clusters)
                                 : cl_launch_l<float, float, 4>(0, P, pl.warps, pl.cl, a, true, &clusters));
      break;
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return clusters > 0 ? 1 : 0;
}

void launch_sptrsv_blk_multi(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                             int in_f32, void *x, int out_f32, size_t vstride, int nrhs, int *tickets, int *status,
                             const int *done_flag, bool prefilled) {
  BlkPlanDev P = plan_dev(pl, val);
  // rows of a block kept in shared memory: the whole block when it fits
  P.win = window_rows(pl, vt);
  const int cl = cluster_size(pl, vt);
  int grid = pl.grid;
  if (cl > 1) {
    // whole clusters, at most one per group of cl blocks
    const int groups = (pl.nblocks + cl - 1) / cl;
    grid = std::max(1, std::min(groups, std::max(1, grid / cl))) * cl;
  } else {
    if (grid > pl.nblocks) grid = pl.nblocks;
    if (grid < 1) grid = 1;
  }
  if (!prefilled) {
    const size_t vec16 = ((size_t)pl.n * (out_f32 ? 4 : 8) + 15) / 16;
    const int fgrid = (int)std::max<size_t>(1, std::min<size_t>((size_t)num_sms() * 4, (vec16 + 255) / 256));
    k_fill_unsolved<<<fgrid, 256, 0, s>>>(x, out_f32, pl.n, vstride, nrhs, done_flag);
  }
  BlkArgs a{b, in_f32, x, out_f32, vstride, nrhs, tickets, status, done_flag, pl.max_units, pl.lower, cl};
  switch (vt) {
    case VType::F64: blk_launch_r<double, double>(s, pl.R, P, pl.warps, grid, a); break;
    case VType::F32: blk_launch_r<float, float>(s, pl.R, P, pl.warps, grid, a); break;
    case VType::BF16: blk_launch_r<float, __nv_bfloat16>(s, pl.R, P, pl.warps, grid, a); break;
  }
}

void launch_sptrsv_blk(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                       int in_f32, void *x, int out_f32, Control *ctrl, int slot, bool honor_done, bool prefilled) {
  launch_sptrsv_blk_multi(s, pl, val, vt, b, in_f32, x, out_f32, 0, 1, ctrl->tickets[slot], &ctrl->status,
                          honor_done ? &ctrl->done : nullptr, prefilled);
}

}  // namespace lace
