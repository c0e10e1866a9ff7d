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
// round robin in local-level order (a chunk's level is one more than that of
// its dependencies in the block), so the lowest unsolved chunk can always
// proceed.
//
// Each warp prepares its next chunks while other warps solve, three deep:
// the chunk after next has its record and row pointers loaded, the next one
// its entries and right-hand side, and when a chunk is done the next one is
// classified (window slot or row of another block per entry) and scaled by
// the reciprocal of the diagonal.  What is left on the dependency chain is
// reading the dependencies, one fused multiply-add per entry, the scan, and
// the stores.
//
// For a lexicographic 7-point stencil with R = 4 (a chunk = one x-line) and
// blocks of whole planes, every x-line is one scan, the j- and k-direction
// dependencies inside a block are shared-memory reads, and only a block's
// first plane reads rows of another CTA.
#include <algorithm>

#include "internal.h"

namespace lace {

template <typename T>
__device__ __forceinline__ void st_out(void *x, int out_f32, int i, T v) {
  if (out_f32) ((volatile float *)x)[i] = (float)v;
  else ((volatile double *)x)[i] = (double)v;
}

// shared memory a CTA may use for its block's solved rows
constexpr int kSptrsvSmemMax = 160 * 1024;

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

// CSR entries of a row loaded ahead of the row's turn; longer rows read the
// rest when they are solved
template <int R>
struct BlkSlots {
  static constexpr int S = R == 1 ? 6 : (R == 2 ? 4 : (R == 4 ? 3 : 2));
};

struct BlkPlanDev {
  int n, nblocks;
  const int *row, *col;
  const void *val;
  int unit;
  const int4 *blk;   // {first unit, end unit, local levels, lowest row}
  const int4 *urec;  // {chunk, local level | serial << 30, 0, 0}
  int win;           // rows of a block kept in shared memory (0: none), plus a spare slot
  int rec_off;       // byte offset of the staged unit records in dynamic shared memory
};

// A chunk of the block whose record and row pointers are loaded.
template <int R>
struct UnitHead {
  int k;  // index in the block's unit list; -1: none
  int4 rec;
  int e0[R], e1[R];
};
// Loaded entries of a chunk, before classification.
template <typename VT, int R, int S>
struct UnitRaw {
  int cc[R][S];
  VT vv[R][S];
  unsigned long long braw[R];  // b_i: FP64 bits, or FP32 bits in the low word
};
// A chunk ready to solve.  Per row: bs = b/d, aps = -a_{i,prev}/d, rd = 1/d,
// and the loaded entries scaled by 1/d with where their dependency is read:
// code >= 0 a window slot, code <= -2 row -(code+2) of the output, -1 none.
// Bit r of rest: row r has dependencies among the entries not loaded.
template <typename CT, int R, int S>
struct UnitReady {
  int k;
  int4 rec;
  CT bs[R], aps[R], rd[R];
  int code[R][S];
  CT vs[R][S];
  int e0[R], e1[R];
  int rest;
};

template <int R, bool LOWER>
__device__ __forceinline__ void unit_head(UnitHead<R> &h, int k, int nunits, const int4 *s_rec,
                                          const BlkPlanDev &P, int lane) {
  constexpr int CS = 32 * R;
  h.k = k < nunits ? k : -1;
  if (h.k < 0) return;
  h.rec = s_rec[k];
  const int base = h.rec.x * CS, cnt = min(CS, P.n - base);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int pos = lane * R + r;
    h.e0[r] = 0;
    h.e1[r] = 0;
    if (pos < cnt) {
      const int i = LOWER ? base + pos : base + cnt - 1 - pos;
      h.e0[r] = P.row[i];
      h.e1[r] = P.row[i + 1];
    }
  }
}

template <typename VT, int R, int S, bool LOWER>
__device__ __forceinline__ void unit_load(UnitRaw<VT, R, S> &w, const UnitHead<R> &h, const BlkPlanDev &P,
                                          const void *b, int in_f32, int lane) {
  constexpr int CS = 32 * R;
  if (h.k < 0) return;
  const VT *val = (const VT *)P.val;
  const int base = h.rec.x * CS, cnt = min(CS, P.n - base);
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int pos = lane * R + r;
    w.braw[r] = 0;
    if (pos < cnt) {
      const int i = LOWER ? base + pos : base + cnt - 1 - pos;
      if (in_f32) w.braw[r] = ((const unsigned *)b)[i];
      else w.braw[r] = ((const unsigned long long *)b)[i];
    }
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const int e = h.e0[r] + t;
      w.cc[r][t] = -1;
      if (e < h.e1[r]) {
        w.cc[r][t] = P.col[e];
        w.vv[r][t] = val[e];
      }
    }
  }
}

template <typename CT, typename VT, int R, int S, bool LOWER>
__device__ __forceinline__ void unit_classify(UnitReady<CT, R, S> &u, const UnitRaw<VT, R, S> &w,
                                              const UnitHead<R> &h, const BlkPlanDev &P, int in_f32,
                                              int lane, int row0, unsigned brows, unsigned win) {
  constexpr int CS = 32 * R;
  u.k = h.k;
  u.rec = h.rec;
  if (u.k < 0) return;
  const VT *val = (const VT *)P.val;
  const int c = h.rec.x;
  const bool serial = (h.rec.y >> 30) != 0;
  const int base = c * CS, cnt = min(CS, P.n - base);
  u.rest = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int pos = lane * R + r;
    const int i = LOWER ? base + pos : base + cnt - 1 - pos;
    const int prev = LOWER ? i - 1 : i + 1;
    u.e0[r] = h.e0[r];
    u.e1[r] = h.e1[r];
    CT d = (CT)1, ap = (CT)0;
    auto where = [&](int jc, CT v) -> int {
      if (jc == i) {
        if (!P.unit) d = v;
        return -1;
      }
      if (LOWER ? (jc > i) : (jc < i)) return -1;
      if (jc / CS == c) {
        if (!serial && jc == prev) ap = v;
        return -1;
      }
      const unsigned slot = (unsigned)(jc - row0);
      return (slot < brows && slot < win) ? (int)slot : -jc - 2;
    };
#pragma unroll
    for (int t = 0; t < S; ++t) {
      const CT v = cvt<CT>(w.vv[r][t]);
      u.code[r][t] = w.cc[r][t] >= 0 ? where(w.cc[r][t], v) : -1;
      u.vs[r][t] = v;
    }
    // the diagonal (last in a CSRL row) may lie beyond the loaded entries
    for (int e = h.e0[r] + S; e < h.e1[r]; ++e)
      if (where(P.col[e], cvt<CT>(val[e])) != -1) u.rest |= 1 << r;
    const CT rd = P.unit ? (CT)1 : rcp_rn(d);
    const CT bb = in_f32 ? (CT)__uint_as_float((unsigned)w.braw[r])
                         : (CT)__longlong_as_double((long long)w.braw[r]);
    u.rd[r] = rd;
    u.bs[r] = pos < cnt ? bb * rd : (CT)0;
    u.aps[r] = -ap * rd;
#pragma unroll
    for (int t = 0; t < S; ++t) u.vs[r][t] *= rd;
  }
}

// blockIdx.y selects one of several right-hand sides (vectors vstride
// elements apart, each filled with the unsolved pattern beforehand); each has
// its own ticket counter tickets[rhs]; tickets[gridDim.y] counts exiting CTAs.
template <typename CT, typename VT, int R, bool LOWER>
__global__ void __launch_bounds__(512) k_sptrsv_blk(BlkPlanDev P, const void *b_, int in_f32, void *x_,
                                                    int out_f32, size_t vstride, int *tickets,
                                                    const int *done_flag, int *status) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  constexpr int CS = 32 * R;
  constexpr int S = BlkSlots<R>::S;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  CT *xs = reinterpret_cast<CT *>(smem_raw);
  int4 *s_rec = reinterpret_cast<int4 *>(smem_raw + P.rec_off);
  __shared__ int s_blk;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nw = blockDim.x >> 5;
  const int rhs = blockIdx.y;
  const void *b = (const char *)b_ + (size_t)rhs * vstride * (in_f32 ? 4 : 8);
  void *x = (char *)x_ + (size_t)rhs * vstride * (out_f32 ? 4 : 8);
  const VT *val = (const VT *)P.val;
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) s_blk = atomicAdd(&tickets[rhs], 1);
    __syncthreads();
    const int bk = s_blk;
    if (bk >= P.nblocks) break;
    const int4 B = P.blk[bk];
    const int nunits = B.y - B.x, row0 = B.w;
    const unsigned brows = (unsigned)(nunits * CS);
    const unsigned win = min(brows, (unsigned)P.win);
    for (int u = threadIdx.x; u < nunits; u += blockDim.x) s_rec[u] = P.urec[B.x + u];
    for (unsigned s = threadIdx.x; s < win; s += blockDim.x) xs[s] = unsolved_value<CT>();
    if (threadIdx.x == 0) xs[win] = (CT)0;  // the spare slot: always solved
    __syncthreads();
    // a warp's chunks are k = warp, warp + nw, ...: ub is ready to solve;
    // the entries of the next one (rw, with its head rh) are in flight, and
    // the record and row pointers of the one after that (hd)
    UnitReady<CT, R, S> ub;
    UnitRaw<VT, R, S> rw;
    UnitHead<R> rh, hd;
    {
      UnitHead<R> h0;
      unit_head<R, LOWER>(h0, warp, nunits, s_rec, P, lane);
      unit_load<VT, R, S, LOWER>(rw, h0, P, b, in_f32, lane);
      rh.k = -1;
      if (h0.k >= 0) unit_head<R, LOWER>(rh, h0.k + nw, nunits, s_rec, P, lane);
      unit_classify<CT, VT, R, S, LOWER>(ub, rw, h0, P, in_f32, lane, row0, brows, win);
      unit_load<VT, R, S, LOWER>(rw, rh, P, b, in_f32, lane);
      hd.k = -1;
      if (rh.k >= 0) unit_head<R, LOWER>(hd, rh.k + nw, nunits, s_rec, P, lane);
    }
    while (ub.k >= 0) {
      const int c = ub.rec.x;
      const bool serial = (ub.rec.y >> 30) != 0;
      const int base = c * CS;
      const int cnt = min(CS, P.n - base);
      CT A[R], Bv[R], X[R];
      int rows[R];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int pos = lane * R + r;
        rows[r] = pos < cnt ? (LOWER ? base + pos : base + cnt - 1 - pos) : -1;
        A[r] = serial ? (CT)0 : ub.aps[r];
        X[r] = (CT)0;
      }
      // Wait for the chunk's dependencies with the whole warp in lock step
      // (lanes spinning on different branches of a diverged warp would wait
      // for the scheduler to switch between them): each pass reads all of a
      // phase's dependencies and forms the sums, and the warp leaves when
      // every lane saw them solved.  Phase A: rows of other blocks (and
      // dependencies beyond the loaded entries), read through L2; they are
      // usually solved before the warp gets here.  Phase B: rows of this block
      // from the window, branch free - an entry that is not a window
      // dependency reads the always-solved spare slot with weight 0.
      bool far = false;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        Bv[r] = ub.bs[r];
        far |= (ub.rest >> r) & 1;
#pragma unroll
        for (int t = 0; t < S; ++t) far |= ub.code[r][t] <= -2;
      }
      if (__any_sync(0xffffffffu, far)) {
        for (int spins = 0;; ++spins) {
          bool ok = true;
#pragma unroll
          for (int r = 0; r < R; ++r) {
            CT acc = ub.bs[r];
#pragma unroll
            for (int t = 0; t < S; ++t)
              if (ub.code[r][t] <= -2) acc -= ub.vs[r][t] * read_dep<CT>(xs, x, out_f32, ub.code[r][t], ok);
            if (ub.rest & (1 << r))
              for (int e = ub.e0[r] + S; e < ub.e1[r]; ++e) {
                const int i = rows[r], jc = P.col[e];
                if (jc == i || (LOWER ? (jc > i) : (jc < i)) || jc / CS == c) continue;
                const unsigned slot = (unsigned)(jc - row0);
                const int code = (slot < brows && slot < win) ? (int)slot : -jc - 2;
                acc -= cvt<CT>(val[e]) * ub.rd[r] * read_dep<CT>(xs, x, out_f32, code, ok);
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
      for (int spins = 0;; ++spins) {
        bool ok = true;
        CT acc[R];
#pragma unroll
        for (int r = 0; r < R; ++r) {
          acc[r] = Bv[r];
#pragma unroll
          for (int t = 0; t < S; ++t) {
            const int code = ub.code[r][t];
            const CT v = ((const volatile CT *)xs)[code >= 0 ? code : (int)win];
            ok &= !is_unsolved(v);
            acc[r] -= (code >= 0 ? ub.vs[r][t] : (CT)0) * v;
          }
        }
        if (__all_sync(0xffffffffu, ok)) {
#pragma unroll
          for (int r = 0; r < R; ++r) Bv[r] = acc[r];
          break;
        }
        if (spins > kMaxSpins || ((spins & 1023) == 1023 && (*(const volatile int *)status & kStatusSpinTimeout))) {
          if (lane == 0) atomicOr(status, kStatusSpinTimeout);
          break;
        }
      }
      if (!serial) {
        // x_p = A_p x_{p-1} + B_p along the chunk: a warp-wide affine scan
        CT ca = (CT)1, cb = (CT)0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          cb = A[r] * cb + Bv[r];
          ca = A[r] * ca;
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const CT pa = __shfl_up_sync(0xffffffffu, ca, o);
          const CT pb = __shfl_up_sync(0xffffffffu, cb, o);
          if (lane >= o) {
            cb = ca * pb + cb;
            ca = ca * pa;
          }
        }
        CT xin = __shfl_up_sync(0xffffffffu, cb, 1);
        if (lane == 0) xin = (CT)0;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          xin = A[r] * xin + Bv[r];
          X[r] = xin;
        }
      } else {
        // position by position: the owner's value is final, the later rows
        // of the chunk subtract it
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
              for (int e = ub.e0[r]; e < ub.e1[r]; ++e)
                if (P.col[e] == rowp) Bv[r] -= cvt<CT>(val[e]) * ub.rd[r] * xp;
          }
        }
      }
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (rows[r] >= 0) {
          const CT v = as_solved(X[r]);
          const unsigned slot = (unsigned)(rows[r] - row0);
          if (slot < win) ((volatile CT *)xs)[slot] = v;
          st_out<CT>(x, out_f32, rows[r], v);
        }
      // advance the pipeline: classify the next chunk (its entries were
      // loaded one chunk ago), load the entries of the one after, and the
      // record and row pointers of the one after that
      unit_classify<CT, VT, R, S, LOWER>(ub, rw, rh, P, in_f32, lane, row0, brows, win);
      rh = hd;
      unit_load<VT, R, S, LOWER>(rw, rh, P, b, in_f32, lane);
      hd.k = -1;
      if (rh.k >= 0) unit_head<R, LOWER>(hd, rh.k + nw, nunits, s_rec, P, lane);
    }
  }
  // the CTA that leaves last re-arms the tickets
  if (threadIdx.x == 0) {
    const int nrhs = gridDim.y;
    const int e = atomicAdd(&tickets[nrhs], 1);
    if (e == (int)(gridDim.x * gridDim.y) - 1) {
      for (int r = 0; r <= nrhs; ++r) tickets[r] = 0;
      __threadfence();
    }
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
};

template <typename CT, typename VT, int R>
static void blk_launch(cudaStream_t s, const BlkPlanDev &P, int warps, int grid, const BlkArgs &a) {
  dim3 g(grid, a.nrhs);
  const size_t sm = (size_t)P.rec_off + (size_t)a.max_units * sizeof(int4);
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
  P.unit = pl.unit;
  P.blk = pl.blk;
  P.urec = pl.urec;
  P.win = 0;
  P.rec_off = 0;
  return P;
}

void launch_sptrsv_blk_multi(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                             int in_f32, void *x, int out_f32, size_t vstride, int nrhs, int *tickets, int *status,
                             const int *done_flag) {
  BlkPlanDev P = plan_dev(pl, val);
  // rows of a block kept in shared memory: the whole block when it fits
  const size_t rows = (size_t)pl.cpb * 32 * pl.R;
  const size_t esz = vt == VType::F64 ? 8 : 4;
  P.win = rows * esz <= (size_t)kSptrsvSmemMax ? (int)rows : 0;
  P.rec_off = (int)(((size_t)(P.win + 1) * esz + 15) & ~(size_t)15);  // window + spare slot
  int grid = pl.grid;
  if (grid > pl.nblocks) grid = pl.nblocks;
  if (grid < 1) grid = 1;
  const size_t vec16 = ((size_t)pl.n * (out_f32 ? 4 : 8) + 15) / 16;
  const int fgrid = (int)std::max<size_t>(1, std::min<size_t>((size_t)num_sms() * 4, (vec16 + 255) / 256));
  k_fill_unsolved<<<fgrid, 256, 0, s>>>(x, out_f32, pl.n, vstride, nrhs, done_flag);
  BlkArgs a{b, in_f32, x, out_f32, vstride, nrhs, tickets, status, done_flag, pl.max_units, pl.lower};
  switch (vt) {
    case VType::F64: blk_launch_r<double, double>(s, pl.R, P, pl.warps, grid, a); break;
    case VType::F32: blk_launch_r<float, float>(s, pl.R, P, pl.warps, grid, a); break;
    case VType::BF16: blk_launch_r<float, __nv_bfloat16>(s, pl.R, P, pl.warps, grid, a); break;
  }
}

void launch_sptrsv_blk(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                       int in_f32, void *x, int out_f32, Control *ctrl, int slot, bool honor_done) {
  launch_sptrsv_blk_multi(s, pl, val, vt, b, in_f32, x, out_f32, 0, 1, ctrl->tickets[slot], &ctrl->status,
                          honor_done ? &ctrl->done : nullptr);
}

}  // namespace lace
