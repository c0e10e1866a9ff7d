// Block-scheduled sync-free SpTRSV.
//
// The rows of one triangle are cut into chunks of 32*R consecutive rows (one
// warp each, lane l the R rows l*R.. in solve order; "scan" chunks whose only
// in-chunk dependency is the previous row are solved with a warp-wide affine
// scan, others position by position).  Consecutive chunks (in solve order)
// form blocks; one CTA owns a block at a time (taken by atomic ticket, in
// solve order).  Inside a block the chunks are processed by local level - a
// chunk's level is one more than that of its dependencies in the same block -
// with a CTA barrier between levels, so dependencies inside a block cost a
// barrier instead of a round trip through L2.  A chunk that depends on rows of
// an earlier block waits until that block's published progress (levels done,
// 64-bit epoch-tagged counter) covers the dependency's level: one relaxed poll
// per distinct block, bounded, then an acquire fence.  A block of one chunk
// with one warp is the classic warp-level sync-free solve.
//
// For a lexicographic 7-point stencil with R = 4 (a chunk = one x-line) and
// blocks of several planes, every x-line is one scan, the j- and k-direction
// dependencies inside a block are barrier steps, and only a block's first
// plane waits on another CTA.
#include "internal.h"

namespace lace {

template <typename T>
__device__ __forceinline__ T ld_in(const void *b, int in_f32, int i) {
  return in_f32 ? (T)((const float *)b)[i] : (T)((const double *)b)[i];
}
template <typename T>
__device__ __forceinline__ void st_out(void *x, int out_f32, int i, T v) {
  if (out_f32) ((float *)x)[i] = (float)v;
  else ((double *)x)[i] = (double)v;
}
// x written by another CTA (after the acquire): read through L2
template <typename T>
__device__ __forceinline__ T ld_x_l2(const void *x, int f32, int i) {
  return f32 ? (T)__ldcg(((const float *)x) + i) : (T)__ldcg(((const double *)x) + i);
}
// x written by this CTA (ordered by the CTA barrier)
template <typename T>
__device__ __forceinline__ T ld_x_cta(const void *x, int f32, int i) {
  return f32 ? (T)((const volatile float *)x)[i] : (T)((const volatile double *)x)[i];
}

__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void fence_acquire() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }

// shared memory a CTA may use for its block's solved rows
constexpr int kSptrsvSmemMax = 160 * 1024;

struct BlkPlanDev {
  int n, nchunks, nblocks;
  const int *row, *col;
  const void *val;
  int unit, lower;
  const int *blk_lvl_ptr;   // [nblocks+1] offsets into lvl_ptr
  const int *lvl_ptr;       // level -> offset into units
  const int *units;         // chunk ids ordered by (block, level)
  const int *chunk_blk;     // chunk -> block (solve order index)
  const int *blk_row0;      // block -> lowest row it holds
  const int *req_ptr;       // chunk -> offsets into req_blk / req_lvl
  const int *req_blk;       // blocks a chunk waits on
  const int *req_lvl;       // ... and how many levels of them
  const uint8_t *kind;      // 0 scan, 1 serial
  unsigned long long *progress;  // per block: (epoch << 32) | levels done
  int win;                  // rows of a block kept in shared memory (0: none)
};

// blockIdx.y selects one of several right-hand sides (vectors vstride
// elements apart); each has its own tickets (tickets[rhs]) and progress
// counters (progress + rhs * nblocks); tickets[gridDim.y] counts exiting CTAs.
//
// Every row a block solves is also kept in shared memory (P.win rows from the
// block's lowest row), so a dependency inside the block is a shared-memory
// read after the level barrier; other blocks' rows are read from L2 after
// their progress is seen.  With several warps the last one only publishes the
// block's progress (one release store per level), so the fence latency stays
// off the warps that solve the next level.
template <typename CT, typename VT, int R, bool LOWER>
__global__ void __launch_bounds__(512) k_sptrsv_blk(BlkPlanDev P, const void *b_, int in_f32, void *x_,
                                                    int out_f32, size_t vstride, int *tickets,
                                                    int *epoch_slot, const int *done_flag, int *status) {
  if (done_flag != nullptr && *(volatile const int *)done_flag) return;
  extern __shared__ unsigned char smem_raw[];
  CT *xs = reinterpret_cast<CT *>(smem_raw);
  constexpr int CS = 32 * R;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  const bool publisher_warp = nwarps > 1 && warp == nwarps - 1;
  const int nw = nwarps > 1 ? nwarps - 1 : 1;  // warps that solve
  const int rhs = blockIdx.y;
  const void *b = (const char *)b_ + (size_t)rhs * vstride * (in_f32 ? 4 : 8);
  void *x = (char *)x_ + (size_t)rhs * vstride * (out_f32 ? 4 : 8);
  P.progress += (size_t)rhs * P.nblocks;
  const unsigned long long ep = (unsigned long long)(unsigned)(*(volatile int *)epoch_slot + 1);
  __shared__ int s_blk;
  const VT *val = (const VT *)P.val;
  while (true) {
    __syncthreads();
    if (threadIdx.x == 0) s_blk = atomicAdd(&tickets[rhs], 1);
    __syncthreads();
    const int bk = s_blk;
    if (bk >= P.nblocks) break;
    const int l0 = P.blk_lvl_ptr[bk], l1 = P.blk_lvl_ptr[bk + 1];
    const int row0 = P.blk_row0[bk];
    for (int lv = l0; lv < l1; ++lv) {
      if (!publisher_warp) {
        for (int u = P.lvl_ptr[lv] + warp; u < P.lvl_ptr[lv + 1]; u += nw) {
          const int c = P.units[u];
          // cross-block requirements: one lane per required block
          const int r0 = P.req_ptr[c], nr = P.req_ptr[c + 1] - r0;
          for (int q = lane; q < nr; q += 32) {
            const int ob = P.req_blk[r0 + q];
            const unsigned long long need = (ep << 32) | (unsigned)P.req_lvl[r0 + q];
            int spins = 0;
            while (ld_relaxed_u64(&P.progress[ob]) < need) {
              if (++spins > kMaxSpins) {
                atomicOr(status, kStatusSpinTimeout);
                break;
              }
              if (spins > 32) __nanosleep(32);
            }
          }
          __syncwarp();
          if (nr > 0) fence_acquire();
          const int base = c * CS;
          const int cnt = min(CS, P.n - base);
          const bool serial = P.kind[c] != 0;
          CT A[R], B[R], X[R];
          int rows[R];
#pragma unroll
          for (int r = 0; r < R; ++r) {
            const int pos = lane * R + r;
            A[r] = (CT)1;
            B[r] = (CT)0;
            rows[r] = -1;
            if (pos >= cnt) continue;
            const int i = LOWER ? base + pos : base + cnt - 1 - pos;
            rows[r] = i;
            const int prev = LOWER ? i - 1 : i + 1;
            CT acc = ld_in<CT>(b, in_f32, i);
            CT d = (CT)1, ap = (CT)0;
            for (int e = P.row[i]; e < P.row[i + 1]; ++e) {
              const int jc = P.col[e];
              if (jc == i) {
                if (!P.unit) d = cvt<CT>(val[e]);
                continue;
              }
              if (LOWER ? (jc > i) : (jc < i)) continue;
              const int cj = jc / CS;
              if (cj == c) {
                if (!serial && pos > 0 && jc == prev) ap = cvt<CT>(val[e]);
                continue;
              }
              const unsigned slot = (unsigned)(jc - row0);
              CT xv;
              if (slot < (unsigned)P.win && P.chunk_blk[cj] == bk)
                xv = ((volatile CT *)xs)[slot];
              else
                xv = ld_x_l2<CT>(x, out_f32, jc);
              acc -= cvt<CT>(val[e]) * xv;
            }
            if (!serial) {
              A[r] = -ap / d;
              B[r] = acc / d;
            } else {
              A[r] = d;
              B[r] = acc;
            }
          }
          if (!serial) {
            CT ca = (CT)1, cb = (CT)0;
#pragma unroll
            for (int r = 0; r < R; ++r) {
              cb = A[r] * cb + B[r];
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
              xin = A[r] * xin + B[r];
              X[r] = xin;
            }
          } else {
            for (int p = 0; p < cnt; ++p) {
              const int owner = p / R, rr = p % R;
              CT xp = (CT)0;
#pragma unroll
              for (int r = 0; r < R; ++r)
                if (lane == owner && r == rr) xp = B[r] / A[r];
              xp = __shfl_sync(0xffffffffu, xp, owner);
              const int rowp = LOWER ? base + p : base + cnt - 1 - p;
#pragma unroll
              for (int r = 0; r < R; ++r) {
                const int pos = lane * R + r;
                if (pos == p) X[r] = xp;
                if (pos > p && pos < cnt) {
                  const int i = rows[r];
                  for (int e = P.row[i]; e < P.row[i + 1]; ++e)
                    if (P.col[e] == rowp) B[r] -= cvt<CT>(val[e]) * xp;
                }
              }
            }
          }
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (rows[r] >= 0) {
              st_out<CT>(x, out_f32, rows[r], X[r]);
              const unsigned slot = (unsigned)(rows[r] - row0);
              if (slot < (unsigned)P.win) xs[slot] = X[r];
            }
        }
      }
      // level done: visible to the CTA now, to other CTAs after the release
      __syncthreads();
      if ((publisher_warp || nwarps == 1) && lane == 0)
        st_release_u64(&P.progress[bk], (ep << 32) | (unsigned)(lv - l0 + 1));
    }
  }
  // the CTA that leaves last re-arms the tickets and publishes the epoch
  if (threadIdx.x == 0) {
    const int nrhs = gridDim.y;
    const int e = atomicAdd(&tickets[nrhs], 1);
    if (e == (int)(gridDim.x * gridDim.y) - 1) {
      for (int r = 0; r <= nrhs; ++r) tickets[r] = 0;
      *epoch_slot = (int)ep;
      __threadfence();
    }
  }
}

struct BlkArgs {
  const void *b;
  int in_f32;
  void *x;
  int out_f32;
  size_t vstride;
  int nrhs;
  int *tickets, *epoch_slot, *status;
  const int *dfl;
};

template <typename CT, typename VT, int R>
static void blk_launch(cudaStream_t s, const BlkPlanDev &P, int warps, int grid, const BlkArgs &a) {
  dim3 g(grid, a.nrhs);
  const size_t sm = (size_t)P.win * sizeof(CT);
  if (P.lower) {
    auto fn = k_sptrsv_blk<CT, VT, R, true>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    fn<<<g, 32 * warps, sm, s>>>(P, a.b, a.in_f32, a.x, a.out_f32, a.vstride, a.tickets, a.epoch_slot, a.dfl,
                                 a.status);
  } else {
    auto fn = k_sptrsv_blk<CT, VT, R, false>;
    if (sm > 48 * 1024) cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    fn<<<g, 32 * warps, sm, s>>>(P, a.b, a.in_f32, a.x, a.out_f32, a.vstride, a.tickets, a.epoch_slot, a.dfl,
                                 a.status);
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

static BlkPlanDev plan_dev(const TriBlkPlan &pl, const void *val);

// several right-hand sides at once: b/x hold nrhs vectors vstride apart;
// tickets has nrhs+1 ints, progress nrhs*nblocks counters (both zeroed)
void launch_sptrsv_blk_multi(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                             int in_f32, void *x, int out_f32, size_t vstride, int nrhs, int *tickets,
                             unsigned long long *progress, int *epoch_slot, int *status, const int *done_flag) {
  BlkPlanDev P = plan_dev(pl, val);
  P.progress = progress;
  // rows of a block kept in shared memory: the whole block when it fits
  const size_t rows = (size_t)pl.cpb * 32 * pl.R;
  const size_t esz = vt == VType::F64 ? 8 : 4;
  P.win = rows * esz <= (size_t)kSptrsvSmemMax ? (int)rows : 0;
  int grid = pl.grid;
  if (grid > pl.nblocks) grid = pl.nblocks;
  if (grid < 1) grid = 1;
  BlkArgs a{b, in_f32, x, out_f32, vstride, nrhs, tickets, epoch_slot, status, done_flag};
  switch (vt) {
    case VType::F64: blk_launch_r<double, double>(s, pl.R, P, pl.warps, grid, a); break;
    case VType::F32: blk_launch_r<float, float>(s, pl.R, P, pl.warps, grid, a); break;
    case VType::BF16: blk_launch_r<float, __nv_bfloat16>(s, pl.R, P, pl.warps, grid, a); break;
  }
}

static BlkPlanDev plan_dev(const TriBlkPlan &pl, const void *val) {
  BlkPlanDev P;
  P.n = pl.n;
  P.nchunks = pl.nchunks;
  P.nblocks = pl.nblocks;
  P.row = pl.row;
  P.col = pl.col;
  P.val = val;
  P.unit = pl.unit;
  P.lower = pl.lower;
  P.blk_lvl_ptr = pl.blk_lvl_ptr;
  P.lvl_ptr = pl.lvl_ptr;
  P.units = pl.units;
  P.chunk_blk = pl.chunk_blk;
  P.req_ptr = pl.req_ptr;
  P.req_blk = pl.req_blk;
  P.req_lvl = pl.req_lvl;
  P.kind = pl.kind;
  P.progress = pl.progress;
  P.blk_row0 = pl.blk_row0;
  P.win = 0;
  return P;
}

void launch_sptrsv_blk(cudaStream_t s, const TriBlkPlan &pl, const void *val, VType vt, const void *b,
                       int in_f32, void *x, int out_f32, Control *ctrl, int slot, bool honor_done) {
  launch_sptrsv_blk_multi(s, pl, val, vt, b, in_f32, x, out_f32, 0, 1, ctrl->tickets[slot], pl.progress,
                          &ctrl->trsv_epoch[slot], &ctrl->status, honor_done ? &ctrl->done : nullptr);
}

}  // namespace lace
