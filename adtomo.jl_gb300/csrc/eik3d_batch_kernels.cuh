// eik3d_batch_kernels.cuh -- kernels of the batched misfit + gradient plan.
//
// A persistent grid of CTAs, each split into warp groups.  A group takes one
// solve at a time from a work counter (solves pre-sorted largest grid first)
// and runs that solve's whole forward (or adjoint) alone, so no group ever
// waits for another: the only synchronisation is a named barrier of the
// group's warps between brick levels.  Inside a solve the group's warps sweep
// the dirty bricks of one level concurrently (eik3d_brick.cuh); several
// groups per SM keep the SM busy while one solve's level has little work.
//
// Brick skipping (exact): a brick is swept in an ordering only if it, or one
// of its six face neighbours, changed since the brick was last swept.  A
// sweep of a brick whose cells and halo are unchanged since its last sweep
// reproduces the same values (the update reads only those), so skipping it
// leaves every result bit-identical to sweeping everything.
#pragma once
#include "eik3d_brick.cuh"

// Register budgets of the persistent sweep kernels: threads per CTA the
// compiler must fit, 65536 / (threads) registers per thread.  The forward
// tile needs 16 KB of shared memory per warp, so 12 warps (two solves of 6
// warps) fit an SM when a thread has at most 170 registers; the adjoint
// tiles (23 KB per warp) hold it to 9 warps, so it is left unconstrained.
#ifndef ADT_FWD_MAXT
#define ADT_FWD_MAXT 384
#endif
#define ADT_FWD_BOUNDS __launch_bounds__(ADT_FWD_MAXT, 1)

namespace adt {

template <class T>
struct FieldDev {
  Geom g;
  double h;
  const T* f;               // FP32: slowness; FP64: f h per cell
  const T* f2;              // FP64: f f h h per cell (f h and f f h h formed once
                            // per evaluation in the reference's order); FP32: unused
  const double* f64;        // slowness, FP64 (gradient)
  const double* vel0;       // fixed velocity model for the near-source values, FP64
  const uint32_t* bricks;   // level-ordered bricks
  const int* lstart;        // nlev + 1
  const double* sta;        // receivers, 3 per station
  int nsta;
  // floor(2^64 / d) + 1 for d = n * l and d = l: x / d = __umul64hi(x, .) for
  // every 32-bit x (division by an invariant integer by multiplication; the
  // error term x (d M - 2^64) / (d 2^64) stays below 1 / d when x < 2^32)
  unsigned long long div_nl, div_l;
};

struct SolveDev {
  int field;
  int gidx;                 // index in the caller's solve list
  int xc, xf, yc, yf, zc, zf;  // ceil / floor of the source coordinates
  double sx, sy, sz;
  double v0[8];             // initial values at the 8 nodes, FP64 (src init kernel)
  int64_t u_off;            // cell offset in the chunk buffers
  int64_t meta_off;         // brick offset in the chunk meta buffer
  int64_t obs_off;          // pick offset
  int64_t seed_off;         // seed slot offset (8 per station) in the chunk seed buffer
};

// Per-cell record of the causal-order adjoint (eik3d_adj_causal.cuh): the
// adjoint value and the cell's active upwind difference along each axis,
// u_c - min(neighbours) (0 when the axis is inactive).  A user r of cell c
// along axis a has c as its smaller neighbour there, so r's difference along
// a is exactly u_r - u_c: the records hold every weight of the adjoint rows.
template <class T>
struct alignas(4 * sizeof(T)) CausalRec {
  T lam, d[3];
};

template <class T>
struct BatchArgs {
  const FieldDev<T>* fields;
  SolveDev* solves;         // all solves (global index)
  const int* order;         // chunk solves to run, largest first (global indices)
  int n_solves;             // in this chunk
  T* u;                     // chunk travel times
  T* lam;                   // chunk adjoint variables
  uint16_t* code;           // chunk adjoint codes
  int* meta;                // chunk brick meta: mod[nb] then proc[nb] per solve
  int64_t* seed_idx;        // chunk seeds (sorted, merged)
  T* seed_val;
  T* gdense;                // chunk seed values as a dense field (0 off the seeds), or null
  int* n_seed;              // per chunk-local solve... indexed by global solve
  T* snap;                  // per-CTA snapshot (reference stopping rule), or null
  int64_t snap_stride;
  int* next;                // work counter
  adt_solve_status* status; // per global solve
  unsigned long long* counters;  // [0] fwd cell updates [1] fwd bricks [2] adj updates [3] adj bricks
  unsigned long long* cost;  // per solve: bricks swept in this evaluation (orders the next one)
  double tol;
  float wake;               // FP32 forward: decrease at or below which a brick wakes no one
  float adj_wake;           // FP32 adjoint: relative change at or below which it wakes no one
  int max_iter;
  int adj_max_iter;
  int ref_compat;
  int near_r;
  int group_warps;          // warps per group (one solve per group)
  int meta_smem;            // 1: brick meta of the running solve in shared memory
  int max_nb;               // bricks of the largest field (shared-memory meta size)
  int adj_order_filter;     // 1: adjoint sweeps a brick only in the orderings its flow allows
  int fwd_order_filter;     // 1: FP32 forward sweeps a brick only in the orderings its
                            //    learned upwind directions allow
  uint32_t* meta32;         // causal-order adjoint: code bits and outstanding users, blocked layout
  CausalRec<T>* rec;        // causal-order adjoint: lambda and upwind differences, blocked layout
  int* queue;               // causal-order adjoint: cells in evaluation order, one int per chunk cell
};

// Per-group scalars at the start of dynamic shared memory.
struct GroupShared {
  int q;
  int changed;
  unsigned long long err;
  int lo[2], hi[2];  // level range with pending bricks at the start of an ordering (run_ordering)
  int lchg[3];       // a brick of level d changed in this ordering: lchg[d % 3]
};

// Empty level ranges for both orderings' slots (run_ordering), at the start
// of a solve, before the barrier that precedes its sweeps.
__device__ __forceinline__ void group_reset_range(GroupShared* gs) {
  gs->lo[0] = gs->lo[1] = INT_MAX;
  gs->hi[0] = gs->hi[1] = -1;
}

__device__ __forceinline__ void group_sync(int grp, int nthreads) {
  asm volatile("bar.sync %0, %1;\n" ::"r"(grp + 1), "r"(nthreads) : "memory");
}

// Brick metadata of one solve: arrays of one int per brick.  Both sweeps keep
// mod and proc (timestamps of the last change and of the last sweep); the
// adjoint adds flow (the directions in which adjoint values enter the
// brick's cells, which orderings it is swept in) and the FP32 forward its
// learned upwind directions (fmask, run_ordering).  The global meta buffer
// holds META_ARRAYS_MAX arrays per solve.
constexpr int META_ARRAYS_FWD = 3;
constexpr int META_ARRAYS_ADJ = 3;
constexpr int META_ARRAYS_MAX = 3;

// Dynamic shared memory: [G GroupShared][G * narr * max_nb meta ints][warp tiles]
__host__ __device__ inline size_t group_hdr_bytes(int G, int meta_smem, int max_nb, int narr) {
  size_t b = ((size_t)G * sizeof(GroupShared) + 15) / 16 * 16;
  if (meta_smem) b += ((size_t)G * narr * max_nb * sizeof(int) + 15) / 16 * 16;
  return b;
}

// Initial value of the implicit u0 in the compute precision: 1000, or the
// FP64 near-source value at the 8 nodes around the source (k_src_init;
// scripts/gene_obs.jl:42-51, scripts/inversion.jl:52-60), converted.  Only
// those eight nodes convert; every other cell takes the constant.
template <class T>
__device__ __forceinline__ T u0_t(const SolveDev& s, int i, int j, int k) {
  const bool xi = (i == s.xc) || (i == s.xf);
  const bool yj = (j == s.yc) || (j == s.yf);
  const bool zk = (k == s.zc) || (k == s.zf);
  if (__builtin_expect(xi && yj && zk, 0)) {
    const int a = (i == s.xc) ? 0 : 1, b = (j == s.yc) ? 0 : 1, c = (k == s.zc) ? 0 : 1;
    return (T)s.v0[a * 4 + b * 2 + c];
  }
  return T(1000);
}

template <class T>
__device__ __forceinline__ unsigned long long to_ordered(T v);
template <>
__device__ __forceinline__ unsigned long long to_ordered<float>(float v) {
  return (unsigned long long)__float_as_uint(v);
}
template <>
__device__ __forceinline__ unsigned long long to_ordered<double>(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
template <class T>
__device__ __forceinline__ T from_ordered(unsigned long long b);
template <>
__device__ __forceinline__ float from_ordered<float>(unsigned long long b) {
  return __uint_as_float((unsigned)b);
}
template <>
__device__ __forceinline__ double from_ordered<double>(unsigned long long b) {
  return __longlong_as_double((long long)b);
}

// Does brick b = (bx, by, bz) need a sweep at time t of its level?  It does
// if it changed in its own last sweep, or a face neighbour changed after that.
//
// Every warp of the group evaluates this for the whole level while other
// warps may already be sweeping bricks of the same level, and all must get
// the same answer.  Face neighbours lie in the levels before and after, which
// do not change during the level.  The brick's own words are written only by
// the warp that sweeps it, and only after that warp found it dirty: it sets
// proc = t, then mod = t if something changed.  A reader sees either the old
// words (dirty, as the sweeper found), proc == t (dirty by the first test) or
// the old proc with mod == t (dirty by the second), so the answer is the same.
//
// feeds: which face neighbours can change the brick's values (bit 0: x-,
// 1: x+, 2: y-, 3: y+, 4: z-, 5: z+); 63 for the forward, where any
// neighbour may become a cell's upwind neighbour.  The adjoint passes its
// flow bits: a brick none of whose cells is used by a cell across a face
// reads that face's adjoint values only with zero weight, so a change there
// cannot change the brick.
__device__ __forceinline__ bool brick_dirty(const int* mod_, const int* proc_, const Geom& g,
                                            int b, int bx, int by, int bz, int t, int feeds = 63) {
  const volatile int* mod = mod_;
  const volatile int* proc = proc_;
  const int pr = proc[b];
  if (pr == t) return true;
  bool v = mod[b] >= pr;
  const int sx = g.nby * g.nbz;
  if ((feeds & 1) && bx > 0) v |= mod[b - sx] > pr;
  if ((feeds & 2) && bx < g.nbx - 1) v |= mod[b + sx] > pr;
  if ((feeds & 4) && by > 0) v |= mod[b - g.nbz] > pr;
  if ((feeds & 8) && by < g.nby - 1) v |= mod[b + g.nbz] > pr;
  if ((feeds & 16) && bz > 0) v |= mod[b - 1] > pr;
  if ((feeds & 32) && bz < g.nbz - 1) v |= mod[b + 1] > pr;
  return v;
}

// Orderings of the adjoint sweeps that follow a brick's flow.  The adjoint
// system is triangular: lambda flows from a cell to its upwind neighbour
// (from user r to c), so a sweep carries it within one pass only when it
// visits r before c.  flow holds the user bits of the brick's cells, OR-ed
// (bit 0: the x- neighbour uses a cell, so lambda flows along +x and needs an
// ordering with si = +1; bit 1: along -x, si = -1; bits 2-3 y, 4-5 z).  An
// ordering is kept when it agrees with every axis whose flow has one
// direction; an axis with both directions (or none) constrains nothing.
// Skipping the other orderings is exact: a skipped dirty brick stays dirty
// (its timestamps do not move) and is swept in an allowed ordering of the
// same or the next iteration, and the solve stops only after an iteration in
// which nothing changed, so at the end every cell satisfies its equation --
// and the triangular system has exactly one such solution.
__host__ __device__ __forceinline__ int adjoint_flow_forbidden(int si, int sj, int sk) {
  return (si > 0 ? 2 : 1) | (sj > 0 ? 8 : 4) | (sk > 0 ? 32 : 16);
}
__host__ __device__ __forceinline__ bool adjoint_flow_allowed(int flow, int forbid) {
  const int both = flow & (flow >> 1) & 0x15;
  return ((flow & ~(both | (both << 1))) & forbid) == 0;
}

// ------------------------------------------------------------------ forward
// Group layout helpers shared by the forward and adjoint kernels.
struct GroupCtx {
  int NW, GW, G, warp, lane, grp, gw, gthreads;
  GroupShared* gs;
  int* smeta;  // this group's meta (narr * max_nb ints) or null
  unsigned char* tiles;
};

template <class T>
__device__ __forceinline__ GroupCtx group_ctx(const BatchArgs<T>& A, unsigned char* smem,
                                              int narr) {
  GroupCtx c;
  c.NW = blockDim.x >> 5;
  c.GW = A.group_warps;
  c.G = c.NW / c.GW;
  c.warp = threadIdx.x >> 5;
  c.lane = threadIdx.x & 31;
  c.grp = c.warp / c.GW;
  c.gw = c.warp - c.grp * c.GW;
  c.gthreads = c.GW * 32;
  c.gs = reinterpret_cast<GroupShared*>(smem) + c.grp;
  const size_t g0 = ((size_t)c.G * sizeof(GroupShared) + 15) / 16 * 16;
  c.smeta = A.meta_smem
                ? reinterpret_cast<int*>(smem + g0) + (size_t)c.grp * narr * A.max_nb
                : nullptr;
  c.tiles = smem + group_hdr_bytes(c.G, A.meta_smem, A.max_nb, narr);
  return c;
}

// Take the next solve for this group (or -1 when the queue is empty).  The
// first solve of every group is assigned statically, so every SM gets a
// solve before any SM gets a second: group 0 of CTA b takes solve b, and the
// solves of each later round go to the CTAs whose earlier solves are the
// lightest (solves are ordered heaviest first), the heaviest of the round to
// the last CTA.  The heaviest solves then run alone on their SM and the
// lighter ones share, which shortens the longest SM.  Later solves come from
// the shared counter.
template <class T>
__device__ __forceinline__ int group_next(const BatchArgs<T>& A, const GroupCtx& c, bool& first) {
  int q;
  if (first) {
    first = false;
    const int C = (int)gridDim.x, b = (int)blockIdx.x;
    if (c.grp == 0) {
      q = b;
    } else {
      const int r0 = c.grp * C;                          // first solve of this round
      const int cnt = min(C, max(A.n_solves - r0, 0));   // solves in this round
      q = b >= C - cnt ? r0 + (C - 1 - b) : A.n_solves;  // none for the heavier CTAs
    }
  } else {
    if (c.gw == 0 && c.lane == 0) c.gs->q = atomicAdd(A.next, 1) + c.G * (int)gridDim.x;
    group_sync(c.grp, c.gthreads);
    q = c.gs->q;
    group_sync(c.grp, c.gthreads);
  }
  return q < A.n_solves ? q : -1;
}

// One ordering of one solve, level by level (bricks of level bx+by+bz in
// the ordering's own coordinates are independent; a level's sweeps read the
// previous level's new values and the next level's old ones -- the
// Gauss-Seidel data flow of the reference's loop).  For each level every
// warp of the group forms the level's dirty-brick mask itself (one lane per
// brick, 32 bricks at a time, brick_dirty) and sweeps the dirty bricks of
// rank gw, gw + GW, ...: equal shares however the dirty bricks are spread,
// without a barrier before the level; one named barrier after it.
//
// body(p, fbits) sweeps one dirty brick and returns whether it changed; this
// function keeps the brick's timestamps (t = ts0 + level) and counters.
//
// flow (adjoint only, else null): per brick, the directions in which adjoint
// values enter its cells (user bits of adjoint_flow_allowed); a dirty brick
// is swept only in the orderings that follow them, and only changes of the
// face neighbours that feed it make it dirty (brick_dirty).  flow is written
// before the sweeps and not during them, so every warp still reads the same
// mask.
//
// fmask (FP32 forward only, else null): per brick, the upwind directions its
// changing sweeps have seen, learned during the solve (FWD_FLOW_KNOWN set
// once one has), with the level time of the last write (modulo 2^24) in the
// bits above 8.  A dirty brick with a known mask is swept only in the
// orderings that follow it.  The sweeper writes the entry while other warps
// may still be testing the brick in the same level; an entry written at the
// current level time reads as allowed, which is what the sweeper found before
// it swept, so all warps still agree.  (An entry 2^24 level steps old also
// reads as allowed: a spare sweep, never a missed one.)  body(p, fbits) returns the sweep's upwind bits
// (absolute, as the adjoint's flow bits) in fbits.
constexpr int FWD_FLOW_KNOWN = 0x80;

template <int BK, class Body>
__device__ __forceinline__ void run_ordering(const GroupCtx& c, const Geom& g, const uint32_t* bricks,
                                             const int* lstart, int* mod, int* proc,
                                             const int* flow, int* fmask, int ts0, int si, int sj,
                                             int sk, unsigned long long& cnt_upd,
                                             unsigned long long& cnt_brk, Body&& body) {
  const int lane = c.lane;
  const int forbid = (flow || fmask) ? adjoint_flow_forbidden(si, sj, sk) : 0;
  // does brick b need a sweep at level time t (dirty, and allowed by the filters)?
  auto pending = [&](int b, int bx, int by, int bz, int t) -> bool {
    if (flow) {
      const int fl = ((const volatile int*)flow)[b];
      return adjoint_flow_allowed(fl, forbid) && brick_dirty(mod, proc, g, b, bx, by, bz, t, fl);
    }
    if (fmask) {
      const int e = ((const volatile int*)fmask)[b];
      return brick_dirty(mod, proc, g, b, bx, by, bz, t) &&
             (!(e & FWD_FLOW_KNOWN) || ((unsigned)e >> 8) == ((unsigned)t & 0xFFFFFFu) ||
              adjoint_flow_allowed(e & 63, forbid));
    }
    return brick_dirty(mod, proc, g, b, bx, by, bz, t);
  };
  // Level range.  Before any sweep of this ordering, a brick needs one only if
  // it is pending now; during the ordering a brick can become pending only
  // when a face neighbour of the previous level changes (the next level's
  // neighbours have not been swept yet).  So the ordering starts at the
  // lowest pending level and stops after the highest one as soon as a level
  // changes nothing.  Every warp scans a share of the bricks; the range and
  // the per-level change flags live in the group's shared scalars, read only
  // after the barriers that close their writes (lchg[d % 3] is reset during
  // level d - 1, written during level d, read after its barrier).
  const int par = (ts0 / g.nlev) & 1;
  if (c.gw == 0 && lane == 0) {
    c.gs->lchg[0] = c.gs->lchg[1] = c.gs->lchg[2] = 0;
  }
  {
    int lo = INT_MAX, hi = -1;
    const int nb = g.nbx * g.nby * g.nbz;
    for (int b = c.gw * 32 + lane; b < nb; b += c.gthreads) {
      const int bx = b / (g.nby * g.nbz), by = (b / g.nbz) % g.nby, bz = b % g.nbz;
      if (pending(b, bx, by, bz, INT_MIN)) {
        const int lv = (si > 0 ? bx : g.nbx - 1 - bx) + (sj > 0 ? by : g.nby - 1 - by) +
                       (sk > 0 ? bz : g.nbz - 1 - bz);
        lo = min(lo, lv);
        hi = max(hi, lv);
      }
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lane == 0 && hi >= 0) {
      atomicMin(&c.gs->lo[par], lo);
      atomicMax(&c.gs->hi[par], hi);
    }
  }
  group_sync(c.grp, c.gthreads);
  const int dlo = c.gs->lo[par], dhi = c.gs->hi[par];
  if (c.gw == 0 && lane == 0) {  // the next ordering's range (nobody reads it any more)
    c.gs->lo[par ^ 1] = INT_MAX;
    c.gs->hi[par ^ 1] = -1;
  }
  for (int d = dlo; d < g.nlev; ++d) {
    if (d > dhi && !c.gs->lchg[(d - 1) % 3]) break;
    if (c.gw == 0 && lane == 0) c.gs->lchg[(d + 1) % 3] = 0;
    const int t = ts0 + d;
    const int q0 = lstart[d], q1 = lstart[d + 1];
    int slot = 0;
    for (int c0 = q0; c0 < q1; c0 += 32) {
      const int qq = c0 + lane;
      uint32_t packed = 0;
      bool dv = false;
      if (qq < q1) {
        packed = bricks[qq];
        int rx, ry, rz;
        unpack_brick(packed, rx, ry, rz);
        const int bx = si > 0 ? rx : g.nbx - 1 - rx;
        const int by = sj > 0 ? ry : g.nby - 1 - ry;
        const int bz = sk > 0 ? rz : g.nbz - 1 - rz;
        dv = pending((bx * g.nby + by) * g.nbz + bz, bx, by, bz, t);
      }
      unsigned m = __ballot_sync(0xffffffffu, dv);
      while (m) {
        const int bit = __ffs(m) - 1;
        m &= m - 1;
        const uint32_t pk = __shfl_sync(0xffffffffu, packed, bit);
        if (slot == c.gw) {
          const BrickPos p = brick_pos<BK>(g, pk, si, sj, sk);
          uint32_t fbits = 0;
          const bool ch = body(p, fbits);
          __syncwarp();
          if (lane == 0) {
            const int b = (p.bx * g.nby + p.by) * g.nbz + p.bz;
            proc[b] = t;
            if (ch) {
              mod[b] = t;
              c.gs->lchg[d % 3] = 1;
            }
            if (fmask && fbits) {
              const int old = fmask[b];
              fmask[b] = (int)((((unsigned)t & 0xFFFFFFu) << 8) | FWD_FLOW_KNOWN |
                               ((old & FWD_FLOW_KNOWN) ? (old & 63) : 0) | fbits);
            }
            cnt_upd += (unsigned long long)p.ni * p.nj * p.nk;
            cnt_brk += 1;
          }
        }
        if (++slot == c.GW) slot = 0;
      }
    }
    group_sync(c.grp, c.gthreads);
  }
}

// Select the sweep instantiation for the ordering's directions and the
// near-source flag.
template <int BK, int SI, int SJ, int SKD, bool FLOW>
__device__ __forceinline__ bool fwd_f32_dir(float* S, const float* F, const BrickPos& p, bool nr,
                                            float h, double hd, const NearBox& box, int lane,
                                            float& md, uint32_t& fbits) {
  return nr ? sweep_brick_fwd_f32<BK, SI, SJ, SKD, true, FLOW>(S, F, p, h, hd, box, lane, md,
                                                               fbits)
            : sweep_brick_fwd_f32<BK, SI, SJ, SKD, false, FLOW>(S, F, p, h, hd, box, lane, md,
                                                                fbits);
}

template <int BK, bool FLOW>
__device__ __forceinline__ bool dispatch_fwd_f32(float* S, const float* F, const BrickPos& p,
                                                 int si, int sj, int sk, bool nr, float h,
                                                 double hd, const NearBox& box, int lane,
                                                 float& md, uint32_t& fb) {
  switch ((si < 0) | ((sj < 0) << 1) | ((sk < 0) << 2)) {
    case 0: return fwd_f32_dir<BK, 1, 1, 1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    case 1: return fwd_f32_dir<BK, -1, 1, 1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    case 2: return fwd_f32_dir<BK, 1, -1, 1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    case 3: return fwd_f32_dir<BK, -1, -1, 1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    case 4: return fwd_f32_dir<BK, 1, 1, -1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    case 5: return fwd_f32_dir<BK, -1, 1, -1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    case 6: return fwd_f32_dir<BK, 1, -1, -1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
    default: return fwd_f32_dir<BK, -1, -1, -1, FLOW>(S, F, p, nr, h, hd, box, lane, md, fb);
  }
}

template <class T, int BK, int MODE>
__global__ void ADT_FWD_BOUNDS k_batch_fwd(BatchArgs<T> A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GroupCtx c = group_ctx(A, smem, META_ARRAYS_FWD);
  if (c.grp >= c.G) return;
  const int lane = c.lane;
  // per warp: the travel-time tile, then one interior tile (f), or two with
  // MODE_EXACT_CST (f h, f f h h); fwd_warp_smem sizes the same layout
  constexpr int NI = MODE == MODE_EXACT_CST ? 2 : 1;
  T* S = reinterpret_cast<T*>(c.tiles) + c.warp * (tile_elems(BK) + NI * itile_elems(BK));
  T* F = S + tile_elems(BK);
  unsigned long long cnt_upd = 0, cnt_brk = 0;
  bool first = true;
  for (;;) {
    const int q = group_next(A, c, first);
    if (q < 0) break;
    const int gsol = A.order[q];
    const SolveDev& sd = A.solves[gsol];
    const FieldDev<T> fd = A.fields[sd.field];
    const Geom g = fd.g;
    const T h = (T)fd.h;
    const unsigned long long brk0 = cnt_brk;
    T* u = A.u + sd.u_off;
    const int nb = g.nbx * g.nby * g.nbz;
    int* mod = c.smeta ? c.smeta : A.meta + sd.meta_off;
    int* proc = mod + (c.smeta ? A.max_nb : nb);
    int* fmask = (MODE == MODE_STABLE && A.fwd_order_filter) ? proc + (c.smeta ? A.max_nb : nb)
                                                               : nullptr;
    // u = u0 (column-wise: lanes along k)
    for (int64_t col = c.gw; col < (int64_t)g.m * g.n; col += c.GW) {
      const int i = (int)(col / g.n), j = (int)(col % g.n);
      T* uc = u + col * g.l;
      for (int k = lane; k < g.l; k += 32) uc[k] = u0_t<T>(sd, i, j, k);
    }
    // Only the bricks whose cells or halo hold a source node start dirty.
    // Every other cell starts at 1000 with all its neighbours at 1000, and
    // with f h > 0 no candidate falls below 1000, so such a brick cannot
    // change until a neighbour does: skipping it is exact, like every other
    // skip.  (The halo counts: a brick next to a source node changes in its
    // first sweep even while the source's own brick has not been swept.)
    auto near = [](int x0, int x1, int b, int B) {
      return (x0 >= b * B - 1 && x0 <= b * B + B) || (x1 >= b * B - 1 && x1 <= b * B + B);
    };
    for (int b = c.gw * 32 + lane; b < nb; b += c.gthreads) {
      const int bx = b / (g.nby * g.nbz), by = (b / g.nbz) % g.nby, bz = b % g.nbz;
      const bool src = near(sd.xf, sd.xc, bx, BI) && near(sd.yf, sd.yc, by, BJ) &&
                       near(sd.zf, sd.zc, bz, BK);
      mod[b] = src ? -1 : -2;
      proc[b] = -1;
      if (fmask) fmask[b] = 0;
    }
    if (c.gw == 0 && lane == 0) group_reset_range(c.gs);
    NearBox box;
    box.i0 = max(0, sd.xf - A.near_r);
    box.i1 = min(g.m - 1, sd.xc + A.near_r);
    box.j0 = max(0, sd.yf - A.near_r);
    box.j1 = min(g.n - 1, sd.yc + A.near_r);
    box.k0 = max(0, sd.zf - A.near_r);
    box.k1 = min(g.l - 1, sd.zc + A.near_r);
    const bool use_near = (A.near_r >= 0) && (MODE == MODE_STABLE);
    const bool vec = (g.l % 4) == 0;
    T* snap = A.snap ? A.snap + (int64_t)(blockIdx.x * c.G + c.grp) * A.snap_stride : nullptr;
    group_sync(c.grp, c.gthreads);
    int it;
    bool conv = false;
    T err = T(0);
    for (it = 0; it < A.max_iter; ++it) {
      if (c.gw == 0 && lane == 0) c.gs->err = 0ull;
      if (snap)
        for (int64_t x = c.gw * 32 + lane; x < g.ncell; x += c.gthreads) snap[x] = u[x];
      group_sync(c.grp, c.gthreads);
      T md = T(0);
      for (int o = 0; o < 8; ++o) {
        int si, sj, sk;
        ordering3(o, si, sj, sk);
        const int CS = tile_col_stride(BK, sj == sk);
        run_ordering<BK>(c, g, fd.bricks, fd.lstart, mod, proc, nullptr, fmask,
                         (it * 8 + o) * g.nlev, si, sj, sk, cnt_upd, cnt_brk,
                         [&](const BrickPos& p, uint32_t& fbits) -> bool {
          bool ch;
          if constexpr (MODE == MODE_STABLE && sizeof(T) == 4) {
            if (vec) {
              load_tile_f32_async<BK>(S, u, g, p, CS, lane);
              load_interior_f32_async<BK>(F, fd.f, g, p, CS, lane);
              cp_async_wait_all();
              __syncwarp();
              const bool nr = use_near && box.hits(p);
              float mbb = 0.0f;  // this brick's largest decrease (per lane)
              ch = fmask ? dispatch_fwd_f32<BK, true>(S, F, p, si, sj, sk, nr, (float)h, fd.h, box,
                                                      lane, mbb, fbits)
                         : dispatch_fwd_f32<BK, false>(S, F, p, si, sj, sk, nr, (float)h, fd.h,
                                                       box, lane, mbb, fbits);
              md = fmaxf(md, mbb);
              if (ch) store_interior_f32_vec<BK>(S, u, g, p, CS, lane);
              // the brick's own cells keep every decrease; only a brick that moved by
              // more than `wake` marks itself and its neighbours for the next sweeps
              if (ch && A.wake > 0.0f) ch = __any_sync(0xffffffffu, mbb > A.wake);
            } else {
              load_halo_tile<T, BK>(S, u, g, p, CS, lane);
              load_interior<T, BK>(F, fd.f, g, p, CS, lane);
              cp_async_wait_all();
              __syncwarp();
              ch = sweep_brick_fwd<T, BK, MODE>(S, F, g, p, si, sj, sk, CS, h, fd.h, box,
                                                use_near && box.hits(p), lane, md);
              if (ch) store_interior<T, BK>(S, u, g, p, CS, lane);
            }
          } else {
            load_halo_tile<T, BK>(S, u, g, p, CS, lane);
            load_interior<T, BK>(F, fd.f, g, p, CS, lane);
            if constexpr (MODE == MODE_EXACT_CST)
              load_interior<T, BK>(F + itile_elems(BK), fd.f2, g, p, CS, lane);
            cp_async_wait_all();
            __syncwarp();
            ch = sweep_brick_fwd<T, BK, MODE>(S, F, g, p, si, sj, sk, CS, h, fd.h, box,
                                              use_near && box.hits(p), lane, md);
            if (ch) store_interior<T, BK>(S, u, g, p, CS, lane);
          }
          return ch;
        });
      }
      if (snap) {
        T mx = T(0);
        for (int64_t x = c.gw * 32 + lane; x < g.ncell; x += c.gthreads) {
          const T dd = u[x] > snap[x] ? u[x] - snap[x] : snap[x] - u[x];
          mx = rmax(dd, mx);
        }
        md = mx;
      }
      md = warp_max(md);
      if (lane == 0) atomicMax(&c.gs->err, to_ordered<T>(md));
      group_sync(c.grp, c.gthreads);
      err = from_ordered<T>(c.gs->err);
      group_sync(c.grp, c.gthreads);
      if ((double)err < A.tol) {
        conv = true;
        break;
      }
    }
    if (lane == 0 && cnt_brk > brk0) atomicAdd(&A.cost[sd.gidx], cnt_brk - brk0);
    if (c.gw == 0 && lane == 0) {
      adt_solve_status& st = A.status[sd.gidx];
      st.iters = conv ? it + 1 : it;
      st.converged = conv ? 1 : 0;
      st.final_err = (double)err;
    }
  }
  if (lane == 0 && cnt_brk) {
    atomicAdd(&A.counters[0], cnt_upd);
    atomicAdd(&A.counters[1], cnt_brk);
  }
}

// ---------------------------------------------------------- misfit, seeds
// One CTA per solve of the chunk.  Samples u at the receivers with the
// branch structure of scripts/inversion.jl:64-95, forms the weighted misfit
// (missing picks t_obs == -1 skipped, :81) and the sensitivities dL/du at
// the (up to 8) nodes of each receiver; equal nodes are merged in
// (receiver, node) order so the seed values are independent of scheduling.
//
// The merge arrays live in shared memory, or, for receiver counts too large
// for it (scratch != null), in a per-CTA slice of global scratch of
// `scratch_stride` bytes; the bitonic sort is the same either way.
static_assert(8LL * ADT_BATCH_MAX_RECEIVERS <= (1LL << 20), "merge key entry field");

template <class T>
__global__ void k_batch_misfit(BatchArgs<T> A, const double* __restrict__ t_obs,
                               const double* __restrict__ weight, double* __restrict__ t_pred,
                               double* __restrict__ solve_misfit, unsigned char* scratch,
                               int64_t scratch_stride) {
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  unsigned char* smem = scratch ? scratch + (int64_t)blockIdx.x * scratch_stride : smem_dyn;
  const int gs = A.order[blockIdx.x];
  const SolveDev sd = A.solves[gs];
  const FieldDev<T> fd = A.fields[sd.field];
  const Geom g = fd.g;
  const T* u = A.u + sd.u_off;
  const int S = fd.nsta;
  int E = 8 * S;
  int P = 1;
  while (P < E) P <<= 1;
  long long* key = reinterpret_cast<long long*>(smem);
  double* val = reinterpret_cast<double*>(key + P);
  double* mis = val + P;
  for (int q = threadIdx.x; q < S; q += blockDim.x) {
    const double x = fd.sta[3 * q], y = fd.sta[3 * q + 1], z = fd.sta[3 * q + 2];
    const int x1 = (int)floor(x), x2 = (int)ceil(x);
    const int y1 = (int)floor(y), y2 = (int)ceil(y);
    const int z1 = (int)floor(z), z2 = (int)ceil(z);
    auto U = [&](int i, int j, int k) -> double {
      return (double)u[((int64_t)i * g.n + j) * g.l + k];
    };
    double t11, t12, t21, t22, wx1, wx2, wy1, wy2, wz1, wz2;
    if (x1 == x2) {
      t11 = U(x1, y1, z1); t12 = U(x1, y1, z2); t21 = U(x1, y2, z1); t22 = U(x1, y2, z2);
      wx1 = 1.0; wx2 = 0.0;
    } else {
      wx1 = x2 - x; wx2 = x - x1;
      t11 = __dadd_rn(__dmul_rn(wx1, U(x1, y1, z1)), __dmul_rn(wx2, U(x2, y1, z1)));
      t12 = __dadd_rn(__dmul_rn(wx1, U(x1, y1, z2)), __dmul_rn(wx2, U(x2, y1, z2)));
      t21 = __dadd_rn(__dmul_rn(wx1, U(x1, y2, z1)), __dmul_rn(wx2, U(x2, y2, z1)));
      t22 = __dadd_rn(__dmul_rn(wx1, U(x1, y2, z2)), __dmul_rn(wx2, U(x2, y2, z2)));
    }
    double t1, t2;
    if (y1 == y2) {
      t1 = t11; t2 = t12; wy1 = 1.0; wy2 = 0.0;
    } else {
      wy1 = y2 - y; wy2 = y - y1;
      t1 = __dadd_rn(__dmul_rn(wy1, t11), __dmul_rn(wy2, t21));
      t2 = __dadd_rn(__dmul_rn(wy1, t12), __dmul_rn(wy2, t22));
    }
    double t;
    if (z1 == z2) {
      t = t1; wz1 = 1.0; wz2 = 0.0;
    } else {
      wz1 = z2 - z; wz2 = z - z1;
      t = __dadd_rn(__dmul_rn(wz1, t1), __dmul_rn(wz2, t2));
    }
    const int64_t o = sd.obs_off + q;
    t_pred[o] = t;
    const double to = t_obs[o], w = weight[o];
    double dt = 0.0, mq = 0.0;
    if (to != -1.0) {
      const double r = __dsub_rn(to, t);
      mq = __dmul_rn(__dmul_rn(w, r), r);
      dt = __dmul_rn(__dmul_rn(-2.0, w), r);
    }
    mis[q] = mq;
    const int xi[2] = {x1, x2}, yi[2] = {y1, y2}, zi[2] = {z1, z2};
    const double xw[2] = {wx1, wx2}, yw[2] = {wy1, wy2}, zw[2] = {wz1, wz2};
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
          const int e = q * 8 + a * 4 + b * 2 + c;
          const double wt = __dmul_rn(__dmul_rn(xw[a], yw[b]), zw[c]);
          const double v = __dmul_rn(dt, wt);
          const long long cell = ((long long)xi[a] * g.n + yi[b]) * g.l + zi[c];
          // zero contributions leave the accumulated value unchanged: drop them
          // (cell, entry) in one key: entry < 8 * ADT_BATCH_MAX_RECEIVERS = 2^19
          key[e] = (v == 0.0) ? LLONG_MAX : (cell << 20) | e;
          val[e] = v;
        }
  }
  for (int e = E + threadIdx.x; e < P; e += blockDim.x) key[e] = LLONG_MAX;
  __syncthreads();
  // bitonic sort of (key, val) ascending; keys are unique except LLONG_MAX
  for (int k = 2; k <= P; k <<= 1)
    for (int jj = k >> 1; jj > 0; jj >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int ixj = i ^ jj;
        if (ixj > i) {
          const bool up = ((i & k) == 0);
          const long long ki = key[i], kj = key[ixj];
          if ((ki > kj) == up) {
            key[i] = kj;
            key[ixj] = ki;
            const double tv = val[i];
            val[i] = val[ixj];
            val[ixj] = tv;
          }
        }
      }
      __syncthreads();
    }
  if (threadIdx.x == 0) {
    double m = 0.0;
    for (int q = 0; q < S; ++q) m = __dadd_rn(m, mis[q]);
    solve_misfit[sd.gidx] = m;
    int ns = 0;
    long long cur = -1;
    double acc = 0.0;
    int64_t* sidx = A.seed_idx + sd.seed_off;
    T* sval = A.seed_val + sd.seed_off;
    for (int e = 0; e < P; ++e) {
      const long long kk = key[e];
      if (kk == LLONG_MAX) break;
      const long long cell = kk >> 20;
      if (cell != cur) {
        if (cur >= 0) {
          sidx[ns] = cur;
          sval[ns] = (T)acc;
          if (A.gdense) A.gdense[sd.u_off + cur] = (T)acc;
          ++ns;
        }
        cur = cell;
        acc = 0.0;
      }
      acc = __dadd_rn(acc, val[e]);
    }
    if (cur >= 0) {
      sidx[ns] = cur;
      sval[ns] = (T)acc;
      if (A.gdense) A.gdense[sd.u_off + cur] = (T)acc;
      ++ns;
    }
    A.n_seed[sd.gidx] = ns;
  }
}

// ------------------------------------------------------------------ adjoint
template <class T>
__device__ __forceinline__ int upwind_side_t(const T* u, int64_t c, int pos, int ext, int64_t st,
                                             T uc) {
  int side;
  T a;
  if (pos == 0) {
    side = 2;
    a = u[c + st];
  } else if (pos == ext - 1) {
    side = 1;
    a = u[c - st];
  } else {
    const T up = u[c + st], um = u[c - st];
    if (up > um) {
      side = 1;
      a = um;
    } else {
      side = 2;
      a = up;
    }
  }
  return (uc > a) ? side : 0;
}

// Codes of four consecutive cells of one column (FP32, l % 4 == 0), from
// 16-byte loads: the same rule as upwind_side_t and the fixed-cell test,
// with out-of-grid neighbours read as +inf (so the edge cases fall out of the
// comparisons).  Writes the four codes (one 8-byte store) and lambda = 0.
// Split into the loads (p1_load; u is read-only in the adjoint kernel, so
// through the read-only path) and the rest (p1_store), so that a caller can
// issue the loads of several groups of cells before it waits for any.
struct P1Loads {
  float4 c4, xm, xp, ym, yp;
  float zm, zp;
};

__device__ __forceinline__ P1Loads p1_load(const float* __restrict__ u, const Geom& g, int64_t x,
                                           int i, int j, int k) {
  const float INF = __int_as_float(0x7f800000);
  const float4 INF4 = make_float4(INF, INF, INF, INF);
  const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
  P1Loads r;
  r.c4 = __ldg(reinterpret_cast<const float4*>(u + x));
  r.xm = i > 0 ? __ldg(reinterpret_cast<const float4*>(u + x - sI)) : INF4;
  r.xp = i < g.m - 1 ? __ldg(reinterpret_cast<const float4*>(u + x + sI)) : INF4;
  r.ym = j > 0 ? __ldg(reinterpret_cast<const float4*>(u + x - sJ)) : INF4;
  r.yp = j < g.n - 1 ? __ldg(reinterpret_cast<const float4*>(u + x + sJ)) : INF4;
  r.zm = k > 0 ? __ldg(u + x - 1) : INF;
  r.zp = k + 4 < g.l ? __ldg(u + x + 4) : INF;
  return r;
}

__device__ __forceinline__ void p1_store(const P1Loads& r, uint16_t* code, float* lam,
                                         const SolveDev& sd, int64_t x, int i, int j, int k) {
  const float uc[4] = {r.c4.x, r.c4.y, r.c4.z, r.c4.w};
  const float vxm[4] = {r.xm.x, r.xm.y, r.xm.z, r.xm.w}, vxp[4] = {r.xp.x, r.xp.y, r.xp.z, r.xp.w};
  const float vym[4] = {r.ym.x, r.ym.y, r.ym.z, r.ym.w}, vyp[4] = {r.yp.x, r.yp.y, r.yp.z, r.yp.w};
  uint32_t packed[2] = {0u, 0u};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const float um[3] = {vxm[q], vym[q], q == 0 ? r.zm : uc[q - 1]};
    const float up[3] = {vxp[q], vyp[q], q == 3 ? r.zp : uc[q + 1]};
    uint32_t cd = 0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {  // upwind side: the smaller neighbour, ties to +1
      const bool minus = up[ax] > um[ax];
      const float a = minus ? um[ax] : up[ax];
      cd |= (uc[q] > a ? (minus ? 1u : 2u) : 0u) << (2 * ax);
    }
    if (uc[q] == u0_t<float>(sd, i, j, k + q) || cd == 0) cd = CODE_FIXED;
    packed[q >> 1] |= cd << (16 * (q & 1));
  }
  *reinterpret_cast<uint2*>(code + x) = make_uint2(packed[0], packed[1]);
  *reinterpret_cast<float4*>(lam + x) = make_float4(0.f, 0.f, 0.f, 0.f);
}

// User bits of four consecutive cells (pass 2) from 8-byte loads of the
// codes: neighbour r uses c when r is not fixed and its upwind side along
// the axis points at c.  p2_load / p2_store split as in pass 1; the codes are
// read through the ordinary path (pass 2 rewrites their user bits, never the
// bits read here).  p2_store returns one byte per cell (cell q in bits
// 8q..8q+7): its user bits, or REM_FIXED for a fixed cell (the outstanding-
// user bytes of the causal-order adjoint, and the flow bits of the sweeps).
struct P2Loads {
  uint2 c4, xm, xp, ym, yp;
  uint32_t zm, zp;
};

__device__ __forceinline__ P2Loads p2_load(const uint16_t* code, const Geom& g, int64_t x, int i,
                                           int j, int k) {
  const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
  auto ld4 = [&](int64_t y) -> uint2 { return *reinterpret_cast<const uint2*>(code + y); };
  const uint2 fixed4 = make_uint2(CODE_FIXED | (CODE_FIXED << 16), CODE_FIXED | (CODE_FIXED << 16));
  P2Loads r;
  r.c4 = ld4(x);
  r.xm = i > 0 ? ld4(x - sI) : fixed4;
  r.xp = i < g.m - 1 ? ld4(x + sI) : fixed4;
  r.ym = j > 0 ? ld4(x - sJ) : fixed4;
  r.yp = j < g.n - 1 ? ld4(x + sJ) : fixed4;
  r.zm = k > 0 ? (uint32_t)code[x - 1] : CODE_FIXED;
  r.zp = k + 4 < g.l ? (uint32_t)code[x + 4] : CODE_FIXED;
  return r;
}

__device__ __forceinline__ uint32_t p2_store(const P2Loads& r, uint16_t* code, int64_t x) {
  auto c16 = [](uint2 v, int q) -> uint32_t {
    return ((q < 2 ? v.x : v.y) >> (16 * (q & 1))) & 0xffffu;
  };
  auto uses = [](uint32_t cr, int ax, uint32_t want) -> bool {
    return !(cr & CODE_FIXED) && ((cr >> (2 * ax)) & 3u) == want;
  };
  uint32_t packed[2] = {0u, 0u};
  uint32_t bytes = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    uint32_t cd = c16(r.c4, q);
    if (cd & CODE_FIXED) {
      bytes |= (uint32_t)REM_FIXED << (8 * q);
    } else {
      uint32_t us = 0;
      if (uses(c16(r.xm, q), 0, 2u)) us |= 1u;
      if (uses(c16(r.xp, q), 0, 1u)) us |= 2u;
      if (uses(c16(r.ym, q), 1, 2u)) us |= 4u;
      if (uses(c16(r.yp, q), 1, 1u)) us |= 8u;
      if (uses(q == 0 ? r.zm : c16(r.c4, q - 1), 2, 2u)) us |= 16u;
      if (uses(q == 3 ? r.zp : c16(r.c4, q + 1), 2, 1u)) us |= 32u;
      cd |= us << CODE_USERS;
      bytes |= us << (8 * q);
    }
    packed[q >> 1] |= cd << (16 * (q & 1));
  }
  *reinterpret_cast<uint2*>(code + x) = make_uint2(packed[0], packed[1]);
  return bytes;
}

// OR of the user bits in a word of four p2_store bytes.
__device__ __forceinline__ uint32_t users_of4(uint32_t bytes) {
  return (bytes | (bytes >> 8) | (bytes >> 16) | (bytes >> 24)) & 0x3fu;
}

template <int BK>
__device__ __forceinline__ bool dispatch_adj_f32(const float* U, float* L, const uint16_t* C,
                                                 const float* gcell, const Geom& g,
                                                 const BrickPos& p, int si, int sj, int sk,
                                                 int lane, float eps, bool seeds, bool& sig) {
#define ADT_ADJ_CASE(SI, SJ, SK)                                                              \
  return seeds ? sweep_brick_adj_f32<BK, SI, SJ, SK, true>(U, L, C, gcell, g, p, lane, eps, sig) \
               : sweep_brick_adj_f32<BK, SI, SJ, SK, false>(U, L, C, gcell, g, p, lane, eps, sig)
  switch ((si < 0) | ((sj < 0) << 1) | ((sk < 0) << 2)) {
    case 0: ADT_ADJ_CASE(1, 1, 1);
    case 1: ADT_ADJ_CASE(-1, 1, 1);
    case 2: ADT_ADJ_CASE(1, -1, 1);
    case 3: ADT_ADJ_CASE(-1, -1, 1);
    case 4: ADT_ADJ_CASE(1, 1, -1);
    case 5: ADT_ADJ_CASE(-1, 1, -1);
    case 6: ADT_ADJ_CASE(1, -1, -1);
    default: ADT_ADJ_CASE(-1, -1, -1);
  }
#undef ADT_ADJ_CASE
}

template <class T, int BK>
__global__ void k_batch_adj(BatchArgs<T> A) {
  extern __shared__ __align__(16) unsigned char smem[];
  const GroupCtx c = group_ctx(A, smem, META_ARRAYS_ADJ);
  if (c.grp >= c.G) return;
  const int lane = c.lane;
  constexpr size_t WS = (2 * tile_elems(BK)) * sizeof(T) + itile_elems(BK) * sizeof(uint16_t);
  T* U = reinterpret_cast<T*>(c.tiles + c.warp * WS);
  T* L = U + tile_elems(BK);
  uint16_t* C = reinterpret_cast<uint16_t*>(L + tile_elems(BK));
  unsigned long long cnt_upd = 0, cnt_brk = 0;
  constexpr bool EXACT = sizeof(T) == 8;
  bool first = true;
  for (;;) {
    const int q = group_next(A, c, first);
    if (q < 0) break;
    const int gsol = A.order[q];
    const SolveDev& sd = A.solves[gsol];
    const unsigned long long brk0 = cnt_brk;
    const FieldDev<T> fd = A.fields[sd.field];
    const Geom g = fd.g;
    const T* u = A.u + sd.u_off;
    T* lam = A.lam + sd.u_off;
    uint16_t* code = A.code + sd.u_off;
    const int nb = g.nbx * g.nby * g.nbz;
    int* mod = c.smeta ? c.smeta : A.meta + sd.meta_off;
    int* proc = mod + (c.smeta ? A.max_nb : nb);
    int* flow = proc + (c.smeta ? A.max_nb : nb);
    const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
    const bool vec = (g.l % 8) == 0;
    // pass 1: upwind sides and fixed cells; lambda = 0
    const bool vec4 = sizeof(T) == 4 && (g.l % 4) == 0;
    if constexpr (sizeof(T) == 4) {
      // two groups of four cells per step, all their loads issued first
      if (vec4)
        for (int64_t e = c.gw * 32 + lane; e < g.ncell / 4; e += 2 * c.gthreads) {
          const int64_t e2 = e + c.gthreads;
          const bool two = e2 < g.ncell / 4;
          const int64_t col = e / (g.l / 4), col2 = (two ? e2 : e) / (g.l / 4);
          const int i = (int)(col / g.n), j = (int)(col % g.n), k = (int)(4 * e - col * g.l);
          const int i2 = (int)(col2 / g.n), j2 = (int)(col2 % g.n);
          const int k2 = (int)(4 * (two ? e2 : e) - col2 * g.l);
          const P1Loads a = p1_load(u, g, 4 * e, i, j, k);
          const P1Loads b = p1_load(u, g, 4 * (two ? e2 : e), i2, j2, k2);
          p1_store(a, code, lam, sd, 4 * e, i, j, k);
          if (two) p1_store(b, code, lam, sd, 4 * e2, i2, j2, k2);
        }
    }
    for (int64_t col = vec4 ? (int64_t)g.m * g.n : c.gw; col < (int64_t)g.m * g.n; col += c.GW) {
      const int i = (int)(col / g.n), j = (int)(col % g.n);
      for (int k = lane; k < g.l; k += 32) {
        const int64_t x = col * g.l + k;
        const T uc = u[x];
        const int sx = upwind_side_t(u, x, i, g.m, sI, uc);
        const int sy = upwind_side_t(u, x, j, g.n, sJ, uc);
        const int sz = upwind_side_t(u, x, k, g.l, (int64_t)1, uc);
        uint16_t cd = (uint16_t)(sx | (sy << 2) | (sz << 4));
        if (uc == u0_t<T>(sd, i, j, k) || (sx | sy | sz) == 0) cd = CODE_FIXED;
        code[x] = cd;
        lam[x] = T(0);
      }
    }
    for (int b = c.gw * 32 + lane; b < nb; b += c.gthreads) {
      mod[b] = -2;
      proc[b] = -1;
      flow[b] = 0;
    }
    if (c.gw == 0 && lane == 0) group_reset_range(c.gs);
    group_sync(c.grp, c.gthreads);
    // pass 2: users (reads only the low bits of neighbours, writes own high bits);
    // each brick's flow collects its cells' user bits
    auto add_flow = [&](int i, int j, int k, uint32_t us) {
      if (!us) return;
      int* fb = flow + ((i / BI) * g.nby + (j / BJ)) * g.nbz + (k / BK);
      if ((((const volatile int*)fb)[0] & (int)us) != (int)us) atomicOr(fb, (int)us);
    };
    if constexpr (sizeof(T) == 4) {
      if (vec4)
        for (int64_t e = c.gw * 32 + lane; e < g.ncell / 4; e += 2 * c.gthreads) {
          const int64_t e2 = e + c.gthreads;
          const bool two = e2 < g.ncell / 4;
          const int64_t col = e / (g.l / 4), col2 = (two ? e2 : e) / (g.l / 4);
          const int i = (int)(col / g.n), j = (int)(col % g.n), k = (int)(4 * e - col * g.l);
          const int i2 = (int)(col2 / g.n), j2 = (int)(col2 % g.n);
          const int k2 = (int)(4 * (two ? e2 : e) - col2 * g.l);
          const P2Loads a = p2_load(code, g, 4 * e, i, j, k);
          const P2Loads b = p2_load(code, g, 4 * (two ? e2 : e), i2, j2, k2);
          add_flow(i, j, k, users_of4(p2_store(a, code, 4 * e)));
          if (two) add_flow(i2, j2, k2, users_of4(p2_store(b, code, 4 * e2)));
        }
    }
    for (int64_t col = vec4 ? (int64_t)g.m * g.n : c.gw; col < (int64_t)g.m * g.n; col += c.GW) {
      const int i = (int)(col / g.n), j = (int)(col % g.n);
      for (int k = lane; k < g.l; k += 32) {
        const int64_t x = col * g.l + k;
        const uint16_t cd = code[x];
        if (cd & CODE_FIXED) continue;
        uint16_t us = 0;
        auto uses = [&](int64_t r, int ax, int want) -> bool {
          const uint16_t cr = code[r];
          return !(cr & CODE_FIXED) && (((cr >> (2 * ax)) & 3) == want);
        };
        if (i > 0 && uses(x - sI, 0, 2)) us |= 1;
        if (i < g.m - 1 && uses(x + sI, 0, 1)) us |= 2;
        if (j > 0 && uses(x - sJ, 1, 2)) us |= 4;
        if (j < g.n - 1 && uses(x + sJ, 1, 1)) us |= 8;
        if (k > 0 && uses(x - 1, 2, 2)) us |= 16;
        if (k < g.l - 1 && uses(x + 1, 2, 1)) us |= 32;
        code[x] = (uint16_t)(cd | (us << CODE_USERS));
        add_flow(i, j, k, us);
      }
    }
    group_sync(c.grp, c.gthreads);
    // seeds: mark cells and make their bricks dirty
    const int ns = A.n_seed[sd.gidx];
    const int64_t* sidx = A.seed_idx + sd.seed_off;
    const T* sval = A.seed_val + sd.seed_off;
    for (int e = c.gw * 32 + lane; e < ns; e += c.gthreads) {
      const int64_t x = sidx[e];
      const uint16_t cd = code[x];
      if (cd & CODE_FIXED) continue;
      code[x] = (uint16_t)(cd | CODE_SEED);
      const int i = (int)(x / sI), j = (int)((x / sJ) % g.n), k = (int)(x % g.l);
      mod[((i / BI) * g.nby + (j / BJ)) * g.nbz + (k / BK)] = -1;
    }
    group_sync(c.grp, c.gthreads);
    int it;
    bool conv = false;
    for (it = 0; it < A.adj_max_iter; ++it) {
      if (c.gw == 0 && lane == 0) c.gs->changed = 0;
      group_sync(c.grp, c.gthreads);
      bool any = false;
      for (int o = 0; o < 8; ++o) {
        int si, sj, sk;
        ordering3(o, si, sj, sk);
        const int CS = tile_col_stride(BK, sj == sk);
        run_ordering<BK>(c, g, fd.bricks, fd.lstart, mod, proc, A.adj_order_filter ? flow : nullptr,
                         nullptr, (it * 8 + o) * g.nlev, si, sj, sk, cnt_upd, cnt_brk,
                         [&](const BrickPos& p, uint32_t&) -> bool {
          bool ch;
          if constexpr (sizeof(T) == 4) {
            if (vec) {
              load_tile_f32_async<BK>(U, u, g, p, CS, lane);
              load_tile_f32_async<BK>(L, lam, g, p, CS, lane, 0.0f);
              const bool seeds = load_codes_vec<BK>(C, code, g, p, CS, lane);
              cp_async_wait_all();
              __syncwarp();
              bool sig;
              ch = dispatch_adj_f32<BK>(U, L, C, A.gdense + sd.u_off, g, p, si, sj, sk, lane,
                                        A.adj_wake, seeds, sig);
              if (ch) store_interior_f32_vec<BK>(L, lam, g, p, CS, lane);
              ch = sig;  // only a significant change wakes neighbours and extends the solve
            } else {
              load_halo_tile<T, BK>(U, u, g, p, CS, lane);
              load_halo_tile<T, BK>(L, lam, g, p, CS, lane);
              load_interior<uint16_t, BK>(C, code, g, p, CS, lane);
              cp_async_wait_all();
              __syncwarp();
              ch = sweep_brick_adj<T, BK, EXACT, false>(U, L, C, nullptr, sidx, sval, ns, g, p, si,
                                                        sj, sk, CS, lane);
              if (ch) store_interior<T, BK>(L, lam, g, p, CS, lane);
            }
          } else {
            load_halo_tile<T, BK>(U, u, g, p, CS, lane);
            load_halo_tile<T, BK>(L, lam, g, p, CS, lane);
            load_interior<uint16_t, BK>(C, code, g, p, CS, lane);
            cp_async_wait_all();
            __syncwarp();
            ch = sweep_brick_adj<T, BK, EXACT, false>(U, L, C, nullptr, sidx, sval, ns, g, p, si,
                                                      sj, sk, CS, lane);
            if (ch) store_interior<T, BK>(L, lam, g, p, CS, lane);
          }
          any |= ch;
          return ch;
        });
      }
      if (any && lane == 0) c.gs->changed = 1;
      group_sync(c.grp, c.gthreads);
      const bool changed = c.gs->changed != 0;
      group_sync(c.grp, c.gthreads);
      if (!changed) {
        conv = true;
        break;
      }
    }
    if (A.gdense)  // leave the dense seed field all zero for the next evaluation
      for (int e = c.gw * 32 + lane; e < ns; e += c.gthreads) A.gdense[sd.u_off + sidx[e]] = T(0);
    if (lane == 0 && cnt_brk > brk0) atomicAdd(&A.cost[sd.gidx], cnt_brk - brk0);
    if (c.gw == 0 && lane == 0) {
      adt_solve_status& st = A.status[sd.gidx];
      st.adj_iters = conv ? it + 1 : it;
      st.adj_converged = conv ? 1 : 0;
    }
  }
  if (lane == 0 && cnt_brk) {
    atomicAdd(&A.counters[2], cnt_upd);
    atomicAdd(&A.counters[3], cnt_brk);
  }
}

// --------------------------------------------------------------- gradient
// grad[c] += sum over the chunk's solves on this field (in solve order) of
// -lambda_s[c] * (-2 f h h), in FP64 (Eikonal3D.cpp:163-166,244-246).
// - FP64 plans form every product and add it in solve order, as the oracle's
//   batch does (bit-identical).
// - FP32 plans add the solves' -lambda (exact conversions, FP64 sum in solve
//   order, carried across chunks in grad) and k_grad_scale multiplies by
//   -2 f h h once after the last chunk: half the FP64 operations, no less
//   accurate, and the same bits however the solves are chunked.
// Loads are issued eight solves ahead of the adds.  lambda of cell c of the
// solve at u_off is lam[(u_off + c) * lam_stride]: stride 1 for the sweeps'
// lambda array, 4 for the causal-order adjoint's records.
template <class T>
__global__ void k_batch_grad(const T* __restrict__ lam, int lam_stride,
                             const int64_t* __restrict__ u_off, int n_solves,
                             const double* __restrict__ f64, double h, int64_t ncell,
                             double* __restrict__ grad, int blocked_n, int blocked_l) {
  constexpr int U = 8;
  const BlkMap bm = make_blkmap(blocked_n, blocked_l);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
       c += (int64_t)gridDim.x * blockDim.x) {
    // lc: the cell's slot in lam (blocked_n > 0: the causal-order adjoint's
    // records in the blocked layout, BlkMap)
    int64_t lc = c;
    if (blocked_n > 0) {
      const int64_t nl = (int64_t)blocked_n * blocked_l;
      const int i = (int)(c / nl), j = (int)((c - i * nl) / blocked_l);
      lc = blk_index(bm, i, j, (int)(c - i * nl - (int64_t)j * blocked_l));
    }
    const double rhs =
        sizeof(T) == 4 ? 0.0 : __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f64[c]), h), h);
    double G = grad[c];
    int s = 0;
    for (; s + U <= n_solves; s += U) {
      double l[U];
#pragma unroll
      for (int q = 0; q < U; ++q) l[q] = (double)lam[(u_off[s + q] + lc) * lam_stride];
#pragma unroll
      for (int q = 0; q < U; ++q)
        G = sizeof(T) == 4 ? __dadd_rn(G, -l[q]) : __dadd_rn(G, __dmul_rn(-l[q], rhs));
    }
    for (; s < n_solves; ++s) {
      const double l = (double)lam[(u_off[s] + lc) * lam_stride];
      G = sizeof(T) == 4 ? __dadd_rn(G, -l) : __dadd_rn(G, __dmul_rn(-l, rhs));
    }
    grad[c] = G;
  }
}

// FP32 plans, after the last chunk: grad[c] = (sum of -lambda) * (-2 f h h).
__global__ void k_grad_scale(const double* __restrict__ f64, double h, int64_t ncell,
                             double* __restrict__ grad) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
       c += (int64_t)gridDim.x * blockDim.x)
    grad[c] = __dmul_rn(grad[c], __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f64[c]), h), h));
}

// Order each chunk's solves for the next evaluation by this evaluation's
// cost (bricks swept, forward + adjoint), most expensive first, ties by solve
// index.  With the persistent kernels' static first assignment (group_next)
// and work counter, that is longest-first scheduling.  Only the schedule changes; every
// sum over solves keeps its own fixed order, so results do not.  One CTA per
// chunk; chunks of more than ORDER_MAX solves keep their order.
constexpr int ORDER_MAX = 4096;

__global__ void k_order_by_cost(int* order, const long long* chunk_off, const int* chunk_cnt,
                                const unsigned long long* cost) {
  __shared__ unsigned long long key[ORDER_MAX];
  __shared__ int idx[ORDER_MAX];
  const int c = blockIdx.x, n = chunk_cnt[c];
  if (n > ORDER_MAX || n < 2) return;
  int* o = order + chunk_off[c];
  int P = 1;
  while (P < n) P <<= 1;
  for (int i = threadIdx.x; i < P; i += blockDim.x) {
    if (i < n) {
      idx[i] = o[i];
      key[i] = cost[o[i]];
    } else {
      idx[i] = INT_MAX;
      key[i] = 0;
    }
  }
  __syncthreads();
  // bitonic sort: cost descending, then index ascending
  for (int k = 2; k <= P; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int i = threadIdx.x; i < P; i += blockDim.x) {
        const int p = i ^ j;
        if (p > i) {
          const bool before = key[i] > key[p] || (key[i] == key[p] && idx[i] < idx[p]);
          if (before != ((i & k) == 0)) {
            const unsigned long long tk = key[i];
            key[i] = key[p];
            key[p] = tk;
            const int ti = idx[i];
            idx[i] = idx[p];
            idx[p] = ti;
          }
        }
      }
      __syncthreads();
    }
  for (int i = threadIdx.x; i < n; i += blockDim.x) o[i] = idx[i];
}

}  // namespace adt
