// eik3d_adj_causal.cuh -- the 3D adjoint solved once, in causal order,
// instead of by sweeps until nothing changes: the batched plan's
// (k_batch_adj_causal) and the single-event op's (k_single_adj_causal).
//
// The adjoint system of one solve (Eikonal3D.cpp:96-198, which assembles it
// and factors it with SparseLU) is triangular in travel-time order: cell c's
// row couples it only to its users, the neighbours whose active upwind side
// along an axis is c, and a user's travel time is strictly larger than c's
// (a side is taken only towards a smaller neighbour).  The users relation is
// therefore acyclic, and one pass in reverse causal order solves the system
// exactly: every cell is evaluated once, after all its users (Kahn's
// algorithm on that graph).
//
// One CTA runs one solve at a time (solves from the chunk's work counter).
// Per cell the kernel keeps a 32-bit meta word (upwind sides, fixed, seed,
// user bits, and the user bits still outstanding in bits 16-21) and a record
// {lambda, upwind difference per axis} (CausalRec), both in the blocked
// layout of 2 x 2 x 2 cell groups (BlkMap), which keeps most of a cell's
// neighbourhood in its own 128-byte line:
//  - pass 1 reads the travel times once (coalesced) and writes the sides,
//    the fixed flag and the differences; pass 2 the user bits, from the
//    neighbours' meta words;
//  - the cells without users open the solve's queue (every slot starts at -1);
//  - every thread then takes the next queue slot, waits until a cell is
//    written there, evaluates it from its own record and its users' records
//    (a user's difference along the axis is its weight u_r - u_c) and clears
//    its bit in each upwind neighbour's outstanding bits (atomicAnd on the
//    meta word); the thread whose clear empties them appends that cell to the
//    queue.  No barrier between cells: a cell is evaluated as soon as its last
//    user is and a thread has taken its slot.
// Ordering: a cell's adjoint value is stored before its release atomics,
// which are acq_rel at CTA scope, and the releasing thread writes the queue
// slot with a release store that the evaluating thread reads with an acquire
// load, so every user's value is visible when the cell is evaluated.
// Progress: slots are taken and written in order, and while a taken slot is
// unwritten some cell is still unevaluated; the unevaluated cell with the
// largest travel time has all its users evaluated, so it has been queued and
// its slot's thread can go on.  Every wait is also bounded
// (CAUSAL_WAIT_CYCLES); one that runs out marks the solve unconverged instead
// of hanging, and the other waits then stop too.
//
// A cell is evaluated with the sweeping adjoint's formula, the same
// operations in the same order on the same operands (FP32: adj_cell_f32 and
// the sweep step; FP64: sweep_brick_adj's exact form, which the oracle
// follows), so the result is the sweeps' exact fixed point, bit for bit (up
// to the sign of a zero), with one evaluation per cell instead of one per
// sweep that reaches it.
#pragma once
#include "causal_sync.cuh"
#include "eik3d_batch_kernels.cuh"

// Threads per CTA the kernels are compiled for: FP32 1024 (at most 64
// registers; the kernel needs about 42), FP64 512 (its doubles need more).
#ifndef ADT_CAUSAL_MAXT
#define ADT_CAUSAL_MAXT 1024
#endif
#define ADT_CAUSAL_BOUNDS(T) __launch_bounds__(sizeof(T) == 8 ? ADT_CAUSAL_MAXT / 2 : ADT_CAUSAL_MAXT)

namespace adt {

// Meta word: bits 0-15 the adjoint code (adt_common.cuh), bits 16-21 the
// user bits whose users are not evaluated yet.
constexpr int META_OUT = 16;

struct CausalShared {
  int q;
  int head;      // next queue slot to take
  int tail;      // queue slots written so far
  int nonfixed;  // non-fixed cells of the running solve (each is queued once)
  int err;       // a wait on a queue slot ran out of its budget
  int pad;
};

// (i, j, k) of cell x of a field (x < 2^31), by multiplications.
__device__ __forceinline__ void cell_ijk(uint32_t x, const Geom& g, unsigned long long div_nl,
                                         unsigned long long div_l, int& i, int& j, int& k) {
  const uint32_t nl = (uint32_t)g.n * (uint32_t)g.l;
  const uint32_t ii = (uint32_t)__umul64hi((unsigned long long)x, div_nl);
  const uint32_t r = x - ii * nl;
  const uint32_t jj = (uint32_t)__umul64hi((unsigned long long)r, div_l);
  i = (int)ii;
  j = (int)jj;
  k = (int)(r - jj * (uint32_t)g.l);
}

template <class T>
__device__ __forceinline__ T inf_value() {
  if constexpr (sizeof(T) == 4)
    return __int_as_float(0x7f800000);
  else
    return __longlong_as_double(0x7ff0000000000000LL);
}

// Seed value of a cell with the seed bit, from the solve's sorted seed list.
template <class T>
__device__ __forceinline__ T seed_lookup(const int64_t* idx, const T* val, int ns, int64_t key) {
  int lo = 0, hi = ns - 1;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (idx[mid] < key) lo = mid + 1; else hi = mid;
  }
  return val[lo];
}

// Side code and upwind difference of one axis from the two neighbours (+inf
// off the grid): the side is the smaller neighbour (ties to +1) when u_c
// exceeds it (upwind_side_t's rule); the difference u_c - min is formed as
// the FP32 sweep forms it (fmaxf(u_c - fminf(.), 0)) and, in FP64, as the
// oracle's diagonal does (u_c - a when active, else 0).
template <class T>
__device__ __forceinline__ void axis_side(T uc, T um, T up, uint32_t& side, T& d) {
  const bool minus = up > um;
  const T a = minus ? um : up;
  side = uc > a ? (minus ? 1u : 2u) : 0u;
  if constexpr (sizeof(T) == 4)
    d = fmaxf(uc - fminf(um, up), 0.0f);
  else
    d = uc > a ? __dsub_rn(uc, a) : 0.0;
}

// The adjoint value of one non-fixed cell: meta word mt, its own upwind
// differences dc, its users' upwind differences towards it (w, 0 for a
// neighbour that is not a user) and adjoint values (ln, 0 likewise), in the
// order x-, x+, y-, y+, z-, z+; gs: the seed value (0 without one).
// FP32: lambda = fma(P_x + P_y, c2, fma(P_z, c2, c0)), P_a = fma(w_{a+},
// lambda_{a+}, w_{a-} lambda_{a-}), c2 = rcp(d), c0 = 0.5 g c2 -- the
// sweeping adjoint's order for every sweep direction (adj_cell_f32).
// FP64: (g + sum_users 2 (u_r - u_c) lambda_r) / sum_sides 2 (u_c - u_side)
// in the oracle's order (sweep_brick_adj with EXACT).
template <class T>
__device__ __forceinline__ T causal_lambda(uint32_t mt, const T (&dc)[3], const T (&w)[6],
                                           const T (&ln)[6], T gs) {
  if constexpr (sizeof(T) == 4) {
    const float px = fmaf(w[1], ln[1], w[0] * ln[0]);
    const float py = fmaf(w[3], ln[3], w[2] * ln[2]);
    const float pz = fmaf(w[5], ln[5], w[4] * ln[4]);
    float d = dc[0];
    d += dc[1];
    d += dc[2];
    const float c2 = rcp_approx(d);
    const float c0 = 0.5f * gs * c2;
    return fmaf(px + py, c2, fmaf(pz, c2, c0));
  } else {
    double acc = gs;
#pragma unroll
    for (int q = 0; q < 6; ++q)
      if (mt & (1u << (CODE_USERS + q))) acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(2.0, w[q]), ln[q]));
    // d = 0 + t_x + t_y + t_z over the active axes; every t is positive, so
    // the first addition (0 + t = t) is left out
    double d = 0.0;
    bool any = false;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax)
      if ((mt >> (2 * ax)) & 3u) {
        const double t = __dmul_rn(2.0, dc[ax]);
        d = any ? __dadd_rn(d, t) : t;
        any = true;
      }
    return fi_div(acc, d);
  }
}

// Pass 1 over one solve's cells: upwind sides, fixed flag (u ==
// u0_of(x, i, j, k) or no active axis), upwind differences and lambda = 0
// into the blocked meta words and records, and empty queue slots.  Reads the
// travel times in their own order (coalesced).
template <class T, class U0>
__device__ __forceinline__ void causal_pass1(const T* __restrict__ u, const Geom& g,
                                             unsigned long long div_nl, unsigned long long div_l,
                                             const BlkMap& bm, uint32_t* meta, CausalRec<T>* rec,
                                             int* queue, U0 u0_of, int tid, int nth) {
  const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
  const T INF = inf_value<T>();
  for (int x = tid; x < (int)g.ncell; x += nth) {
    int i, j, k;
    cell_ijk((uint32_t)x, g, div_nl, div_l, i, j, k);
    const T uc = u[x];
    const T un[6] = {i > 0 ? u[x - sI] : INF, i < g.m - 1 ? u[x + sI] : INF,
                     j > 0 ? u[x - sJ] : INF, j < g.n - 1 ? u[x + sJ] : INF,
                     k > 0 ? u[x - 1] : INF, k < g.l - 1 ? u[x + 1] : INF};
    uint32_t cd = 0;
    CausalRec<T> rc;
    rc.lam = T(0);
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      uint32_t side;
      axis_side(uc, un[2 * ax], un[2 * ax + 1], side, rc.d[ax]);
      cd |= side << (2 * ax);
    }
    if (uc == u0_of(x, i, j, k) || cd == 0) cd = CODE_FIXED;
    const int b = blk_index(bm, i, j, k);
    meta[b] = cd;
    rec[b] = rc;
    queue[x] = -1;
  }
}

// Pass 2 over one solve's cells: user bits (and as outstanding bits) from
// the neighbours' meta words, and the cells without users appended to the
// queue (counted in *tail) by their blocked slots.  Every thread of the CTA
// calls it (warp-uniform loop); returns the thread's count of non-fixed cells.
__device__ __forceinline__ int causal_pass2(const Geom& g, unsigned long long div_nl,
                                            unsigned long long div_l, const BlkMap& bm,
                                            uint32_t* meta, int* queue, int* tail, int lane, int warp,
                                            int nth) {
  const int ncell = (int)g.ncell;
  int nf = 0;
  for (int x0 = warp * 32; x0 < ncell; x0 += nth) {
    const int x = x0 + lane;
    uint32_t by = REM_FIXED;
    int b = 0;
    if (x < ncell) {
      int i, j, k;
      cell_ijk((uint32_t)x, g, div_nl, div_l, i, j, k);
      b = blk_index(bm, i, j, k);
      const uint32_t cd = meta[b];
      if (!(cd & CODE_FIXED)) {
        auto uses = [&](int a, int dir, uint32_t want) -> bool {
          const uint32_t cr = meta[blk_step(bm, b, a, dir)];
          return !(cr & CODE_FIXED) && ((cr >> (2 * a)) & 3u) == want;
        };
        uint32_t us = 0;
        if (i > 0 && uses(0, -1, 2u)) us |= 1u;
        if (i < g.m - 1 && uses(0, 1, 1u)) us |= 2u;
        if (j > 0 && uses(1, -1, 2u)) us |= 4u;
        if (j < g.n - 1 && uses(1, 1, 1u)) us |= 8u;
        if (k > 0 && uses(2, -1, 2u)) us |= 16u;
        if (k < g.l - 1 && uses(2, 1, 1u)) us |= 32u;
        // only the high bits change: a neighbour reading this word
        // concurrently sees the same side bits either way
        meta[b] = cd | (us << CODE_USERS) | (us << META_OUT);
        by = us;
      }
    }
    nf += by != REM_FIXED;
    const int pos = warp_append(by == 0u ? 1 : 0, tail, lane);
    if (by == 0u) queue[pos] = b;
  }
  return nf;
}

// The evaluation in causal order (every thread of the CTA): take the next
// queue slot, wait for its cell, evaluate it from its record and its users'
// records, release its upwind neighbours and queue the ones released.
// Cells are blocked slots; seed_of(slot, meta word) gives the cell's seed value.  Ends when every
// non-fixed cell has been taken (S.nonfixed) or a wait ran out (S.err).
template <class T, class Seed>
__device__ __forceinline__ void causal_evaluate(CausalShared& S, const BlkMap& bm, uint32_t* meta,
                                                CausalRec<T>* rec, int* queue, Seed seed_of) {
  const int nonfixed = S.nonfixed;
  for (;;) {
    const int slot = take_slots(1, &S.head);
    if (slot >= nonfixed) break;
    int x = ld_acquire_cta(queue + slot);
    if (x < 0) {
      const long long t0 = clock64();
      do {
        __nanosleep(64);
        x = ld_acquire_cta(queue + slot);
      } while (x < 0 && clock64() - t0 < CAUSAL_WAIT_CYCLES &&
               !*reinterpret_cast<volatile int*>(&S.err));
      if (x < 0) {  // out of budget, or another thread's was
        atomicOr(&S.err, 1);
        break;
      }
    }
    const uint32_t mt = meta[x];
    const CausalRec<T> rc = rec[x];
    const T dc[3] = {rc.d[0], rc.d[1], rc.d[2]};
    // the users' records: adjoint value (final) and upwind difference
    // towards this cell (its weight)
    T w[6], ln[6];
    const uint32_t us = mt >> CODE_USERS;
#pragma unroll
    for (int t = 0; t < 6; ++t) {
      w[t] = T(0);
      ln[t] = T(0);
      if ((us >> t) & 1u) {
        const CausalRec<T> rr = rec[blk_step(bm, x, t >> 1, t & 1 ? 1 : -1)];
        w[t] = rr.d[t >> 1];
        ln[t] = rr.lam;
      }
    }
    rec[x].lam = causal_lambda<T>(mt, dc, w, ln, seed_of(x, mt));
    // release the upwind neighbours (their outstanding bit for this cell)
    uint32_t rel = 0;
    int np = 0;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const uint32_t side = (mt >> (2 * a)) & 3u;
      if (side) {
        const int tq = blk_step(bm, x, a, side == 1 ? -1 : 1);
        const uint32_t bit = side == 1 ? (2u << (2 * a)) : (1u << (2 * a));
        const uint32_t old = atom_and_acq_rel_cta(meta + tq, ~(bit << META_OUT));
        const uint32_t ob = (old >> META_OUT) & 0x3fu;
        if ((ob & bit) && !(ob & ~bit)) {
          rel |= 1u << a;
          ++np;
        }
      }
    }
    int pos = take_slots(np, &S.tail);
#pragma unroll
    for (int a = 0; a < 3; ++a)
      if ((rel >> a) & 1u) {
        const uint32_t side = (mt >> (2 * a)) & 3u;
        st_release_cta(queue + pos++, blk_step(bm, x, a, side == 1 ? -1 : 1));
      }
  }
}

// Every non-fixed cell queued and evaluated, and no wait ran out.
__device__ __forceinline__ bool causal_complete(const CausalShared& S) {
  return S.err == 0 && S.tail == S.nonfixed && S.head >= S.nonfixed;
}

template <class T>
__global__ void ADT_CAUSAL_BOUNDS(T) k_batch_adj_causal(BatchArgs<T> A) {
  __shared__ CausalShared S;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
  unsigned long long upd = 0;
  int q = blockIdx.x;
  while (q < A.n_solves) {
    const int gsol = A.order[q];
    const SolveDev& sd = A.solves[gsol];
    const FieldDev<T> fd = A.fields[sd.field];
    const Geom g = fd.g;
    const BlkMap bm = make_blkmap(g.n, g.l);
    // per-solve regions hold max(cells, blocked slots) (batch_create)
    uint32_t* meta = A.meta32 + sd.u_off;
    CausalRec<T>* rec = A.rec + sd.u_off;
    int* queue = A.queue + sd.u_off;
    if (tid == 0) {
      S.head = S.tail = 0;
      S.nonfixed = 0;
      S.err = 0;
    }
    // pass 1: sides, fixed cells, upwind differences; lambda = 0
    causal_pass1<T>(A.u + sd.u_off, g, fd.div_nl, fd.div_l, bm, meta, rec, queue,
                    [&](int, int i, int j, int k) { return u0_t<T>(sd, i, j, k); }, tid, nth);
    __syncthreads();
    // pass 2: user bits and the cells nobody uses
    int nf = causal_pass2(g, fd.div_nl, fd.div_l, bm, meta, queue, &S.tail, lane, warp, nth);
    nf = __reduce_add_sync(0xffffffffu, nf);
    if (lane == 0 && nf) atomicAdd(&S.nonfixed, nf);
    __syncthreads();
    // seeds: mark the seeded non-fixed cells
    const int ns = A.n_seed[sd.gidx];
    const int64_t* sidx = A.seed_idx + sd.seed_off;
    const T* sval = A.seed_val + sd.seed_off;
    for (int e = tid; e < ns; e += nth) {
      int i, j, k;
      cell_ijk((uint32_t)sidx[e], g, fd.div_nl, fd.div_l, i, j, k);
      const int b = blk_index(bm, i, j, k);
      const uint32_t cd = meta[b];
      if (!(cd & CODE_FIXED)) meta[b] = cd | CODE_SEED;
    }
    __syncthreads();
    // evaluation in causal order; a seeded cell's value is found by its
    // position in the solve's own order
    causal_evaluate<T>(S, bm, meta, rec, queue, [&](int b, uint32_t mt) -> T {
      if (!(mt & CODE_SEED)) return T(0);
      int i, j, k;
      blk_cell(bm, b, i, j, k);
      const int64_t x = ((int64_t)i * g.n + j) * g.l + k;
      if constexpr (sizeof(T) == 4)
        return A.gdense ? A.gdense[sd.u_off + x] : seed_lookup(sidx, sval, ns, x);
      else
        return seed_lookup(sidx, sval, ns, x);
    });
    __syncthreads();
    if (A.gdense)  // leave the dense seed field all zero for the next evaluation
      for (int e = tid; e < ns; e += nth) A.gdense[sd.u_off + sidx[e]] = T(0);
    if (tid == 0) {
      adt_solve_status& st = A.status[sd.gidx];
      st.adj_iters = 1;
      // every non-fixed cell queued and evaluated, no wait ran out
      st.adj_converged = causal_complete(S) ? 1 : 0;
      upd += (unsigned long long)S.tail;
      S.q = atomicAdd(A.next, 1) + (int)gridDim.x;
    }
    __syncthreads();
    q = S.q;
    __syncthreads();  // S.q read by all before the next solve's tid 0 writes S
  }
  if (tid == 0 && upd) atomicAdd(&A.counters[2], upd);
}

// The single-event adjoint (EikonalThreeDGrad, Eikonal3D.cpp:96-198) in
// causal order, one CTA: u0 is the op's explicit array (fixed cells: u ==
// u0 or no active axis) and every non-fixed cell starts from its grad_u
// value, as the oracle's substitution does, so lambda is the oracle's bit
// for bit.  meta and rec hold blk_slots(m, n, l) entries (blocked layout),
// queue one per cell.  *complete = 1 when every non-fixed cell was evaluated.
__global__ void __launch_bounds__(ADT_CAUSAL_MAXT / 2)
    k_single_adj_causal(const double* __restrict__ u, const double* __restrict__ u0,
                        const double* __restrict__ grad_u, Geom g, unsigned long long div_nl,
                        unsigned long long div_l, uint32_t* meta, CausalRec<double>* rec, int* queue,
                        int* complete) {
  __shared__ CausalShared S;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    S.head = S.tail = 0;
    S.nonfixed = 0;
    S.err = 0;
  }
  const BlkMap bm = make_blkmap(g.n, g.l);
  causal_pass1<double>(u, g, div_nl, div_l, bm, meta, rec, queue,
                       [&](int x, int, int, int) { return u0[x]; }, tid, nth);
  __syncthreads();
  int nf = causal_pass2(g, div_nl, div_l, bm, meta, queue, &S.tail, lane, warp, nth);
  nf = __reduce_add_sync(0xffffffffu, nf);
  if (lane == 0 && nf) atomicAdd(&S.nonfixed, nf);
  __syncthreads();
  causal_evaluate<double>(S, bm, meta, rec, queue, [&](int b, uint32_t) {
    int i, j, k;
    blk_cell(bm, b, i, j, k);
    return grad_u[((int64_t)i * g.n + j) * g.l + k];
  });
  __syncthreads();
  if (tid == 0) *complete = causal_complete(S) ? 1 : 0;
}

}  // namespace adt
