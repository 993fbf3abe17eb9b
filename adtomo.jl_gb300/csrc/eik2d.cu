// eik2d.cu -- 2D fast sweeping (FP64, reference arithmetic) and its adjoint.
//
// Grid (n+1) x (m+1), index j*(m+1)+i (Eikonal.h:30-48).  One CTA per solve.
// Each of the 4 orderings (I,J), (iI,J), (iI,iJ), (I,iJ) (Eikonal.h:74-77) is
// run as a wavefront over the anti-diagonals i' + j' = s of that ordering:
// every cell on a diagonal depends only on the previous diagonal, which is
// the Gauss-Seidel data flow of the reference's i-outer / j-inner loop, so
// travel times are bit-identical.  The source cell is skipped and pinned to 0.
// Stop when ||u - u_old|| / ||u_old|| < 1e-8, at most 100 iterations
// (Eikonal.h:71-86).  Nodes none of whose neighbours changed since their last
// update are skipped (exact); the travel times and those change flags live in
// shared memory for grids up to FWD2_SMEM_NODES nodes.
//
// Adjoint (Eikonal.h:95-200): lambda_c = (g_c + sum_users 2 (u_r - u_c)
// lambda_r) / d_c with the source row the identity.  The system is
// triangular in travel-time order, so each row is solved once, after its
// users: level by level in shared memory (k_eik2d_adjoint_levels), with a
// queue in global memory for larger grids (k_eik2d_adjoint_causal), and by
// the same diagonal sweeps until a full iteration changes nothing above 2^30
// nodes (k_eik2d_adjoint).  A non-source cell without an active axis makes
// the reference's matrix singular; it is reported as ADT_ESINGULAR.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "eik2d.h"
#include "eik3d_common_host.h"
#include "causal_sync.cuh"
#include "eik_local.cuh"
#include "fp64_int.cuh"

namespace adt {

namespace {

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  if (threadIdx.x == 0) red[32] = t;
  __syncthreads();
  return red[32];
}

__device__ __forceinline__ void ord2(int o, int& si, int& sj) {
  si = (o == 1 || o == 2) ? -1 : 1;
  sj = (o >= 2) ? -1 : 1;
}

// Travel times and change flags of a solve stay in shared memory up to this
// many nodes (9 bytes each).
constexpr int FWD2_SMEM_NODES = 25600;
// The adjoint by levels keeps lambda, the queue and the flags in shared
// memory up to ADJ2_SMEM_NODES nodes (13 bytes each), and the travel times
// too, with a 16-bit queue, up to ADJ2_STAGE_U_NODES (19 bytes each).
constexpr int ADJ2_SMEM_NODES = 17600;
constexpr int ADJ2_STAGE_U_NODES = 12200;

}  // namespace

// Per-node constants of the 2D update, formed once per call in the
// reference's operation order (Eikonal.h:14-20): x = f h, y = 2 f f h h.
__global__ void k_eik2d_cells(const double* __restrict__ f, int64_t N, double h,
                              double2* __restrict__ cst) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < N;
       p += (int64_t)gridDim.x * blockDim.x) {
    const double fv = f[p];
    cst[p] = make_double2(__dmul_rn(fv, h),
                          __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(2.0, fv), fv), h), h));
  }
}

// Exact work skipping: a node's update reads only its four neighbours, so a
// node none of whose neighbours changed since its last update would compute
// the same candidate again, which cannot lower it.  dirty[c] says a
// neighbour of c changed since c was last updated (all set at the start);
// an update clears the node's flag, and a node that decreases sets its
// neighbours' flags.  Neighbours lie on the adjacent anti-diagonals, so
// within a wavefront step no flag is set and cleared at once, and the
// travel times are bit for bit those of updating every node.
//
// SMEM: the solve's travel times and flags live in dynamic shared memory
// (grids up to FWD2_SMEM_NODES nodes), written to u_all at the end;
// otherwise u_all and dirty_all (N bytes per solve) hold them.
template <bool SMEM>
__global__ void __launch_bounds__(512)
    k_eik2d_forward(const double2* __restrict__ cst, int m, int n, const int* __restrict__ srcx,
                    const int* __restrict__ srcy, double* __restrict__ u_all,
                    double* __restrict__ prev_all, uint8_t* __restrict__ dirty_all,
                    int* __restrict__ iters, int* __restrict__ conv, double* __restrict__ errs) {
  extern __shared__ double s_u[];
  __shared__ double red[33];
  const int w = m + 1;
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  const int sol = blockIdx.x;
  double* u = SMEM ? s_u : u_all + sol * N;
  uint8_t* dirty = SMEM ? reinterpret_cast<uint8_t*>(s_u + N) : dirty_all + sol * N;
  double* prev = prev_all + sol * N;
  const int ix = srcx[sol], jx = srcy[sol];
  for (int64_t p = threadIdx.x; p < N; p += blockDim.x) {
    const int i = (int)(p % w), j = (int)(p / w);
    const double v = (i == ix && j == jx) ? 0.0 : 100000.0;
    u[p] = v;
    prev[p] = v;
    dirty[p] = 1;
  }
  __syncthreads();
  int it, done = 0;
  double err = 0.0;
  for (it = 0; it < 100; ++it) {
    for (int o = 0; o < 4; ++o) {
      int si, sj;
      ord2(o, si, sj);
      for (int s = 0; s <= m + n; ++s) {
        const int a0 = max(0, s - n), a1 = min(m, s);
        for (int a = a0 + (int)threadIdx.x; a <= a1; a += blockDim.x) {
          const int b = s - a;
          const int i = si > 0 ? a : m - a;
          const int j = sj > 0 ? b : n - b;
          if (i == ix && j == jx) continue;
          const int c = j * w + i;
          if (!dirty[c]) continue;
          dirty[c] = 0;
          const double2 k = cst[c];
          double ax, by;
          if (i == 0) ax = u[c + 1];
          else if (i == m) ax = u[c - 1];
          else ax = min_nn(u[c + 1], u[c - 1]);
          if (j == 0) by = u[c + w];
          else if (j == n) by = u[c - w];
          else by = min_nn(u[c - w], u[c + w]);
          const double un = upd2_exact(ax, by, k.x, k.y);
          if (lt_nn(un, u[c])) {  // rmin(u[c], un)
            u[c] = un;
            if (i > 0) dirty[c - 1] = 1;
            if (i < m) dirty[c + 1] = 1;
            if (j > 0) dirty[c - w] = 1;
            if (j < n) dirty[c + w] = 1;
          }
        }
        __syncthreads();
      }
    }
    double dd = 0.0, pp = 0.0;
    for (int64_t p = threadIdx.x; p < N; p += blockDim.x) {
      const double d = __dsub_rn(u[p], prev[p]);
      dd = __dadd_rn(dd, __dmul_rn(d, d));
      pp = __dadd_rn(pp, __dmul_rn(prev[p], prev[p]));
    }
    dd = block_sum(dd, red);
    pp = block_sum(pp, red);
    err = __ddiv_rn(__dsqrt_rn(dd), __dsqrt_rn(pp));
    if (err < 1e-8) {
      done = 1;
      break;
    }
    for (int64_t p = threadIdx.x; p < N; p += blockDim.x) prev[p] = u[p];
    __syncthreads();
  }
  if (SMEM)
    for (int64_t p = threadIdx.x; p < N; p += blockDim.x) u_all[sol * N + p] = u[p];
  if (threadIdx.x == 0) {
    iters[sol] = done ? it + 1 : it;
    conv[sol] = done;
    errs[sol] = err;
  }
}

// Upwind neighbour index along one axis (edge rule, ties to the +1 side).
__device__ __forceinline__ int64_t upw2(const double* u, int64_t p, int pos, int last, int64_t st) {
  if (pos == 0) return p + st;
  if (pos == last) return p - st;
  return (u[p + st] > u[p - st]) ? p - st : p + st;
}

__global__ void k_eik2d_adjoint(const double* __restrict__ gu, const double* __restrict__ u,
                                const double* __restrict__ f, int m, int n, double h, int ix,
                                int jx, double* __restrict__ lam, double* __restrict__ grad_f,
                                int* __restrict__ status) {
  __shared__ int s_changed, s_singular;
  const int w = m + 1;
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  const int64_t src = (int64_t)jx * w + ix;
  for (int64_t p = threadIdx.x; p < N; p += blockDim.x) lam[p] = 0.0;
  if (threadIdx.x == 0) s_singular = 0;
  __syncthreads();
  int it, done = 0;
  for (it = 0; it < 10000; ++it) {
    if (threadIdx.x == 0) s_changed = 0;
    __syncthreads();
    for (int o = 0; o < 4; ++o) {
      int si, sj;
      ord2(o, si, sj);
      for (int s = 0; s <= m + n; ++s) {
        const int a0 = max(0, s - n), a1 = min(m, s);
        for (int a = a0 + (int)threadIdx.x; a <= a1; a += blockDim.x) {
          const int b = s - a;
          const int i = si > 0 ? a : m - a;
          const int j = sj > 0 ? b : n - b;
          const int64_t c = (int64_t)j * w + i;
          double acc = gu[c];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int ri = i + (q == 0 ? -1 : q == 1 ? 1 : 0);
            const int rj = j + (q == 2 ? -1 : q == 3 ? 1 : 0);
            if (ri < 0 || ri > m || rj < 0 || rj > n) continue;
            const int64_t r = (int64_t)rj * w + ri;
            if (r == src) continue;
            const int64_t nb = (q < 2) ? upw2(u, r, ri, m, 1) : upw2(u, r, rj, n, w);
            if (nb != c || !(u[r] > u[c])) continue;
            acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(2.0, __dsub_rn(u[r], u[c])), lam[r]));
          }
          double d;
          if (c == src) {
            d = 1.0;
          } else {
            d = 0.0;
            const int64_t nx = upw2(u, c, i, m, 1), ny = upw2(u, c, j, n, w);
            if (u[c] > u[nx]) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(u[c], u[nx])));
            if (u[c] > u[ny]) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(u[c], u[ny])));
          }
          if (d == 0.0) {
            s_singular = 1;
            continue;
          }
          const double l = fi_div(acc, d);
          if (!(l == lam[c])) {
            lam[c] = l;
            s_changed = 1;
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (s_singular) break;
    if (!s_changed) {
      done = 1;
      break;
    }
    __syncthreads();
  }
  for (int64_t p = threadIdx.x; p < N; p += blockDim.x) {
    // dFdf = -2 f h h, 0 at the source; grad_f = -lambda * dFdf (Eikonal.h:100-104,196-198)
    const double dfdf = (p == src) ? 0.0 : __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f[p]), h), h);
    grad_f[p] = __dmul_rn(-lam[p], dfdf);
  }
  if (threadIdx.x == 0) status[0] = s_singular ? -1 : (done ? it + 1 : 0);
}

// One row of the 2D adjoint (Eikonal.h:95-200) for cell x, whose users (bits
// x-, x+, y-, y+ in us) are evaluated: lambda_x = (g_x + sum_users
// 2 (u_r - u_x) lambda_r) / d_x, d_x = sum over the upwind axes of
// 2 (u_x - u_upwind) (1 at the source), in k_eik2d_adjoint's order.  Also
// returns the upwind neighbours (nx, ny) and which axes are upwind.
__device__ __forceinline__ double adj2_row(const double* __restrict__ gu,
                                           const double* __restrict__ u, const double* lam, int x,
                                           uint32_t us, int m, int n, int src, int& nx, int& ny,
                                           bool& ax, bool& ay) {
  const int w = m + 1;
  const int i = x % w, j = x / w;
  double acc = gu[x];
#pragma unroll
  for (int q = 0; q < 4; ++q)
    if ((us >> q) & 1u) {
      const int r = x + (q == 0 ? -1 : q == 1 ? 1 : q == 2 ? -w : w);
      acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(2.0, __dsub_rn(u[r], u[x])), lam[r]));
    }
  nx = (int)upw2(u, x, i, m, 1);
  ny = (int)upw2(u, x, j, n, w);
  ax = x != src && u[x] > u[nx];
  ay = x != src && u[x] > u[ny];
  double d;
  if (x == src) {
    d = 1.0;
  } else {
    // 0 + t is t for the positive t of an upwind axis: the first term needs
    // no addition
    const double tx = ax ? __dmul_rn(2.0, __dsub_rn(u[x], u[nx])) : 0.0;
    const double ty = ay ? __dmul_rn(2.0, __dsub_rn(u[x], u[ny])) : 0.0;
    d = (ax && ay) ? __dadd_rn(tx, ty) : (ax ? tx : ty);
  }
  return fi_div(acc, d);
}

// Users of cell c (bits x-, x+, y-, y+): the non-source neighbours whose
// upwind neighbour along the axis is c; singular: c is not the source and
// has no upwind axis (its row has no diagonal).
__device__ __forceinline__ uint32_t adj2_users(const double* __restrict__ u, int c, int m, int n,
                                               int src, bool& singular) {
  const int w = m + 1;
  const int i = c % w, j = c / w;
  uint32_t us = 0;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const int ri = i + (q == 0 ? -1 : q == 1 ? 1 : 0);
    const int rj = j + (q == 2 ? -1 : q == 3 ? 1 : 0);
    if (ri < 0 || ri > m || rj < 0 || rj > n) continue;
    const int r = rj * w + ri;
    if (r == src) continue;
    const int64_t nb = (q < 2) ? upw2(u, r, ri, m, 1) : upw2(u, r, rj, n, w);
    if (nb == c && u[r] > u[c]) us |= 1u << q;
  }
  singular = c != src && !(u[c] > u[upw2(u, c, i, m, 1)]) && !(u[c] > u[upw2(u, c, j, n, w)]);
  return us;
}

// The 2D adjoint in causal order by levels, one CTA, for grids up to
// ADJ2_SMEM_NODES nodes: the rows of k_eik2d_adjoint solved once, every cell
// after its users (Kahn's algorithm on the users graph, acyclic since a
// user's travel time is strictly larger), one level of the graph per round.
// Round r evaluates the cells queued in round r - 1 (all their users are in
// earlier rounds), clears their bits in their upwind neighbours' flag sets
// and queues the neighbours whose sets empty; a barrier ends the round.
// lambda, the queue and the flags (one byte per cell: users in bits 0-3, not
// yet evaluated in 4-7, four cells to a 32-bit word for the atomics) live in
// dynamic shared memory; with STAGE_U (grids up to ADJ2_STAGE_U_NODES
// nodes) the travel times are copied there as well and the queue holds
// 16-bit cell indices.  The formula and summation order are
// k_eik2d_adjoint's, so lambda is the same, bit for bit.  No thread waits on
// another except at the barriers; the rounds end when one queues nothing.
// status: 1 done, -1 a non-source cell has no upwind direction, 0 cells left
// unevaluated (impossible for travel times from the forward).
template <bool STAGE_U>
__global__ void __launch_bounds__(512)
    k_eik2d_adjoint_levels(const double* __restrict__ gu, const double* __restrict__ u_g,
                           const double* __restrict__ f, int m, int n, double h, int ix, int jx,
                           double* __restrict__ grad_f, int* __restrict__ status) {
  using QT = typename std::conditional<STAGE_U, uint16_t, int>::type;
  extern __shared__ __align__(16) unsigned char adj_smem[];
  __shared__ int s_cnt[3], s_singular;
  const int w = m + 1;
  const int N = (m + 1) * (n + 1);
  const int src = jx * w + ix;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
  double* lam = reinterpret_cast<double*>(adj_smem);
  double* u_s = lam + N;
  const double* u = STAGE_U ? u_s : u_g;
  QT* queue = reinterpret_cast<QT*>(adj_smem + (size_t)N * (STAGE_U ? 16 : 8));
  // 32-bit flag words after the queue, at a multiple of 4 bytes
  uint32_t* word =
      reinterpret_cast<uint32_t*>(adj_smem + ((size_t)N * (STAGE_U ? 18 : 12) + 3) / 4 * 4);
  uint8_t* flag = reinterpret_cast<uint8_t*>(word);
  if (tid == 0) {
    s_cnt[0] = s_cnt[1] = s_cnt[2] = 0;
    s_singular = 0;
  }
  if (STAGE_U)
    for (int p = tid; p < N; p += nth) u_s[p] = u_g[p];
  __syncthreads();
  // level 0: the cells without users
  for (int c0 = warp * 32; c0 < N; c0 += nth) {
    const int c = c0 + lane;
    uint32_t us = 0;
    if (c < N) {
      bool sing;
      us = adj2_users(u, c, m, n, src, sing);
      flag[c] = (uint8_t)(us | (us << 4));
      if (sing) s_singular = 1;
    }
    const int pos = warp_append((c < N && us == 0) ? 1 : 0, &s_cnt[0], lane);
    if (c < N && us == 0) queue[pos] = (QT)c;
  }
  __syncthreads();
  int lo = 0, hi = s_cnt[0];
  if (!s_singular) {
    // round r appends to s_cnt[(r + 1) % 3]; thread 0 clears the counter of
    // round r + 1 before the barrier ending round r (its last readers passed
    // the barrier ending round r - 1)
    for (int r = 0; lo < hi; ++r) {
      int* cnt = &s_cnt[(r + 1) % 3];
      if (tid == 0) s_cnt[(r + 2) % 3] = 0;
      for (int k0 = lo; k0 < hi; k0 += nth) {
        const int k = k0 + tid;
        int rel[2] = {-1, -1}, np = 0;
        if (k < hi) {
          const int x = queue[k];
          int nx, ny;
          bool ax, ay;
          lam[x] = adj2_row(gu, u, lam, x, flag[x] & 15u, m, n, src, nx, ny, ax, ay);
          // release the upwind neighbours this cell is a user of: x+ (1)
          // or x- (0) seen from nx, y+ (3) or y- (2) seen from ny
          const int nbs[2] = {nx, ny};
          const bool act[2] = {ax, ay};
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            if (!act[a]) continue;
            const int nb = nbs[a];
            const int q = a == 0 ? (nb < x ? 1 : 0) : (nb < x ? 3 : 2);
            const int sh = 8 * (nb & 3);
            const uint32_t bit = (1u << (q + 4)) << sh;
            const uint32_t old = atomicAnd(word + (nb >> 2), ~bit);
            if ((old & bit) && !(old & ~bit & (0xf0u << sh))) rel[a] = nb, ++np;
          }
        }
        const int pos = hi + warp_append(np, cnt, lane);
        int o = pos;
        for (int a = 0; a < 2; ++a)
          if (rel[a] >= 0) queue[o++] = (QT)rel[a];
      }
      __syncthreads();
      lo = hi;
      hi += *cnt;
    }
  }
  __syncthreads();
  const bool done = !s_singular && hi == N;
  for (int p = tid; p < N; p += nth) {
    // dFdf = -2 f h h, 0 at the source; grad_f = -lambda * dFdf (Eikonal.h:100-104,196-198)
    const double dfdf = (p == src) ? 0.0 : __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f[p]), h), h);
    grad_f[p] = done ? __dmul_rn(-lam[p], dfdf) : 0.0;
  }
  if (tid == 0) status[0] = s_singular ? -1 : (done ? 1 : 0);
}

// The 2D adjoint in causal order for larger grids, one CTA, without
// barriers: threads take queue slots and wait for their cells (bounded by
// CAUSAL_WAIT_CYCLES); lambda, the queue and the flag sets (one 32-bit word
// per cell: users in bits 0-3, not yet evaluated in 8-11) are global.  Each
// evaluated non-source cell clears its bit in its upwind neighbours' sets
// (acq_rel atomics at CTA scope); the thread that empties a set queues that
// cell (release store; slots are read with acquire loads).  status as
// k_eik2d_adjoint_levels, 0 also when a wait ran out.
__global__ void __launch_bounds__(512)
    k_eik2d_adjoint_causal(const double* __restrict__ gu, const double* __restrict__ u,
                           const double* __restrict__ f, int m, int n, double h, int ix, int jx,
                           double* lam, double* __restrict__ grad_f, uint32_t* word, int* queue,
                           int* __restrict__ status) {
  __shared__ int s_head, s_tail, s_err, s_singular;
  const int w = m + 1;
  const int N = (m + 1) * (n + 1);
  const int src = jx * w + ix;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_head = s_tail = 0;
    s_err = s_singular = 0;
  }
  for (int p = tid; p < N; p += nth) queue[p] = -1;
  __syncthreads();
  // users of each cell, cells without users queued, singular rows found
  for (int c0 = warp * 32; c0 < N; c0 += nth) {
    const int c = c0 + lane;
    uint32_t us = 0;
    if (c < N) {
      bool sing;
      us = adj2_users(u, c, m, n, src, sing);
      word[c] = us | (us << 8);
      if (sing) s_singular = 1;
    }
    const int pos = warp_append((c < N && us == 0) ? 1 : 0, &s_tail, lane);
    if (c < N && us == 0) queue[pos] = c;
  }
  __syncthreads();
  if (!s_singular) {
    for (;;) {
      const int slot = take_slots(1, &s_head);
      if (slot >= N) break;
      int x = ld_acquire_cta(queue + slot);
      if (x < 0) {
        const long long t0 = clock64();
        do {
          __nanosleep(64);
          x = ld_acquire_cta(queue + slot);
        } while (x < 0 && clock64() - t0 < CAUSAL_WAIT_CYCLES &&
                 !*reinterpret_cast<volatile int*>(&s_err));
        if (x < 0) {  // out of budget, or another thread's was
          atomicOr(&s_err, 1);
          break;
        }
      }
      int nx, ny;
      bool ax, ay;
      lam[x] = adj2_row(gu, u, lam, x, word[x] & 15u, m, n, src, nx, ny, ax, ay);
      // release the upwind neighbours this cell is a user of
      int rel[2] = {-1, -1}, np = 0;
      const int nbs[2] = {nx, ny};
      const bool act[2] = {ax, ay};
#pragma unroll
      for (int a = 0; a < 2; ++a) {
        if (!act[a]) continue;
        const int nb = nbs[a];
        // this cell seen from nb: x+ (1) or x- (0), y+ (3) or y- (2)
        const int q = a == 0 ? (nb < x ? 1 : 0) : (nb < x ? 3 : 2);
        const uint32_t bit = (1u << q) << 8;
        const uint32_t old = atom_and_acq_rel_cta(word + nb, ~bit);
        if ((old & bit) && !(old & ~bit & 0xf00u)) {
          rel[a] = nb;
          ++np;
        }
      }
      int pos = take_slots(np, &s_tail);
      for (int a = 0; a < 2; ++a)
        if (rel[a] >= 0) st_release_cta(queue + pos++, rel[a]);
    }
  }
  __syncthreads();
  const bool done = !s_singular && !s_err && s_tail == N;
  for (int p = tid; p < N; p += nth) {
    // dFdf = -2 f h h, 0 at the source; grad_f = -lambda * dFdf (Eikonal.h:100-104,196-198)
    const double dfdf = (p == src) ? 0.0 : __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f[p]), h), h);
    grad_f[p] = done ? __dmul_rn(-lam[p], dfdf) : 0.0;
  }
  if (tid == 0) status[0] = s_singular ? -1 : (done ? 1 : 0);
}

namespace {
// Device workspaces of the 2D solves, kept per device between calls (grown,
// never shrunk); a call holds its device's lock while it uses them.
struct Eik2dWork {
  std::mutex mu;
  DevBuf prev, dirty, cst, stat, lam, word, queue;
};
Eik2dWork& work2d(int dev) {
  static Eik2dWork* w = new Eik2dWork[64];
  return w[dev & 63];
}
}  // namespace

int eik2d_forward_batch(const double* d_f, int m, int n, double h, int count, const int* d_srcx,
                        const int* d_srcy, double* d_u, adt_solve_status* st, cudaStream_t stream) {
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  int dev = 0;
  ADT_CUDA(cudaGetDevice(&dev));
  Eik2dWork& W = work2d(dev);
  std::lock_guard<std::mutex> lock(W.mu);
  ADT_CUDA(W.prev.reserve((size_t)count * N * sizeof(double)));
  ADT_CUDA(W.cst.reserve((size_t)N * sizeof(double2)));
  ADT_CUDA(W.stat.reserve((size_t)count * (2 * sizeof(int) + sizeof(double))));
  double* d_err = W.stat.as<double>();
  int* d_iters = reinterpret_cast<int*>(d_err + count);
  int* d_conv = d_iters + count;
  double2* cst = W.cst.as<double2>();
  k_eik2d_cells<<<(int)std::min<int64_t>((N + 255) / 256, 1024), 256, 0, stream>>>(d_f, N, h, cst);
  ADT_CUDA(cudaGetLastError());
  // a wavefront holds at most min(m, n) + 1 nodes
  const int thr = std::max(64, std::min(512, (std::min(m, n) + 32) / 32 * 32));
  if (N <= FWD2_SMEM_NODES) {
    const int smem = (int)(N * (sizeof(double) + 1));
    ADT_CUDA(cudaFuncSetAttribute(k_eik2d_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  smem));
    k_eik2d_forward<true><<<count, thr, smem, stream>>>(cst, m, n, d_srcx, d_srcy, d_u,
                                                        W.prev.as<double>(), nullptr, d_iters,
                                                        d_conv, d_err);
  } else {
    ADT_CUDA(W.dirty.reserve((size_t)count * N));
    k_eik2d_forward<false><<<count, thr, 0, stream>>>(cst, m, n, d_srcx, d_srcy, d_u,
                                                      W.prev.as<double>(), W.dirty.as<uint8_t>(),
                                                      d_iters, d_conv, d_err);
  }
  ADT_CUDA(cudaGetLastError());
  std::vector<char> hs((size_t)count * (2 * sizeof(int) + sizeof(double)));
  ADT_CUDA(cudaMemcpyAsync(hs.data(), W.stat.p, hs.size(), cudaMemcpyDeviceToHost, stream));
  ADT_CUDA(cudaStreamSynchronize(stream));
  const double* er = reinterpret_cast<const double*>(hs.data());
  const int* it = reinterpret_cast<const int*>(er + count);
  const int* cv = it + count;
  if (st)
    for (int k = 0; k < count; ++k) {
      st[k].iters = it[k];
      st[k].converged = cv[k];
      st[k].final_err = er[k];
      st[k].adj_iters = 0;
      st[k].adj_converged = 0;
    }
  return ADT_OK;
}

int eik2d_adjoint(const double* d_gu, const double* d_u, const double* d_f, int m, int n, double h,
                  int ix, int jx, double* d_gf, cudaStream_t stream) {
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  int dev = 0;
  ADT_CUDA(cudaGetDevice(&dev));
  Eik2dWork& W = work2d(dev);
  std::lock_guard<std::mutex> lock(W.mu);
  ADT_CUDA(W.lam.reserve((size_t)N * sizeof(double)));
  ADT_CUDA(W.stat.reserve(sizeof(int)));
  int* d_stat = W.stat.as<int>();
  if (N <= ADJ2_STAGE_U_NODES) {  // causal order by levels, travel times staged
    const int smem = (int)((N * 18 + 3) / 4 * 4 + (N + 3) / 4 * 4);
    ADT_CUDA(cudaFuncSetAttribute(k_eik2d_adjoint_levels<true>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    k_eik2d_adjoint_levels<true><<<1, 256, smem, stream>>>(d_gu, d_u, d_f, m, n, h, ix, jx, d_gf,
                                                           d_stat);
  } else if (N <= ADJ2_SMEM_NODES) {  // causal order by levels
    const int smem = (int)(N * 12 + (N + 3) / 4 * 4);
    ADT_CUDA(cudaFuncSetAttribute(k_eik2d_adjoint_levels<false>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    k_eik2d_adjoint_levels<false><<<1, 256, smem, stream>>>(d_gu, d_u, d_f, m, n, h, ix, jx, d_gf,
                                                            d_stat);
  } else if (N < (1 << 30)) {  // causal order: every cell once
    ADT_CUDA(W.word.reserve((size_t)N * sizeof(uint32_t)));
    ADT_CUDA(W.queue.reserve((size_t)N * sizeof(int)));
    k_eik2d_adjoint_causal<<<1, 512, 0, stream>>>(d_gu, d_u, d_f, m, n, h, ix, jx,
                                                  W.lam.as<double>(), d_gf, W.word.as<uint32_t>(),
                                                  W.queue.as<int>(), d_stat);
  } else {
    k_eik2d_adjoint<<<1, 256, 0, stream>>>(d_gu, d_u, d_f, m, n, h, ix, jx, W.lam.as<double>(),
                                           d_gf, d_stat);
  }
  ADT_CUDA(cudaGetLastError());
  int s = 0;
  ADT_CUDA(cudaMemcpyAsync(&s, d_stat, sizeof(int), cudaMemcpyDeviceToHost, stream));
  ADT_CUDA(cudaStreamSynchronize(stream));
  if (s < 0) return set_error(ADT_ESINGULAR, "2D adjoint: a non-source cell has no upwind direction");
  if (s == 0) return set_error(ADT_ENOCONV, "2D adjoint did not complete");
  return ADT_OK;
}

}  // namespace adt
