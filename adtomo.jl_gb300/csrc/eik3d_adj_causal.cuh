// eik3d_adj_causal.cuh -- the batched plan's adjoint solved once, in causal
// order, instead of by sweeps until nothing changes.
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
// One CTA runs one solve at a time (solves from the chunk's work counter):
//  - pass 1 forms the side codes and fixed cells, pass 2 the user bits (the
//    same code passes as the sweeping adjoint) and, per cell, a byte of the
//    user bits still outstanding (REM_FIXED for a fixed cell, never released);
//  - the cells without users are frontier 0 in the solve's queue;
//  - round r evaluates frontier r.  Each evaluated cell clears its bit in the
//    byte of each upwind neighbour (atomicAnd on the word of four bytes), and
//    the thread whose clear empties a byte appends that cell to frontier
//    r + 1; a CTA barrier ends the round, which publishes the round's adjoint
//    values and queue entries to the next.
// On the 128x128x64 layered + checkerboard workload a solve takes about 350
// rounds of about 3000 cells (2.9 users per cell).
//
// A cell is evaluated with the sweeping adjoint's formula, the same
// operations in the same order (FP32: adj_cell_f32 and the sweep step; FP64:
// sweep_brick_adj's exact form, which the oracle follows), so the result is
// the sweeps' exact fixed point, bit for bit (up to the sign of a zero), with
// one evaluation per cell instead of one per sweep that reaches it.
#pragma once
#include "eik3d_batch_kernels.cuh"

// Threads per CTA the kernel is compiled for: FP32 1024 (64 registers, two
// 512-thread solves per SM), FP64 512 (its doubles need more registers).
#ifndef ADT_CAUSAL_MAXT
#define ADT_CAUSAL_MAXT 1024
#endif
#define ADT_CAUSAL_BOUNDS(T) __launch_bounds__(sizeof(T) == 8 ? ADT_CAUSAL_MAXT / 2 : ADT_CAUSAL_MAXT)

namespace adt {

struct CausalShared {
  int q;
  int cnt[3];    // frontier sizes: frontier r's in cnt[r % 3]
  int nonfixed;  // non-fixed cells of the running solve (each is evaluated once)
  int pad;
};

// All 32 lanes call with their entry counts; returns this lane's first slot
// in a list whose length is counted in *len (one shared atomic per warp).
__device__ __forceinline__ int warp_append(int np, int* len, int lane) {
  int incl = np;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int v = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += v;
  }
  const int total = __shfl_sync(0xffffffffu, incl, 31);
  int wb = 0;
  if (lane == 31 && total) wb = atomicAdd(len, total);
  wb = __shfl_sync(0xffffffffu, wb, 31);
  return wb + incl - np;
}

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

// The adjoint value of one non-fixed cell from its neighbours (un: x-, x+,
// y-, y+, z-, z+; +inf off the grid) and its users' adjoint values (ln, 0
// for a neighbour that is not a user); gs: the seed value (0 without one).
// FP32: lambda = fma(P_x + P_y, c2, fma(P_z, c2, c0)), P_a = fma(w_{a+},
// lambda_{a+}, w_{a-} lambda_{a-}), c2 = rcp(d), c0 = 0.5 g c2 -- the
// sweeping adjoint's order for every sweep direction (adj_cell_f32).
// FP64: (g + sum_users 2 (u_r - u_c) lambda_r) / sum_sides 2 (u_c - u_side)
// in the oracle's order (sweep_brick_adj with EXACT).
template <class T>
__device__ __forceinline__ T causal_lambda(uint32_t cd, T uc, const T (&un)[6], const T (&ln)[6],
                                           T gs) {
  if constexpr (sizeof(T) == 4) {
    const uint32_t us = cd >> CODE_USERS;
    float w[6];
#pragma unroll
    for (int q = 0; q < 6; ++q) w[q] = ((us >> q) & 1u) ? un[q] - uc : 0.0f;
    const float px = fmaf(w[1], ln[1], w[0] * ln[0]);
    const float py = fmaf(w[3], ln[3], w[2] * ln[2]);
    const float pz = fmaf(w[5], ln[5], w[4] * ln[4]);
    float d = fmaxf(uc - fminf(un[0], un[1]), 0.0f);
    d += fmaxf(uc - fminf(un[2], un[3]), 0.0f);
    d += fmaxf(uc - fminf(un[4], un[5]), 0.0f);
    const float c2 = rcp_approx(d);
    const float c0 = 0.5f * gs * c2;
    return fmaf(px + py, c2, fmaf(pz, c2, c0));
  } else {
    double acc = gs;
#pragma unroll
    for (int q = 0; q < 6; ++q)
      if (cd & (1u << (CODE_USERS + q)))
        acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(2.0, __dsub_rn(un[q], uc)), ln[q]));
    double d = 0.0;
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
      const uint32_t side = (cd >> (2 * ax)) & 3u;
      if (side) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(uc, side == 1 ? un[2 * ax] : un[2 * ax + 1])));
    }
    return __ddiv_rn(acc, d);
  }
}

// NB: queue entries per thread per pass over a frontier (their loads are
// issued together).
template <class T, int NB>
__global__ void ADT_CAUSAL_BOUNDS(T) k_batch_adj_causal(BatchArgs<T> A) {
  __shared__ CausalShared S;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
  const int nwarps = nth >> 5;
  unsigned long long upd = 0;
  int q = blockIdx.x;
  while (q < A.n_solves) {
    const int gsol = A.order[q];
    const SolveDev& sd = A.solves[gsol];
    const FieldDev<T> fd = A.fields[sd.field];
    const Geom g = fd.g;
    const T* __restrict__ u = A.u + sd.u_off;
    T* lam = A.lam + sd.u_off;
    uint16_t* code = A.code + sd.u_off;
    uint32_t* rem = A.rem + (sd.u_off >> 2);  // u_off is a multiple of 16
    uint8_t* rem8 = reinterpret_cast<uint8_t*>(rem);
    int* queue = A.queue + sd.u_off;
    const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
    const int ncell = (int)g.ncell;
    const bool vec4 = sizeof(T) == 4 && (g.l % 4) == 0;
    if (tid == 0) {
      S.cnt[0] = S.cnt[1] = S.cnt[2] = 0;
      S.nonfixed = 0;
    }
    // pass 1: upwind sides and fixed cells; lambda = 0
    if constexpr (sizeof(T) == 4) {
      if (vec4)
        for (int e = tid; e < ncell / 4; e += nth) {
          const int64_t col = e / (g.l / 4);
          const int i = (int)(col / g.n), j = (int)(col % g.n), k = (int)(4 * (int64_t)e - col * g.l);
          p1_store(p1_load(u, g, 4 * (int64_t)e, i, j, k), code, lam, sd, 4 * (int64_t)e, i, j, k);
        }
    }
    if (!vec4)
      for (int64_t col = warp; col < (int64_t)g.m * g.n; col += nwarps) {
        const int i = (int)(col / g.n), j = (int)(col % g.n);
        for (int k = lane; k < g.l; k += 32) {
          const int64_t x = col * g.l + k;
          const T uc = u[x];
          const int sx = upwind_side_t(u, x, i, g.m, sI, uc);
          const int sy = upwind_side_t(u, x, j, g.n, sJ, uc);
          const int sz = upwind_side_t(u, x, k, g.l, (int64_t)1, uc);
          uint16_t cd = (uint16_t)(sx | (sy << 2) | (sz << 4));
          if (uc == (T)u0_at(sd, i, j, k) || (sx | sy | sz) == 0) cd = CODE_FIXED;
          code[x] = cd;
          lam[x] = T(0);
        }
      }
    __syncthreads();
    // pass 2: user bits, outstanding-user bytes, frontier 0 (the cells nobody
    // uses).  Warp-uniform loops (warp_append needs all lanes).
    int nf = 0;
    if (vec4) {
      for (int e0 = warp * 32; e0 < ncell / 4; e0 += nth) {
        const int e = e0 + lane;
        uint32_t bytes = 0x80808080u;
        if (e < ncell / 4) {
          const int64_t col = e / (g.l / 4);
          const int i = (int)(col / g.n), j = (int)(col % g.n), k = (int)(4 * (int64_t)e - col * g.l);
          bytes = p2_store(p2_load(code, g, 4 * (int64_t)e, i, j, k), code, 4 * (int64_t)e);
          rem[e] = bytes;
        }
        int np = 0;
#pragma unroll
        for (int b = 0; b < 4; ++b) {
          const uint32_t by = (bytes >> (8 * b)) & 0xffu;
          np += by == 0u;
          nf += by != REM_FIXED;
        }
        int pos = warp_append(np, &S.cnt[0], lane);
#pragma unroll
        for (int b = 0; b < 4; ++b)
          if (((bytes >> (8 * b)) & 0xffu) == 0u) queue[pos++] = 4 * e + b;
      }
    } else {
      for (int x0 = warp * 32; x0 < ncell; x0 += nth) {
        const int x = x0 + lane;
        uint32_t by = REM_FIXED;
        if (x < ncell) {
          int i, j, k;
          cell_ijk((uint32_t)x, g, fd.div_nl, fd.div_l, i, j, k);
          const uint16_t cd = code[x];
          if (!(cd & CODE_FIXED)) {
            uint32_t us = 0;
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
            // only the high bits change: a neighbour reading this code
            // concurrently sees the same side bits either way
            code[x] = (uint16_t)(cd | (us << CODE_USERS));
            by = us;
          }
          rem8[x] = (uint8_t)by;
        }
        nf += by != REM_FIXED;
        const int pos = warp_append(by == 0u ? 1 : 0, &S.cnt[0], lane);
        if (by == 0u) queue[pos] = x;
      }
    }
    nf = __reduce_add_sync(0xffffffffu, nf);
    if (lane == 0 && nf) atomicAdd(&S.nonfixed, nf);
    __syncthreads();
    // seeds: mark the seeded non-fixed cells
    const int ns = A.n_seed[sd.gidx];
    const int64_t* sidx = A.seed_idx + sd.seed_off;
    const T* sval = A.seed_val + sd.seed_off;
    for (int e = tid; e < ns; e += nth) {
      const int64_t x = sidx[e];
      const uint16_t cd = code[x];
      if (!(cd & CODE_FIXED)) code[x] = (uint16_t)(cd | CODE_SEED);
    }
    __syncthreads();
    // rounds
    const T INF = inf_value<T>();
    const int st3[3] = {(int)sI, (int)sJ, 1};
    int base = 0;
    for (int r = 0;; ++r) {
      const int size = S.cnt[r % 3];
      if (size == 0) break;
      if (tid == 0) S.cnt[(r + 2) % 3] = 0;  // frontier r - 1's, read by all before the last barrier
      int* len = &S.cnt[(r + 1) % 3];
      const int nbase = base + size;
      for (int e0 = 0; e0 < size; e0 += NB * nth) {
        int x[NB];
        bool ok[NB];
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          const int e = e0 + b * nth + tid;
          ok[b] = e < size;
          x[b] = ok[b] ? queue[base + e] : 0;
        }
        uint32_t cd[NB];
        T uc[NB], un[NB][6];
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          cd[b] = 0u;
          uc[b] = T(0);
#pragma unroll
          for (int t = 0; t < 6; ++t) un[b][t] = INF;
          if (ok[b]) {
            int i, j, k;
            cell_ijk((uint32_t)x[b], g, fd.div_nl, fd.div_l, i, j, k);
            const T* p = u + x[b];
            cd[b] = code[x[b]];
            uc[b] = __ldg(p);
            if (i > 0) un[b][0] = __ldg(p - sI);
            if (i < g.m - 1) un[b][1] = __ldg(p + sI);
            if (j > 0) un[b][2] = __ldg(p - sJ);
            if (j < g.n - 1) un[b][3] = __ldg(p + sJ);
            if (k > 0) un[b][4] = __ldg(p - 1);
            if (k < g.l - 1) un[b][5] = __ldg(p + 1);
          }
        }
        // release the upwind neighbours (their outstanding bit for this cell)
        uint32_t rel = 0;
        int np = 0;
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
          for (int a = 0; a < 3; ++a) {
            const uint32_t side = (cd[b] >> (2 * a)) & 3u;
            if (side) {
              const int tq = x[b] + (side == 1 ? -st3[a] : st3[a]);
              const uint32_t bit = side == 1 ? (2u << (2 * a)) : (1u << (2 * a));
              const uint32_t sh = 8u * ((uint32_t)tq & 3u);
              const uint32_t old = atomicAnd_block(rem + (tq >> 2), ~(bit << sh));
              const uint32_t ob = (old >> sh) & 0xffu;
              if ((ob & bit) && !(ob & ~bit)) {
                rel |= 1u << (3 * b + a);
                ++np;
              }
            }
          }
        // the users' adjoint values (final: evaluated in earlier rounds)
        T ln[NB][6];
#pragma unroll
        for (int b = 0; b < NB; ++b) {
          const uint32_t us = cd[b] >> CODE_USERS;
#pragma unroll
          for (int t = 0; t < 6; ++t) {
            const int off = (t & 1 ? 1 : -1) * st3[t >> 1];
            ln[b][t] = ((us >> t) & 1u) ? lam[x[b] + off] : T(0);
          }
        }
#pragma unroll
        for (int b = 0; b < NB; ++b)
          if (ok[b]) {
            T gs = T(0);
            if (cd[b] & CODE_SEED) {
              if constexpr (sizeof(T) == 4)
                gs = A.gdense ? A.gdense[sd.u_off + x[b]] : seed_lookup(sidx, sval, ns, (int64_t)x[b]);
              else
                gs = seed_lookup(sidx, sval, ns, (int64_t)x[b]);
            }
            lam[x[b]] = causal_lambda<T>(cd[b], uc[b], un[b], ln[b], gs);
          }
        int pos = nbase + warp_append(np, len, lane);
#pragma unroll
        for (int b = 0; b < NB; ++b)
#pragma unroll
          for (int a = 0; a < 3; ++a)
            if ((rel >> (3 * b + a)) & 1u) {
              const uint32_t side = (cd[b] >> (2 * a)) & 3u;
              queue[pos++] = x[b] + (side == 1 ? -st3[a] : st3[a]);
            }
      }
      __syncthreads();
      base = nbase;
    }
    if (A.gdense)  // leave the dense seed field all zero for the next evaluation
      for (int e = tid; e < ns; e += nth) A.gdense[sd.u_off + sidx[e]] = T(0);
    if (tid == 0) {
      adt_solve_status& st = A.status[sd.gidx];
      st.adj_iters = 1;
      st.adj_converged = base == S.nonfixed ? 1 : 0;  // else the users graph had a cycle
      upd += (unsigned long long)base;
      S.q = atomicAdd(A.next, 1) + (int)gridDim.x;
    }
    __syncthreads();
    q = S.q;
    __syncthreads();  // S.q read by all before the next solve's tid 0 writes S
  }
  if (tid == 0 && upd) atomicAdd(&A.counters[2], upd);
}

}  // namespace adt
