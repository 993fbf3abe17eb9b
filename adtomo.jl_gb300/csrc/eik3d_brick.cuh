// eik3d_brick.cuh -- one warp sweeps one brick of the 3D grid.
//
// A brick is 8 (i) x 4 (j) columns x BK cells along k.  Lane L owns column
// (li, lj) = (L >> 2, L & 3), mirrored so that the sweep direction always
// runs from lane 0 outwards, and walks its column in the sweep's k direction
// with a skew of s = li + lj steps.  At step tau every lane updates the cell
// at k' = tau - s, so the 32 cells of a step lie on one local hyperplane
// i + j + k = const of the ordering: a cell's upstream neighbours (one index
// back along each axis) were updated at the previous step and its downstream
// neighbours not yet -- exactly the Gauss-Seidel data flow of the reference's
// lexicographic loop (Eikonal3D.cpp:35-57).  Bricks are visited in any order
// that respects the same dependencies (brick levels bx+by+bz), so the result
// is the reference's, bit for bit, when the per-cell arithmetic is.
//
// The brick and a one-cell halo are staged in shared memory with cp.async
// (layout in adt_common.cuh, bank-conflict-free for every ordering); the
// interior is written back with coalesced stores.
#pragma once
#include "adt_common.cuh"
#include "eik_local.cuh"

namespace adt {

constexpr int SKEW = (BI - 1) + (BJ - 1);

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

template <class T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src);
template <>
__device__ __forceinline__ void cp_async_elem<float>(float* dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(dst)), "l"(src));
}
template <>
__device__ __forceinline__ void cp_async_elem<double>(double* dst, const double* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem_u32(dst)), "l"(src));
}
template <>
__device__ __forceinline__ void cp_async_elem<uint16_t>(uint16_t* dst, const uint16_t* src) {
  *dst = *src;  // 2-byte copies are not supported by cp.async
}
__device__ __forceinline__ void cp_async_wait_all() {
  asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Position of one brick for one ordering.
struct BrickPos {
  int i0, j0, k0;  // first node
  int ni, nj, nk;  // valid extents (<= BI, BJ, BK)
  int bx, by, bz;  // actual brick coordinates
};

template <int BK>
__device__ __forceinline__ BrickPos brick_pos(const Geom& g, uint32_t packed, int si, int sj,
                                              int sk) {
  int rx, ry, rz;
  unpack_brick(packed, rx, ry, rz);
  BrickPos p;
  p.bx = si > 0 ? rx : g.nbx - 1 - rx;
  p.by = sj > 0 ? ry : g.nby - 1 - ry;
  p.bz = sk > 0 ? rz : g.nbz - 1 - rz;
  p.i0 = p.bx * BI;
  p.j0 = p.by * BJ;
  p.k0 = p.bz * BK;
  p.ni = min(BI, g.m - p.i0);
  p.nj = min(BJ, g.n - p.j0);
  p.nk = min(BK, g.l - p.k0);
  return p;
}

// Stage a brick and its in-grid halo (faces only) into the tile S.
// Out-of-grid halo slots are never read (edge rule redirects to the interior
// neighbour), so they are left untouched.
template <class T, int BK>
__device__ __forceinline__ void load_halo_tile(T* S, const T* __restrict__ src, const Geom& g,
                                               const BrickPos& p, int CS, int lane) {
  constexpr int RS = tile_row_stride(BK);
  for (int col = 0; col < (BI + 2) * (BJ + 2); ++col) {
    const int ci = col / (BJ + 2), cj = col - ci * (BJ + 2);
    const bool hx = (ci == 0 || ci == BI + 1), hy = (cj == 0 || cj == BJ + 1);
    if (hx && hy) continue;  // corner columns are not neighbours of any cell
    const int i = p.i0 + ci - 1, j = p.j0 + cj - 1;
    if (i < 0 || i >= g.m || j < 0 || j >= g.n) continue;
    if (!hx && !hy && (ci > p.ni || cj > p.nj)) continue;
    const T* gcol = src + ((int64_t)i * g.n + j) * g.l + p.k0;
    T* scol = S + ci * RS + cj * CS + 1;
    for (int kk = lane; kk < p.nk; kk += 32) cp_async_elem(scol + kk, gcol + kk);
    if (!hx && !hy) {  // k halo of interior columns
      if (lane == 0 && p.k0 > 0) cp_async_elem(scol - 1, gcol - 1);
      if (lane == 1 && p.k0 + BK < g.l) cp_async_elem(scol + BK, gcol + BK);
    }
  }
}

// Stage the interior of a brick (no halo) into an interior tile.
template <class T, int BK>
__device__ __forceinline__ void load_interior(T* S, const T* __restrict__ src, const Geom& g,
                                              const BrickPos& p, int CS, int lane) {
  constexpr int IRS = itile_row_stride(BK);
  for (int col = 0; col < BI * BJ; ++col) {
    const int ci = col / BJ, cj = col - ci * BJ;
    if (ci >= p.ni || cj >= p.nj) continue;
    const T* gcol = src + ((int64_t)(p.i0 + ci) * g.n + (p.j0 + cj)) * g.l + p.k0;
    T* scol = S + ci * IRS + cj * CS;
    for (int kk = lane; kk < p.nk; kk += 32) cp_async_elem(scol + kk, gcol + kk);
  }
}

// Write the interior of a halo tile back to global memory.
template <class T, int BK>
__device__ __forceinline__ void store_interior(const T* S, T* __restrict__ dst, const Geom& g,
                                               const BrickPos& p, int CS, int lane) {
  constexpr int RS = tile_row_stride(BK);
  for (int col = 0; col < BI * BJ; ++col) {
    const int ci = col / BJ, cj = col - ci * BJ;
    if (ci >= p.ni || cj >= p.nj) continue;
    T* gcol = dst + ((int64_t)(p.i0 + ci) * g.n + (p.j0 + cj)) * g.l + p.k0;
    const T* scol = S + (ci + 1) * RS + (cj + 1) * CS + 1;
    for (int kk = lane; kk < p.nk; kk += 32) gcol[kk] = scol[kk];
  }
}

// Zero the interior + halo of a tile (used for lambda of never-touched bricks).
template <class T, int BK>
__device__ __forceinline__ void zero_tile(T* S, int lane) {
  for (int e = lane; e < tile_elems(BK); e += 32) S[e] = T(0);
}

// Source box for the FP64 near-source update of the FP32 path.
struct NearBox {
  int i0, i1, j0, j1, k0, k1;  // inclusive; empty when i0 > i1
  __device__ __forceinline__ bool hits(const BrickPos& p) const {
    return !(i1 < p.i0 || i0 >= p.i0 + p.ni || j1 < p.j0 || j0 >= p.j0 + p.nj || k1 < p.k0 ||
             k0 >= p.k0 + p.nk);
  }
  __device__ __forceinline__ bool has(int i, int j, int k) const {
    return i >= i0 && i <= i1 && j >= j0 && j <= j1 && k >= k0 && k <= k1;
  }
};

enum SweepMode { MODE_EXACT = 0, MODE_STABLE = 1 };

// Forward sweep of one staged brick.  Returns the per-lane largest decrease
// and whether any cell changed (any lane).
template <class T, int BK, int MODE>
__device__ __forceinline__ bool sweep_brick_fwd(T* S, const T* F, const Geom& g, const BrickPos& p,
                                                int si, int sj, int sk, int CS, T h, double hd,
                                                const NearBox& nb, bool near, int lane,
                                                T& maxdec) {
  constexpr int RS = tile_row_stride(BK);
  constexpr int IRS = itile_row_stride(BK);
  const int li = lane >> 2, lj = lane & 3;
  const int pi = si > 0 ? li : BI - 1 - li;
  const int pj = sj > 0 ? lj : BJ - 1 - lj;
  const int s = li + lj;
  const int i = p.i0 + pi, j = p.j0 + pj;
  const bool colok = (pi < p.ni) && (pj < p.nj);
  const int own = (pi + 1) * RS + (pj + 1) * CS + 1;
  // one-sided neighbour at the grid edge (Eikonal3D.cpp:47-52): read the
  // interior neighbour twice
  const int oxm = own + ((i == 0) ? RS : -RS);
  const int oxp = own + ((i == g.m - 1) ? -RS : RS);
  const int oym = own + ((j == 0) ? CS : -CS);
  const int oyp = own + ((j == g.n - 1) ? -CS : CS);
  const int fo = pi * IRS + pj * CS;
  bool changed = false;
#pragma unroll 2
  for (int tau = 0; tau < BK + SKEW; ++tau) {
    const int kk = tau - s;
    const int k = sk > 0 ? kk : BK - 1 - kk;
    if (colok && kk >= 0 && kk < BK && k < p.nk) {
      const int kg = p.k0 + k;
      const T uo = S[own + k];
      const T ax = rmin(S[oxp + k], S[oxm + k]);
      const T ay = rmin(S[oyp + k], S[oym + k]);
      const T az = rmin(S[own + k + ((kg == g.l - 1) ? -1 : 1)], S[own + k + ((kg == 0) ? 1 : -1)]);
      const T fc = F[fo + k];
      T un;
      if (MODE == MODE_EXACT) {
        un = (T)upd3_exact((double)ax, (double)ay, (double)az, (double)fc, hd);
      } else {
        if (near && nb.has(i, j, kg))
          un = (T)upd3_stable<double>((double)ax, (double)ay, (double)az, (double)fc * hd);
        else
          un = upd3_stable<T>(ax, ay, az, fc * h);
      }
      const T v = rmin(un, uo);
      S[own + k] = v;
      if (!(v == uo)) {
        changed = true;
        const T d = uo - v;
        maxdec = (d > maxdec) ? d : maxdec;
      }
    }
    __syncwarp();
  }
  return __any_sync(0xffffffffu, changed);
}

// Adjoint sweep of one staged brick: lambda_c = (g_c + sum_users 2 (u_r - u_c)
// lambda_r) / d_c with d_c = sum_active 2 (u_c - u_upwind), fixed cells keep
// lambda = 0 (Eikonal3D.cpp:113-196 solved by reverse sweeps; Eikonal.h:95-200
// in 2D).  The summation order (x-, x+, y-, y+, z-, z+; diagonal x, y, z)
// matches the oracle.  G is the dense seed tile (DENSE) or the solve's sorted
// seed list (idx/val, n_seed) otherwise.
template <class T, int BK, bool EXACT, bool DENSE>
__device__ __forceinline__ bool sweep_brick_adj(const T* U, T* L, const uint16_t* CODE, const T* G,
                                                const int64_t* seed_idx, const T* seed_val,
                                                int n_seed, const Geom& g, const BrickPos& p,
                                                int si, int sj, int sk, int CS, int lane) {
  constexpr int RS = tile_row_stride(BK);
  constexpr int IRS = itile_row_stride(BK);
  const int li = lane >> 2, lj = lane & 3;
  const int pi = si > 0 ? li : BI - 1 - li;
  const int pj = sj > 0 ? lj : BJ - 1 - lj;
  const int s = li + lj;
  const bool colok = (pi < p.ni) && (pj < p.nj);
  const int own = (pi + 1) * RS + (pj + 1) * CS + 1;
  const int io = pi * IRS + pj * CS;
  const int64_t gcol = ((int64_t)(p.i0 + pi) * g.n + (p.j0 + pj)) * g.l + p.k0;
  const int nstep[6] = {-RS, RS, -CS, CS, -1, 1};
  bool changed = false;
#pragma unroll 1
  for (int tau = 0; tau < BK + SKEW; ++tau) {
    const int kk = tau - s;
    const int k = sk > 0 ? kk : BK - 1 - kk;
    if (colok && kk >= 0 && kk < BK && k < p.nk) {
      const uint16_t code = CODE[io + k];
      if (!(code & CODE_FIXED)) {
        const int a = own + k;
        const T uc = U[a];
        T acc = T(0);
        if (code & CODE_SEED) {
          if (DENSE) {
            acc = G[io + k];
          } else {
            const int64_t key = gcol + k;
            int lo = 0, hi = n_seed - 1;
            while (lo < hi) {
              const int mid = (lo + hi) >> 1;
              if (seed_idx[mid] < key) lo = mid + 1; else hi = mid;
            }
            acc = seed_val[lo];
          }
        }
#pragma unroll
        for (int q = 0; q < 6; ++q) {
          if (code & (1u << (CODE_USERS + q))) {
            const int r = a + nstep[q];
            if (EXACT)
              acc = (T)__dadd_rn((double)acc,
                                 __dmul_rn(__dmul_rn(2.0, __dsub_rn((double)U[r], (double)uc)),
                                           (double)L[r]));
            else
              acc += T(2) * (U[r] - uc) * L[r];
          }
        }
        T d = T(0);
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          const int side = (code >> (2 * ax)) & 3;
          if (side) {
            const T uu = U[a + (side == 1 ? nstep[2 * ax] : nstep[2 * ax + 1])];
            if (EXACT)
              d = (T)__dadd_rn((double)d, __dmul_rn(2.0, __dsub_rn((double)uc, (double)uu)));
            else
              d += T(2) * (uc - uu);
          }
        }
        const T lam = EXACT ? (T)__ddiv_rn((double)acc, (double)d) : acc / d;
        if (!(lam == L[a])) {
          L[a] = lam;
          changed = true;
        }
      }
    }
    __syncwarp();
  }
  return __any_sync(0xffffffffu, changed);
}

template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const T w = __shfl_xor_sync(0xffffffffu, v, o);
    v = (w > v) ? w : v;
  }
  return v;
}

}  // namespace adt
