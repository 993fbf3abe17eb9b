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

// MODE_EXACT_CST: the exact update with F holding f h per cell and the next
// interior tile (F + itile_elems(BK)) f f h h.
enum SweepMode { MODE_EXACT = 0, MODE_STABLE = 1, MODE_EXACT_CST = 2 };

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
      // the exact modes (FP64) select by integer compares (travel times are
      // never NaN; fp64_int.cuh), off the FP64 unit
      auto tmin = [](T x, T y) -> T {
        if constexpr (MODE != MODE_STABLE) return min_nn(x, y);
        else return rmin(x, y);
      };
      const T ax = tmin(S[oxp + k], S[oxm + k]);
      const T ay = tmin(S[oyp + k], S[oym + k]);
      const T az = tmin(S[own + k + ((kg == g.l - 1) ? -1 : 1)], S[own + k + ((kg == 0) ? 1 : -1)]);
      const T fc = F[fo + k];
      T un;
      if (MODE == MODE_EXACT) {
        un = (T)upd3_exact((double)ax, (double)ay, (double)az, (double)fc, hd);
      } else if (MODE == MODE_EXACT_CST) {
        un = (T)upd3_exact_fh((double)ax, (double)ay, (double)az, (double)fc,
                              (double)F[fo + k + itile_elems(BK)]);
      } else {
        if (near && nb.has(i, j, kg))
          un = (T)upd3_stable<double>((double)ax, (double)ay, (double)az, (double)fc * hd);
        else
          un = upd3_stable<T>(ax, ay, az, fc * h);
      }
      const T v = tmin(un, uo);
      S[own + k] = v;
      bool same;
      if constexpr (MODE != MODE_STABLE) same = eq_nn(v, uo);
      else same = v == uo;
      if (!same) {
        changed = true;
        const T d = uo - v;
        maxdec = (d > maxdec) ? d : maxdec;
      }
    }
    __syncwarp();
  }
  return __any_sync(0xffffffffu, changed);
}

// ---------------------------------------------------------------------------
// FP32 staging for grids whose k extent is a multiple of 4 (every brick
// column segment starts on a 16-byte boundary).  The 56 columns of a halo
// tile (32 interior, 24 face columns) are split into 4-float chunks; lane t
// takes chunks t, t+32, ...  Out-of-grid cells of the halo are written as
// `ghost`: +inf for travel times, so min(neighbour pair) falls back to the
// single interior neighbour exactly as the reference's edge rule does, and 0
// for adjoint variables, whose ghosts are only ever multiplied by a zero
// weight.  Travel times, adjoint variables and codes are written during the
// kernel by other warps, so they are read through the coherent path (cp.async
// and ordinary loads), never the read-only one.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void halo_col(int c, int& ci, int& cj) {
  if (c < BI * BJ) {  // interior
    ci = (c >> 2) + 1;
    cj = (c & 3) + 1;
  } else {
    const int h = c - BI * BJ;  // 0..23
    if (h < 8) {                // x faces
      ci = (h < 4) ? 0 : BI + 1;
      cj = (h & 3) + 1;
    } else {  // y faces, the two faces of a row interleaved: consecutive columns of one
              // staging copy then start in different bank residues (2-way instead of
              // 4-way conflicts; all-equal residues within a face)
      const int q = h - 8;
      ci = (q >> 1) + 1;
      cj = (q & 1) ? BJ + 1 : 0;
    }
  }
}

template <int BK>
__device__ __forceinline__ void store_interior_f32_vec(const float* S, float* __restrict__ dst,
                                                       const Geom& g, const BrickPos& p, int CS,
                                                       int lane) {
  constexpr int RS = tile_row_stride(BK);
  constexpr int CH = BK / 4;
  constexpr int PER = BI * BJ * CH / 32;
  if constexpr (BK == 32) {
    if (p.ni == BI && p.nj == BJ && p.nk == BK) {  // full brick: same copies, no checks
      const int gq = lane >> 3, k = 4 * (lane & 7);
      const int64_t nl = (int64_t)g.n * g.l;
      float* dp = dst + ((int64_t)p.i0 * g.n + (p.j0 + gq)) * g.l + p.k0 + k;
      const float* s = S + RS + (gq + 1) * CS + 1 + k;
#pragma unroll
      for (int t = 0; t < BI; ++t) {
        const float* st = s + t * RS;
        *reinterpret_cast<float4*>(dp) = make_float4(st[0], st[1], st[2], st[3]);
        dp += nl;
      }
      return;
    }
  }
#pragma unroll
  for (int t = 0; t < PER; ++t) {
    const int e = lane + 32 * t;
    const int c = e / CH, ch = e - (e / CH) * CH;
    const int ci = c >> 2, cj = c & 3, k = 4 * ch;
    if (ci < p.ni && cj < p.nj && k < p.nk) {
      const float* s = S + (ci + 1) * RS + (cj + 1) * CS + 1 + k;
      *reinterpret_cast<float4*>(dst + ((int64_t)(p.i0 + ci) * g.n + (p.j0 + cj)) * g.l + p.k0 +
                                 k) = make_float4(s[0], s[1], s[2], s[3]);
    }
  }
}

// Asynchronous staging (cp.async, 4 bytes per copy): every element of a tile
// is requested before any is waited for, so a brick pays the load latency
// once instead of once per batch of register loads.  The padded tile layout
// (odd column stride) rules out 16-byte copies; out-of-grid ghosts are plain
// shared stores.  The caller waits with cp_async_wait_all() + __syncwarp().
__device__ __forceinline__ void cp_async4(uint32_t dst, const float* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void sts4(uint32_t dst, float v) {
  asm volatile("st.shared.f32 [%0], %1;\n" ::"r"(dst), "f"(v) : "memory");
}

template <int BK>
__device__ __forceinline__ void load_tile_f32_async(float* S, const float* src, const Geom& g,
                                                    const BrickPos& p, int CS, int lane,
                                                    float ghost = INFINITY) {
  constexpr int RS = tile_row_stride(BK);
  constexpr int CH = BK / 4;
  constexpr int NCOL = BI * BJ + 2 * BI + 2 * BJ;  // 56
  constexpr int PER = NCOL * CH / 32;              // chunks per lane (exact)
  static_assert(NCOL * CH % 32 == 0, "tile chunking");
  const uint32_t s0 = smem_u32(S);
  {  // k halo of the interior columns (lane c takes interior column c)
    const int hci = (lane >> 2) + 1, hcj = (lane & 3) + 1;
    const int i = p.i0 + hci - 1, j = p.j0 + hcj - 1;
    const uint32_t d = s0 + 4u * (uint32_t)(hci * RS + hcj * CS);
    const bool in = i < g.m && j < g.n;
    const float* col = in ? src + ((int64_t)i * g.n + j) * g.l + p.k0 : src;
    if (in && p.k0 > 0) cp_async4(d, col - 1); else sts4(d, ghost);
    const uint32_t dh = d + 4u * (uint32_t)(1 + p.nk);
    if (in && p.k0 + p.nk < g.l) cp_async4(dh, col + p.nk); else sts4(dh, ghost);
  }
  if constexpr (BK == 32) {
    if (p.i0 >= 1 && p.j0 >= 1 && p.i0 + BI + 1 <= g.m && p.j0 + BJ + 1 <= g.n && p.nk == BK) {
      // whole halo inside the grid: the copies of the loop below (halo_col's
      // columns, lane group gq = lane / 8 on column gq of each group of four),
      // with per-lane bases and constant offsets instead of per-copy checks
      const int gq = lane >> 3, k = 4 * (lane & 7);
      const int64_t nl = (int64_t)g.n * g.l;
      // columns 1..BJ of rows 0..BI+1 (interior rows and both x faces)
      const float* sp = src + ((int64_t)(p.i0 - 1) * g.n + (p.j0 + gq)) * g.l + p.k0 + k;
      const uint32_t da = s0 + 4u * (uint32_t)((gq + 1) * CS + 1 + k);
#pragma unroll
      for (int ci = 0; ci < BI + 2; ++ci) {
        const uint32_t dd = da + 4u * (uint32_t)(ci * RS);
        cp_async4(dd, sp);
        cp_async4(dd + 4, sp + 1);
        cp_async4(dd + 8, sp + 2);
        cp_async4(dd + 12, sp + 3);
        sp += nl;
      }
      // y faces: columns 0 and BJ+1 of rows 1..BI, interleaved as in halo_col
      const int cib = (gq >> 1) + 1, cjb = (gq & 1) ? BJ + 1 : 0;
      sp = src + ((int64_t)(p.i0 + cib - 1) * g.n + (p.j0 + cjb - 1)) * g.l + p.k0 + k;
      const uint32_t db = s0 + 4u * (uint32_t)(cib * RS + cjb * CS + 1 + k);
#pragma unroll
      for (int r = 0; r < BI / 2; ++r) {
        const uint32_t dd = db + 4u * (uint32_t)(2 * r * RS);
        cp_async4(dd, sp);
        cp_async4(dd + 4, sp + 1);
        cp_async4(dd + 8, sp + 2);
        cp_async4(dd + 12, sp + 3);
        sp += 2 * nl;
      }
      return;
    }
  }
#pragma unroll
  for (int t = 0; t < PER; ++t) {
    const int e = lane + 32 * t;
    const int c = e / CH, ch = e - (e / CH) * CH;
    int ci, cj;
    halo_col(c, ci, cj);
    const int i = p.i0 + ci - 1, j = p.j0 + cj - 1, k = 4 * ch;
    const uint32_t d = s0 + 4u * (uint32_t)(ci * RS + cj * CS + 1 + k);
    if (i >= 0 && i < g.m && j >= 0 && j < g.n && k < p.nk) {
      const float* sp = src + ((int64_t)i * g.n + j) * g.l + p.k0 + k;
      cp_async4(d, sp);
      cp_async4(d + 4, sp + 1);
      cp_async4(d + 8, sp + 2);
      cp_async4(d + 12, sp + 3);
    } else {
      sts4(d, ghost);
      sts4(d + 4, ghost);
      sts4(d + 8, ghost);
      sts4(d + 12, ghost);
    }
  }
}

template <int BK>
__device__ __forceinline__ void load_interior_f32_async(float* S, const float* src, const Geom& g,
                                                        const BrickPos& p, int CS, int lane) {
  constexpr int IRS = itile_row_stride(BK);
  constexpr int CH = BK / 4;
  constexpr int PER = BI * BJ * CH / 32;
  const uint32_t s0 = smem_u32(S);
  if constexpr (BK == 32) {
    if (p.ni == BI && p.nj == BJ && p.nk == BK) {  // full brick: same copies, no checks
      const int gq = lane >> 3, k = 4 * (lane & 7);
      const int64_t nl = (int64_t)g.n * g.l;
      const float* sp = src + ((int64_t)p.i0 * g.n + (p.j0 + gq)) * g.l + p.k0 + k;
      const uint32_t da = s0 + 4u * (uint32_t)(gq * CS + k);
#pragma unroll
      for (int t = 0; t < BI; ++t) {
        const uint32_t dd = da + 4u * (uint32_t)(t * IRS);
        cp_async4(dd, sp);
        cp_async4(dd + 4, sp + 1);
        cp_async4(dd + 8, sp + 2);
        cp_async4(dd + 12, sp + 3);
        sp += nl;
      }
      return;
    }
  }
#pragma unroll
  for (int t = 0; t < PER; ++t) {
    const int e = lane + 32 * t;
    const int c = e / CH, ch = e - (e / CH) * CH;
    const int ci = c >> 2, cj = c & 3, k = 4 * ch;
    if (ci < p.ni && cj < p.nj && k < p.nk) {
      const float* sp = src + ((int64_t)(p.i0 + ci) * g.n + (p.j0 + cj)) * g.l + p.k0 + k;
      const uint32_t d = s0 + 4u * (uint32_t)(ci * IRS + cj * CS + k);
      cp_async4(d, sp);
      cp_async4(d + 4, sp + 1);
      cp_async4(d + 8, sp + 2);
      cp_async4(d + 12, sp + 3);
    }
  }
}

// Hardware square root (MUFU, ~1 ulp), for the FP32 path only.
__device__ __forceinline__ float sqrt_approx(float x) {
  float r;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Three-input minimum and maximum (one instruction each on sm_100 and later).
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Branch-free FP32 form of upd3_stable: all three candidate roots are
// formed and the first admissible one selected, so lanes on different
// branches do not serialise.  Arranged for a short dependency path from ax
// and ay, which arrive last (other lanes' results of the previous step):
// - the sort uses three-input min/max;
// - the three-axis root (u - ax)^2 + (u - ay)^2 + (u - az)^2 = F^2 is
//   symmetric in the three values, so it is formed relative to az (this
//   lane's own, available early) instead of the sorted minimum:
//   u = az + (bx + by + sqrt(3F^2 - bx^2 - by^2 - (bx - by)^2)) / 3 with
//   b = a - az; it is only selected when every value is finite;
// - the two-axis root x2 = lo + (d2 + r2)/2 is admissible while x2 <= hi,
//   tested as r2 <= 2 d3 - d2 (the two roots agree on that boundary).
__device__ __forceinline__ float upd3_f32(float ax, float ay, float az, float fh) {
  const float lo = fmin3f(ax, ay, az);
  const float hi = fmax3f(ax, ay, az);
  const float mid = fmin3f(fmaxf(ax, ay), fmaxf(ax, az), fmaxf(ay, az));
  const float F2 = fh * fh;
  const float d2 = mid - lo;
  const float d3 = hi - lo;
  const float x1 = lo + fh;
  // 2F^2 - d2^2 < 0 only when d2 > F, where x1 <= mid selects x1: no clamp
  const float r2 = sqrt_approx(fmaf(-d2, d2, 2.0f * F2));
  const float x2 = fmaf(0.5f, d2 + r2, lo);
  const float bx = ax - az, by = ay - az, bxy = ax - ay;
  const float disc = fmaf(-bxy, bxy, fmaf(-by, by, fmaf(-bx, bx, 3.0f * F2)));
  const float r3 = sqrt_approx(fmaxf(disc, 0.0f));
  const float x3 = fmaf(bx + by + r3, 1.0f / 3.0f, az);
  return (x1 <= mid) ? x1 : ((r2 <= fmaf(2.0f, d3, -d2)) ? x2 : x3);
}

// Shared-memory accesses with a 32-bit shared-window address and a
// compile-time byte offset (one instruction each, no address arithmetic).
template <int OFF>
__device__ __forceinline__ float lds(uint32_t a) {
  float v;
  asm volatile("ld.shared.f32 %0, [%1+%2];\n" : "=f"(v) : "r"(a), "n"(OFF));
  return v;
}
__device__ __forceinline__ void sts_if(bool p, uint32_t a, float v) {
  asm volatile(
      "{\n .reg .pred q;\n setp.ne.b32 q, %0, 0;\n @q st.shared.f32 [%1], %2;\n}\n" ::"r"((int)p),
      "r"(a), "f"(v)
      : "memory");
}

// FP32 forward sweep of one staged brick (the batched path), for tiles
// staged by load_tile_f32_vec (out-of-grid ghosts are +inf, so every
// neighbour pair is a plain min).  Same data flow as sweep_brick_fwd, as a
// software pipeline.  At step tau the lane's cell is kk = tau - s; of its
// neighbours only the two upstream ones across columns (x and y, written by
// other lanes one step earlier) and the z-upstream one (this lane's own
// previous result, kept in a register) are new.  The downstream neighbours
// and the slowness cannot change before this step, so they are loaded one
// step ahead, and each step's dependency path is just: two shared loads, the
// local solve, the store.  Lanes outside their window [0, nk) run the same
// code on cells of their own column extended past the brick (still inside
// this warp's tiles, by the tile layout) and only the store is predicated:
// the carried old value at kk = -1 is the halo cell, so the z-upstream value
// entering the window is right without a special case.  SI, SJ, SKD: sweep
// directions; NEAR: cells in the source box update in FP64.
//
// FLOW: also collect the upwind directions of the written cells into fbits
// (bit 0: some cell's active x neighbour is its x- one, so values travel
// along +x; bit 1: along -x; bits 2-3 y, 4-5 z).  An axis is active when the
// new value exceeds the smaller neighbour along it; that neighbour is the
// upwind one (ties: the sweep-upstream one).
template <int BK, int SI, int SJ, int SKD, bool NEAR, bool FLOW = false>
__device__ __forceinline__ bool sweep_brick_fwd_f32(float* S, const float* F, const BrickPos& p,
                                                    float h, double hd, const NearBox& nb,
                                                    int lane, float& maxdec, uint32_t& fbits) {
  constexpr int RS = tile_row_stride(BK);
  constexpr int IRS = itile_row_stride(BK);
  constexpr int CS = tile_col_stride(BK, SJ == SKD);
  constexpr int DZ = 4 * SKD;                       // bytes per step along the column
  constexpr int XU = -4 * RS * SI, XD = 4 * RS * SI;  // byte offsets, upstream / downstream
  constexpr int YU = -4 * CS * SJ, YD = 4 * CS * SJ;
  const int li = lane >> 2, lj = lane & 3;
  const int pi = SI > 0 ? li : BI - 1 - li;
  const int pj = SJ > 0 ? lj : BJ - 1 - lj;
  const int s = li + lj;
  const bool colok = (pi < p.ni) && (pj < p.nj);
  const int nk = colok ? p.nk : 0;
  const int kb = SKD > 0 ? 0 : p.nk - 1;
  // addresses of the lane's cell at tau = 0 (kk = -s)
  uint32_t a = smem_u32(S + (pi + 1) * RS + (pj + 1) * CS + 1 + kb) - DZ * s;
  uint32_t fa = smem_u32(F + pi * IRS + pj * CS + kb) - DZ * s;
  float uo = lds<0>(a);      // old value of the cell
  float prev = lds<-DZ>(a);  // value of the z-upstream cell
  float dn = lds<DZ>(a), xd = lds<XD>(a), yd = lds<YD>(a);
  float fc = lds<0>(fa);
  float mb = 0.0f;
  uint32_t fl = 0;  // sweep-relative upwind bits: 1/2 x up-/downstream, 4/8 y, 16/32 z
  const int nsteps = p.nk + SKEW;
#pragma unroll 4
  for (int tau = 0; tau < nsteps; ++tau) {
    const int kk = tau - s;
    const bool act = (unsigned)kk < (unsigned)nk;
    const float xu = lds<XU>(a), yu = lds<YU>(a);
    // next step's stable operands
    const float n_dn = lds<2 * DZ>(a), n_xd = lds<XD + DZ>(a), n_yd = lds<YD + DZ>(a);
    const float n_fc = lds<DZ>(fa);
    const float az = fminf(prev, dn);
    const float ax = fminf(xu, xd);
    const float ay = fminf(yu, yd);
    float un;
    if (NEAR && act && nb.has(p.i0 + pi, p.j0 + pj, p.k0 + kb + SKD * kk))
      un = (float)upd3_stable<double>((double)ax, (double)ay, (double)az, (double)fc * hd);
    else
      un = upd3_f32(ax, ay, az, fc * h);
    const bool wr = act && (un < uo);
    sts_if(wr, a, un);
    mb = fmaxf(mb, act ? uo - un : 0.0f);
    if constexpr (FLOW) {
      const uint32_t bx = (un > ax) ? ((xu <= xd) ? 1u : 2u) : 0u;
      const uint32_t by = (un > ay) ? ((yu <= yd) ? 4u : 8u) : 0u;
      const uint32_t bz = (un > az) ? ((prev <= dn) ? 16u : 32u) : 0u;
      fl |= wr ? (bx | by | bz) : 0u;
    }
    prev = wr ? un : uo;
    uo = dn;
    dn = n_dn;
    xd = n_xd;
    yd = n_yd;
    fc = n_fc;
    a += (uint32_t)DZ;  // wraps for a negative step
    fa += (uint32_t)DZ;
    __syncwarp();
  }
  maxdec = fmaxf(maxdec, mb);
  if constexpr (FLOW) {
    // to absolute directions: the sweep-upstream side is the minus side of a
    // positive sweep direction
    uint32_t r = __reduce_or_sync(0xffffffffu, fl);
    if (SI < 0) r = (r & ~3u) | ((r & 1u) << 1) | ((r >> 1) & 1u);
    if (SJ < 0) r = (r & ~12u) | ((r & 4u) << 1) | ((r >> 1) & 4u);
    if (SKD < 0) r = (r & ~48u) | ((r & 16u) << 1) | ((r >> 1) & 16u);
    fbits = r;
  }
  return __any_sync(0xffffffffu, mb > 0.0f);
}

// Interior codes (uint16) with 16-byte vector loads: 8 codes per chunk.
// Needs the k extent to be a multiple of 8 (16-byte aligned column segments).
// Returns whether any code of the brick has the seed bit (warp-uniform).
template <int BK>
__device__ __forceinline__ bool load_codes_vec(uint16_t* S, const uint16_t* src,
                                               const Geom& g, const BrickPos& p, int CS, int lane) {
  constexpr int IRS = itile_row_stride(BK);
  constexpr int CH = BK / 8;
  constexpr int PER = BI * BJ * CH / 32;
  uint4 v[PER];
  int dst[PER];
  bool ok[PER];
  if (BK == 32 && p.ni == BI && p.nj == BJ && p.nk == BK) {
    // full brick: the same loads (chunk c = lane / 4 + 8 t is row 2 t + lane / 16,
    // column (lane / 4) mod 4, cells 8 (lane mod 4) ..), one base per lane
    const int ci = lane >> 4, cj = (lane >> 2) & 3, k = 8 * (lane & 3);
    const int64_t nl2 = 2 * (int64_t)g.n * g.l;
    const uint16_t* sp = src + ((int64_t)(p.i0 + ci) * g.n + (p.j0 + cj)) * g.l + p.k0 + k;
    const int d0 = ci * IRS + cj * CS + k;
#pragma unroll
    for (int t = 0; t < PER; ++t) {
      v[t] = *(reinterpret_cast<const uint4*>(sp));
      sp += nl2;
      dst[t] = d0 + 2 * t * IRS;
      ok[t] = true;
    }
  } else {
#pragma unroll
    for (int t = 0; t < PER; ++t) {
      const int e = lane + 32 * t;
      const int c = e / CH, ch = e - (e / CH) * CH;
      const int ci = c >> 2, cj = c & 3, k = 8 * ch;
      ok[t] = ci < p.ni && cj < p.nj && k < p.nk;
      if (ok[t])
        v[t] = *(reinterpret_cast<const uint4*>(
            src + ((int64_t)(p.i0 + ci) * g.n + (p.j0 + cj)) * g.l + p.k0 + k));
      dst[t] = ci * IRS + cj * CS + k;
    }
  }
  constexpr uint32_t SEED2 = (uint32_t)CODE_SEED | ((uint32_t)CODE_SEED << 16);
  uint32_t seeds = 0;
#pragma unroll
  for (int t = 0; t < PER; ++t)
    if (ok[t]) seeds |= (v[t].x | v[t].y | v[t].z | v[t].w) & SEED2;
#pragma unroll
  for (int t = 0; t < PER; ++t)
    if (ok[t]) {
      uint16_t* d = S + dst[t];
      d[0] = (uint16_t)(v[t].x & 0xffffu);
      d[1] = (uint16_t)(v[t].x >> 16);
      d[2] = (uint16_t)(v[t].y & 0xffffu);
      d[3] = (uint16_t)(v[t].y >> 16);
      d[4] = (uint16_t)(v[t].z & 0xffffu);
      d[5] = (uint16_t)(v[t].z >> 16);
      d[6] = (uint16_t)(v[t].w & 0xffffu);
      d[7] = (uint16_t)(v[t].w >> 16);
    }
  return __any_sync(0xffffffffu, seeds != 0);
}

__device__ __forceinline__ uint32_t ldsu16(uint32_t a) {
  unsigned short v;
  asm volatile("ld.shared.u16 %0, [%1];\n" : "=h"(v) : "r"(a));
  return (uint32_t)v;
}
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// Per-cell constants of one FP32 adjoint update, formed one step ahead.
// The user terms w_q lambda_q (w_q = u_q - u_c for a user q, else 0) are
// combined in one fixed order whatever the sweep direction:
//   lambda = fma(P_x + P_y, c2, fma(P_z, c2, c0)),
//   P_a = fma(w_{a+}, lambda_{a+}, w_{a-} lambda_{a-}),
// so a cell evaluates to the same bits in every ordering and the sweeps
// reach an exact fixed point (an order that followed the sweep would make
// the orderings disagree in the last bit and never settle).  Per axis one
// lambda is new in the sweep (the upstream neighbour) and one is old: when
// the new one is the minus neighbour, P = fma(a, b, w_u lambda_u) with
// (a, b) = (w_d, lambda_d); when it is the plus neighbour, P = fma(w_u,
// lambda_u, a) with a = w_d lambda_d.  The z term is this lane's own and
// is folded into the constant first, which keeps it off the path from the
// other lanes' values.
struct AdjCellF32 {
  float wx, ax, bx, wy, ay, by, wz, az, bz;
  float c2, c0;
  bool wrok;  // active, not fixed
};

template <int S>
__device__ __forceinline__ float adj_pair(float w_u, float l_u, float a, float b) {
  return S > 0 ? fmaf(a, b, w_u * l_u) : fmaf(w_u, l_u, a);
}

// lambda_c = (g_c + 2 sum_users (u_r - u_c) lambda_r) / (2 sum_active (u_c - u_upwind))
// for the cell with the given code and neighbours (xu/xd: upstream /
// downstream along x for the sweep, likewise y and z).  Inactive terms are
// selected away (selects, not products, so +inf ghosts never turn into NaN);
// the adjoint tile's ghosts are 0, so their zero weights multiply zeros.
template <int SI, int SJ, int SKD, bool SEEDS>
__device__ __forceinline__ AdjCellF32 adj_cell_f32(uint32_t code, float uc, float uxu, float uxd,
                                                   float uyu, float uyd, float uzu, float uzd,
                                                   float lxd, float lyd, float lzd, bool act,
                                                   int64_t cell, const float* gcell) {
  // user bits (absolute: x-, x+, y-, y+, z-, z+) of the upstream /
  // downstream neighbours of this sweep
  constexpr uint32_t XU = SI > 0 ? 1u : 2u, XD = SI > 0 ? 2u : 1u;
  constexpr uint32_t YU = SJ > 0 ? 4u : 8u, YD = SJ > 0 ? 8u : 4u;
  constexpr uint32_t ZU = SKD > 0 ? 16u : 32u, ZD = SKD > 0 ? 32u : 16u;
  const uint32_t us = code >> CODE_USERS;
  AdjCellF32 c;
  c.wx = (us & XU) ? uxu - uc : 0.0f;
  c.wy = (us & YU) ? uyu - uc : 0.0f;
  c.wz = (us & ZU) ? uzu - uc : 0.0f;
  const float w_xd = (us & XD) ? uxd - uc : 0.0f;
  const float w_yd = (us & YD) ? uyd - uc : 0.0f;
  const float w_zd = (us & ZD) ? uzd - uc : 0.0f;
  if (SI > 0) { c.ax = w_xd; c.bx = lxd; } else { c.ax = w_xd * lxd; c.bx = 0.0f; }
  if (SJ > 0) { c.ay = w_yd; c.by = lyd; } else { c.ay = w_yd * lyd; c.by = 0.0f; }
  if (SKD > 0) { c.az = w_zd; c.bz = lzd; } else { c.az = w_zd * lzd; c.bz = 0.0f; }
  // The diagonal needs no side codes: an axis is active exactly when u_c
  // exceeds the smaller neighbour, which is the upwind one (the codes' tie
  // rule picks between equal values), and out-of-grid ghosts are +inf.
  float d = fmaxf(uc - fminf(uxu, uxd), 0.0f);
  d += fmaxf(uc - fminf(uyu, uyd), 0.0f);
  d += fmaxf(uc - fminf(uzu, uzd), 0.0f);
  c.c2 = rcp_approx(d);
  if constexpr (SEEDS) {
    const float gs = (act && (code & CODE_SEED)) ? gcell[cell] : 0.0f;
    c.c0 = 0.5f * gs * c.c2;
  } else {
    c.c0 = 0.0f;
  }
  c.wrok = act && !(code & CODE_FIXED);
  return c;
}

// FP32 adjoint sweep of one staged brick (tiles from the vector loaders), as a
// software pipeline like sweep_brick_fwd_f32: u and the codes are read-only
// during the sweep and the downstream adjoint values cannot change before the
// step that reads them, so everything but the x and y upstream adjoint values
// is loaded, and the cell's constants formed, one step ahead.  A step's
// dependency path is two shared loads, at most five FMA-pipe operations and
// the store.  U and L
// share one tile layout; SI, SJ, SKD: sweep directions.
//
// Returns whether any lambda of the brick changed (the tile must be written
// back); `sig` tells whether one changed by more than eps relative
// (|new - old| > eps |new|), which is what wakes the brick's neighbours.
// With eps = 0 the two are the same.  SEEDS = false for a brick whose staged
// codes carry no seed bit: no seed value is looked up.
template <int BK, int SI, int SJ, int SKD, bool SEEDS>
__device__ __forceinline__ bool sweep_brick_adj_f32(const float* U, float* L, const uint16_t* C,
                                                    const float* gcell, const Geom& g,
                                                    const BrickPos& p, int lane, float eps,
                                                    bool& sig) {
  constexpr int RS = tile_row_stride(BK);
  constexpr int IRS = itile_row_stride(BK);
  constexpr int CS = tile_col_stride(BK, SJ == SKD);
  constexpr int DZ = 4 * SKD, DC = 2 * SKD;
  constexpr int XU = -4 * RS * SI, XD = 4 * RS * SI;
  constexpr int YU = -4 * CS * SJ, YD = 4 * CS * SJ;
  const int li = lane >> 2, lj = lane & 3;
  const int pi = SI > 0 ? li : BI - 1 - li;
  const int pj = SJ > 0 ? lj : BJ - 1 - lj;
  const int s = li + lj;
  const bool colok = (pi < p.ni) && (pj < p.nj);
  const int nk = colok ? p.nk : 0;
  const int kb = SKD > 0 ? 0 : p.nk - 1;
  const int own = (pi + 1) * RS + (pj + 1) * CS + 1 + kb;
  // addresses of the lane's cell at tau = 0 (kk = -s)
  uint32_t ua = smem_u32(U + own) - DZ * s;
  uint32_t la = smem_u32(L + own) - DZ * s;
  uint32_t ca = smem_u32(C + pi * IRS + pj * CS + kb) - DC * s;
  const int64_t gcol = ((int64_t)(p.i0 + pi) * g.n + (p.j0 + pj)) * g.l + p.k0 + kb;
  float uc = lds<0>(ua), uzd = lds<DZ>(ua);
  float lold = lds<0>(la), lzd = lds<DZ>(la);
  float lzu = lds<-DZ>(la);
  AdjCellF32 cur = adj_cell_f32<SI, SJ, SKD, SEEDS>(
      ldsu16(ca), uc, lds<XU>(ua), lds<XD>(ua), lds<YU>(ua), lds<YD>(ua), lds<-DZ>(ua), uzd,
      lds<XD>(la), lds<YD>(la), lzd, (unsigned)(-s) < (unsigned)nk, gcol - SKD * s, gcell);
  bool changed = false;
  float rmax = -1.0f;  // largest |new - old| - eps |new| over this lane's writes
  const int nsteps = p.nk + SKEW;
#pragma unroll 4
  for (int tau = 0; tau < nsteps; ++tau) {
    const float lxu = lds<XU>(la), lyu = lds<YU>(la);
    // next cell's operands
    const uint32_t n_code = ldsu16(ca + (uint32_t)DC);
    const float n_uxu = lds<DZ + XU>(ua), n_uxd = lds<DZ + XD>(ua);
    const float n_uyu = lds<DZ + YU>(ua), n_uyd = lds<DZ + YD>(ua);
    const float n_uzd = lds<2 * DZ>(ua);
    const float n_lxd = lds<DZ + XD>(la), n_lyd = lds<DZ + YD>(la);
    const float n_lzd = lds<2 * DZ>(la);
    // lambda = (P_x + P_y) c2 + (P_z c2 + c0): P_z is this lane's own (early)
    const float pz = fmaf(adj_pair<SKD>(cur.wz, lzu, cur.az, cur.bz), cur.c2, cur.c0);
    const float pxy = adj_pair<SI>(cur.wx, lxu, cur.ax, cur.bx) +
                      adj_pair<SJ>(cur.wy, lyu, cur.ay, cur.by);
    const float lam = fmaf(pxy, cur.c2, pz);
    const bool wr = cur.wrok && (lam != lold);
    sts_if(wr, la, lam);
    changed |= wr;
    const float rel = fmaf(-eps, fabsf(lam), fabsf(lam - lold));
    rmax = wr ? fmaxf(rmax, rel) : rmax;
    lzu = wr ? lam : lold;
    const int kn = tau + 1 - s;
    cur = adj_cell_f32<SI, SJ, SKD, SEEDS>(n_code, uzd, n_uxu, n_uxd, n_uyu, n_uyd, uc, n_uzd, n_lxd,
                                    n_lyd, n_lzd, (unsigned)kn < (unsigned)nk, gcol + SKD * kn,
                                    gcell);
    uc = uzd;
    uzd = n_uzd;
    lold = lzd;
    lzd = n_lzd;
    ua += (uint32_t)DZ;  // wraps for a negative step
    la += (uint32_t)DZ;
    ca += (uint32_t)DC;
    __syncwarp();
  }
  const bool any = __any_sync(0xffffffffu, changed);
  sig = eps > 0.0f ? __any_sync(0xffffffffu, rmax > 0.0f) : any;
  return any;
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
        const T lam = EXACT ? (T)fi_div((double)acc, (double)d) : acc / d;
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
