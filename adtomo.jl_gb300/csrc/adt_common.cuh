// adt_common.cuh -- shared definitions for the GB300 Eikonal library.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/adtomo_gpu.h"

namespace adt {

// Set the thread-local error message and return the code.
int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

#define ADT_CUDA(call)                                      \
  do {                                                      \
    cudaError_t adt_e_ = (call);                            \
    if (adt_e_ != cudaSuccess) return adt::cuda_error(adt_e_, #call); \
  } while (0)

// Reference min/max semantics (std::min(a,b) = (b < a) ? b : a).
template <class T>
__host__ __device__ __forceinline__ T rmin(T a, T b) {
  return (b < a) ? b : a;
}
template <class T>
__host__ __device__ __forceinline__ T rmax(T a, T b) {
  return (a < b) ? b : a;
}

// Brick geometry used by every 3D sweep: 8 (i) x 4 (j) columns, one lane per
// column, BK cells deep along k (the contiguous axis).
constexpr int BI = 8;
constexpr int BJ = 4;
// Brick depth of the plain single-solve 3D path (the batched plan chooses its
// own).  16: a level of one solve holds few bricks, each on its own SM, and a
// level lasts one brick's chain of FP64 steps (16 + 10 steps, against 42 for
// 32 cells).
constexpr int SBK = 16;

// Shared-memory tile of one brick with a one-cell halo on every side:
// column (pi, pj) for pi in [-1, BI], pj in [-1, BJ]; slot k+1 for k in
// [-1, BK].  addr = (pi+1)*row + (pj+1)*col + (k+1).
// The wavefront of one step touches cells on a local hyperplane; with
// row = 0 (mod 32) and col = 9 (mod 16) when the j and k sweep directions
// agree (7 (mod 16) otherwise), the 32 cells of every step and of each of
// their six neighbour sets fall in 32 distinct banks for all 8 orderings
// (checked exhaustively for BK = 16, 32, 64).
__host__ __device__ constexpr int tile_col_stride(int BK, bool same_dir) {
  return ((BK + 2 + 15 - (same_dir ? 9 : 7)) / 16) * 16 + (same_dir ? 9 : 7);
}
__host__ __device__ constexpr int tile_col_stride_max(int BK) {
  return tile_col_stride(BK, true) > tile_col_stride(BK, false) ? tile_col_stride(BK, true)
                                                                 : tile_col_stride(BK, false);
}
__host__ __device__ constexpr int tile_row_stride(int BK) {
  return ((6 * tile_col_stride_max(BK) + 31) / 32) * 32;
}
__host__ __device__ constexpr int tile_elems(int BK) { return (BI + 2) * tile_row_stride(BK); }
// Interior-only tile (slowness, seeds, codes): no halo.
__host__ __device__ constexpr int itile_row_stride(int BK) {
  return ((BJ * tile_col_stride_max(BK) + 31) / 32) * 32;
}
__host__ __device__ constexpr int itile_elems(int BK) { return BI * itile_row_stride(BK); }

// Packed brick coordinates in "sweep-relative" form (level = bx + by + bz).
__host__ __device__ __forceinline__ uint32_t pack_brick(int bx, int by, int bz) {
  return (uint32_t)bx | ((uint32_t)by << 11) | ((uint32_t)bz << 22);
}
__host__ __device__ __forceinline__ void unpack_brick(uint32_t p, int& bx, int& by, int& bz) {
  bx = (int)(p & 2047u);
  by = (int)((p >> 11) & 2047u);
  bz = (int)(p >> 22);
}

// The 8 orderings in the reference's sequence (Eikonal3D.cpp:59-68).
__host__ __device__ __forceinline__ void ordering3(int o, int& si, int& sj, int& sk) {
  // (+,+,+) (-,+,+) (-,-,+) (+,-,+) (+,-,-) (+,+,-) (-,+,-) (-,-,-):
  // bit o of each mask marks a negative direction.
  si = ((0xC6u >> o) & 1u) ? -1 : 1;
  sj = ((0x9Cu >> o) & 1u) ? -1 : 1;
  sk = ((0xF0u >> o) & 1u) ? -1 : 1;
}

// Per-cell adjoint code (uint16):
//   bits 0-1 / 2-3 / 4-5: upwind side along x / y / z (0 inactive, 1 minus, 2 plus)
//   bit 6: fixed cell (identity row: travel time equals its initial value, or
//          no active axis -- Eikonal3D.cpp:126-130,168-171)
//   bit 7: seeded (non-zero misfit sensitivity at this cell)
//   bits 8-13: users -- the neighbour at x-, x+, y-, y+, z-, z+ uses this cell
//          as its active upwind neighbour (so its lambda feeds this cell's)
constexpr uint16_t CODE_FIXED = 1u << 6;
constexpr uint16_t CODE_SEED = 1u << 7;
constexpr int CODE_USERS = 8;
// Outstanding-user byte of a fixed cell in the causal-order adjoint: never
// cleared by a user, so the cell is never queued.
constexpr uint32_t REM_FIXED = 0x80u;

// Geometry of one field as seen by the kernels.
struct Geom {
  int m, n, l;        // nodes
  int nbx, nby, nbz;  // bricks
  int nlev;           // levels per ordering = nbx + nby + nbz - 2
  int64_t ncell;
};

inline Geom make_geom(int m, int n, int l, int BK) {
  Geom g;
  g.m = m;
  g.n = n;
  g.l = l;
  g.nbx = (m + BI - 1) / BI;
  g.nby = (n + BJ - 1) / BJ;
  g.nbz = (l + BK - 1) / BK;
  g.nlev = g.nbx + g.nby + g.nbz - 2;
  g.ncell = (int64_t)m * n * l;
  return g;
}

// Blocked cell layout of the causal-order adjoint's per-cell words and
// records: groups of 2 x 2 x 2 cells stored together (eight 16-byte FP32
// records fill one 128-byte line), groups in (i, j, k) order.  A cell's
// neighbour along an axis lies in its own group when the coordinate's low
// bit allows and in the adjacent group otherwise, so half of a cell's
// neighbourhood shares its line.  Grids with odd extents leave the unused
// slots of their last groups untouched (no in-grid cell refers to them).
struct BlkMap {
  int nj2, nk2;  // groups along j and k
  int gi;        // slots per group step along i: nj2 * nk2 * 8
};
__host__ __device__ inline BlkMap make_blkmap(int n, int l) {
  BlkMap b;
  b.nj2 = (n + 1) / 2;
  b.nk2 = (l + 1) / 2;
  b.gi = b.nj2 * b.nk2 * 8;
  return b;
}
// Slots of one solve in the blocked layout (< 2^31 where it is used).
__host__ __device__ inline int64_t blk_slots(int m, int n, int l) {
  return (int64_t)((m + 1) / 2) * ((n + 1) / 2) * ((l + 1) / 2) * 8;
}
__host__ __device__ __forceinline__ int blk_index(const BlkMap& b, int i, int j, int k) {
  return ((i >> 1) * b.nj2 + (j >> 1)) * b.nk2 * 8 + (k >> 1) * 8 +
         (((i & 1) << 2) | ((j & 1) << 1) | (k & 1));
}
// The slot of the neighbour of slot s along axis a (0: i, 1: j, 2: k) in
// direction +1 (dir > 0) or -1; the caller knows that neighbour is in the grid.
__host__ __device__ __forceinline__ int blk_step(const BlkMap& b, int s, int a, int dir) {
  const int bit = 4 >> a;
  const int gs = a == 0 ? b.gi : (a == 1 ? b.nk2 * 8 : 8);
  if (dir > 0) return (s & bit) ? s - bit + gs : s + bit;
  return (s & bit) ? s - bit : s + bit - gs;
}
// (i, j, k) of slot s (plain divisions: used for the few seeded cells).
__host__ __device__ __forceinline__ void blk_cell(const BlkMap& b, int s, int& i, int& j, int& k) {
  const int g = s >> 3, w = s & 7;
  const int gjk = b.nj2 * b.nk2;
  const int I = g / gjk, r = g - I * gjk, J = r / b.nk2, K = r - J * b.nk2;
  i = 2 * I + (w >> 2);
  j = 2 * J + ((w >> 1) & 1);
  k = 2 * K + (w & 1);
}

}  // namespace adt
