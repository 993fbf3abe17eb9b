// eik3d_single_kernels.h -- kernels and launch constants of the plain FP64
// single-solve 3D path (defined in eik3d_single.cu).
#pragma once
#include "eik3d_brick.cuh"

namespace adt {

// Warps (bricks) per CTA.  One: a level has few bricks, and the FP64
// arithmetic of each brick runs at the rate of one SM's FP64 pipe, so every
// brick gets an SM of its own.
constexpr int FWD_WPB = 1;
constexpr int ADJ_WPB = 1;
// the forward's tiles: travel times with halo, then two interior tiles (f, or
// f h and f f h h)
constexpr size_t FWD_WARP_SMEM = (tile_elems(SBK) + 2 * itile_elems(SBK)) * sizeof(double);
constexpr size_t ADJ_WARP_SMEM =
    (2 * tile_elems(SBK) + itile_elems(SBK)) * sizeof(double) + itile_elems(SBK) * sizeof(uint16_t);

// One level of one ordering: one warp per brick of the level.  With stamps
// (per brick: the time of its last sweep, then of its last change; zeros at
// the start) a brick is swept only if its last sweep changed it or a face
// neighbour changed after that sweep: otherwise every cell already satisfies
// its update and a sweep would change nothing (exact).  t: this launch's
// time, larger than any before it; the bricks of one level are not face
// neighbours, so no stamp is read and written by the same launch.
// fcst: per cell f h (ncell doubles) then f f h h (ncell more), formed once
// per solve by k_fwd_cells, or nullptr to form them from f in every update.
__global__ void k_level_fwd(double* __restrict__ u, const double* __restrict__ f,
                            const double* __restrict__ fcst, Geom g,
                            const uint32_t* __restrict__ bricks, int q0, int cnt, int o, double h,
                            int* __restrict__ stamps, int t);
// fcst[c] = f h, fcst[ncell + c] = f f h h in the reference's order
// (Eikonal3D.cpp:11-28).
__global__ void k_fwd_cells(const double* __restrict__ f, double h, int64_t ncell,
                            double* __restrict__ fcst);
// max |a - b| as the bit pattern of a non-negative double (atomicMax into *out).
__global__ void k_maxdiff(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                          unsigned long long* out);

}  // namespace adt
