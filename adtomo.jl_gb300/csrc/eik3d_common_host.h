// eik3d_common_host.h -- host helpers shared by the 3D drivers.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "adt_common.cuh"

namespace adt {

// Bricks of a grid in sweep-relative coordinates, grouped by level
// bx + by + bz.  The same list serves all 8 orderings (brick_pos mirrors).
struct LevelList {
  std::vector<uint32_t> bricks;
  std::vector<int> start;  // nlev + 1 entries
};

inline LevelList make_levels(const Geom& g) {
  LevelList L;
  L.start.assign(g.nlev + 1, 0);
  std::vector<int> cnt(g.nlev, 0);
  for (int x = 0; x < g.nbx; ++x)
    for (int y = 0; y < g.nby; ++y)
      for (int z = 0; z < g.nbz; ++z) ++cnt[x + y + z];
  for (int d = 0; d < g.nlev; ++d) L.start[d + 1] = L.start[d] + cnt[d];
  L.bricks.resize(L.start[g.nlev]);
  std::vector<int> pos(L.start.begin(), L.start.end() - 1);
  for (int x = 0; x < g.nbx; ++x)
    for (int y = 0; y < g.nby; ++y)
      for (int z = 0; z < g.nbz; ++z) L.bricks[pos[x + y + z]++] = pack_brick(x, y, z);
  return L;
}

// Simple owning device buffer.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  // Grow to at least n bytes (contents are not preserved).
  cudaError_t reserve(size_t n) {
    if (n <= bytes) return cudaSuccess;
    release();
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaSuccess) bytes = n;
    else p = nullptr;
    return e;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

}  // namespace adt
