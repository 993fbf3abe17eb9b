// eik3d_noalloc.cu -- the 3D FP64 forward without any device allocation.
//
// Some callers cannot allocate device memory themselves: code running
// inside a framework that owns the whole device heap through its own
// allocator (and forbids cudaMalloc beside it), real-time or embedded hosts
// whose memory budget is fixed at start-up, and callers that must not risk
// an allocation failure (or an allocator synchronisation) in the middle of a
// run.  adt_eikonal_three_d_device_noalloc serves them: it runs the same
// kernels as adt_eikonal_three_d_device, on caller-provided device inputs
// and outputs, and takes its scratch (the previous iterate for the stopping
// rule, the brick level list and the error word) from the file-scope array
// below instead of cudaMalloc.
//
// Properties a caller must know:
//  - The array is a fixed ADT_NOALLOC_SCRATCH_BYTES per device (about 2.2 MB)
//    and stays resident on every device that loads the library until the
//    process exits.  Grids above ADT_NOALLOC_MAX_CELLS cells are rejected
//    with ADT_EINVAL before any device work.
//  - The first call on a device looks up the array's device address
//    (cudaGetSymbolAddress, with that device current) and caches it; make
//    that first call before any stream capture on that device.
//  - Every call on a device uses the same array, so calls must not overlap on
//    the GPU.  Calls from several host threads are serialised by a per-device
//    mutex; the call returns only after its work on `stream` has finished.
//  - Nothing is left for the next call to rely on: the previous iterate is
//    overwritten each iteration, the level list on each call, and the error
//    word is cleared before each use.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "eik3d_single_kernels.h"

namespace adt {

namespace {

// Scratch layout: [previous iterate: MAX_CELLS doubles][brick list: MAX_CELLS/8
// uint32 (a brick covers at least 8 cells of any legal grid)][error word]
constexpr size_t NA_UOLD_BYTES = (size_t)ADT_NOALLOC_MAX_CELLS * sizeof(double);
constexpr size_t NA_BRICK_BYTES = (size_t)(ADT_NOALLOC_MAX_CELLS / 8) * sizeof(uint32_t);
constexpr size_t NA_ERR_OFF = NA_UOLD_BYTES + NA_BRICK_BYTES;
static_assert(NA_ERR_OFF + 256 <= ADT_NOALLOC_SCRATCH_BYTES, "scratch layout");

static __device__ __align__(256) unsigned char adt_noalloc_scratch[ADT_NOALLOC_SCRATCH_BYTES];

// Host-side level list of the grid, in fixed storage (no heap use either):
// at most MAX_CELLS/8 bricks and, with m <= 8*2047, n <= 4*2047 and at most
// MAX_CELLS cells, fewer than 4096 levels.
constexpr int NA_MAX_BRICKS = ADT_NOALLOC_MAX_CELLS / 8;
constexpr int NA_MAX_LEVELS = 4096;

struct NoAllocDevice {
  std::mutex mu;
  unsigned char* base = nullptr;  // device address of adt_noalloc_scratch
  bool attr_set = false;
  uint32_t bricks[NA_MAX_BRICKS];
  int start[NA_MAX_LEVELS + 1];
};

// Bricks grouped by level bx+by+bz (same order as make_levels).
bool na_levels(const Geom& g, NoAllocDevice& D) {
  const int64_t nb = (int64_t)g.nbx * g.nby * g.nbz;
  if (nb > NA_MAX_BRICKS || g.nlev > NA_MAX_LEVELS) return false;
  for (int d = 0; d <= g.nlev; ++d) D.start[d] = 0;
  for (int x = 0; x < g.nbx; ++x)
    for (int y = 0; y < g.nby; ++y)
      for (int z = 0; z < g.nbz; ++z) ++D.start[x + y + z + 1];
  for (int d = 0; d < g.nlev; ++d) D.start[d + 1] += D.start[d];
  int pos[NA_MAX_LEVELS];
  for (int d = 0; d < g.nlev; ++d) pos[d] = D.start[d];
  for (int x = 0; x < g.nbx; ++x)
    for (int y = 0; y < g.nby; ++y)
      for (int z = 0; z < g.nbz; ++z) D.bricks[pos[x + y + z]++] = pack_brick(x, y, z);
  return true;
}
constexpr int NA_MAX_DEVICES = 16;
NoAllocDevice& na_device(int dev) {
  static NoAllocDevice d[NA_MAX_DEVICES];
  return d[dev];
}

// The solve itself, on the locked device D.  Sets `enqueued` once work has
// been queued on `st`, so that the caller can drain the stream when an
// error cuts the call short.
int na_solve(NoAllocDevice& D, const double* u0, const double* f, double h, const Geom& g,
             double tol, int verbose, double* u, adt_solve_status* status, cudaStream_t st,
             bool& enqueued) {
  if (!D.base) {  // once per device, with that device current
    void* p = nullptr;
    ADT_CUDA(cudaGetSymbolAddress(&p, adt_noalloc_scratch));
    D.base = static_cast<unsigned char*>(p);
  }
  if (!D.attr_set) {
    ADT_CUDA(cudaFuncSetAttribute(k_level_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(FWD_WPB * FWD_WARP_SMEM)));
    D.attr_set = true;
  }
  if (!na_levels(g, D)) return set_error(ADT_EINVAL, "eikonal3d_noalloc: grid has too many bricks");
  const int nbricks = D.start[g.nlev];
  double* uold = reinterpret_cast<double*>(D.base);
  uint32_t* bricks = reinterpret_cast<uint32_t*>(D.base + NA_UOLD_BYTES);
  unsigned long long* err_word = reinterpret_cast<unsigned long long*>(D.base + NA_ERR_OFF);
  const size_t bytes = (size_t)g.ncell * sizeof(double);
  enqueued = true;
  ADT_CUDA(cudaMemcpyAsync(bricks, D.bricks, nbricks * sizeof(uint32_t), cudaMemcpyHostToDevice,
                           st));
  ADT_CUDA(cudaMemcpyAsync(u, u0, bytes, cudaMemcpyDeviceToDevice, st));
  int it = 0, done = 0;
  double err = 0.0;
  for (it = 0; it < 20; ++it) {  // the reference's iteration cap (Eikonal3D.cpp:74)
    ADT_CUDA(cudaMemcpyAsync(uold, u, bytes, cudaMemcpyDeviceToDevice, st));
    for (int o = 0; o < 8; ++o)
      for (int d = 0; d < g.nlev; ++d) {
        const int cnt = D.start[d + 1] - D.start[d];
        k_level_fwd<<<(cnt + FWD_WPB - 1) / FWD_WPB, FWD_WPB * 32, FWD_WPB * FWD_WARP_SMEM, st>>>(
            u, f, nullptr, g, bricks, D.start[d], cnt, o, h, nullptr, 0);
      }
    ADT_CUDA(cudaGetLastError());
    ADT_CUDA(cudaMemsetAsync(err_word, 0, sizeof(unsigned long long), st));
    const int blocks = (int)((g.ncell + 255) / 256 < 4096 ? (g.ncell + 255) / 256 : 4096);
    k_maxdiff<<<blocks, 256, 0, st>>>(u, uold, g.ncell, err_word);
    unsigned long long bits = 0;
    ADT_CUDA(cudaMemcpyAsync(&bits, err_word, sizeof bits, cudaMemcpyDeviceToHost, st));
    ADT_CUDA(cudaStreamSynchronize(st));
    std::memcpy(&err, &bits, sizeof err);
    if (verbose) printf("Iteration %d, Error = %0.6e\n", it, err);
    if (err < tol) {
      done = 1;
      break;
    }
  }
  if (status) {
    status->iters = done ? it + 1 : it;
    status->converged = done;
    status->final_err = err;
    status->adj_iters = 0;
    status->adj_converged = 0;
  }
  return ADT_OK;
}

}  // namespace
}  // namespace adt

using namespace adt;

extern "C" int adt_eikonal_three_d_device_noalloc(const double* u0, const double* f, double h,
                                                  int64_t m, int64_t n, int64_t l, double tol,
                                                  int verbose, double* u,
                                                  adt_solve_status* status, void* stream) {
  if (m < 2 || n < 2 || l < 2)
    return set_error(ADT_EINVAL, "eikonal3d_noalloc: need m, n, l >= 2 (got %lld x %lld x %lld)",
                     (long long)m, (long long)n, (long long)l);
  // each extent is bounded before the product is formed, so the product
  // cannot overflow
  if (m > BI * 2047 || n > BJ * 2047 || l > (int64_t)ADT_NOALLOC_MAX_CELLS ||
      m * n * l > (int64_t)ADT_NOALLOC_MAX_CELLS)
    return set_error(ADT_EINVAL,
                     "eikonal3d_noalloc: %lld x %lld x %lld cells exceed the fixed scratch limit "
                     "of %d cells (use adt_eikonal_three_d_device for larger grids)",
                     (long long)m, (long long)n, (long long)l, ADT_NOALLOC_MAX_CELLS);
  // brick coordinates are packed in 11/11/10 bits (pack_brick)
  if (make_geom((int)m, (int)n, (int)l, SBK).nbz > 1023)
    return set_error(ADT_EINVAL, "eikonal3d_noalloc: l = %lld is too deep (at most %d)",
                     (long long)l, SBK * 1023);
  if (!(h > 0.0) || !std::isfinite(h))
    return set_error(ADT_EINVAL, "eikonal3d_noalloc: h must be finite and > 0");
  if (!(tol >= 0.0)) return set_error(ADT_EINVAL, "eikonal3d_noalloc: tol must be >= 0");
  if (!u0 || !f || !u) return set_error(ADT_EINVAL, "eikonal3d_noalloc: null array");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(ADT_ENODEV, "no CUDA device available");
  }
  int dev = 0;
  ADT_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NA_MAX_DEVICES)
    return set_error(ADT_EINVAL, "eikonal3d_noalloc: device %d beyond the supported %d", dev,
                     NA_MAX_DEVICES);
  NoAllocDevice& D = na_device(dev);
  std::lock_guard<std::mutex> lock(D.mu);
  cudaStream_t st = (cudaStream_t)stream;
  bool enqueued = false;
  const int rc = na_solve(D, u0, f, h, make_geom((int)m, (int)n, (int)l, SBK), tol, verbose, u,
                          status, st, enqueued);
  // On an error after work was queued, wait for that work before the lock is
  // released: a later call must not reuse the scratch under it.  The error
  // of the wait itself is not reported over the first one.
  if (rc != ADT_OK && enqueued) {
    cudaStreamSynchronize(st);
    cudaGetLastError();
  }
  return rc;
}
