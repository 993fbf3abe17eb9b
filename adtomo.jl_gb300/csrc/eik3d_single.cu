// eik3d_single.cu -- the plain FP64 single-solve 3D path.
//
// One solve per call, FP64 with the reference's arithmetic, no batching and
// no CUDA graph: the host loops over iterations, the 8 orderings and the
// brick levels of each ordering, launching one kernel per level (one warp per
// brick).  The stopping rule is the reference's: max |u - u_old| over an
// iteration < tol, at most max_iter (20) iterations (Eikonal3D.cpp:71-88).
// The adjoint assembles nothing: per-cell codes describe the upwind structure
// and reverse sweeps solve A^T lambda = grad_u until a full iteration changes
// no lambda (the system is triangular in descending travel time, so sweeps
// reach the exact solution).
#include <cstdio>
#include <cstring>
#include <mutex>

#include "eik3d_brick.cuh"
#include "eik3d_batch.h"
#include "eik3d_common_host.h"
#include "eik3d_single.h"
#include "eik3d_single_kernels.h"

namespace adt {

__global__ void k_fwd_cells(const double* __restrict__ f, double h, int64_t ncell,
                            double* __restrict__ fcst) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double fv = f[c];
    fcst[c] = __dmul_rn(fv, h);
    fcst[ncell + c] = __dmul_rn(__dmul_rn(__dmul_rn(fv, fv), h), h);
  }
}

__global__ void k_level_fwd(double* __restrict__ u, const double* __restrict__ f,
                            const double* __restrict__ fcst, Geom g,
                            const uint32_t* __restrict__ bricks, int q0, int cnt, int o, double h,
                            int* __restrict__ stamps, int t) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = blockIdx.x * (blockDim.x >> 5) + warp;
  if (q >= cnt) return;
  double* S = reinterpret_cast<double*>(smem + warp * FWD_WARP_SMEM);
  double* F = S + tile_elems(SBK);
  int si, sj, sk;
  ordering3(o, si, sj, sk);
  const int CS = tile_col_stride(SBK, sj == sk);
  const BrickPos p = brick_pos<SBK>(g, bricks[q0 + q], si, sj, sk);
  const int id = (p.bx * g.nby + p.by) * g.nbz + p.bz;
  if (stamps) {  // exact brick skipping
    const int swept = stamps[2 * id];
    bool dirty = stamps[2 * id + 1] >= swept;
    auto newer = [&](int x, int y, int z) { return stamps[2 * ((x * g.nby + y) * g.nbz + z) + 1] > swept; };
    dirty = dirty || (p.bx > 0 && newer(p.bx - 1, p.by, p.bz)) ||
            (p.bx < g.nbx - 1 && newer(p.bx + 1, p.by, p.bz)) ||
            (p.by > 0 && newer(p.bx, p.by - 1, p.bz)) ||
            (p.by < g.nby - 1 && newer(p.bx, p.by + 1, p.bz)) ||
            (p.bz > 0 && newer(p.bx, p.by, p.bz - 1)) ||
            (p.bz < g.nbz - 1 && newer(p.bx, p.by, p.bz + 1));
    if (!dirty) return;
  }
  load_halo_tile<double, SBK>(S, u, g, p, CS, lane);
  if (fcst) {
    load_interior<double, SBK>(F, fcst, g, p, CS, lane);
    load_interior<double, SBK>(F + itile_elems(SBK), fcst + g.ncell, g, p, CS, lane);
  } else {
    load_interior<double, SBK>(F, f, g, p, CS, lane);
  }
  cp_async_wait_all();
  __syncwarp();
  double md = 0.0;
  NearBox nb{1, 0, 1, 0, 1, 0};
  const bool ch =
      fcst ? sweep_brick_fwd<double, SBK, MODE_EXACT_CST>(S, F, g, p, si, sj, sk, CS, h, h, nb,
                                                          false, lane, md)
           : sweep_brick_fwd<double, SBK, MODE_EXACT>(S, F, g, p, si, sj, sk, CS, h, h, nb, false,
                                                      lane, md);
  if (ch) store_interior<double, SBK>(S, u, g, p, CS, lane);
  if (stamps && lane == 0) {
    stamps[2 * id] = t;
    if (ch) stamps[2 * id + 1] = t;
  }
}

// max |a - b| as the bit pattern of a non-negative double.
__global__ void k_maxdiff(const double* __restrict__ a, const double* __restrict__ b, int64_t n,
                          unsigned long long* out) {
  double mx = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    mx = rmax(fabs(a[i] - b[i]), mx);
  mx = warp_max(mx);
  __shared__ double red[32];
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = mx;
  __syncthreads();
  if (threadIdx.x < 32) {
    double v = (threadIdx.x < (blockDim.x >> 5)) ? red[threadIdx.x] : 0.0;
    v = warp_max(v);
    if (threadIdx.x == 0) atomicMax(out, (unsigned long long)__double_as_longlong(v));
  }
}

// Upwind side along one axis (1 = minus, 2 = plus) with the edge rule and
// ties to the plus side (Eikonal3D.cpp:189-197); 0 if not active.
template <class T>
__device__ __forceinline__ int upwind_side(const T* u, int64_t c, int pos, int ext, int64_t st,
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

// Pass 1 of the adjoint codes: upwind sides, fixed and seed bits.
__global__ void k_code1(const double* __restrict__ u, const double* __restrict__ u0,
                        const double* __restrict__ gdense, Geom g, uint16_t* __restrict__ code) {
  const int64_t N = g.ncell;
  const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / sI), j = (int)((c / sJ) % g.n), k = (int)(c % g.l);
    const double uc = u[c];
    const int sx = upwind_side(u, c, i, g.m, sI, uc);
    const int sy = upwind_side(u, c, j, g.n, sJ, uc);
    const int sz = upwind_side(u, c, k, g.l, (int64_t)1, uc);
    uint16_t cd = (uint16_t)(sx | (sy << 2) | (sz << 4));
    if (uc == u0[c] || (sx | sy | sz) == 0) cd = CODE_FIXED;
    else if (gdense[c] != 0.0) cd |= CODE_SEED;
    code[c] = cd;
  }
}

// Pass 2: which neighbours use this cell as their active upwind neighbour.
__device__ __forceinline__ uint16_t users_bits(const uint16_t* code, int64_t c, int i, int j,
                                               int k, const Geom& g) {
  const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
  uint16_t us = 0;
  auto uses = [&](int64_t r, int ax, int want) -> bool {
    const uint16_t cr = code[r];
    return !(cr & CODE_FIXED) && (((cr >> (2 * ax)) & 3) == want);
  };
  if (i > 0 && uses(c - sI, 0, 2)) us |= 1;
  if (i < g.m - 1 && uses(c + sI, 0, 1)) us |= 2;
  if (j > 0 && uses(c - sJ, 1, 2)) us |= 4;
  if (j < g.n - 1 && uses(c + sJ, 1, 1)) us |= 8;
  if (k > 0 && uses(c - 1, 2, 2)) us |= 16;
  if (k < g.l - 1 && uses(c + 1, 2, 1)) us |= 32;
  return us;
}

__global__ void k_code2(const uint16_t* __restrict__ code1, uint16_t* __restrict__ code, Geom g) {
  const int64_t N = g.ncell;
  const int64_t sI = (int64_t)g.n * g.l, sJ = g.l;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < N;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int i = (int)(c / sI), j = (int)((c / sJ) % g.n), k = (int)(c % g.l);
    const uint16_t cd = code1[c];
    code[c] = (cd & CODE_FIXED) ? cd : (uint16_t)(cd | (users_bits(code1, c, i, j, k, g) << CODE_USERS));
  }
}

__global__ void k_level_adj(const double* __restrict__ u, double* __restrict__ lam,
                            const uint16_t* __restrict__ code, const double* __restrict__ gdense,
                            Geom g, const uint32_t* __restrict__ bricks, int q0, int cnt, int o,
                            int* changed) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = blockIdx.x * (blockDim.x >> 5) + warp;
  if (q >= cnt) return;
  unsigned char* base = smem + warp * ADJ_WARP_SMEM;
  double* U = reinterpret_cast<double*>(base);
  double* L = U + tile_elems(SBK);
  double* G = L + tile_elems(SBK);
  uint16_t* C = reinterpret_cast<uint16_t*>(G + itile_elems(SBK));
  int si, sj, sk;
  ordering3(o, si, sj, sk);
  const int CS = tile_col_stride(SBK, sj == sk);
  const BrickPos p = brick_pos<SBK>(g, bricks[q0 + q], si, sj, sk);
  load_halo_tile<double, SBK>(U, u, g, p, CS, lane);
  load_halo_tile<double, SBK>(L, lam, g, p, CS, lane);
  load_interior<double, SBK>(G, gdense, g, p, CS, lane);
  load_interior<uint16_t, SBK>(C, code, g, p, CS, lane);
  cp_async_wait_all();
  __syncwarp();
  const bool ch = sweep_brick_adj<double, SBK, true, true>(U, L, C, G, nullptr, nullptr, 0, g, p, si,
                                                           sj, sk, CS, lane);
  if (ch) {
    store_interior<double, SBK>(L, lam, g, p, CS, lane);
    if (lane == 0) atomicExch(changed, 1);
  }
}

// lambda of cell c: lam[c] for the sweeps' array; with blocked_n > 0 the
// causal-order adjoint's records (4 doubles each, lambda first) in the
// blocked layout of an m x blocked_n x blocked_l grid.
__global__ void k_grad(const double* __restrict__ lam, int blocked_n, int blocked_l,
                       const double* __restrict__ f, const double* __restrict__ u,
                       const double* __restrict__ u0, const double* __restrict__ gu, double h,
                       int64_t n, double* __restrict__ grad_f, double* __restrict__ grad_u0) {
  const BlkMap bm = make_blkmap(blocked_n, blocked_l);
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    int64_t lc = c;
    if (blocked_n > 0) {
      const int64_t nl = (int64_t)blocked_n * blocked_l;
      const int i = (int)(c / nl), j = (int)((c - i * nl) / blocked_l);
      lc = 4 * (int64_t)blk_index(bm, i, j, (int)(c - i * nl - (int64_t)j * blocked_l));
    }
    // rhs = -2 f h h ; grad_f = -lambda * rhs  (Eikonal3D.cpp:163-166,244-246)
    const double rhs = __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f[c]), h), h);
    grad_f[c] = __dmul_rn(-lam[lc], rhs);
    if (grad_u0) grad_u0[c] = (u[c] == u0[c]) ? gu[c] : 0.0;
  }
}

namespace {
struct SingleWork {
  std::mutex mu;
  DevBuf uold, lam, code1, code, levels, scalar;
  DevBuf stamps;  // forward brick skipping: per brick, last sweep and last change
  DevBuf fcst;    // forward: f h and f f h h per cell
  DevBuf meta, rec, queue;  // causal-order adjoint
  int lev_m = -1, lev_n = -1, lev_l = -1;
  LevelList host_levels;
};
SingleWork& work(int dev) {
  static SingleWork w[64];
  return w[dev & 63];
}

int ensure_levels(SingleWork& W, const Geom& g, cudaStream_t st) {
  if (W.lev_m == g.m && W.lev_n == g.n && W.lev_l == g.l) return ADT_OK;
  W.host_levels = make_levels(g);
  ADT_CUDA(W.levels.reserve(W.host_levels.bricks.size() * sizeof(uint32_t)));
  ADT_CUDA(cudaMemcpyAsync(W.levels.p, W.host_levels.bricks.data(),
                           W.host_levels.bricks.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, st));
  ADT_CUDA(cudaStreamSynchronize(st));
  W.lev_m = g.m;
  W.lev_n = g.n;
  W.lev_l = g.l;
  return ADT_OK;
}

int grid_for(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)(b < 4096 ? (b > 0 ? b : 1) : 4096);
}
}  // namespace

int eik3d_single_forward(const double* d_u0, const double* d_f, double h, int m, int n, int l,
                         double tol, int max_iter, int verbose, double* d_u, adt_solve_status* st,
                         cudaStream_t stream) {
  int dev = 0;
  ADT_CUDA(cudaGetDevice(&dev));
  SingleWork& W = work(dev);
  std::lock_guard<std::mutex> lock(W.mu);
  const Geom g = make_geom(m, n, l, SBK);
  const size_t bytes = (size_t)g.ncell * sizeof(double);
  int rc = ensure_levels(W, g, stream);
  if (rc) return rc;
  ADT_CUDA(W.uold.reserve(bytes));
  ADT_CUDA(W.scalar.reserve(sizeof(unsigned long long)));
  const int64_t nbricks = (int64_t)g.nbx * g.nby * g.nbz;
  ADT_CUDA(W.stamps.reserve((size_t)nbricks * 2 * sizeof(int)));
  ADT_CUDA(cudaMemsetAsync(W.stamps.p, 0, (size_t)nbricks * 2 * sizeof(int), stream));
  ADT_CUDA(W.fcst.reserve(2 * bytes));
  k_fwd_cells<<<grid_for(g.ncell), 256, 0, stream>>>(d_f, h, g.ncell, W.fcst.as<double>());
  static bool attr_set[64] = {false};
  if (!attr_set[dev & 63]) {
    ADT_CUDA(cudaFuncSetAttribute(k_level_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(FWD_WPB * FWD_WARP_SMEM)));
    ADT_CUDA(cudaFuncSetAttribute(k_level_adj, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(ADJ_WPB * ADJ_WARP_SMEM)));
    attr_set[dev & 63] = true;
  }
  ADT_CUDA(cudaMemcpyAsync(d_u, d_u0, bytes, cudaMemcpyDeviceToDevice, stream));
  const uint32_t* lv = W.levels.as<uint32_t>();
  const std::vector<int>& start = W.host_levels.start;
  unsigned long long* d_err = W.scalar.as<unsigned long long>();
  int it = 0, done = 0;
  double err = 0.0;
  for (it = 0; it < max_iter; ++it) {
    ADT_CUDA(cudaMemcpyAsync(W.uold.p, d_u, bytes, cudaMemcpyDeviceToDevice, stream));
    for (int o = 0; o < 8; ++o)
      for (int d = 0; d < g.nlev; ++d) {
        const int cnt = start[d + 1] - start[d];
        const int blocks = (cnt + FWD_WPB - 1) / FWD_WPB;
        k_level_fwd<<<blocks, FWD_WPB * 32, FWD_WPB * FWD_WARP_SMEM, stream>>>(
            d_u, d_f, W.fcst.as<double>(), g, lv, start[d], cnt, o, h, W.stamps.as<int>(),
            1 + (it * 8 + o) * g.nlev + d);
      }
    ADT_CUDA(cudaGetLastError());
    ADT_CUDA(cudaMemsetAsync(d_err, 0, sizeof(unsigned long long), stream));
    k_maxdiff<<<grid_for(g.ncell), 256, 0, stream>>>(d_u, W.uold.as<double>(), g.ncell, d_err);
    unsigned long long bits = 0;
    ADT_CUDA(cudaMemcpyAsync(&bits, d_err, sizeof bits, cudaMemcpyDeviceToHost, stream));
    ADT_CUDA(cudaStreamSynchronize(stream));
    memcpy(&err, &bits, sizeof err);
    if (verbose) printf("Iteration %d, Error = %0.6e\n", it, err);
    if (err < tol) {
      done = 1;
      break;
    }
  }
  if (st) {
    st->iters = done ? it + 1 : it;
    st->converged = done;
    st->final_err = err;
    st->adj_iters = 0;
    st->adj_converged = 0;
  }
  return ADT_OK;
}

int eik3d_single_adjoint(const double* d_gu, const double* d_u, const double* d_u0,
                         const double* d_f, double h, int m, int n, int l, int max_iter,
                         double* d_gu0, double* d_gf, int* iters_out, int* converged_out,
                         cudaStream_t stream) {
  int dev = 0;
  ADT_CUDA(cudaGetDevice(&dev));
  SingleWork& W = work(dev);
  std::lock_guard<std::mutex> lock(W.mu);
  const Geom g = make_geom(m, n, l, SBK);
  if (blk_slots(m, n, l) < ((int64_t)1 << 31)) {
    // causal order: every cell evaluated once, after its users, in one CTA
    // (the same per-cell formula as the sweeps below, so the same bits)
    ADT_CUDA(W.scalar.reserve(sizeof(unsigned long long)));
    const int64_t slots = blk_slots(m, n, l);
    ADT_CUDA(W.meta.reserve((size_t)slots * sizeof(uint32_t)));
    ADT_CUDA(W.rec.reserve((size_t)slots * CAUSAL_REC64_BYTES));
    ADT_CUDA(W.queue.reserve((size_t)g.ncell * sizeof(int)));
    int* d_complete = W.scalar.as<int>();
    int rc;
    if ((rc = causal_single_adjoint(d_u, d_u0, d_gu, m, n, l, W.meta.as<uint32_t>(), W.rec.p,
                                    W.queue.as<int>(), d_complete, stream)))
      return rc;
    k_grad<<<grid_for(g.ncell), 256, 0, stream>>>(W.rec.as<double>(), n, l, d_f, d_u, d_u0, d_gu, h,
                                                  g.ncell, d_gf, d_gu0);
    ADT_CUDA(cudaGetLastError());
    int complete = 0;
    ADT_CUDA(cudaMemcpyAsync(&complete, d_complete, sizeof(int), cudaMemcpyDeviceToHost, stream));
    ADT_CUDA(cudaStreamSynchronize(stream));
    if (iters_out) *iters_out = 1;
    if (converged_out) *converged_out = complete;
    return ADT_OK;
  }
  // larger grids: reverse level sweeps until nothing changes
  int rc = ensure_levels(W, g, stream);
  if (rc) return rc;
  ADT_CUDA(W.lam.reserve((size_t)g.ncell * sizeof(double)));
  ADT_CUDA(W.code1.reserve((size_t)g.ncell * sizeof(uint16_t)));
  ADT_CUDA(W.code.reserve((size_t)g.ncell * sizeof(uint16_t)));
  ADT_CUDA(W.scalar.reserve(sizeof(unsigned long long)));
  static bool attr_set[64] = {false};
  if (!attr_set[dev & 63]) {
    ADT_CUDA(cudaFuncSetAttribute(k_level_fwd, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(FWD_WPB * FWD_WARP_SMEM)));
    ADT_CUDA(cudaFuncSetAttribute(k_level_adj, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)(ADJ_WPB * ADJ_WARP_SMEM)));
    attr_set[dev & 63] = true;
  }
  double* lam = W.lam.as<double>();
  uint16_t* code = W.code.as<uint16_t>();
  k_code1<<<grid_for(g.ncell), 256, 0, stream>>>(d_u, d_u0, d_gu, g, W.code1.as<uint16_t>());
  k_code2<<<grid_for(g.ncell), 256, 0, stream>>>(W.code1.as<uint16_t>(), code, g);
  ADT_CUDA(cudaMemsetAsync(lam, 0, (size_t)g.ncell * sizeof(double), stream));
  ADT_CUDA(cudaGetLastError());
  const uint32_t* lv = W.levels.as<uint32_t>();
  const std::vector<int>& start = W.host_levels.start;
  int* d_changed = W.scalar.as<int>();
  int it = 0, done = 0;
  for (it = 0; it < max_iter; ++it) {
    ADT_CUDA(cudaMemsetAsync(d_changed, 0, sizeof(int), stream));
    for (int o = 0; o < 8; ++o)
      for (int d = 0; d < g.nlev; ++d) {
        const int cnt = start[d + 1] - start[d];
        const int blocks = (cnt + ADJ_WPB - 1) / ADJ_WPB;
        k_level_adj<<<blocks, ADJ_WPB * 32, ADJ_WPB * ADJ_WARP_SMEM, stream>>>(
            d_u, lam, code, d_gu, g, lv, start[d], cnt, o, d_changed);
      }
    ADT_CUDA(cudaGetLastError());
    int changed = 0;
    ADT_CUDA(cudaMemcpyAsync(&changed, d_changed, sizeof(int), cudaMemcpyDeviceToHost, stream));
    ADT_CUDA(cudaStreamSynchronize(stream));
    if (!changed) {
      done = 1;
      break;
    }
  }
  k_grad<<<grid_for(g.ncell), 256, 0, stream>>>(lam, 0, 0, d_f, d_u, d_u0, d_gu, h, g.ncell, d_gf, d_gu0);
  ADT_CUDA(cudaGetLastError());
  ADT_CUDA(cudaStreamSynchronize(stream));
  if (iters_out) *iters_out = done ? it + 1 : it;
  if (converged_out) *converged_out = done;
  return ADT_OK;
}

}  // namespace adt
