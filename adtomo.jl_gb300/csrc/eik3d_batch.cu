// eik3d_batch.cu -- the batched misfit + gradient plan (adt_batch_*).
//
// One evaluation = for every chunk of solves: persistent forward kernel,
// receiver sampling + misfit + seeds, persistent adjoint kernel, FP64
// gradient accumulation; then the misfit sum.  The sequence is captured once
// into a CUDA graph and replayed per evaluation.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <memory>
#include <numeric>
#include <vector>

#include "eik3d_batch.h"
#include "eik3d_adj_causal.cuh"
#include "eik3d_batch_kernels.cuh"
#include "eik3d_common_host.h"
#include "eik3d_single_kernels.h"

namespace adt {

namespace {

__global__ void k_to_t_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

// FP64 near-source initial values at the 8 nodes (i, j, k) around each
// source, from the distance r = sqrt(dx^2+dy^2+dz^2) (dx = x - i, ...):
//  - default (vel == 0): r * f * h with one slowness per depth plane, taken
//    from the evaluation's slowness at the (ceil x, ceil y) column
//    (scripts/gene_obs.jl:42-51: slowness_pu / slowness_pd);
//  - vel != 0: r * h / vel0[i, j, k], vel0 a fixed velocity model
//    (scripts/inversion.jl:52-60).
template <class T>
__global__ void k_src_init(SolveDev* solves, int n, const FieldDev<T>* fields, int vel,
                           unsigned long long* cost) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  cost[s] = 0;  // bricks swept by this evaluation's sweeps, for the next one's order
  SolveDev& sd = solves[s];
  const FieldDev<T>& fd = fields[sd.field];
  const int xs[2] = {sd.xc, sd.xf}, ys[2] = {sd.yc, sd.yf}, zs[2] = {sd.zc, sd.zf};
  for (int a = 0; a < 2; ++a)
    for (int b = 0; b < 2; ++b)
      for (int c = 0; c < 2; ++c) {
        const double dx = sd.sx - xs[a], dy = sd.sy - ys[b], dz = sd.sz - zs[c];
        const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)),
                                              __dmul_rn(dz, dz)));
        double v;
        if (vel) {
          const int64_t p = ((int64_t)xs[a] * fd.g.n + ys[b]) * fd.g.l + zs[c];
          v = __ddiv_rn(__dmul_rn(r, fd.h), fd.vel0[p]);
        } else {
          const int64_t q = ((int64_t)sd.xc * fd.g.n + sd.yc) * fd.g.l + zs[c];
          v = __dmul_rn(__dmul_rn(r, fd.f64[q]), fd.h);
        }
        sd.v0[a * 4 + b * 2 + c] = v;
      }
}

__global__ void k_misfit_sum(const double* __restrict__ m, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < n; ++i) s = __dadd_rn(s, m[i]);
    *out = s;
  }
}

int grid1d(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 8192));
}

// per warp: the travel-time tile with halo and the interior slowness tile
// (FP64: two interior tiles, f h and f f h h); k_batch_fwd places the warps'
// tiles with the same stride
template <class T>
size_t fwd_warp_smem(int bk) {
  const int ni = sizeof(T) == 8 ? 2 : 1;
  const int t = bk == 64 ? tile_elems(64) + ni * itile_elems(64)
                         : bk == 16 ? tile_elems(16) + ni * itile_elems(16)
                                    : tile_elems(32) + ni * itile_elems(32);
  return (size_t)t * sizeof(T);
}
template <class T>
size_t adj_warp_smem(int bk) {
  const int te = bk == 64 ? tile_elems(64) : bk == 16 ? tile_elems(16) : tile_elems(32);
  const int ie = bk == 64 ? itile_elems(64) : bk == 16 ? itile_elems(16) : itile_elems(32);
  return 2 * (size_t)te * sizeof(T) + (size_t)ie * sizeof(uint16_t);
}

// Multipliers of the causal-order adjoint's cell-index divisions (FieldDev).
template <class T>
void set_divisors(FieldDev<T>& fd) {
  const unsigned long long nl = (unsigned long long)fd.g.n * fd.g.l, l = fd.g.l;  // both >= 2
  fd.div_nl = ~0ULL / nl + 1;
  fd.div_l = ~0ULL / l + 1;
}

}  // namespace

// Kernel entry points per (T, BK), resolved at plan creation.
struct KernelSet {
  const void* fwd;
  const void* adj;
  const void* adj_causal;
  const void* misfit;
  const void* grad;
};

template <class T>
static KernelSet kernels_for(int bk) {
  constexpr int MODE = sizeof(T) == 8 ? MODE_EXACT_CST : MODE_STABLE;
  KernelSet k;
  if (bk == 64) {
    k.fwd = (const void*)&k_batch_fwd<T, 64, MODE>;
    k.adj = (const void*)&k_batch_adj<T, 64>;
  } else if (bk == 16) {
    k.fwd = (const void*)&k_batch_fwd<T, 16, MODE>;
    k.adj = (const void*)&k_batch_adj<T, 16>;
  } else {
    k.fwd = (const void*)&k_batch_fwd<T, 32, MODE>;
    k.adj = (const void*)&k_batch_adj<T, 32>;
  }
  k.adj_causal = (const void*)&k_batch_adj_causal<T>;
  k.misfit = (const void*)&k_batch_misfit<T>;
  k.grad = (const void*)&k_batch_grad<T>;
  return k;
}

struct BatchPlan {
  int dev = 0;
  cudaStream_t stream = nullptr;
  adt_batch_opts opts;
  int bk = 32;
  bool f64 = false;
  size_t esz = 4;
  // fields
  int nf = 0;
  std::vector<Geom> geoms;
  std::vector<double> h;
  std::vector<int> nsta;
  std::vector<int64_t> cell_off, sta_off;
  std::vector<int64_t> cell_off_t;  // FP32 slowness copy: per-field offsets padded to 16 cells
  int64_t ncell_t_total = 0;
  int64_t ncell_total = 0;
  // solves
  int ns = 0;
  std::vector<int> solve_field;
  std::vector<int64_t> obs_off;
  int64_t nobs = 0;
  std::vector<SolveDev> solves;
  struct Chunk {
    int first, count;
    std::vector<int> order;                           // largest first
    std::vector<std::vector<int64_t>> field_uoff;     // per field, solve order
    int64_t dev_order_off;
    std::vector<int64_t> dev_uoff_off;                // per field offset into d_uoff
  };
  std::vector<Chunk> chunks;
  // device
  DevBuf d_slow64, d_vel0, d_slowT, d_sta, d_tobs, d_w, d_tpred, d_grad, d_smis, d_mis, d_status;
  DevBuf d_levels, d_lstart, d_fields, d_solves, d_order, d_uoff;
  DevBuf d_nseed, d_snap, d_next, d_counters;
  // Buffers of the solves resident at once (one chunk).  With overlapping
  // chunks there are two sets: chunk c uses set c % 2 on stream c % 2, so the
  // next chunk's forward runs beside this chunk's adjoint.
  struct ChunkBufs {
    DevBuf u, lam, code, meta, sidx, sval;
    DevBuf gdense;       // FP32 path: seed values as a dense field per chunk solve (zero elsewhere)
    DevBuf mis_scratch;  // seed merge arrays when they exceed shared memory
    DevBuf meta32, rec, queue;  // causal-order adjoint: meta words, records, frontiers
  };
  ChunkBufs cb[2];
  int nsets = 1;
  cudaStream_t stream2 = nullptr;    // second chunk stream (overlapping chunks)
  std::vector<cudaEvent_t> ev_sync;  // [0] fork, [1 + c] gradient of chunk c added
  DevBuf d_cost, d_chunk_off, d_chunk_cnt;  // per-solve cost; chunk slices of d_order
  int64_t mis_stride = 0;
  int64_t snap_stride = 0;
  std::vector<adt_solve_status> h_status;
  int uploaded = 0;  // bits: 1 slowness, 2 t_obs, 4 weight
  bool src_vel = false;  // near-source values from d_vel0 (batch_set_source_velocity)
  // launch shapes
  KernelSet ks;
  int fwd_warps = 8, adj_warps = 4, fwd_ctas = 0, adj_ctas = 0;
  int fwd_gw = 4, fwd_groups = 2, adj_gw = 2, adj_groups = 4;
  bool causal = false;  // adjoint in causal order (k_batch_adj_causal, one solve per CTA)
  bool dual = false;    // both adjoint solvers available (FP32 with ADT_ADJ_AUTO): the
                        // autotuner keeps the faster
  const void* adj_kern[2] = {nullptr, nullptr};  // [0] sweeps, [1] causal order
  int adj_regs_k[2] = {0, 0}, adj_maxt_k[2] = {1024, 1024};
  int max_nb = 0, meta_smem = 0;
  int sm_count = 0, fwd_regs = 0, adj_regs = 0, adj_maxt = 1024;
  size_t smem_budget = 0, fwd_wbytes = 0, adj_wbytes = 0;
  size_t fwd_smem = 0, adj_smem = 0, mis_smem = 0;
  // graph and timing
  cudaGraphExec_t graph = nullptr;
  std::vector<cudaEvent_t> ev;  // per chunk: fwd0 fwd1 adj0 adj1; then total0 total1
  bool ran = false;
  ~BatchPlan() {
    if (graph) cudaGraphExecDestroy(graph);
    for (auto e : ev) cudaEventDestroy(e);
    for (auto e : ev_sync) cudaEventDestroy(e);
    if (stream2) cudaStreamDestroy(stream2);
    if (stream) cudaStreamDestroy(stream);
  }
};

void batch_opts_default(adt_batch_opts* o) {
  std::memset(o, 0, sizeof(*o));
  o->precision = ADT_F32;
  o->tol = 1e-6;
  o->max_iter = 200;
  o->adj_max_iter = 200;
  o->ref_compat = 0;
  o->near_src_f64 = 2;
  o->chunk = 0;
  o->bk = 0;
  o->warps = 0;
  o->groups = 0;
  o->use_graph = 1;
  o->wake_tol = 0.0;
  o->adj_wake_tol = 0.0;
  o->adj_order_filter = 1;
  o->fwd_order_filter = 1;
  o->overlap_chunks = 0;
  o->adj_warps = 0;
  o->adj_groups = 0;
  o->adj_solver = ADT_ADJ_AUTO;
}

static int enqueue(BatchPlan& P, bool capturing);

// Launch shape of one sweep kernel: `gw` warps per solve (warp group) and as
// many groups per CTA as shared memory, registers and `max_threads` allow
// (at most `groups_req` when > 0); confirmed with the occupancy calculator.
static int fit_shape(const void* fn, size_t warp_bytes, int regs, int max_threads, int meta_smem,
                     int max_nb, int narr, size_t budget, int gw_req, int groups_req, int& gw,
                     int& groups, size_t& smem) {
  const int max_warps = std::min(max_threads / 32, 65536 / std::max(1, regs * 32));
  gw = std::max(1, std::min(gw_req, max_warps));
  for (;;) {
    int G = 1;
    while (G < 15 &&
           group_hdr_bytes(G + 1, meta_smem, max_nb, narr) + (size_t)(G + 1) * gw * warp_bytes <= budget &&
           (G + 1) * gw <= max_warps)
      ++G;
    if (group_hdr_bytes(G, meta_smem, max_nb, narr) + (size_t)G * gw * warp_bytes <= budget) {
      if (groups_req > 0) G = std::min(G, groups_req);
      for (; G >= 1; --G) {  // shrink until one CTA fits
        smem = group_hdr_bytes(G, meta_smem, max_nb, narr) + (size_t)G * gw * warp_bytes;
        ADT_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        int occ = 0;
        ADT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, G * gw * 32, smem));
        if (occ >= 1) {
          groups = G;
          return ADT_OK;
        }
      }
    }
    // no group count fits at this width (shared memory, or the occupancy
    // calculator's register and carve-out limits): try a narrower group
    if (gw == 1) return set_error(ADT_EINVAL, "batch: no launch shape fits on this device");
    --gw;
  }
}

// Set both sweep kernels' launch shapes (0 = default width / as many groups
// as fit) and drop a captured graph that used the old ones.  Defaults,
// measured on the 256-event 128x128x64 workload: the forward runs two solves
// of 6 warps per SM (its register cap allows 12 warps), the adjoint two
// solves of 4 warps (its tiles allow 9).
static int apply_shapes(BatchPlan* P, int fwd_gw, int fwd_groups, int adj_gw, int adj_groups) {
  int rc;
  if ((rc = fit_shape(P->ks.fwd, P->fwd_wbytes, P->fwd_regs, ADT_FWD_MAXT, P->meta_smem, P->max_nb,
                      META_ARRAYS_FWD, P->smem_budget, fwd_gw > 0 ? fwd_gw : (P->f64 ? 2 : 6), fwd_groups,
                      P->fwd_gw, P->fwd_groups, P->fwd_smem)))
    return rc;
  if (P->causal) {  // one solve per CTA of adj_gw warps, static shared memory only
    const int max_warps = std::min(P->adj_maxt / 32, 65536 / std::max(1, P->adj_regs * 32));
    P->adj_gw = std::max(1, std::min(adj_gw > 0 ? adj_gw : 32, max_warps));
    P->adj_groups = 1;
    P->adj_smem = 0;
  } else if ((rc = fit_shape(P->ks.adj, P->adj_wbytes, P->adj_regs, 1024, P->meta_smem, P->max_nb,
                             META_ARRAYS_ADJ, P->smem_budget, adj_gw > 0 ? adj_gw : (P->f64 ? 2 : 4),
                             adj_groups, P->adj_gw, P->adj_groups, P->adj_smem))) {
    return rc;
  }
  P->fwd_warps = P->fwd_gw * P->fwd_groups;
  P->adj_warps = P->adj_gw * P->adj_groups;
  int occ_f = 0, occ_a = 0;
  ADT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_f, P->ks.fwd, P->fwd_warps * 32,
                                                         P->fwd_smem));
  ADT_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_a, P->ks.adj, P->adj_warps * 32,
                                                         P->adj_smem));
  P->fwd_ctas = std::max(1, occ_f) * P->sm_count;
  P->adj_ctas = std::max(1, occ_a) * P->sm_count;
  if (P->graph) {
    cudaGraphExecDestroy(P->graph);
    P->graph = nullptr;
  }
  return ADT_OK;
}

// Make the sweeps (causal = false) or the causal-order solve the adjoint of
// the next evaluations (both must have been set up at plan creation).
static void select_solver(BatchPlan* P, bool causal) {
  P->causal = causal;
  P->ks.adj = P->adj_kern[causal ? 1 : 0];
  P->adj_regs = P->adj_regs_k[causal ? 1 : 0];
  P->adj_maxt = P->adj_maxt_k[causal ? 1 : 0];
  if (P->graph) {
    cudaGraphExecDestroy(P->graph);
    P->graph = nullptr;
  }
}

int batch_check_args(int32_t n_fields, const int32_t* dims, const double* hh, const int32_t* nsta,
                     int32_t n_solves, const int32_t* solve_field, const double* src_xyz,
                     const adt_batch_opts* opts) {
  adt_batch_opts o;
  batch_opts_default(&o);
  if (opts) o = *opts;
  if (n_fields < 1 || n_solves < 1 || !dims || !hh || !nsta || !solve_field || !src_xyz)
    return set_error(ADT_EINVAL, "batch: need at least one field and one solve");
  if (o.precision != ADT_F32 && o.precision != ADT_F64)
    return set_error(ADT_EINVAL, "batch: precision must be ADT_F32 or ADT_F64");
  if (o.ref_compat && o.precision != ADT_F64)
    return set_error(ADT_EINVAL, "batch: ref_compat needs ADT_F64");
  if (o.max_iter < 1 || o.adj_max_iter < 1 || o.max_iter > 100000 || o.adj_max_iter > 100000 ||
      !(o.tol >= 0.0))
    return set_error(ADT_EINVAL, "batch: bad iteration caps (1..100000) or tolerance");
  if (!(o.wake_tol >= 0.0) || !std::isfinite(o.wake_tol) || !(o.adj_wake_tol >= 0.0) ||
      !std::isfinite(o.adj_wake_tol))
    return set_error(ADT_EINVAL, "batch: wake_tol and adj_wake_tol must be finite and >= 0");
  if (o.bk != 0 && o.bk != 16 && o.bk != 32 && o.bk != 64)
    return set_error(ADT_EINVAL, "batch: bk must be 0, 16, 32 or 64");
  if (o.adj_solver != ADT_ADJ_SWEEPS && o.adj_solver != ADT_ADJ_CAUSAL &&
      o.adj_solver != ADT_ADJ_AUTO)
    return set_error(ADT_EINVAL, "batch: adj_solver must be ADT_ADJ_AUTO, ADT_ADJ_SWEEPS or "
                     "ADT_ADJ_CAUSAL");
  return ADT_OK;
}

int batch_create(BatchPlan** out, int32_t n_fields, const int32_t* dims, const double* hh,
                 const int32_t* nsta, const double* sta_xyz, int32_t n_solves,
                 const int32_t* solve_field, const double* src_xyz, const adt_batch_opts* opts) {
  *out = nullptr;
  int rc0 = batch_check_args(n_fields, dims, hh, nsta, n_solves, solve_field, src_xyz, opts);
  if (rc0) return rc0;
  adt_batch_opts o;
  batch_opts_default(&o);
  if (opts) o = *opts;
  auto P = std::make_unique<BatchPlan>();
  P->opts = o;
  if (o.ref_compat) P->opts.max_iter = std::min(o.max_iter, 20);
  P->f64 = o.precision == ADT_F64;
  P->esz = P->f64 ? 8 : 4;
  int minl = INT_MAX;
  for (int f = 0; f < n_fields; ++f) {
    const int m = dims[3 * f], n = dims[3 * f + 1], l = dims[3 * f + 2];
    if (m < 2 || n < 2 || l < 2 || m > BI * 2047 || n > BJ * 2047)
      return set_error(ADT_EINVAL, "batch: field %d has bad dimensions %d x %d x %d", f, m, n, l);
    if (!(hh[f] > 0.0) || !std::isfinite(hh[f]))
      return set_error(ADT_EINVAL, "batch: field %d has bad spacing", f);
    if (nsta[f] < 0 || nsta[f] > ADT_BATCH_MAX_RECEIVERS)
      return set_error(ADT_EINVAL, "batch: field %d has %d receivers (0..%d supported)", f,
                       nsta[f], ADT_BATCH_MAX_RECEIVERS);
    minl = std::min(minl, l);
  }
  (void)minl;
  P->bk = o.bk ? o.bk : 32;
  P->nf = n_fields;
  // ADT_ADJ_AUTO: the causal-order solve, and in FP32 also the sweeps, for
  // the autotuner to choose between
  P->causal = o.adj_solver == ADT_ADJ_CAUSAL || o.adj_solver == ADT_ADJ_AUTO;
  P->dual = o.adj_solver == ADT_ADJ_AUTO && o.precision == ADT_F32;
  for (int f = 0; f < n_fields; ++f)
    if (P->causal && blk_slots(dims[3 * f], dims[3 * f + 1], dims[3 * f + 2]) >= ((int64_t)1 << 31)) {
      if (o.adj_solver == ADT_ADJ_CAUSAL)
        return set_error(ADT_EINVAL, "batch: the causal-order adjoint needs fewer than 2^31 cells "
                         "per field (field %d)", f);
      P->causal = P->dual = false;  // automatic choice: the sweeps
    }
  int64_t sofs = 0;
  for (int f = 0; f < n_fields; ++f) {
    const Geom g = make_geom(dims[3 * f], dims[3 * f + 1], dims[3 * f + 2], P->bk);
    if (g.nbz > 1023) return set_error(ADT_EINVAL, "batch: field %d is too deep", f);
    // brick timestamps count level steps, (iteration * 8 + ordering) * levels + level,
    // in an int
    if ((int64_t)(std::max(P->opts.max_iter, o.adj_max_iter) + 1) * 8 * g.nlev >= INT_MAX)
      return set_error(ADT_EINVAL, "batch: field %d has too many brick levels (%d) for the "
                       "iteration caps", f, g.nlev);
    P->geoms.push_back(g);
    P->h.push_back(hh[f]);
    P->nsta.push_back(nsta[f]);
    P->cell_off.push_back(P->ncell_total);
    P->cell_off_t.push_back(P->ncell_t_total);
    P->sta_off.push_back(sofs);
    P->ncell_total += g.ncell;
    P->ncell_t_total += (g.ncell + 15) / 16 * 16;
    for (int q = 0; q < nsta[f]; ++q) {
      const double* x = sta_xyz + 3 * (sofs + q);
      if (!(x[0] >= 0 && x[0] <= g.m - 1 && x[1] >= 0 && x[1] <= g.n - 1 && x[2] >= 0 && x[2] <= g.l - 1))
        return set_error(ADT_EINVAL, "batch: receiver %d of field %d is outside the grid", q, f);
    }
    sofs += nsta[f];
  }
  P->ns = n_solves;
  P->obs_off.resize(n_solves + 1, 0);
  P->solves.resize(n_solves);
  for (int s = 0; s < n_solves; ++s) {
    const int f = solve_field[s];
    if (f < 0 || f >= n_fields) return set_error(ADT_EINVAL, "batch: solve %d names field %d", s, f);
    const Geom& g = P->geoms[f];
    const double* x = src_xyz + 3 * s;
    if (!(x[0] >= 0 && x[0] <= g.m - 1 && x[1] >= 0 && x[1] <= g.n - 1 && x[2] >= 0 && x[2] <= g.l - 1))
      return set_error(ADT_EINVAL, "batch: source of solve %d is outside its grid", s);
    SolveDev sd;
    std::memset(&sd, 0, sizeof sd);
    sd.field = f;
    sd.gidx = s;
    sd.sx = x[0];
    sd.sy = x[1];
    sd.sz = x[2];
    sd.xc = (int)std::ceil(x[0]);
    sd.xf = (int)std::floor(x[0]);
    sd.yc = (int)std::ceil(x[1]);
    sd.yf = (int)std::floor(x[1]);
    sd.zc = (int)std::ceil(x[2]);
    sd.zf = (int)std::floor(x[2]);
    P->solves[s] = sd;
    P->solve_field.push_back(f);
    P->obs_off[s + 1] = P->obs_off[s] + nsta[f];
    P->solves[s].obs_off = P->obs_off[s];
  }
  P->nobs = P->obs_off[n_solves];
  // chunks of consecutive solves
  const int C = (o.chunk > 0 && o.chunk < n_solves) ? o.chunk : n_solves;
  int64_t max_cells = 0, max_bricks = 0, max_seeds = 0;
  int64_t order_total = 0, uoff_total = 0;
  for (int c0 = 0; c0 < n_solves; c0 += C) {
    BatchPlan::Chunk ch;
    ch.first = c0;
    ch.count = std::min(C, n_solves - c0);
    ch.order.resize(ch.count);
    std::iota(ch.order.begin(), ch.order.end(), c0);
    std::stable_sort(ch.order.begin(), ch.order.end(), [&](int a, int b) {
      return P->geoms[P->solve_field[a]].ncell > P->geoms[P->solve_field[b]].ncell;
    });
    int64_t cells = 0, bricks = 0, seeds = 0;
    ch.field_uoff.assign(n_fields, {});
    for (int s = c0; s < c0 + ch.count; ++s) {
      const Geom& g = P->geoms[P->solve_field[s]];
      P->solves[s].u_off = cells;
      P->solves[s].meta_off = bricks;
      P->solves[s].seed_off = seeds;
      ch.field_uoff[P->solve_field[s]].push_back(cells);
      // 64-byte aligned solves (the FP32 path uses 16-byte accesses), each
      // also holding the causal-order adjoint's blocked slots
      const int64_t span = P->causal ? std::max(g.ncell, blk_slots(g.m, g.n, g.l)) : g.ncell;  // causal or dual
      cells += (span + 15) / 16 * 16;
      bricks += (int64_t)META_ARRAYS_MAX * g.nbx * g.nby * g.nbz;
      seeds += 8LL * P->nsta[P->solve_field[s]];
    }
    max_cells = std::max(max_cells, cells);
    max_bricks = std::max(max_bricks, bricks);
    max_seeds = std::max(max_seeds, seeds);
    ch.dev_order_off = order_total;
    order_total += ch.count;
    for (int f = 0; f < n_fields; ++f) {
      ch.dev_uoff_off.push_back(uoff_total);
      uoff_total += (int64_t)ch.field_uoff[f].size();
    }
    P->chunks.push_back(std::move(ch));
  }
  // device setup
  ADT_CUDA(cudaGetDevice(&P->dev));
  ADT_CUDA(cudaStreamCreateWithFlags(&P->stream, cudaStreamNonBlocking));
  const size_t es = P->esz;
  auto R = [&](DevBuf& b, size_t bytes) -> int {
    cudaError_t e = b.reserve(std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return set_error(ADT_ENOMEM, "batch: cudaMalloc of %zu bytes failed", bytes);
    return ADT_OK;
  };
  int rc;
#define R_(b, n) \
  if ((rc = R(b, n))) return rc;
  R_(P->d_slow64, P->ncell_total * 8);
  R_(P->d_vel0, P->ncell_total * 8);
  // FP32: the slowness in FP32; FP64: f h and f f h h per cell
  R_(P->d_slowT, P->f64 ? 2 * P->ncell_total * 8 : P->ncell_t_total * 4);
  R_(P->d_sta, (size_t)sofs * 3 * 8);
  R_(P->d_tobs, P->nobs * 8);
  R_(P->d_w, P->nobs * 8);
  R_(P->d_tpred, P->nobs * 8);
  R_(P->d_grad, P->ncell_total * 8);
  R_(P->d_smis, (size_t)n_solves * 8);
  R_(P->d_mis, 8);
  R_(P->d_status, (size_t)n_solves * sizeof(adt_solve_status));
  R_(P->d_solves, (size_t)n_solves * sizeof(SolveDev));
  R_(P->d_order, (size_t)order_total * 4);
  R_(P->d_uoff, (size_t)std::max<int64_t>(uoff_total, 1) * 8);
  // two buffer sets only when there is a second chunk to overlap with (the
  // reference stopping rule's per-CTA snapshots are shared, so not there)
  P->nsets = (o.overlap_chunks && P->chunks.size() > 1 && !o.ref_compat) ? 2 : 1;
  for (int k = 0; k < P->nsets; ++k) {
    BatchPlan::ChunkBufs& B = P->cb[k];
    R_(B.u, (size_t)max_cells * es);
    if (!P->causal || P->dual) {  // the causal-order adjoint keeps lambda in its records
      R_(B.lam, (size_t)max_cells * es);
      R_(B.code, (size_t)max_cells * 2);
    }
    R_(B.meta, (size_t)max_bricks * 4);
    R_(B.sidx, (size_t)std::max<int64_t>(max_seeds, 1) * 8);
    R_(B.sval, (size_t)std::max<int64_t>(max_seeds, 1) * es);
    if (!P->f64) {
      R_(B.gdense, (size_t)max_cells * es);
      ADT_CUDA(cudaMemset(B.gdense.p, 0, (size_t)max_cells * es));
    }
    if (P->causal || P->dual) {
      R_(B.meta32, (size_t)max_cells * 4);
      R_(B.rec, (size_t)max_cells * 4 * es);
      R_(B.queue, (size_t)max_cells * 4);
    }
  }
  if (P->nsets == 2) {
    ADT_CUDA(cudaStreamCreateWithFlags(&P->stream2, cudaStreamNonBlocking));
    P->ev_sync.resize(1 + P->chunks.size());
    for (auto& e : P->ev_sync) ADT_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  R_(P->d_nseed, (size_t)n_solves * 4);
  R_(P->d_next, (size_t)2 * P->chunks.size() * 4);
  R_(P->d_counters, 4 * 8);
  // level lists per field
  std::vector<uint32_t> lv;
  std::vector<int> ls;
  std::vector<int64_t> lv_off, ls_off;
  for (int f = 0; f < n_fields; ++f) {
    LevelList L = make_levels(P->geoms[f]);
    lv_off.push_back((int64_t)lv.size());
    ls_off.push_back((int64_t)ls.size());
    lv.insert(lv.end(), L.bricks.begin(), L.bricks.end());
    ls.insert(ls.end(), L.start.begin(), L.start.end());
  }
  R_(P->d_levels, lv.size() * 4);
  R_(P->d_lstart, ls.size() * 4);
  ADT_CUDA(cudaMemcpy(P->d_levels.p, lv.data(), lv.size() * 4, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(P->d_lstart.p, ls.data(), ls.size() * 4, cudaMemcpyHostToDevice));
  if (sofs) ADT_CUDA(cudaMemcpy(P->d_sta.p, sta_xyz, (size_t)sofs * 3 * 8, cudaMemcpyHostToDevice));
  // fields
  if (P->f64) {
    std::vector<FieldDev<double>> fdv(n_fields);
    for (int f = 0; f < n_fields; ++f) {
      fdv[f].g = P->geoms[f];
      fdv[f].h = P->h[f];
      fdv[f].f64 = P->d_slow64.as<double>() + P->cell_off[f];
      fdv[f].vel0 = P->d_vel0.as<double>() + P->cell_off[f];
      fdv[f].f = P->d_slowT.as<double>() + 2 * P->cell_off[f];  // f h, then f f h h
      fdv[f].f2 = fdv[f].f + P->geoms[f].ncell;
      fdv[f].bricks = P->d_levels.as<uint32_t>() + lv_off[f];
      fdv[f].lstart = P->d_lstart.as<int>() + ls_off[f];
      fdv[f].sta = P->d_sta.as<double>() + 3 * P->sta_off[f];
      fdv[f].nsta = P->nsta[f];
      set_divisors(fdv[f]);
    }
    R_(P->d_fields, n_fields * sizeof(FieldDev<double>));
    ADT_CUDA(cudaMemcpy(P->d_fields.p, fdv.data(), n_fields * sizeof(FieldDev<double>), cudaMemcpyHostToDevice));
    P->ks = kernels_for<double>(P->bk);
  } else {
    std::vector<FieldDev<float>> fdv(n_fields);
    for (int f = 0; f < n_fields; ++f) {
      fdv[f].g = P->geoms[f];
      fdv[f].h = P->h[f];
      fdv[f].f64 = P->d_slow64.as<double>() + P->cell_off[f];
      fdv[f].vel0 = P->d_vel0.as<double>() + P->cell_off[f];
      fdv[f].f = P->d_slowT.as<float>() + P->cell_off_t[f];  // 64-byte aligned (16-byte loads)
      fdv[f].f2 = nullptr;
      fdv[f].bricks = P->d_levels.as<uint32_t>() + lv_off[f];
      fdv[f].lstart = P->d_lstart.as<int>() + ls_off[f];
      fdv[f].sta = P->d_sta.as<double>() + 3 * P->sta_off[f];
      fdv[f].nsta = P->nsta[f];
      set_divisors(fdv[f]);
    }
    R_(P->d_fields, n_fields * sizeof(FieldDev<float>));
    ADT_CUDA(cudaMemcpy(P->d_fields.p, fdv.data(), n_fields * sizeof(FieldDev<float>), cudaMemcpyHostToDevice));
    P->ks = kernels_for<float>(P->bk);
  }
  ADT_CUDA(cudaMemcpy(P->d_solves.p, P->solves.data(), n_solves * sizeof(SolveDev), cudaMemcpyHostToDevice));
  {
    std::vector<int> ord;
    std::vector<int64_t> uo;
    for (auto& ch : P->chunks) {
      ord.insert(ord.end(), ch.order.begin(), ch.order.end());
      for (int f = 0; f < n_fields; ++f) uo.insert(uo.end(), ch.field_uoff[f].begin(), ch.field_uoff[f].end());
    }
    ADT_CUDA(cudaMemcpy(P->d_order.p, ord.data(), ord.size() * 4, cudaMemcpyHostToDevice));
    std::vector<long long> coff;
    std::vector<int> ccnt;
    for (auto& ch : P->chunks) {
      coff.push_back((long long)ch.dev_order_off);
      ccnt.push_back(ch.count);
    }
    R_(P->d_chunk_off, coff.size() * sizeof(long long));
    R_(P->d_chunk_cnt, ccnt.size() * sizeof(int));
    R_(P->d_cost, (size_t)n_solves * sizeof(unsigned long long));
    ADT_CUDA(cudaMemcpy(P->d_chunk_off.p, coff.data(), coff.size() * sizeof(long long),
                        cudaMemcpyHostToDevice));
    ADT_CUDA(cudaMemcpy(P->d_chunk_cnt.p, ccnt.data(), ccnt.size() * sizeof(int),
                        cudaMemcpyHostToDevice));
    ADT_CUDA(cudaMemset(P->d_cost.p, 0, (size_t)n_solves * sizeof(unsigned long long)));
    if (!uo.empty()) ADT_CUDA(cudaMemcpy(P->d_uoff.p, uo.data(), uo.size() * 8, cudaMemcpyHostToDevice));
  }
  // launch shapes: warp groups (one solve each) per CTA, as many as fit
  ADT_CUDA(cudaDeviceGetAttribute(&P->sm_count, cudaDevAttrMultiProcessorCount, P->dev));
  int smem_optin = 0;
  ADT_CUDA(cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, P->dev));
  P->smem_budget = (size_t)smem_optin - 1024;
  P->fwd_wbytes = P->f64 ? fwd_warp_smem<double>(P->bk) : fwd_warp_smem<float>(P->bk);
  P->adj_wbytes = P->f64 ? adj_warp_smem<double>(P->bk) : adj_warp_smem<float>(P->bk);
  for (auto& g : P->geoms) P->max_nb = std::max(P->max_nb, g.nbx * g.nby * g.nbz);
  P->meta_smem = ((size_t)META_ARRAYS_MAX * P->max_nb * sizeof(int) <= 16384) ? 1 : 0;
  {
    cudaFuncAttributes fa_f, fa_a;
    ADT_CUDA(cudaFuncGetAttributes(&fa_f, P->ks.fwd));
    P->fwd_regs = fa_f.numRegs;
    P->adj_kern[0] = P->ks.adj;
    P->adj_kern[1] = P->ks.adj_causal;
    for (int k = 0; k < 2; ++k) {
      ADT_CUDA(cudaFuncGetAttributes(&fa_a, P->adj_kern[k]));
      P->adj_regs_k[k] = fa_a.numRegs;
      P->adj_maxt_k[k] = fa_a.maxThreadsPerBlock;
    }
    select_solver(P.get(), P->causal);
  }
  // the causal-order adjoint's width is warps per CTA, not a sweep group's
  const int adj_w0 = o.adj_warps ? o.adj_warps : (P->causal ? 0 : o.warps);
  if ((rc = apply_shapes(P.get(), o.warps, o.groups, adj_w0, o.adj_groups ? o.adj_groups : o.groups)))
    return rc;
  int maxsta = 0;
  for (int f = 0; f < n_fields; ++f) maxsta = std::max(maxsta, P->nsta[f]);
  int pw = 1;
  while (pw < 8 * maxsta) pw <<= 1;
  P->mis_smem = (size_t)pw * 16 + (size_t)maxsta * 8 + 16;
  if (P->mis_smem > 160 * 1024) {  // merge arrays in global scratch, one slice per chunk solve
    P->mis_stride = (int64_t)((P->mis_smem + 255) / 256 * 256);
    int cmax = 0;
    for (auto& ch : P->chunks) cmax = std::max(cmax, ch.count);
    for (int k = 0; k < P->nsets; ++k) R_(P->cb[k].mis_scratch, (size_t)P->mis_stride * cmax);
    P->mis_smem = 0;
  }
  ADT_CUDA(cudaFuncSetAttribute(P->ks.misfit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P->mis_smem));
  if (P->opts.ref_compat) {
    int64_t maxc = 0;
    for (auto& g : P->geoms) maxc = std::max(maxc, g.ncell);
    P->snap_stride = maxc;
    R_(P->d_snap, (size_t)maxc * es * P->fwd_ctas * P->fwd_groups);
  }
#undef R_
  P->ev.resize(4 * P->chunks.size() + 2);
  for (auto& e : P->ev) ADT_CUDA(cudaEventCreate(&e));
  *out = P.release();
  return ADT_OK;
}

void batch_destroy(BatchPlan* P) { delete P; }

template <class T>
static BatchArgs<T> make_args(BatchPlan& P, const BatchPlan::Chunk& ch, int which_counter,
                              int set) {
  const BatchPlan::ChunkBufs& CB = P.cb[set];
  BatchArgs<T> A;
  A.fields = P.d_fields.as<FieldDev<T>>();
  A.solves = P.d_solves.as<SolveDev>();
  A.order = P.d_order.as<int>() + ch.dev_order_off;
  A.n_solves = ch.count;
  A.u = CB.u.as<T>();
  A.lam = CB.lam.as<T>();
  A.code = CB.code.as<uint16_t>();
  A.meta = CB.meta.as<int>();
  A.seed_idx = CB.sidx.as<int64_t>();
  A.seed_val = CB.sval.as<T>();
  A.gdense = P.f64 ? nullptr : CB.gdense.as<T>();
  A.n_seed = P.d_nseed.as<int>();
  A.snap = P.opts.ref_compat ? P.d_snap.as<T>() : nullptr;
  A.snap_stride = P.snap_stride;
  A.next = P.d_next.as<int>() + which_counter;
  A.status = P.d_status.as<adt_solve_status>();
  A.counters = P.d_counters.as<unsigned long long>();
  A.cost = P.d_cost.as<unsigned long long>();
  A.tol = P.opts.tol;
  A.wake = P.f64 ? 0.0f : (float)P.opts.wake_tol;
  A.adj_wake = P.f64 ? 0.0f : (float)P.opts.adj_wake_tol;
  A.max_iter = P.opts.max_iter;
  A.adj_max_iter = P.opts.adj_max_iter;
  A.ref_compat = P.opts.ref_compat;
  A.near_r = P.opts.near_src_f64;
  A.group_warps = which_counter % 2 == 0 ? P.fwd_gw : P.adj_gw;
  A.meta_smem = P.meta_smem;
  A.max_nb = P.max_nb;
  A.adj_order_filter = P.opts.adj_order_filter ? 1 : 0;
  A.fwd_order_filter = (!P.f64 && P.opts.fwd_order_filter) ? 1 : 0;
  A.meta32 = P.causal ? CB.meta32.as<uint32_t>() : nullptr;
  A.rec = P.causal ? CB.rec.as<CausalRec<T>>() : nullptr;
  A.queue = P.causal ? CB.queue.as<int>() : nullptr;
  return A;
}

template <class T>
static int enqueue_t(BatchPlan& P, bool capturing) {
  cudaStream_t st = P.stream;
  // inside a graph capture the timing events must be external event nodes
  const unsigned evf = capturing ? cudaEventRecordExternal : cudaEventRecordDefault;
  for (int f = 0; f < P.nf; ++f)
    if (P.f64)
      k_fwd_cells<<<grid1d(P.geoms[f].ncell), 256, 0, st>>>(
          P.d_slow64.as<double>() + P.cell_off[f], P.h[f], P.geoms[f].ncell,
          P.d_slowT.as<double>() + 2 * P.cell_off[f]);
    else
      k_to_t_f32<<<grid1d(P.geoms[f].ncell), 256, 0, st>>>(P.d_slow64.as<double>() + P.cell_off[f],
                                                           P.d_slowT.as<float>() + P.cell_off_t[f],
                                                           P.geoms[f].ncell);
  k_src_init<T><<<(P.ns + 127) / 128, 128, 0, st>>>(P.d_solves.as<SolveDev>(), P.ns,
                                                     P.d_fields.as<FieldDev<T>>(),
                                                     P.src_vel ? 1 : 0,
                                                     P.d_cost.as<unsigned long long>());
  ADT_CUDA(cudaMemsetAsync(P.d_grad.p, 0, P.ncell_total * 8, st));
  ADT_CUDA(cudaMemsetAsync(P.d_counters.p, 0, 4 * 8, st));
  ADT_CUDA(cudaMemsetAsync(P.d_next.p, 0, 2 * P.chunks.size() * 4, st));
  ADT_CUDA(cudaEventRecordWithFlags(P.ev[4 * P.chunks.size()], st, evf));
  const cudaStream_t st0 = P.stream;
  if (P.nsets == 2) {  // fork the second chunk stream off the prologue
    ADT_CUDA(cudaEventRecord(P.ev_sync[0], st0));
    ADT_CUDA(cudaStreamWaitEvent(P.stream2, P.ev_sync[0], 0));
  }
  for (size_t c = 0; c < P.chunks.size(); ++c) {
    const auto& ch = P.chunks[c];
    // chunk c: buffer set and stream c % 2 with overlapping chunks.  The set's
    // previous chunk (c - 2) ran on the same stream, so its buffers are free.
    const int set = P.nsets == 2 ? (int)(c & 1) : 0;
    st = set ? P.stream2 : st0;
    BatchArgs<T> Af = make_args<T>(P, ch, (int)(2 * c), set);
    BatchArgs<T> Aa = make_args<T>(P, ch, (int)(2 * c + 1), set);
    const int gf = std::min(P.fwd_ctas, ch.count);
    const int ga = std::min(P.adj_ctas, ch.count);
    ADT_CUDA(cudaEventRecordWithFlags(P.ev[4 * c + 0], st, evf));
    {
      void* args[] = {&Af};
      ADT_CUDA(cudaLaunchKernel(P.ks.fwd, dim3(gf), dim3(P.fwd_warps * 32), args, P.fwd_smem, st));
    }
    ADT_CUDA(cudaEventRecordWithFlags(P.ev[4 * c + 1], st, evf));
    {
      const double* tobs = P.d_tobs.as<double>();
      const double* w = P.d_w.as<double>();
      double* tp = P.d_tpred.as<double>();
      double* sm = P.d_smis.as<double>();
      unsigned char* scr = P.mis_stride ? P.cb[set].mis_scratch.as<unsigned char>() : nullptr;
      int64_t stride = P.mis_stride;
      void* args[] = {&Af, &tobs, &w, &tp, &sm, &scr, &stride};
      ADT_CUDA(cudaLaunchKernel(P.ks.misfit, dim3(ch.count), dim3(256), args, P.mis_smem, st));
    }
    ADT_CUDA(cudaEventRecordWithFlags(P.ev[4 * c + 2], st, evf));
    {
      void* args[] = {&Aa};
      ADT_CUDA(cudaLaunchKernel(P.ks.adj, dim3(ga), dim3(P.adj_warps * 32), args, P.adj_smem, st));
    }
    ADT_CUDA(cudaEventRecordWithFlags(P.ev[4 * c + 3], st, evf));
    // the gradient sums chunks in order (fixed summation order): after chunk c - 1's
    if (P.nsets == 2 && c > 0) ADT_CUDA(cudaStreamWaitEvent(st, P.ev_sync[c], 0));
    for (int f = 0; f < P.nf; ++f) {
      const int cnt = (int)ch.field_uoff[f].size();
      if (!cnt) continue;
      // lambda: the sweeps' array, or the causal-order adjoint's records
      const T* lam = P.causal ? P.cb[set].rec.as<T>() : P.cb[set].lam.as<T>();
      int lam_stride = P.causal ? 4 : 1;
      int bn = P.causal ? P.geoms[f].n : 0, bl = P.causal ? P.geoms[f].l : 0;  // blocked records
      const int64_t* uo = P.d_uoff.as<int64_t>() + ch.dev_uoff_off[f];
      const double* f64 = P.d_slow64.as<double>() + P.cell_off[f];
      double hh = P.h[f];
      int64_t nc = P.geoms[f].ncell;
      double* gr = P.d_grad.as<double>() + P.cell_off[f];
      int cc = cnt;
      void* args[] = {&lam, &lam_stride, &uo, &cc, &f64, &hh, &nc, &gr, &bn, &bl};
      ADT_CUDA(cudaLaunchKernel(P.ks.grad, dim3(grid1d(nc)), dim3(256), args, 0, st));
    }
    if (P.nsets == 2) ADT_CUDA(cudaEventRecord(P.ev_sync[c + 1], st));
  }
  st = st0;
  if (P.nsets == 2)  // join: the last gradient (on either stream) is done
    ADT_CUDA(cudaStreamWaitEvent(st0, P.ev_sync[P.chunks.size()], 0));
  if (!P.f64)
    for (int f = 0; f < P.nf; ++f)
      k_grad_scale<<<grid1d(P.geoms[f].ncell), 256, 0, st>>>(
          P.d_slow64.as<double>() + P.cell_off[f], P.h[f], P.geoms[f].ncell,
          P.d_grad.as<double>() + P.cell_off[f]);
  k_misfit_sum<<<1, 32, 0, st>>>(P.d_smis.as<double>(), P.ns, P.d_mis.as<double>());
  k_order_by_cost<<<(int)P.chunks.size(), 256, 0, st>>>(
      P.d_order.as<int>(), P.d_chunk_off.as<long long>(), P.d_chunk_cnt.as<int>(),
      P.d_cost.as<unsigned long long>());
  ADT_CUDA(cudaEventRecordWithFlags(P.ev[4 * P.chunks.size() + 1], st, evf));
  ADT_CUDA(cudaGetLastError());
  return ADT_OK;
}

static int enqueue(BatchPlan& P, bool capturing) {
  return P.f64 ? enqueue_t<double>(P, capturing) : enqueue_t<float>(P, capturing);
}

int batch_upload(BatchPlan* P, const double* slowness, const double* t_obs, const double* weight) {
  if (slowness) {
    for (int64_t i = 0; i < P->ncell_total; ++i)
      if (!(slowness[i] > 0.0) || !std::isfinite(slowness[i]))
        return set_error(ADT_EINVAL, "batch: slowness must be finite and > 0 (cell %lld)", (long long)i);
    ADT_CUDA(cudaMemcpyAsync(P->d_slow64.p, slowness, P->ncell_total * 8, cudaMemcpyHostToDevice, P->stream));
    P->uploaded |= 1;
  }
  if (t_obs) {
    ADT_CUDA(cudaMemcpyAsync(P->d_tobs.p, t_obs, P->nobs * 8, cudaMemcpyHostToDevice, P->stream));
    P->uploaded |= 2;
  }
  if (weight) {
    ADT_CUDA(cudaMemcpyAsync(P->d_w.p, weight, P->nobs * 8, cudaMemcpyHostToDevice, P->stream));
    P->uploaded |= 4;
  }
  return ADT_OK;
}

// Pick the kernels' launch widths by timing them on the uploaded inputs:
// every candidate width runs `reps` evaluations and the fastest forward and
// adjoint kernel times (CUDA events around each kernel) win; the two kernels
// are tuned one after the other.  With both adjoint solvers available (FP32,
// ADT_ADJ_AUTO), each solver's widths are timed and the faster solver is
// kept.  Results do not depend on the width (the bricks of a level, and the
// cells of the causal order, are independent), only the time does; the two
// solvers reach the same fixed point of the adjoint system.
int batch_autotune(BatchPlan* P, int reps) {
  if (P->opts.ref_compat)
    return set_error(ADT_EINVAL, "batch: autotune is not available with ref_compat");
  if ((P->uploaded & 7) != 7)
    return set_error(ADT_EINVAL, "batch: upload slowness, t_obs and weight before autotune");
  reps = std::max(1, std::min(reps, 16));
  const int fwd_c[] = {3, 4, 5, 6, 8, 10, 12};
  const int adj_sweeps[] = {2, 3, 4, 6, 7, 8, 9};
  const int adj_causal[] = {4, 8, 12, 16, 24, 32};  // warps per CTA
  auto measure = [&](float& fwd_ms, float& adj_ms) -> int {
    fwd_ms = adj_ms = 1e30f;
    for (int r = 0; r < reps; ++r) {
      int rc = batch_run_resident(P);
      if (rc) return rc;
      ADT_CUDA(cudaStreamSynchronize(P->stream));
      adt_batch_stats st;
      if ((rc = batch_stats(P, &st))) return rc;
      fwd_ms = std::min(fwd_ms, st.fwd_ms);
      adj_ms = std::min(adj_ms, st.adj_ms);
    }
    return ADT_OK;
  };
  int rc, best_f = P->fwd_gw, best_a = P->adj_gw;
  float best_ft = 1e30f, best_at = 1e30f, ft, at;
  for (int gw : fwd_c) {
    if ((rc = apply_shapes(P, gw, 0, best_a, 0))) return rc;
    if (P->fwd_gw != gw) continue;  // did not fit
    if ((rc = measure(ft, at))) return rc;
    if (ft < best_ft) {
      best_ft = ft;
      best_f = gw;
    }
  }
  // the adjoint: each available solver's widths (with both, the faster solver)
  bool best_causal = P->causal;
  const bool solvers[2] = {false, true};
  for (bool causal : solvers) {
    if (!P->dual && causal != P->causal) continue;
    select_solver(P, causal);
    const int* adj_c = causal ? adj_causal : adj_sweeps;
    const int n_adj = causal ? 6 : 7;
    for (int t = 0; t < n_adj; ++t) {
      const int gw = adj_c[t];
      if ((rc = apply_shapes(P, best_f, 0, gw, 0))) return rc;
      if (P->adj_gw != gw) continue;
      if ((rc = measure(ft, at))) return rc;
      if (at < best_at) {
        best_at = at;
        best_a = gw;
        best_causal = causal;
      }
    }
  }
  select_solver(P, best_causal);
  return apply_shapes(P, best_f, 0, best_a, 0);
}

int batch_set_source_velocity(BatchPlan* P, const double* vel0) {
  if (vel0) {
    for (int64_t i = 0; i < P->ncell_total; ++i)
      if (!(vel0[i] > 0.0) || !std::isfinite(vel0[i]))
        return set_error(ADT_EINVAL, "batch: source velocity must be finite and > 0 (cell %lld)",
                         (long long)i);
    ADT_CUDA(cudaMemcpyAsync(P->d_vel0.p, vel0, P->ncell_total * 8, cudaMemcpyHostToDevice,
                             P->stream));
  }
  ADT_CUDA(cudaStreamSynchronize(P->stream));
  if (P->src_vel != (vel0 != nullptr) && P->graph) {  // the source kernel's argument changes
    cudaGraphExecDestroy(P->graph);
    P->graph = nullptr;
  }
  P->src_vel = vel0 != nullptr;
  return ADT_OK;
}

int batch_run_resident(BatchPlan* P) {
  if (!P->opts.use_graph) {
    int rc = enqueue(*P, false);
    if (rc) return rc;
    P->ran = true;
    return ADT_OK;
  }
  if (!P->graph) {
    cudaGraph_t g = nullptr;
    ADT_CUDA(cudaStreamBeginCapture(P->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue(*P, true);
    cudaError_t e = cudaStreamEndCapture(P->stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&P->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphInstantiate");
  }
  ADT_CUDA(cudaGraphLaunch(P->graph, P->stream));
  P->ran = true;
  return ADT_OK;
}

int batch_download(BatchPlan* P, double* misfit, double* t_pred, double* grad,
                   adt_solve_status* status) {
  if (misfit) ADT_CUDA(cudaMemcpyAsync(misfit, P->d_mis.p, 8, cudaMemcpyDeviceToHost, P->stream));
  if (t_pred) ADT_CUDA(cudaMemcpyAsync(t_pred, P->d_tpred.p, P->nobs * 8, cudaMemcpyDeviceToHost, P->stream));
  if (grad) ADT_CUDA(cudaMemcpyAsync(grad, P->d_grad.p, P->ncell_total * 8, cudaMemcpyDeviceToHost, P->stream));
  P->h_status.resize(P->ns);
  ADT_CUDA(cudaMemcpyAsync(P->h_status.data(), P->d_status.p, P->ns * sizeof(adt_solve_status),
                           cudaMemcpyDeviceToHost, P->stream));
  ADT_CUDA(cudaStreamSynchronize(P->stream));
  if (status) std::memcpy(status, P->h_status.data(), P->ns * sizeof(adt_solve_status));
  return ADT_OK;
}

int batch_stats(BatchPlan* P, adt_batch_stats* s) {
  std::memset(s, 0, sizeof(*s));
  s->bk = P->bk;
  s->warps = P->fwd_gw;
  s->groups = P->fwd_groups;
  s->ctas = P->fwd_ctas;
  s->adj_warps = P->adj_gw;
  s->adj_groups = P->adj_groups;
  s->adj_solver = P->causal ? ADT_ADJ_CAUSAL : ADT_ADJ_SWEEPS;
  s->fwd_ms = s->adj_ms = s->total_ms = -1.f;
  if (!P->ran) return ADT_OK;
  ADT_CUDA(cudaStreamSynchronize(P->stream));
  unsigned long long c[4];
  ADT_CUDA(cudaMemcpy(c, P->d_counters.p, sizeof c, cudaMemcpyDeviceToHost));
  s->fwd_cell_updates = (int64_t)c[0];
  s->fwd_bricks = (int64_t)c[1];
  s->adj_cell_updates = (int64_t)c[2];
  s->adj_bricks = (int64_t)c[3];
  float fw = 0.f, aw = 0.f, tot = 0.f, t;
  for (size_t ch = 0; ch < P->chunks.size(); ++ch) {
    ADT_CUDA(cudaEventElapsedTime(&t, P->ev[4 * ch], P->ev[4 * ch + 1]));
    fw += t;
    ADT_CUDA(cudaEventElapsedTime(&t, P->ev[4 * ch + 2], P->ev[4 * ch + 3]));
    aw += t;
  }
  ADT_CUDA(cudaEventElapsedTime(&tot, P->ev[4 * P->chunks.size()], P->ev[4 * P->chunks.size() + 1]));
  s->fwd_ms = fw;
  s->adj_ms = aw;
  s->total_ms = tot;
  return ADT_OK;
}

void* batch_stream(BatchPlan* P) { return (void*)P->stream; }

static_assert(sizeof(CausalRec<double>) == CAUSAL_REC64_BYTES, "record size");

int causal_single_adjoint(const double* d_u, const double* d_u0, const double* d_grad_u, int m,
                          int n, int l, uint32_t* meta, void* rec, int* queue, int* d_complete,
                          void* stream) {
  const Geom g = make_geom(m, n, l, SBK);
  FieldDev<double> fd;
  std::memset(&fd, 0, sizeof fd);
  fd.g = g;
  set_divisors(fd);
  k_single_adj_causal<<<1, ADT_CAUSAL_MAXT / 2, 0, (cudaStream_t)stream>>>(
      d_u, d_u0, d_grad_u, g, fd.div_nl, fd.div_l, meta, static_cast<CausalRec<double>*>(rec), queue,
      d_complete);
  ADT_CUDA(cudaGetLastError());
  return ADT_OK;
}

void* batch_device_buffer(BatchPlan* P, int which) {
  switch (which) {
    case 0: return P->d_slow64.p;
    case 1: return P->d_grad.p;
    case 2: return P->d_tpred.p;
    case 3: return P->d_mis.p;
    default: return nullptr;
  }
}

}  // namespace adt
