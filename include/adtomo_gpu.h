/*
 * adtomo_gpu.h -- C ABI of the GB300 (sm_103a) Eikonal library libadtomo_gpu.so.
 *
 * Drop-in for the hot path of AI4EPS/ADTomo.jl: the TensorFlow custom ops
 * Eikonal / EikonalGrad (deps/CustomOps/Eikonal/Eikonal.cpp) and
 * EikonalThreeD / EikonalThreeDGrad (deps/CustomOps/Eikonal3D/EikonalThreeD.cpp),
 * which the Julia functions eikonal(...) and eikonal3d(...) of
 * src/eikonal_op.jl load through ADCME.load_op_and_grad.  A Julia caller binds
 * these symbols with ccall; the Python package adtomo_gb300 binds them with
 * ctypes.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Unless a function name ends in _device,
 *    every array is HOST memory owned by the caller; results are on the host
 *    when the call returns (the call is synchronous).
 *  - Layouts are the ops' own flat layouts:
 *      2D: (n+1) x (m+1) grid, index j*(m+1)+i   (Eikonal.h:30-48)
 *      3D: m x n x l grid, C order, index i*n*l + j*l + k (Eikonal3D.cpp:6-8)
 *    A column-major Julia Array (m,n,l) is passed as permutedims(A,(3,2,1)).
 *  - Every function returns ADT_OK (0) or a negative ADT_E* code; the message
 *    of the last error on the calling thread is adt_last_error().
 *  - Inputs are validated before any device work (the reference's DCHECKs are
 *    compiled out under -DNDEBUG; these checks replace them).
 */
#ifndef ADTOMO_GPU_H
#define ADTOMO_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ADT_OK 0
#define ADT_EINVAL (-1)    /* bad size, source index, non-finite or <= 0 slowness, ... */
#define ADT_ENOMEM (-2)    /* device allocation failed */
#define ADT_ECUDA (-3)     /* CUDA runtime error (message names the call) */
#define ADT_ETIMEOUT (-4)  /* a bounded device wait ran out of its budget */
#define ADT_ENOCONV (-5)   /* returned only when the caller asked for strict convergence */
#define ADT_ESINGULAR (-6) /* 2D adjoint: a non-source cell has no upwind direction */
#define ADT_ENODEV (-7)    /* no usable sm_103 device */

/* Per-solve convergence record. */
typedef struct adt_solve_status {
  int32_t iters;     /* forward iterations (one iteration = all orderings) */
  int32_t converged; /* 1 if the stopping rule was met before the iteration cap */
  double final_err;  /* last stopping-rule value */
  int32_t adj_iters; /* adjoint iterations (0 if no adjoint ran); 1 for the causal-order
                        adjoint, which evaluates every cell once (adt_batch_opts.adj_solver) */
  int32_t adj_converged;
} adt_solve_status;

/* Message of the last error on the calling thread ("" if none). */
const char* adt_last_error(void);
/* Library version string. */
const char* adt_version(void);
/* Number of usable devices (0 when none); never fails. */
int adt_device_count(void);
/* Sizes of the structs this header defines, for bindings to check their
 * mirrors against: out[0] = sizeof(adt_solve_status), out[1] =
 * sizeof(adt_batch_opts), out[2] = sizeof(adt_batch_stats).  Writes at most
 * n entries and returns the number of structs (3); never fails. */
int adt_abi_struct_sizes(int64_t* out, int n);
/* Shared-memory tile layout of the 3D brick sweeps (bricks of 8 x 4 columns,
 * bk = 16, 32 or 64 cells deep), in elements: out[0] = row stride of a halo
 * tile, out[1] = row stride of an interior tile, out[2] = column stride when
 * the j and k sweep directions agree, out[3] = when they differ, out[4] =
 * elements of a halo tile, out[5] = of an interior tile.  For checks of the
 * index arithmetic; ADT_EINVAL for another bk. */
int adt_tile_layout(int32_t bk, int32_t* out);

/* The plain ops below take host buffers.  Per device they keep their device
 * staging buffers and solver workspaces between calls (grown to the largest
 * grid seen, never shrunk; a staging buffer above 256 MiB is freed when its
 * call ends), and calls on one device run one at a time.
 *
 * ------------------------------------------------------------------------
 * 2D op: replaces Eikonal (Eikonal.cpp:20-46, Compute :74-127).
 * f: slowness, (n+1)*(m+1) doubles; srcx, srcy: 1-based source node (the op
 * subtracts 1, Eikonal.cpp:125); h: grid spacing.  u: travel times out.
 * FP64, bit-identical to the reference forward (Eikonal.h:54-93): 4 orderings,
 * stop when ||u-u_old||/||u_old|| < 1e-8, at most 100 iterations.  A solve
 * that hits the cap returns ADT_OK with status->converged = 0 (the reference
 * prints "ERROR: Eikonal does not converge!", Eikonal.h:88-90).
 * --------------------------------------------------------------------- */
int adt_eikonal(const double* f, int64_t m, int64_t n, int64_t srcx, int64_t srcy, double h,
                double* u, adt_solve_status* status);

/* 2D gradient op: replaces EikonalGrad (Eikonal.cpp:48-63, Compute :141-221).
 * Returns grad_f = dL/df for dL/du = grad_u at the converged u
 * (Eikonal.h:95-200).  The other gradient outputs of the op are never written
 * by the reference (Eikonal.cpp:187-211) and have no counterpart here. */
int adt_eikonal_grad(const double* grad_u, const double* u, const double* f, int64_t m, int64_t n,
                     int64_t srcx, int64_t srcy, double h, double* grad_f);

/* Batched 2D forward: `count` independent solves on one slowness grid, source
 * k at (srcx[k], srcy[k]) (1-based); u holds count*(n+1)*(m+1) doubles. */
int adt_eikonal_batch(const double* f, int64_t m, int64_t n, int64_t count, const int64_t* srcx,
                      const int64_t* srcy, double h, double* u, adt_solve_status* status);

/* ------------------------------------------------------------------------
 * 3D op: replaces EikonalThreeD (EikonalThreeD.cpp:14-45, Compute :77-140).
 * u0: initial values (upper bounds), f: slowness, both m*n*l doubles; tol:
 * stop when max|u-u_old| over an iteration < tol; at most 20 iterations as in
 * the reference (Eikonal3D.cpp:71-88).  FP64, bit-identical to the reference.
 * verbose != 0 prints the per-iteration error like the reference (:82-84).
 * This is the plain single-solve path: one solve per call, FP64, no batching.
 * --------------------------------------------------------------------- */
int adt_eikonal_three_d(const double* u0, const double* f, double h, int64_t m, int64_t n,
                        int64_t l, double tol, int verbose, double* u, adt_solve_status* status);

/* 3D gradient op: replaces EikonalThreeDGrad (EikonalThreeD.cpp:47-65,
 * Compute :154-250; math Eikonal3D.cpp:96-198).  grad_u0 = grad_u where
 * u == u0 exactly (else 0); grad_f = 2 f h^2 lambda with A^T lambda = grad_u
 * solved by reverse causal sweeps.  tol and verbose are accepted for
 * signature parity and unused, as in the reference. */
int adt_eikonal_three_d_grad(const double* grad_u, const double* u, const double* u0,
                             const double* f, double h, int64_t m, int64_t n, int64_t l,
                             double tol, int verbose, double* grad_u0, double* grad_f);

/* Same two ops on DEVICE pointers, enqueued on `stream` (a cudaStream_t, or
 * NULL for the default stream).  The call returns after the work completes. */
int adt_eikonal_three_d_device(const double* u0, const double* f, double h, int64_t m, int64_t n,
                               int64_t l, double tol, int verbose, double* u,
                               adt_solve_status* status, void* stream);
int adt_eikonal_three_d_grad_device(const double* grad_u, const double* u, const double* u0,
                                    const double* f, double h, int64_t m, int64_t n, int64_t l,
                                    double* grad_u0, double* grad_f, void* stream);

/* The 3D op on DEVICE pointers without any device allocation.  No
 * counterpart in the reference: for callers that cannot call cudaMalloc
 * (a framework owning the device heap through its own allocator, hosts with
 * a memory budget fixed at start-up, callers that must not see an allocation
 * fail mid-run).  Same kernels and results as adt_eikonal_three_d_device; the
 * scratch (previous iterate, brick list, error word) is a fixed array of
 * ADT_NOALLOC_SCRATCH_BYTES in the library, resident on every device that
 * loads it until exit.  Grids above ADT_NOALLOC_MAX_CELLS cells return
 * ADT_EINVAL.  The first call on a device looks up the array's address and
 * should come before any stream capture on that device.  All calls on a
 * device share the array: they must not overlap on the GPU (host threads
 * are serialised by the library; the call returns when its work is done). */
#define ADT_NOALLOC_MAX_CELLS 262144
#define ADT_NOALLOC_SCRATCH_BYTES (2 * 1024 * 1024 + 128 * 1024 + 256)
int adt_eikonal_three_d_device_noalloc(const double* u0, const double* f, double h, int64_t m,
                                       int64_t n, int64_t l, double tol, int verbose, double* u,
                                       adt_solve_status* status, void* stream);

/* ------------------------------------------------------------------------
 * Batched misfit + slowness gradient: the per-evaluation loop of
 * scripts/inversion.jl:46-105 (per-source eikonal3d, trilinear sampling at
 * receivers, weighted L2 misfit with missing picks, gradient) for many
 * sources and several fields (P and S, grids of different size) in one plan.
 *
 *   fields f = 0..n_fields-1: dims[3f..3f+2] = (m,n,l), h[f], nsta[f]
 *       receivers at sta_xyz (3 doubles each, fractional 0-based node
 *       coordinates, concatenated over fields)
 *   solves s = 0..n_solves-1: field solve_field[s], source src_xyz[3s..3s+2]
 *       (fractional 0-based node coordinates).  u0 is 1000 everywhere except
 *       the 8 nodes (i, j, k) around the source (ceil and floor of each
 *       coordinate), which get r * f * h in FP64, r their distance to the
 *       source, f the slowness at (ceil x, ceil y, k): one slowness per depth
 *       plane, as scripts/gene_obs.jl:42-51 builds it
 *       (adt_batch_set_source_velocity switches to scripts/inversion.jl's
 *       rule).  No gradient flows through u0.
 *   picks: t_obs and weight, nsta[solve_field[s]] per solve, concatenated;
 *       t_obs == -1 marks a missing pick (scripts/inversion.jl:81).
 *   outputs: misfit = sum weight*(t_obs - t_pred)^2, t_pred (like t_obs),
 *       grad (concatenated fields, m*n*l doubles each) summed over solves in
 *       FP64, status per solve.
 * --------------------------------------------------------------------- */
#define ADT_F32 0
#define ADT_F64 1
/* adjoint solvers of the batched plan (adt_batch_opts.adj_solver) */
#define ADT_ADJ_SWEEPS 0 /* reverse sweeps until nothing changes (brick skipping, filters) */
#define ADT_ADJ_CAUSAL 1 /* one evaluation per cell in reverse causal order */
#define ADT_ADJ_AUTO 2   /* causal; in FP32 adt_batch_autotune also times the sweeps */
/* Receivers per field.  Up to 1024 the seed merge runs in shared memory;
 * above, in device scratch of about 128 bytes per receiver per resident solve. */
#define ADT_BATCH_MAX_RECEIVERS 65536

typedef struct adt_batch_opts {
  int32_t precision;    /* ADT_F32 (default) or ADT_F64 */
  double tol;           /* forward stop: max travel-time decrease in an iteration < tol (s) */
  int32_t max_iter;     /* forward iteration cap (default 200) */
  int32_t adj_max_iter; /* adjoint iteration cap (default 200) */
  int32_t ref_compat;   /* 1: reference stopping rule max|u-u_old| and cap 20 (F64 only) */
  int32_t near_src_f64; /* FP32: cells within this Chebyshev distance of the source
                           box update in FP64 (default 2; -1 disables) */
  int32_t chunk;        /* solves resident at once; forward fields are recomputed
                           per chunk (0 = all solves at once) */
  int32_t bk;           /* brick depth along k: 0 = default (32), else 16, 32 or 64 */
  int32_t warps;        /* warps per solve (one warp group per solve): 0 = default */
  int32_t groups;       /* solves resident per CTA (warp groups): 0 = as many as fit */
  int32_t use_graph;    /* 1 (default): replay the evaluation as a CUDA graph */
  double wake_tol;      /* FP32 forward: a brick whose largest travel-time decrease in a
                           sweep is at most wake_tol (s) does not wake its neighbours;
                           0 (default) = exact skipping.  Ignored in FP64. */
  double adj_wake_tol;  /* FP32 adjoint: a brick whose largest relative adjoint change
                           |new - old| / |new| in a sweep is at most adj_wake_tol wakes
                           no neighbour and does not extend the solve; 0 (default) =
                           exact (iterate until nothing changes).  Ignored in FP64. */
  int32_t adj_order_filter; /* 1 (default): the adjoint sweeps a brick only in the
                           orderings that follow the directions its adjoint values
                           flow in (exact: same fixed point, same bits); 0: every
                           ordering */
  int32_t fwd_order_filter; /* FP32 forward, 1 (default): a brick is swept only in the
                           orderings that follow the upwind directions its earlier
                           sweeps saw (same fixed point, another iteration path);
                           0: every ordering.  Ignored in FP64, which keeps the
                           reference's iteration path. */
  int32_t overlap_chunks; /* with several chunks, 1: keep two chunks resident so that
                           the next chunk's forward runs beside this chunk's adjoint
                           (twice the chunk memory; same results); 0 (default): one
                           chunk at a time.  Not with ref_compat. */
  int32_t adj_warps;    /* adjoint kernel's warps per solve: 0 = as `warps` */
  int32_t adj_groups;   /* adjoint kernel's solves per CTA: 0 = as `groups` */
  int32_t adj_solver;   /* ADT_ADJ_AUTO (default), ADT_ADJ_SWEEPS or ADT_ADJ_CAUSAL.
                           The adjoint system of a solve is triangular in travel-time order
                           (a cell's row reads only its users, whose travel times
                           are larger), so it is solved by evaluating every cell
                           once, after its users, in rounds of cells whose users
                           are done (one solve per CTA; adj_warps = warps per CTA,
                           adj_groups and the adjoint wake tolerance and filter
                           ignored).  Same formula per cell: the exact sweeps'
                           fixed point.  Needs fewer than 2^31 cells per field.
                           Which is faster depends on the model: one causal pass
                           against the sweeps' iterations, which rough models
                           need more of.  ADT_ADJ_AUTO starts with the causal
                           solve; in FP32 it also keeps the sweeps' buffers and
                           adt_batch_autotune times both and keeps the faster
                           (adt_batch_stats.adj_solver tells which runs).
                           Device memory per cell of each resident solve: sweeps
                           6 bytes, causal 24 (FP32; 40 in FP64), both 30. */
} adt_batch_opts;

typedef struct adt_batch adt_batch;

void adt_batch_opts_default(adt_batch_opts* opts);

int adt_batch_create(adt_batch** out, int32_t n_fields, const int32_t* dims, const double* h,
                     const int32_t* nsta, const double* sta_xyz, int32_t n_solves,
                     const int32_t* solve_field, const double* src_xyz,
                     const adt_batch_opts* opts);
int adt_batch_destroy(adt_batch* b);

/* One evaluation end to end: host inputs are copied to the device, the
 * evaluation runs, host outputs are written.  slowness: concatenated fields
 * (doubles); t_obs/weight as described above.  Any output pointer may be NULL. */
int adt_batch_run(adt_batch* b, const double* slowness, const double* t_obs, const double* weight,
                  double* misfit, double* t_pred, double* grad, adt_solve_status* status);

/* Near-source initial values from a fixed velocity model: the 8 nodes around
 * each source get r * h / vel0[node] (r their distance to the source), as
 * scripts/inversion.jl:52-60 builds u0 from the starting model vel0 and keeps
 * it while the model changes.  vel0: all fields, concatenated like the
 * slowness of adt_batch_run, finite and > 0.  NULL returns to the default
 * rule of scripts/gene_obs.jl (the evaluation's own slowness; see
 * adt_batch_create).  Either way the values are constants of the
 * evaluation: no gradient flows through them. */
int adt_batch_set_source_velocity(adt_batch* b, const double* vel0);

/* Autotuner of the launch shapes: after adt_batch_upload of all three
 * inputs, times the forward and the adjoint kernels over candidate widths
 * (reps evaluations each, 1-16) on those inputs and keeps the fastest of each
 * (visible in adt_batch_stats_get).  With both adjoint solvers available
 * (ADT_ADJ_AUTO in FP32) it times both and keeps the faster solver.  Results
 * do not depend on the width; the two solvers reach the same fixed point of
 * the adjoint system (bit for bit on depths that are multiples of 8).  Not
 * available with ref_compat. */
int adt_batch_autotune(adt_batch* b, int32_t reps);

/* Device-resident use: upload inputs once, run, read outputs later.  upload
 * takes host pointers (NULL leaves that input unchanged); run_resident enqueues
 * one evaluation on the plan's stream without synchronising; download copies
 * outputs to host pointers (NULL skips) after synchronising. */
int adt_batch_upload(adt_batch* b, const double* slowness, const double* t_obs,
                     const double* weight);
int adt_batch_run_resident(adt_batch* b);
int adt_batch_download(adt_batch* b, double* misfit, double* t_pred, double* grad,
                       adt_solve_status* status);
/* The plan's cudaStream_t (for event timing by the caller). */
void* adt_batch_stream(adt_batch* b);
/* Device pointers of the plan's resident buffers (for zero-copy callers):
 * which = 0 slowness (F64), 1 grad (F64), 2 t_pred (F64), 3 misfit (F64, 1). */
void* adt_batch_device_buffer(adt_batch* b, int32_t which);
/* Counters of the last evaluation: cell updates performed by the forward and
 * the adjoint sweeps, bricks processed, and device times in ms of the
 * forward sweep, adjoint sweep, and whole evaluation (measured with CUDA
 * events on the plan's stream; -1 when unavailable). */
typedef struct adt_batch_stats {
  int64_t fwd_cell_updates;
  int64_t adj_cell_updates;
  int64_t fwd_bricks;
  int64_t adj_bricks;
  float fwd_ms;
  float adj_ms;
  float total_ms;
  int32_t bk;
  int32_t warps;  /* warps per solve (group) of the forward kernel */
  int32_t groups; /* solves resident per CTA in the forward kernel */
  int32_t ctas;
  int32_t adj_warps;  /* the same for the adjoint kernel */
  int32_t adj_groups;
  int32_t adj_solver; /* the adjoint solver the evaluations use: ADT_ADJ_SWEEPS or
                         ADT_ADJ_CAUSAL */
} adt_batch_stats;
int adt_batch_stats_get(adt_batch* b, adt_batch_stats* out);

/* ------------------------------------------------------------------------
 * Smoothness penalty of the inversion (replaces the TF graph of
 * scripts/inversion.jl:107-121): penalty = lambda * sum |v - S v| over the
 * m x n x l model v (C order), S the mean over an sh x sh x sv box centred
 * on each cell with circular wrap-around (the reference's tf.concat padding +
 * VALID conv3d).  grad (may be NULL) receives lambda * (s - S s), s =
 * sign(v - S v): the gradient of the penalty with respect to v.  sh and sv
 * are odd; (sh-1)/2 <= m, n and (sv-1)/2 <= l.  FP64 throughout; the sum is
 * reduced in a fixed order, so repeated calls give identical results. */
int adt_smooth_l1(const double* v, int64_t m, int64_t n, int64_t l, int32_t sh, int32_t sv,
                  double lambda, double* penalty, double* grad);
/* The same on device pointers (penalty: one device double), on `stream`. */
int adt_smooth_l1_device(const double* v, int64_t m, int64_t n, int64_t l, int32_t sh,
                         int32_t sv, double lambda, double* penalty, double* grad, void* stream);

/* ------------------------------------------------------------------------
 * 2D-table event location (replaces the torch closure of
 * tests/Eikonal/eikoloc.py:157-206): for every event e, at params[4e..4e+3]
 * = (t0, x, y, z), the loss
 *   mean over its P picks of w huber(t - (t0 + T_P(r, |z| - z_sta)))
 *   + the same over its S picks
 *   + gamma * mean over pick pairs of one phase of w_i w_j huber(dT_ij - dt_ij)
 * and its gradient with respect to (t0, x, y, z).  Picks of event e are
 * [offs[e], offs[e+1]) of sta_xyz (3 per pick), t_obs, phase (0 = P,
 * 1 = S) and weight.  table_p/table_s: m x n travel times on the grid
 * r = r0 + i h, z = z0 + j h, read bilinearly with the cell clamped to the
 * table (eikoloc.py:119-145).  bounds: (xmin, xmax, ymin, ymax, zmin, zmax);
 * the position is clamped to them (a clamped coordinate has no gradient).
 * huber: delta 1 (torch's default).  With gamma != 0 an event may have at most
 * 256 picks.  FP64; host pointers; loss (n_events), grad (4 n_events) out. */
int adt_locate_loss_grad(int32_t n_events, const double* params, const int64_t* offs,
                         const double* sta_xyz, const double* t_obs, const int32_t* phase,
                         const double* weight, const double* table_p, const double* table_s,
                         int32_t m, int32_t n, double r0, double z0, double h,
                         const double* bounds, double gamma, double* loss, double* grad);

#ifdef __cplusplus
}
#endif
#endif
