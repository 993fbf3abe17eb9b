/*
 * eikonal_oracle.h -- CPU restatement of ADTomo.jl's Eikonal hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA library under
 * adtomo.jl_gb300/) links, loads or calls this code.  Only tests/, the smoke
 * check in __graft_entry__.py and the cpu_baseline / reference arm of bench.py
 * use it, and only as the checker or as the timed CPU baseline.
 *
 * Parity status: pinned.  The forward and adjoint are checked against golden
 * vectors produced by the reference's own C++ sources (deps/CustomOps/Eikonal/
 * Eikonal.h and deps/CustomOps/Eikonal3D/Eikonal3D.cpp) compiled by
 * oracle/Makefile into oracle/_ref/, see tests/golden/make_golden.py.
 *
 * Layouts follow the reference ops exactly:
 *   2D: grid of (n+1) rows x (m+1) columns, index j*(m+1)+i   (Eikonal.h:30-48)
 *   3D: grid m x n x l, C order, index i*n*l + j*l + k         (Eikonal3D.cpp:6-8)
 * Source indices given to the 2D functions are 0-based (the TF op subtracts 1,
 * Eikonal.cpp:125,219).
 */
#ifndef ADTOMO_EIKONAL_ORACLE_H
#define ADTOMO_EIKONAL_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 2D forward, Eikonal.h:54-93.  Returns 1 if converged (rel-L2 change < 1e-8
 * within 100 iterations), else 0.  *iters receives the iterations executed. */
int orc_eik2d_forward(const double* f, int m, int n, double h, int ix, int jx,
                      double* u, int* iters);

/* 2D adjoint, Eikonal.h:95-200.  Solves A^T lambda = grad_u exactly by causal
 * (descending travel time) substitution.  Returns 0, or -6 if a non-source
 * cell has no upwind direction (the reference's matrix is singular then). */
int orc_eik2d_backward(const double* grad_u, const double* u, const double* f,
                       int m, int n, double h, int ix, int jx, double* grad_f);

/* 3D forward, Eikonal3D.cpp:71-94 (solve + forward).  max_iter is 20 in the
 * reference (hard-coded at :74).  Returns iterations executed; *final_err is
 * the last max|u - u_old|. */
int orc_eik3d_forward(const double* u0, const double* f, double h, int m, int n,
                      int l, double tol, int max_iter, double* u,
                      double* final_err);

/* 3D adjoint, Eikonal3D.cpp:96-198.  Returns 0. */
int orc_eik3d_backward(const double* grad_u, const double* u, const double* u0,
                       const double* f, double h, int m, int n, int l,
                       double* grad_u0, double* grad_f);

/* Assembled adjoint matrix A (before the transpose) as COO triplets with
 * duplicates kept, for cross-checking the causal solve against a general
 * sparse LU.  Returns the number of triplets written (at most cap), or -1 when
 * cap is too small.  dim==2 uses (m,n,ix,jx); dim==3 uses (m,n,l,u0). */
int64_t orc_assemble(int dim, const double* u, const double* u0, int m, int n,
                     int l, int ix, int jx, int64_t cap, int64_t* rows,
                     int64_t* cols, double* vals, double* rhs_mask);

/* Near-source initial condition: u0 = 1000 everywhere, and the 8 nodes
 * (i, j, k) around the fractional source (sx,sy,sz) (0-based node
 * coordinates; ceil and floor of each) get a value from the distance
 * r = sqrt(dx^2+dy^2+dz^2) (dx = sx - i, ...):
 *   ORC_SRC_GENE_OBS  (a = slowness) r * a[ceil sx, ceil sy, k] * h: one
 *                     slowness per depth plane, taken at the (ceil, ceil)
 *                     column (scripts/gene_obs.jl:42-51);
 *   ORC_SRC_INVERSION (a = velocity) r * h / a[i, j, k]
 *                     (scripts/inversion.jl:52-60, with a = vel0);
 *   ORC_SRC_NODE      (a = slowness) r * a[i, j, k] * h. */
#define ORC_SRC_GENE_OBS 0
#define ORC_SRC_INVERSION 1
#define ORC_SRC_NODE 2
void orc_src_u0(const double* a, int m, int n, int l, double h, double sx,
                double sy, double sz, int mode, double* u0);

/* Trilinear travel-time sample at a fractional node position, with the
 * branch structure of scripts/inversion.jl:64-95 (0-based).  If w is not
 * NULL, the 8 node indices and their weights (dT/du) are written to idx/w;
 * returns the sampled value. */
double orc_sample(const double* u, int m, int n, int l, double x, double y,
                  double z, int64_t* idx, double* w);

/* Batched misfit and slowness gradient over many sources on several fields,
 * the caller pattern of scripts/inversion.jl:46-105 with events as sources.
 *
 *   fields:  n_fields grids, dims[3*f], h[f], slowness concatenated;
 *            stations per field nsta[f], sta_xyz concatenated (3 per station)
 *   solves:  field index, source position src_xyz[3*s]
 *   t_obs / weight: concatenated per solve, nsta[field] entries; t_obs == -1
 *            marks a missing pick (inversion.jl:81)
 *   out:     misfit = sum w (t_obs - t_pred)^2; t_pred (same layout as t_obs);
 *            grad (concatenated fields, summed over solves); iters per solve
 *            (forward iterations executed).  src_mode: the near-source rule
 *            of orc_src_u0; src_model: its array (all fields, concatenated),
 *            or NULL for the evaluation's own slowness (ORC_SRC_GENE_OBS and
 *            ORC_SRC_NODE only).  u0 is treated as a constant
 *            input (inversion.jl builds it from vel0), so no gradient flows
 *            through the near-source initial values.
 * nthreads > 1 runs solves on that many POSIX threads; results do not depend
 * on nthreads except for summation order of the gradient (per-thread partial
 * sums added in thread order).  Returns 0 or a negative error. */
int orc_batch_misfit_grad(int n_fields, const int32_t* dims, const double* h,
                          const double* slowness, const int32_t* nsta,
                          const double* sta_xyz, int n_solves,
                          const int32_t* solve_field, const double* src_xyz,
                          const double* t_obs, const double* weight, double tol,
                          int max_iter, int nthreads, int src_mode,
                          const double* src_model, double* misfit,
                          double* t_pred, double* grad, int32_t* iters);

#ifdef __cplusplus
}
#endif
#endif
