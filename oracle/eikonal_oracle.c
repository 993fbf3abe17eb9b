/*
 * eikonal_oracle.c -- CPU restatement of ADTomo.jl's Eikonal hot path.
 *
 * TEST INFRASTRUCTURE ONLY (see eikonal_oracle.h).  Parity pinned against the
 * reference sources compiled in oracle/_ref (tests/golden).
 *
 * The per-cell arithmetic deliberately keeps the reference's operation order
 * (same products, sums, divisions and square roots in the same sequence), so
 * that the FP64 forward is bit-identical to the reference.  Build with
 * -ffp-contract=off: the reference is compiled for x86-64 without FMA, and
 * aarch64 compilers would otherwise fuse multiply-adds.
 */
#define _GNU_SOURCE
#include "eikonal_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* std::min / std::max semantics of the reference: min(a,b) = (b < a) ? b : a */
static inline double ref_min(double a, double b) { return (b < a) ? b : a; }
static inline double ref_max(double a, double b) { return (a < b) ? b : a; }

/* ------------------------------------------------------------------------ */
/* 2D                                                                        */
/* ------------------------------------------------------------------------ */

/* Two-term upwind update, Eikonal.h:14-20. */
static double upd2(double a, double b, double f, double h) {
  double d = fabs(a - b);
  if (d >= f * h) return ref_min(a, b) + f * h;
  return (a + b + sqrt(2 * f * f * h * h - (a - b) * (a - b))) / 2;
}

/* One Gauss-Seidel ordering, Eikonal.h:22-52: columns i outer (direction si),
 * rows j inner (direction sj); the source cell is skipped; at the grid edge
 * the neighbour candidate is the single interior neighbour. */
static void sweep2(double* u, const double* f, int m, int n, double h, int ix,
                   int jx, int si, int sj) {
  const int w = m + 1;
  for (int a = 0; a <= m; ++a) {
    const int i = si > 0 ? a : m - a;
    for (int b = 0; b <= n; ++b) {
      const int j = sj > 0 ? b : n - b;
      if (i == ix && j == jx) continue;
      double ax, by;
      if (i == 0)
        ax = u[j * w + 1];
      else if (i == m)
        ax = u[j * w + m - 1];
      else
        ax = ref_min(u[j * w + i + 1], u[j * w + i - 1]);
      if (j == 0)
        by = u[w + i];
      else if (j == n)
        by = u[(n - 1) * w + i];
      else
        by = ref_min(u[(j - 1) * w + i], u[(j + 1) * w + i]);
      const double un = upd2(ax, by, f[j * w + i], h);
      u[j * w + i] = ref_min(u[j * w + i], un);
    }
  }
}

int orc_eik2d_forward(const double* f, int m, int n, double h, int ix, int jx,
                      double* u, int* iters) {
  const int w = m + 1;
  const size_t N = (size_t)(m + 1) * (n + 1);
  for (int i = 0; i <= m; ++i)
    for (int j = 0; j <= n; ++j) u[j * w + i] = (i == ix && j == jx) ? 0.0 : 100000.0;
  double* prev = (double*)malloc(N * sizeof(double));
  memcpy(prev, u, N * sizeof(double));
  int converged = 0, it;
  /* orderings (I,J), (iI,J), (iI,iJ), (I,iJ): Eikonal.h:74-77 */
  static const int ord[4][2] = {{1, 1}, {-1, 1}, {-1, -1}, {1, -1}};
  for (it = 0; it < 100; ++it) {
    for (int o = 0; o < 4; ++o) sweep2(u, f, m, n, h, ix, jx, ord[o][0], ord[o][1]);
    double dd = 0.0, pp = 0.0;
    for (size_t p = 0; p < N; ++p) {
      const double d = u[p] - prev[p];
      dd += d * d;
      pp += prev[p] * prev[p];
    }
    const double err = sqrt(dd) / sqrt(pp);
    if (err < 1e-8) {
      converged = 1;
      break;
    }
    memcpy(prev, u, N * sizeof(double));
  }
  free(prev);
  if (iters) *iters = converged ? it + 1 : it;
  return converged;
}

/* Upwind neighbour along one axis for the adjoint, Eikonal.h:116-179 and
 * Eikonal3D.cpp:189-197: the single interior neighbour at an edge, else the
 * smaller of the two with ties going to the +1 side. */
static inline int64_t upwind_nb(const double* u, int64_t p, int pos, int ext,
                                int64_t stride) {
  if (pos == 0) return p + stride;
  if (pos == ext - 1) return p - stride;
  return (u[p + stride] > u[p - stride]) ? p - stride : p + stride;
}

static int cmp_desc_r(const void* a, const void* b, void* ctx) {
  const double* u = (const double*)ctx;
  const double ua = u[*(const int64_t*)a], ub = u[*(const int64_t*)b];
  if (ua > ub) return -1;
  if (ua < ub) return 1;
  return 0;
}

/* Cells sorted by descending travel time.  Every off-diagonal coupling of the
 * adjoint system links a cell to a neighbour with strictly larger travel time
 * (the activity test is a strict '>'), so this order makes A^T triangular.
 * Non-negative doubles order like their bit patterns, so an LSD radix sort on
 * the inverted bits gives the descending order; anything else (negative or
 * NaN travel times) falls back to a comparison sort. */
static int64_t* causal_order(const double* u, int64_t N) {
  int64_t* ord = (int64_t*)malloc((size_t)N * sizeof(int64_t));
  int radix_ok = 1;
  for (int64_t p = 0; p < N; ++p) {
    ord[p] = p;
    if (!(u[p] >= 0.0)) radix_ok = 0;
  }
  if (!radix_ok) {
    qsort_r(ord, (size_t)N, sizeof(int64_t), cmp_desc_r, (void*)u);
    return ord;
  }
  uint64_t* key = (uint64_t*)malloc((size_t)N * sizeof(uint64_t));
  uint64_t* key2 = (uint64_t*)malloc((size_t)N * sizeof(uint64_t));
  int64_t* ord2 = (int64_t*)malloc((size_t)N * sizeof(int64_t));
  for (int64_t p = 0; p < N; ++p) {
    uint64_t b;
    double v = u[p] + 0.0; /* folds -0 into +0 */
    memcpy(&b, &v, sizeof b);
    key[p] = ~b;
  }
  for (int pass = 0; pass < 8; ++pass) {
    const int sh = 8 * pass;
    int64_t cnt[257];
    memset(cnt, 0, sizeof cnt);
    for (int64_t p = 0; p < N; ++p) ++cnt[((key[p] >> sh) & 255u) + 1];
    if (cnt[((key[0] >> sh) & 255u) + 1] == N) continue; /* digit constant */
    for (int d = 0; d < 256; ++d) cnt[d + 1] += cnt[d];
    for (int64_t p = 0; p < N; ++p) {
      const int64_t dst = cnt[(key[p] >> sh) & 255u]++;
      key2[dst] = key[p];
      ord2[dst] = ord[p];
    }
    uint64_t* tk = key; key = key2; key2 = tk;
    int64_t* to = ord; ord = ord2; ord2 = to;
  }
  free(key);
  free(key2);
  free(ord2);
  return ord;
}

int orc_eik2d_backward(const double* grad_u, const double* u, const double* f,
                       int m, int n, double h, int ix, int jx, double* grad_f) {
  const int w = m + 1;
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  const int64_t src = (int64_t)jx * w + ix;
  double* lam = (double*)calloc((size_t)N, sizeof(double));
  int64_t* ord = causal_order(u, N);
  int rc = 0;
  for (int64_t q = 0; q < N; ++q) {
    const int64_t c = ord[q];
    const int i = (int)(c % w), j = (int)(c / w);
    /* column c of A: rows r that use c as their active upwind neighbour */
    double acc = grad_u[c];
    for (int s = 0; s < 4; ++s) {
      int ri = i, rj = j;
      if (s == 0) ri = i - 1;
      if (s == 1) ri = i + 1;
      if (s == 2) rj = j - 1;
      if (s == 3) rj = j + 1;
      if (ri < 0 || ri > m || rj < 0 || rj > n) continue;
      const int64_t r = (int64_t)rj * w + ri;
      if (r == src) continue; /* identity row */
      const int64_t nb = (s < 2) ? upwind_nb(u, r, ri, m + 1, 1) : upwind_nb(u, r, rj, n + 1, w);
      if (nb != c || !(u[r] > u[c])) continue;
      acc += 2 * (u[r] - u[c]) * lam[r];
    }
    double diag;
    if (c == src) {
      diag = 1.0;
    } else {
      diag = 0.0;
      const int64_t nx = upwind_nb(u, c, i, m + 1, 1);
      const int64_t ny = upwind_nb(u, c, j, n + 1, w);
      if (u[c] > u[nx]) diag += 2 * (u[c] - u[nx]);
      if (u[c] > u[ny]) diag += 2 * (u[c] - u[ny]);
    }
    if (diag == 0.0) {
      rc = -6;
      break;
    }
    lam[c] = acc / diag;
  }
  for (int64_t p = 0; p < N; ++p) {
    const double dfdf = (p == src) ? 0.0 : -2 * f[p] * h * h;
    grad_f[p] = -lam[p] * dfdf;
  }
  free(ord);
  free(lam);
  return rc;
}

/* ------------------------------------------------------------------------ */
/* 3D                                                                        */
/* ------------------------------------------------------------------------ */

/* Sorted three-term upwind update, Eikonal3D.cpp:11-28. */
static double upd3(double a1, double a2, double a3, double f, double h) {
  double t;
  if (a1 > a2) { t = a1; a1 = a2; a2 = t; }
  if (a1 > a3) { t = a1; a1 = a3; a3 = t; }
  if (a2 > a3) { t = a2; a2 = a3; a3 = t; }
  double x = a1 + f * h;
  if (x <= a2) return x;
  double B = -(a1 + a2);
  double C = (a1 * a1 + a2 * a2 - f * f * h * h) / 2.0;
  x = (-B + sqrt(B * B - 4 * C)) / 2.0;
  if (x <= a3) return x;
  B = -2.0 * (a1 + a2 + a3) / 3.0;
  C = (a1 * a1 + a2 * a2 + a3 * a3 - f * f * h * h) / 3.0;
  x = (-B + sqrt(B * B - 4 * C)) / 2.0;
  return x;
}

/* Axis candidate: the single interior neighbour at an edge, else the smaller
 * of the two (Eikonal3D.cpp:47-52). */
static inline double axis_min(const double* u, int64_t p, int pos, int ext,
                              int64_t stride) {
  if (pos == 0) return u[p + stride];
  if (pos == ext - 1) return u[p - stride];
  return ref_min(u[p + stride], u[p - stride]);
}

/* One ordering, Eikonal3D.cpp:35-57: i outer, j, k inner; every cell updated. */
static void sweep3(double* u, const double* f, double h, int m, int n, int l,
                   int si, int sj, int sk) {
  const int64_t sI = (int64_t)n * l, sJ = l;
  for (int a = 0; a < m; ++a) {
    const int i = si > 0 ? a : m - 1 - a;
    for (int b = 0; b < n; ++b) {
      const int j = sj > 0 ? b : n - 1 - b;
      for (int c = 0; c < l; ++c) {
        const int k = sk > 0 ? c : l - 1 - c;
        const int64_t p = i * sI + j * sJ + k;
        const double ax = axis_min(u, p, i, m, sI);
        const double ay = axis_min(u, p, j, n, sJ);
        const double az = axis_min(u, p, k, l, 1);
        const double un = upd3(ax, ay, az, f[p], h);
        u[p] = ref_min(un, u[p]);
      }
    }
  }
}

/* The 8 orderings in the reference's sequence, Eikonal3D.cpp:59-68. */
static const int ORD3[8][3] = {{1, 1, 1},  {-1, 1, 1},  {-1, -1, 1}, {1, -1, 1},
                               {1, -1, -1}, {1, 1, -1}, {-1, 1, -1}, {-1, -1, -1}};

int orc_eik3d_forward(const double* u0, const double* f, double h, int m, int n,
                      int l, double tol, int max_iter, double* u,
                      double* final_err) {
  const size_t N = (size_t)m * n * l;
  memcpy(u, u0, N * sizeof(double));
  double* prev = (double*)malloc(N * sizeof(double));
  int it, done = 0;
  double err = 0.0;
  for (it = 0; it < max_iter; ++it) {
    memcpy(prev, u, N * sizeof(double));
    for (int o = 0; o < 8; ++o) sweep3(u, f, h, m, n, l, ORD3[o][0], ORD3[o][1], ORD3[o][2]);
    err = 0.0;
    for (size_t p = 0; p < N; ++p) err = ref_max(fabs(u[p] - prev[p]), err);
    if (err < tol) {
      done = 1;
      break;
    }
  }
  free(prev);
  if (final_err) *final_err = err;
  return done ? it + 1 : it;
}

/* A cell is fixed (identity row, zero seed) when its travel time equals the
 * initial value or when no axis is active, Eikonal3D.cpp:126-130,168-171. */
static int fixed3(const double* u, const double* u0, int64_t p, int i, int j,
                  int k, int m, int n, int l) {
  if (u[p] == u0[p]) return 1;
  const int64_t sI = (int64_t)n * l, sJ = l;
  const double ax = axis_min(u, p, i, m, sI);
  const double ay = axis_min(u, p, j, n, sJ);
  const double az = axis_min(u, p, k, l, 1);
  return !(u[p] > ax || u[p] > ay || u[p] > az);
}

int orc_eik3d_backward(const double* grad_u, const double* u, const double* u0,
                       const double* f, double h, int m, int n, int l,
                       double* grad_u0, double* grad_f) {
  const int64_t N = (int64_t)m * n * l;
  const int64_t sI = (int64_t)n * l, sJ = l;
  for (int64_t p = 0; p < N; ++p) grad_u0[p] = (u[p] == u0[p]) ? grad_u[p] : 0.0;
  unsigned char* fx = (unsigned char*)malloc((size_t)N);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < l; ++k) {
        const int64_t p = i * sI + j * sJ + k;
        fx[p] = (unsigned char)fixed3(u, u0, p, i, j, k, m, n, l);
      }
  double* lam = (double*)calloc((size_t)N, sizeof(double));
  int64_t* ord = causal_order(u, N);
  const int ext[3] = {m, n, l};
  const int64_t str[3] = {sI, sJ, 1};
  for (int64_t q = 0; q < N; ++q) {
    const int64_t c = ord[q];
    if (fx[c]) continue; /* identity row with zero seed: lambda = 0 */
    const int pos[3] = {(int)(c / sI), (int)((c / sJ) % n), (int)(c % l)};
    double acc = grad_u[c];
    for (int ax = 0; ax < 3; ++ax) {
      for (int side = -1; side <= 1; side += 2) {
        const int rp = pos[ax] + side;
        if (rp < 0 || rp >= ext[ax]) continue;
        const int64_t r = c + side * str[ax];
        if (fx[r]) continue; /* couplings to fixed cells are zeroed */
        if (upwind_nb(u, r, rp, ext[ax], str[ax]) != c || !(u[r] > u[c])) continue;
        acc += 2.0 * (u[r] - u[c]) * lam[r];
      }
    }
    double diag = 0.0;
    for (int ax = 0; ax < 3; ++ax) {
      const double a = axis_min(u, c, pos[ax], ext[ax], str[ax]);
      if (u[c] > a) diag += 2.0 * (u[c] - a);
    }
    lam[c] = acc / diag;
  }
  for (int64_t p = 0; p < N; ++p) {
    const double rhs = -2 * f[p] * h * h;
    grad_f[p] = -lam[p] * rhs;
  }
  free(ord);
  free(lam);
  free(fx);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Assembled matrices for the sparse-LU cross-check                          */
/* ------------------------------------------------------------------------ */

#define PUSH(R, C, V)                     \
  do {                                    \
    if (nt >= cap) return -1;             \
    rows[nt] = (R);                       \
    cols[nt] = (C);                       \
    vals[nt] = (V);                       \
    ++nt;                                 \
  } while (0)

int64_t orc_assemble(int dim, const double* u, const double* u0, int m, int n,
                     int l, int ix, int jx, int64_t cap, int64_t* rows,
                     int64_t* cols, double* vals, double* rhs_mask) {
  int64_t nt = 0;
  if (dim == 2) {
    const int w = m + 1;
    for (int j = 0; j <= n; ++j)
      for (int i = 0; i <= m; ++i) {
        const int64_t c = (int64_t)j * w + i;
        rhs_mask[c] = 1.0;
        if (i == ix && j == jx) {
          PUSH(c, c, 1.0);
          continue;
        }
        const int64_t nx = upwind_nb(u, c, i, m + 1, 1);
        if (u[c] > u[nx]) {
          PUSH(c, c, 2 * (u[c] - u[nx]));
          PUSH(c, nx, 2 * (u[nx] - u[c]));
        }
        const int64_t ny = upwind_nb(u, c, j, n + 1, w);
        if (u[c] > u[ny]) {
          PUSH(c, c, 2 * (u[c] - u[ny]));
          PUSH(c, ny, 2 * (u[ny] - u[c]));
        }
      }
    return nt;
  }
  const int64_t sI = (int64_t)n * l, sJ = l, N = (int64_t)m * n * l;
  unsigned char* fx = (unsigned char*)calloc((size_t)N, 1);
  const int ext[3] = {m, n, l};
  const int64_t str[3] = {sI, sJ, 1};
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < n; ++j)
      for (int k = 0; k < l; ++k) {
        const int64_t c = i * sI + j * sJ + k;
        rhs_mask[c] = 1.0;
        fx[c] = (unsigned char)fixed3(u, u0, c, i, j, k, m, n, l);
        if (u[c] == u0[c]) continue;
        const int pos[3] = {i, j, k};
        for (int ax = 0; ax < 3; ++ax) {
          const double a = axis_min(u, c, pos[ax], ext[ax], str[ax]);
          if (u[c] > a) {
            PUSH(c, c, 2.0 * (u[c] - a));
            PUSH(c, upwind_nb(u, c, pos[ax], ext[ax], str[ax]), -2.0 * (u[c] - a));
          }
        }
      }
  for (int64_t t = 0; t < nt; ++t)
    if (fx[rows[t]] || fx[cols[t]]) vals[t] = 0.0;
  for (int64_t c = 0; c < N; ++c)
    if (fx[c]) {
      rhs_mask[c] = 0.0;
      if (nt >= cap) {
        free(fx);
        return -1;
      }
      rows[nt] = c;
      cols[nt] = c;
      vals[nt] = 1.0;
      ++nt;
    }
  free(fx);
  return nt;
}

/* ------------------------------------------------------------------------ */
/* Sources, receivers, misfit                                                */
/* ------------------------------------------------------------------------ */

void orc_src_u0(const double* a, int m, int n, int l, double h, double sx,
                double sy, double sz, int mode, double* u0) {
  const int64_t N = (int64_t)m * n * l;
  for (int64_t p = 0; p < N; ++p) u0[p] = 1000.0;
  const int xs[2] = {(int)ceil(sx), (int)floor(sx)};
  const int ys[2] = {(int)ceil(sy), (int)floor(sy)};
  const int zs[2] = {(int)ceil(sz), (int)floor(sz)};
  /* assignment order of gene_obs.jl:44-51 and inversion.jl:53-60: (u,u,u),
   * (u,u,d), (u,d,u), ... (when a coordinate is integral, both assignments
   * to a node carry the same value) */
  for (int a_ = 0; a_ < 2; ++a_)
    for (int b = 0; b < 2; ++b)
      for (int c = 0; c < 2; ++c) {
        const int i = xs[a_], j = ys[b], k = zs[c];
        const int64_t p = ((int64_t)i * n + j) * l + k;
        const double dx = sx - i, dy = sy - j, dz = sz - k;
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        if (mode == ORC_SRC_INVERSION) {
          /* sqrt(...)*h/vel0[node], inversion.jl:53-60 */
          u0[p] = r * h / a[p];
        } else if (mode == ORC_SRC_GENE_OBS) {
          /* slowness_pu = fvel[ixu,iyu,izu] for the izu plane, slowness_pd =
           * fvel[ixu,iyu,izd] for the izd plane; sqrt(...)*slowness*h,
           * gene_obs.jl:42-51 */
          const int64_t q = ((int64_t)xs[0] * n + ys[0]) * l + k;
          u0[p] = r * a[q] * h;
        } else {
          u0[p] = r * a[p] * h;
        }
      }
}

double orc_sample(const double* u, int m, int n, int l, double x, double y,
                  double z, int64_t* idx, double* w) {
  (void)m;
  const int x1 = (int)floor(x), x2 = (int)ceil(x);
  const int y1 = (int)floor(y), y2 = (int)ceil(y);
  const int z1 = (int)floor(z), z2 = (int)ceil(z);
#define U(i, j, k) u[((int64_t)(i) * n + (j)) * l + (k)]
  double t11, t12, t21, t22, wx1, wx2, wy1, wy2, wz1, wz2;
  if (x1 == x2) {
    t11 = U(x1, y1, z1); t12 = U(x1, y1, z2);
    t21 = U(x1, y2, z1); t22 = U(x1, y2, z2);
    wx1 = 1.0; wx2 = 0.0;
  } else {
    wx1 = x2 - x; wx2 = x - x1;
    t11 = wx1 * U(x1, y1, z1) + wx2 * U(x2, y1, z1);
    t12 = wx1 * U(x1, y1, z2) + wx2 * U(x2, y1, z2);
    t21 = wx1 * U(x1, y2, z1) + wx2 * U(x2, y2, z1);
    t22 = wx1 * U(x1, y2, z2) + wx2 * U(x2, y2, z2);
  }
  double t1, t2;
  if (y1 == y2) {
    t1 = t11; t2 = t12;
    wy1 = 1.0; wy2 = 0.0;
  } else {
    wy1 = y2 - y; wy2 = y - y1;
    t1 = wy1 * t11 + wy2 * t21;
    t2 = wy1 * t12 + wy2 * t22;
  }
  double t;
  if (z1 == z2) {
    t = t1;
    wz1 = 1.0; wz2 = 0.0;
  } else {
    wz1 = z2 - z; wz2 = z - z1;
    t = wz1 * t1 + wz2 * t2;
  }
#undef U
  if (idx && w) {
    const int xi[2] = {x1, x2}, yi[2] = {y1, y2}, zi[2] = {z1, z2};
    const double xw[2] = {wx1, wx2}, yw[2] = {wy1, wy2}, zw[2] = {wz1, wz2};
    int q = 0;
    for (int a = 0; a < 2; ++a)
      for (int b = 0; b < 2; ++b)
        for (int c = 0; c < 2; ++c, ++q) {
          idx[q] = ((int64_t)xi[a] * n + yi[b]) * l + zi[c];
          w[q] = xw[a] * yw[b] * zw[c];
        }
  }
  return t;
}

typedef struct {
  int tid, nthreads;
  int n_fields;
  const int32_t* dims;
  const double* h;
  const double* slowness;
  const int32_t* nsta;
  const double* sta_xyz;
  int n_solves;
  const int32_t* solve_field;
  const double* src_xyz;
  const double* t_obs;
  const double* weight;
  double tol;
  int max_iter;
  int src_mode;
  const double* src_model; /* near-source model (NULL: the slowness) */
  const int64_t* field_off; /* cell offset per field */
  const int64_t* sta_off;   /* station offset per field */
  const int64_t* obs_off;   /* pick offset per solve */
  double* solve_misfit;
  double* t_pred;
  double* grad; /* this thread's partial gradient (all fields) */
  int32_t* iters;
  int rc;
} batch_job_t;

static void* batch_worker(void* arg) {
  batch_job_t* J = (batch_job_t*)arg;
  int64_t maxN = 0;
  for (int fi = 0; fi < J->n_fields; ++fi) {
    const int64_t N = (int64_t)J->dims[3 * fi] * J->dims[3 * fi + 1] * J->dims[3 * fi + 2];
    if (N > maxN) maxN = N;
  }
  double* u0 = (double*)malloc((size_t)maxN * sizeof(double));
  double* u = (double*)malloc((size_t)maxN * sizeof(double));
  double* gu = (double*)malloc((size_t)maxN * sizeof(double));
  double* gu0 = (double*)malloc((size_t)maxN * sizeof(double));
  double* gf = (double*)malloc((size_t)maxN * sizeof(double));
  for (int s = J->tid; s < J->n_solves; s += J->nthreads) {
    const int fi = J->solve_field[s];
    const int m = J->dims[3 * fi], n = J->dims[3 * fi + 1], l = J->dims[3 * fi + 2];
    const int64_t N = (int64_t)m * n * l;
    const double hh = J->h[fi];
    const double* f = J->slowness + J->field_off[fi];
    const double* a = J->src_model ? J->src_model + J->field_off[fi] : f;
    orc_src_u0(a, m, n, l, hh, J->src_xyz[3 * s], J->src_xyz[3 * s + 1], J->src_xyz[3 * s + 2],
               J->src_mode, u0);
    double ferr = 0.0;
    J->iters[s] = orc_eik3d_forward(u0, f, hh, m, n, l, J->tol, J->max_iter, u, &ferr);
    memset(gu, 0, (size_t)N * sizeof(double));
    double mis = 0.0;
    const int S = J->nsta[fi];
    const double* st = J->sta_xyz + 3 * J->sta_off[fi];
    for (int q = 0; q < S; ++q) {
      int64_t idx[8];
      double w[8];
      const double tp = orc_sample(u, m, n, l, st[3 * q], st[3 * q + 1], st[3 * q + 2], idx, w);
      const int64_t o = J->obs_off[s] + q;
      J->t_pred[o] = tp;
      const double to = J->t_obs[o];
      if (to == -1.0) continue;
      const double r = to - tp;
      mis += J->weight[o] * r * r;
      const double dt = -2.0 * J->weight[o] * r;
      for (int c = 0; c < 8; ++c) gu[idx[c]] += dt * w[c];
    }
    J->solve_misfit[s] = mis;
    orc_eik3d_backward(gu, u, u0, f, hh, m, n, l, gu0, gf);
    double* G = J->grad + J->field_off[fi];
    for (int64_t p = 0; p < N; ++p) G[p] += gf[p];
  }
  free(u0);
  free(u);
  free(gu);
  free(gu0);
  free(gf);
  J->rc = 0;
  return NULL;
}

int orc_batch_misfit_grad(int n_fields, const int32_t* dims, const double* h,
                          const double* slowness, const int32_t* nsta,
                          const double* sta_xyz, int n_solves,
                          const int32_t* solve_field, const double* src_xyz,
                          const double* t_obs, const double* weight, double tol,
                          int max_iter, int nthreads, int src_mode,
                          const double* src_model, double* misfit,
                          double* t_pred, double* grad, int32_t* iters) {
  if (src_mode == ORC_SRC_INVERSION && !src_model) return -1;
  if (nthreads < 1) nthreads = 1;
  if (nthreads > n_solves && n_solves > 0) nthreads = n_solves;
  int64_t* field_off = (int64_t*)malloc(sizeof(int64_t) * (n_fields + 1));
  int64_t* sta_off = (int64_t*)malloc(sizeof(int64_t) * (n_fields + 1));
  int64_t* obs_off = (int64_t*)malloc(sizeof(int64_t) * (n_solves + 1));
  field_off[0] = 0;
  sta_off[0] = 0;
  for (int fi = 0; fi < n_fields; ++fi) {
    field_off[fi + 1] = field_off[fi] + (int64_t)dims[3 * fi] * dims[3 * fi + 1] * dims[3 * fi + 2];
    sta_off[fi + 1] = sta_off[fi] + nsta[fi];
  }
  obs_off[0] = 0;
  for (int s = 0; s < n_solves; ++s) obs_off[s + 1] = obs_off[s] + nsta[solve_field[s]];
  const int64_t NT = field_off[n_fields];
  double* solve_misfit = (double*)calloc((size_t)(n_solves > 0 ? n_solves : 1), sizeof(double));
  batch_job_t* jobs = (batch_job_t*)calloc((size_t)nthreads, sizeof(batch_job_t));
  pthread_t* th = (pthread_t*)calloc((size_t)nthreads, sizeof(pthread_t));
  for (int t = 0; t < nthreads; ++t) {
    batch_job_t* J = &jobs[t];
    J->tid = t;
    J->nthreads = nthreads;
    J->n_fields = n_fields;
    J->dims = dims;
    J->h = h;
    J->slowness = slowness;
    J->nsta = nsta;
    J->sta_xyz = sta_xyz;
    J->n_solves = n_solves;
    J->solve_field = solve_field;
    J->src_xyz = src_xyz;
    J->t_obs = t_obs;
    J->weight = weight;
    J->tol = tol;
    J->max_iter = max_iter;
    J->src_mode = src_mode;
    J->src_model = src_model;
    J->field_off = field_off;
    J->sta_off = sta_off;
    J->obs_off = obs_off;
    J->solve_misfit = solve_misfit;
    J->t_pred = t_pred;
    J->grad = (double*)calloc((size_t)NT, sizeof(double));
    J->iters = iters;
    if (nthreads == 1)
      batch_worker(J);
    else
      pthread_create(&th[t], NULL, batch_worker, J);
  }
  if (nthreads > 1)
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  memset(grad, 0, (size_t)NT * sizeof(double));
  for (int t = 0; t < nthreads; ++t) {
    for (int64_t p = 0; p < NT; ++p) grad[p] += jobs[t].grad[p];
    free(jobs[t].grad);
  }
  double tot = 0.0;
  for (int s = 0; s < n_solves; ++s) tot += solve_misfit[s];
  *misfit = tot;
  free(solve_misfit);
  free(jobs);
  free(th);
  free(field_off);
  free(sta_off);
  free(obs_off);
  return 0;
}
