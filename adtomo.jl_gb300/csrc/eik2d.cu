// eik2d.cu -- 2D fast sweeping (FP64, reference arithmetic) and its adjoint.
//
// Grid (n+1) x (m+1), index j*(m+1)+i (Eikonal.h:30-48).  One CTA per solve.
// Each of the 4 orderings (I,J), (iI,J), (iI,iJ), (I,iJ) (Eikonal.h:74-77) is
// run as a wavefront over the anti-diagonals i' + j' = s of that ordering:
// every cell on a diagonal depends only on the previous diagonal, which is
// the Gauss-Seidel data flow of the reference's i-outer / j-inner loop, so
// travel times are bit-identical.  The source cell is skipped and pinned to 0.
// Stop when ||u - u_old|| / ||u_old|| < 1e-8, at most 100 iterations
// (Eikonal.h:71-86).
//
// Adjoint (Eikonal.h:95-200): lambda_c = (g_c + sum_users 2 (u_r - u_c)
// lambda_r) / d_c with the source row the identity, solved by the same
// diagonal sweeps until a full iteration changes nothing.  A non-source cell
// without an active axis makes the reference's matrix singular; it is
// reported as ADT_ESINGULAR.
#include <cstring>

#include "eik2d.h"
#include "eik3d_common_host.h"
#include "causal_sync.cuh"
#include "eik_local.cuh"

namespace adt {

namespace {

__device__ __forceinline__ double block_sum(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double t = 0.0;
  if (threadIdx.x == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  if (threadIdx.x == 0) red[32] = t;
  __syncthreads();
  return red[32];
}

__device__ __forceinline__ void ord2(int o, int& si, int& sj) {
  si = (o == 1 || o == 2) ? -1 : 1;
  sj = (o >= 2) ? -1 : 1;
}

}  // namespace

__global__ void k_eik2d_forward(const double* __restrict__ f, int m, int n, double h,
                                const int* __restrict__ srcx, const int* __restrict__ srcy,
                                double* __restrict__ u_all, double* __restrict__ prev_all,
                                int* __restrict__ iters, int* __restrict__ conv,
                                double* __restrict__ errs) {
  __shared__ double red[33];
  const int w = m + 1;
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  const int sol = blockIdx.x;
  double* u = u_all + sol * N;
  double* prev = prev_all + sol * N;
  const int ix = srcx[sol], jx = srcy[sol];
  for (int64_t p = threadIdx.x; p < N; p += blockDim.x) {
    const int i = (int)(p % w), j = (int)(p / w);
    const double v = (i == ix && j == jx) ? 0.0 : 100000.0;
    u[p] = v;
    prev[p] = v;
  }
  __syncthreads();
  int it, done = 0;
  double err = 0.0;
  for (it = 0; it < 100; ++it) {
    for (int o = 0; o < 4; ++o) {
      int si, sj;
      ord2(o, si, sj);
      for (int s = 0; s <= m + n; ++s) {
        const int a0 = max(0, s - n), a1 = min(m, s);
        for (int a = a0 + (int)threadIdx.x; a <= a1; a += blockDim.x) {
          const int b = s - a;
          const int i = si > 0 ? a : m - a;
          const int j = sj > 0 ? b : n - b;
          if (i == ix && j == jx) continue;
          double ax, by;
          if (i == 0) ax = u[j * w + 1];
          else if (i == m) ax = u[j * w + m - 1];
          else ax = rmin(u[j * w + i + 1], u[j * w + i - 1]);
          if (j == 0) by = u[w + i];
          else if (j == n) by = u[(n - 1) * w + i];
          else by = rmin(u[(j - 1) * w + i], u[(j + 1) * w + i]);
          const double un = upd2_exact(ax, by, f[j * w + i], h);
          u[j * w + i] = rmin(u[j * w + i], un);
        }
        __syncthreads();
      }
    }
    double dd = 0.0, pp = 0.0;
    for (int64_t p = threadIdx.x; p < N; p += blockDim.x) {
      const double d = __dsub_rn(u[p], prev[p]);
      dd = __dadd_rn(dd, __dmul_rn(d, d));
      pp = __dadd_rn(pp, __dmul_rn(prev[p], prev[p]));
    }
    dd = block_sum(dd, red);
    pp = block_sum(pp, red);
    err = __ddiv_rn(__dsqrt_rn(dd), __dsqrt_rn(pp));
    if (err < 1e-8) {
      done = 1;
      break;
    }
    for (int64_t p = threadIdx.x; p < N; p += blockDim.x) prev[p] = u[p];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    iters[sol] = done ? it + 1 : it;
    conv[sol] = done;
    errs[sol] = err;
  }
}

// Upwind neighbour index along one axis (edge rule, ties to the +1 side).
__device__ __forceinline__ int64_t upw2(const double* u, int64_t p, int pos, int last, int64_t st) {
  if (pos == 0) return p + st;
  if (pos == last) return p - st;
  return (u[p + st] > u[p - st]) ? p - st : p + st;
}

__global__ void k_eik2d_adjoint(const double* __restrict__ gu, const double* __restrict__ u,
                                const double* __restrict__ f, int m, int n, double h, int ix,
                                int jx, double* __restrict__ lam, double* __restrict__ grad_f,
                                int* __restrict__ status) {
  __shared__ int s_changed, s_singular;
  const int w = m + 1;
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  const int64_t src = (int64_t)jx * w + ix;
  for (int64_t p = threadIdx.x; p < N; p += blockDim.x) lam[p] = 0.0;
  if (threadIdx.x == 0) s_singular = 0;
  __syncthreads();
  int it, done = 0;
  for (it = 0; it < 10000; ++it) {
    if (threadIdx.x == 0) s_changed = 0;
    __syncthreads();
    for (int o = 0; o < 4; ++o) {
      int si, sj;
      ord2(o, si, sj);
      for (int s = 0; s <= m + n; ++s) {
        const int a0 = max(0, s - n), a1 = min(m, s);
        for (int a = a0 + (int)threadIdx.x; a <= a1; a += blockDim.x) {
          const int b = s - a;
          const int i = si > 0 ? a : m - a;
          const int j = sj > 0 ? b : n - b;
          const int64_t c = (int64_t)j * w + i;
          double acc = gu[c];
#pragma unroll
          for (int q = 0; q < 4; ++q) {
            const int ri = i + (q == 0 ? -1 : q == 1 ? 1 : 0);
            const int rj = j + (q == 2 ? -1 : q == 3 ? 1 : 0);
            if (ri < 0 || ri > m || rj < 0 || rj > n) continue;
            const int64_t r = (int64_t)rj * w + ri;
            if (r == src) continue;
            const int64_t nb = (q < 2) ? upw2(u, r, ri, m, 1) : upw2(u, r, rj, n, w);
            if (nb != c || !(u[r] > u[c])) continue;
            acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(2.0, __dsub_rn(u[r], u[c])), lam[r]));
          }
          double d;
          if (c == src) {
            d = 1.0;
          } else {
            d = 0.0;
            const int64_t nx = upw2(u, c, i, m, 1), ny = upw2(u, c, j, n, w);
            if (u[c] > u[nx]) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(u[c], u[nx])));
            if (u[c] > u[ny]) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(u[c], u[ny])));
          }
          if (d == 0.0) {
            s_singular = 1;
            continue;
          }
          const double l = __ddiv_rn(acc, d);
          if (!(l == lam[c])) {
            lam[c] = l;
            s_changed = 1;
          }
        }
        __syncthreads();
      }
    }
    __syncthreads();
    if (s_singular) break;
    if (!s_changed) {
      done = 1;
      break;
    }
    __syncthreads();
  }
  for (int64_t p = threadIdx.x; p < N; p += blockDim.x) {
    // dFdf = -2 f h h, 0 at the source; grad_f = -lambda * dFdf (Eikonal.h:100-104,196-198)
    const double dfdf = (p == src) ? 0.0 : __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f[p]), h), h);
    grad_f[p] = __dmul_rn(-lam[p], dfdf);
  }
  if (threadIdx.x == 0) status[0] = s_singular ? -1 : (done ? it + 1 : 0);
}

// The 2D adjoint in causal order, one CTA: the rows of k_eik2d_adjoint
// (Eikonal.h:95-200) solved once, every cell after its users (Kahn's
// algorithm on the users graph, acyclic since a user's travel time is
// strictly larger).  A cell's users are the non-source neighbours whose
// upwind neighbour along the axis is the cell; per cell a word holds their
// bits (0-3: x-, x+, y-, y+) and, in bits 8-11, those not yet evaluated.
// Each evaluated non-source cell clears its bit in its upwind neighbours'
// words (acq_rel atomics at CTA scope); the thread that empties a word queues
// that cell (release store; slots are read with acquire loads).  The
// per-cell formula and summation order are k_eik2d_adjoint's, so lambda is
// the same, bit for bit.  status: 1 done, -1 a non-source cell has no upwind
// direction, 0 a wait on the queue ran out (bounded by CAUSAL_WAIT_CYCLES).
__global__ void __launch_bounds__(512)
    k_eik2d_adjoint_causal(const double* __restrict__ gu, const double* __restrict__ u,
                           const double* __restrict__ f, int m, int n, double h, int ix, int jx,
                           double* lam, double* __restrict__ grad_f, uint32_t* word, int* queue,
                           int* __restrict__ status) {
  __shared__ int s_head, s_tail, s_err, s_singular;
  const int w = m + 1;
  const int N = (m + 1) * (n + 1);
  const int src = jx * w + ix;
  const int tid = threadIdx.x, nth = blockDim.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    s_head = s_tail = 0;
    s_err = s_singular = 0;
  }
  for (int p = tid; p < N; p += nth) queue[p] = -1;
  __syncthreads();
  // users of each cell, cells without users queued, singular rows found
  for (int c0 = warp * 32; c0 < N; c0 += nth) {
    const int c = c0 + lane;
    uint32_t us = 0;
    if (c < N) {
      const int i = c % w, j = c / w;
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const int ri = i + (q == 0 ? -1 : q == 1 ? 1 : 0);
        const int rj = j + (q == 2 ? -1 : q == 3 ? 1 : 0);
        if (ri < 0 || ri > m || rj < 0 || rj > n) continue;
        const int r = rj * w + ri;
        if (r == src) continue;
        const int64_t nb = (q < 2) ? upw2(u, r, ri, m, 1) : upw2(u, r, rj, n, w);
        if (nb == c && u[r] > u[c]) us |= 1u << q;
      }
      word[c] = us | (us << 8);
      if (c != src && !(u[c] > u[upw2(u, c, i, m, 1)]) && !(u[c] > u[upw2(u, c, j, n, w)]))
        s_singular = 1;
    }
    const int pos = warp_append((c < N && us == 0) ? 1 : 0, &s_tail, lane);
    if (c < N && us == 0) queue[pos] = c;
  }
  __syncthreads();
  if (!s_singular) {
    for (;;) {
      const int slot = take_slots(1, &s_head);
      if (slot >= N) break;
      int x = ld_acquire_cta(queue + slot);
      if (x < 0) {
        const long long t0 = clock64();
        do {
          __nanosleep(64);
          x = ld_acquire_cta(queue + slot);
        } while (x < 0 && clock64() - t0 < CAUSAL_WAIT_CYCLES &&
                 !*reinterpret_cast<volatile int*>(&s_err));
        if (x < 0) {  // out of budget, or another thread's was
          atomicOr(&s_err, 1);
          break;
        }
      }
      const int i = x % w, j = x / w;
      const uint32_t us = word[x] & 15u;
      double acc = gu[x];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        if ((us >> q) & 1u) {
          const int r = x + (q == 0 ? -1 : q == 1 ? 1 : q == 2 ? -w : w);
          acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(2.0, __dsub_rn(u[r], u[x])), lam[r]));
        }
      double d;
      const int nx = (int)upw2(u, x, i, m, 1), ny = (int)upw2(u, x, j, n, w);
      if (x == src) {
        d = 1.0;
      } else {
        d = 0.0;
        if (u[x] > u[nx]) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(u[x], u[nx])));
        if (u[x] > u[ny]) d = __dadd_rn(d, __dmul_rn(2.0, __dsub_rn(u[x], u[ny])));
      }
      lam[x] = __ddiv_rn(acc, d);
      // release the upwind neighbours this cell is a user of
      int rel[2] = {-1, -1}, np = 0;
      if (x != src) {
        const int nbs[2] = {nx, ny};
#pragma unroll
        for (int a = 0; a < 2; ++a) {
          const int nb = nbs[a];
          if (!(u[x] > u[nb])) continue;
          // this cell seen from nb: x+ (1) or x- (0), y+ (3) or y- (2)
          const int q = a == 0 ? (nb < x ? 1 : 0) : (nb < x ? 3 : 2);
          const uint32_t bit = (1u << q) << 8;
          const uint32_t old = atom_and_acq_rel_cta(word + nb, ~bit);
          if ((old & bit) && !(old & ~bit & 0xf00u)) {
            rel[a] = nb;
            ++np;
          }
        }
      }
      int pos = take_slots(np, &s_tail);
      for (int a = 0; a < 2; ++a)
        if (rel[a] >= 0) st_release_cta(queue + pos++, rel[a]);
    }
  }
  __syncthreads();
  const bool done = !s_singular && !s_err && s_tail == N;
  for (int p = tid; p < N; p += nth) {
    // dFdf = -2 f h h, 0 at the source; grad_f = -lambda * dFdf (Eikonal.h:100-104,196-198)
    const double dfdf = (p == src) ? 0.0 : __dmul_rn(__dmul_rn(__dmul_rn(-2.0, f[p]), h), h);
    grad_f[p] = done ? __dmul_rn(-lam[p], dfdf) : 0.0;
  }
  if (tid == 0) status[0] = s_singular ? -1 : (done ? 1 : 0);
}

int eik2d_forward_batch(const double* d_f, int m, int n, double h, int count, const int* d_srcx,
                        const int* d_srcy, double* d_u, adt_solve_status* st, cudaStream_t stream) {
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  DevBuf prev, b_it, b_cv, b_err;
  ADT_CUDA(prev.reserve((size_t)count * N * sizeof(double)));
  ADT_CUDA(b_it.reserve((size_t)count * sizeof(int)));
  ADT_CUDA(b_cv.reserve((size_t)count * sizeof(int)));
  ADT_CUDA(b_err.reserve((size_t)count * sizeof(double)));
  int* d_iters = b_it.as<int>();
  int* d_conv = b_cv.as<int>();
  double* d_err = b_err.as<double>();
  k_eik2d_forward<<<count, 256, 0, stream>>>(d_f, m, n, h, d_srcx, d_srcy, d_u, prev.as<double>(),
                                             d_iters, d_conv, d_err);
  ADT_CUDA(cudaGetLastError());
  std::vector<int> it(count), cv(count);
  std::vector<double> er(count);
  ADT_CUDA(cudaMemcpyAsync(it.data(), d_iters, count * sizeof(int), cudaMemcpyDeviceToHost, stream));
  ADT_CUDA(cudaMemcpyAsync(cv.data(), d_conv, count * sizeof(int), cudaMemcpyDeviceToHost, stream));
  ADT_CUDA(cudaMemcpyAsync(er.data(), d_err, count * sizeof(double), cudaMemcpyDeviceToHost, stream));
  ADT_CUDA(cudaStreamSynchronize(stream));
  if (st)
    for (int k = 0; k < count; ++k) {
      st[k].iters = it[k];
      st[k].converged = cv[k];
      st[k].final_err = er[k];
      st[k].adj_iters = 0;
      st[k].adj_converged = 0;
    }
  return ADT_OK;
}

int eik2d_adjoint(const double* d_gu, const double* d_u, const double* d_f, int m, int n, double h,
                  int ix, int jx, double* d_gf, cudaStream_t stream) {
  const int64_t N = (int64_t)(m + 1) * (n + 1);
  DevBuf lam, stat;
  ADT_CUDA(lam.reserve((size_t)N * sizeof(double)));
  ADT_CUDA(stat.reserve(sizeof(int)));
  if (N < (1 << 30)) {  // causal order: every cell once
    DevBuf word, queue;
    ADT_CUDA(word.reserve((size_t)N * sizeof(uint32_t)));
    ADT_CUDA(queue.reserve((size_t)N * sizeof(int)));
    k_eik2d_adjoint_causal<<<1, 512, 0, stream>>>(d_gu, d_u, d_f, m, n, h, ix, jx, lam.as<double>(),
                                                  d_gf, word.as<uint32_t>(), queue.as<int>(),
                                                  stat.as<int>());
  } else {
    k_eik2d_adjoint<<<1, 256, 0, stream>>>(d_gu, d_u, d_f, m, n, h, ix, jx, lam.as<double>(), d_gf,
                                           stat.as<int>());
  }
  ADT_CUDA(cudaGetLastError());
  int s = 0;
  ADT_CUDA(cudaMemcpyAsync(&s, stat.p, sizeof(int), cudaMemcpyDeviceToHost, stream));
  ADT_CUDA(cudaStreamSynchronize(stream));
  if (s < 0) return set_error(ADT_ESINGULAR, "2D adjoint: a non-source cell has no upwind direction");
  if (s == 0) return set_error(ADT_ENOCONV, "2D adjoint did not complete");
  return ADT_OK;
}

}  // namespace adt
