// locate.cu -- loss and gradient of the 2D-table event location, all events at once.
//
// tests/Eikonal/eikoloc.py locates each event (origin time t0, position
// x, y, z) by minimising, over its picks,
//   loss = mean_P(w huber(t_obs - (t0 + T_P(r, z')))) + mean_S(...)
//        (+ gamma mean over pick pairs of w_i w_j huber(dT_ij - dt_obs_ij), per phase)
// where r is the horizontal event-station distance, z' = |z| - z_station,
// and T_P, T_S are (r, z) travel-time tables read by bilinear interpolation
// whose cell index is clamped to the table (eikoloc.py:119-145, 148-156,
// 157-206).  The position is clamped to the search bounds before use
// (eikoloc.py:174), so a clamped coordinate gets no gradient.
//
// Here one warp evaluates one event: lanes take its picks, the sums are
// reduced in FP64 in a fixed order, and the gradient with respect to
// (t0, x, y, z) is formed analytically (the derivative of the bilinear form
// inside the clamped cell, of r, of |z|, and of the Huber loss with delta 1).
#include <cmath>
#include <cstdio>

#include "adt_common.cuh"
#include "eik3d_common_host.h"

namespace adt {
namespace {

struct LocTable {
  const double* T;  // m x n, index ir * n + iz
  int m, n;
  double r0, z0, h;
};

// Bilinear value and derivatives at (r, z) with the clamped cell of eikoloc.py:_interp.
__device__ __forceinline__ double interp(const LocTable& t, double r, double z, double& dr,
                                         double& dz) {
  int ir0 = (int)floor((r - t.r0) / t.h);
  int iz0 = (int)floor((z - t.z0) / t.h);
  ir0 = ir0 < 0 ? 0 : (ir0 > t.m - 2 ? t.m - 2 : ir0);
  iz0 = iz0 < 0 ? 0 : (iz0 > t.n - 2 ? t.n - 2 : iz0);
  const double x1 = ir0 * t.h + t.r0, x2 = (ir0 + 1) * t.h + t.r0;
  const double y1 = iz0 * t.h + t.z0, y2 = (iz0 + 1) * t.h + t.z0;
  const double q11 = t.T[(int64_t)ir0 * t.n + iz0], q12 = t.T[(int64_t)ir0 * t.n + iz0 + 1];
  const double q21 = t.T[(int64_t)(ir0 + 1) * t.n + iz0];
  const double q22 = t.T[(int64_t)(ir0 + 1) * t.n + iz0 + 1];
  const double s = 1.0 / ((x2 - x1) * (y2 - y1));
  dr = s * ((q21 - q11) * (y2 - z) + (q22 - q12) * (z - y1));
  dz = s * ((q12 - q11) * (x2 - r) + (q22 - q21) * (r - x1));
  return s * (q11 * (x2 - r) * (y2 - z) + q21 * (r - x1) * (y2 - z) + q12 * (x2 - r) * (z - y1) +
              q22 * (r - x1) * (z - y1));
}

// torch.nn.functional.huber_loss with delta 1: value and derivative in d.
__device__ __forceinline__ double huber(double d, double& g) {
  if (fabs(d) < 1.0) {
    g = d;
    return 0.5 * d * d;
  }
  g = d > 0 ? 1.0 : -1.0;
  return fabs(d) - 0.5;
}

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

constexpr int LOC_MAX_PICKS = 256;  // per event and phase, for the pair term's buffer

__global__ void k_locate(int n_events, const double* __restrict__ params,
                         const int64_t* __restrict__ offs, const double* __restrict__ sta,
                         const double* __restrict__ t_obs, const int32_t* __restrict__ phase,
                         const double* __restrict__ weight, LocTable tp, LocTable ts,
                         const double* __restrict__ bounds, double gamma, double* __restrict__ loss,
                         double* __restrict__ grad) {
  __shared__ double s_tt[4][LOC_MAX_PICKS];
  __shared__ double s_dr[4][3][LOC_MAX_PICKS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * (blockDim.x >> 5) + warp;
  if (e >= n_events) return;
  const double t0 = params[4 * e];
  double p[3], dclamp[3];
  for (int a = 0; a < 3; ++a) {
    const double v = params[4 * e + 1 + a];
    const double lo = bounds[2 * a], hi = bounds[2 * a + 1];
    p[a] = v < lo ? lo : (v > hi ? hi : v);
    dclamp[a] = (v < lo || v > hi) ? 0.0 : 1.0;  // d clamp / d v
    if (p[a] != p[a]) p[a] = 0.0;                  // nan_to_num
  }
  const int64_t b = offs[e], c = offs[e + 1];
  double L = 0.0, G[4] = {0.0, 0.0, 0.0, 0.0};
  for (int ph = 0; ph < 2; ++ph) {
    const LocTable& T = ph == 0 ? tp : ts;
    // count of this phase's picks (mean divisor)
    double cnt = 0.0;
    for (int64_t q = b + lane; q < c; q += 32) cnt += phase[q] == ph ? 1.0 : 0.0;
    cnt = warp_sum(cnt);
    if (cnt == 0.0) continue;
    double l = 0.0, g0 = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
    int np = 0;  // picks of this phase seen so far (for the pair buffer), same on all lanes
    for (int64_t q0 = b; q0 < c; q0 += 32) {
      const int64_t q = q0 + lane;
      const bool mine = q < c && phase[q] == ph;
      double tt = 0.0, dtr = 0.0, dtz = 0.0, ex = 0.0, ey = 0.0, ez = 0.0;
      if (mine) {
        const double dx = p[0] - sta[3 * q], dy = p[1] - sta[3 * q + 1];
        const double r = sqrt(dx * dx + dy * dy);
        const double z = fabs(p[2]) - sta[3 * q + 2];
        tt = interp(T, r, z, dtr, dtz);
        ex = r > 0.0 ? dtr * dx / r : 0.0;  // d tt / d x
        ey = r > 0.0 ? dtr * dy / r : 0.0;
        ez = dtz * (p[2] > 0.0 ? 1.0 : (p[2] < 0.0 ? -1.0 : 0.0));
        double hg;
        const double w = weight[q];
        l += w * huber(t_obs[q] - (t0 + tt), hg);
        // d/d pred of huber(obs - pred) = -hg
        g0 -= w * hg;
        gx -= w * hg * ex;
        gy -= w * hg * ey;
        gz -= w * hg * ez;
      }
      if (gamma != 0.0) {  // keep tt and its gradient for the pair term
        const unsigned m = __ballot_sync(0xffffffffu, mine);
        const int slot = np + __popc(m & ((1u << lane) - 1u));
        if (mine && slot < LOC_MAX_PICKS) {
          s_tt[warp][slot] = tt;
          s_dr[warp][0][slot] = ex;
          s_dr[warp][1][slot] = ey;
          s_dr[warp][2][slot] = ez;
        }
        np += __popc(m);
      }
    }
    l = warp_sum(l);
    L += l / cnt;
    G[0] += warp_sum(g0) / cnt;
    G[1] += warp_sum(gx) / cnt;
    G[2] += warp_sum(gy) / cnt;
    G[3] += warp_sum(gz) / cnt;
    if (gamma != 0.0 && np <= LOC_MAX_PICKS) {
      __syncwarp();
      // the picks of this phase in order, to pair them: gather obs and weights
      double pl = 0.0, pg[3] = {0.0, 0.0, 0.0};
      // index -> pick: walk the event's picks again (same order as the slots)
      for (int i = lane; i < np; i += 32) {
        int64_t qi = -1;
        int k = -1;
        for (int64_t q = b; q < c; ++q)
          if (phase[q] == ph && ++k == i) {
            qi = q;
            break;
          }
        int kj = -1;
        for (int64_t qj = b; qj < c; ++qj) {
          if (phase[qj] != ph) continue;
          const int j = ++kj;
          double hg;
          const double d = (s_tt[warp][i] - s_tt[warp][j]) - (t_obs[qi] - t_obs[qj]);
          const double ww = weight[qi] * weight[qj];
          pl += ww * huber(d, hg);
          for (int a = 0; a < 3; ++a) pg[a] += ww * hg * (s_dr[warp][a][i] - s_dr[warp][a][j]);
        }
      }
      const double npairs = (double)np * (double)np;
      L += gamma * warp_sum(pl) / npairs;
      for (int a = 0; a < 3; ++a) G[1 + a] += gamma * warp_sum(pg[a]) / npairs;
      __syncwarp();
    }
  }
  if (lane == 0) {
    loss[e] = L;
    grad[4 * e] = G[0];
    for (int a = 0; a < 3; ++a) grad[4 * e + 1 + a] = G[1 + a] * dclamp[a];
  }
}

}  // namespace
}  // namespace adt

using namespace adt;

extern "C" int adt_locate_loss_grad(int32_t n_events, const double* params, const int64_t* offs,
                                    const double* sta_xyz, const double* t_obs,
                                    const int32_t* phase, const double* weight,
                                    const double* table_p, const double* table_s, int32_t m,
                                    int32_t n, double r0, double z0, double h,
                                    const double* bounds, double gamma, double* loss,
                                    double* grad) {
  if (n_events < 1 || !params || !offs || !loss || !grad || !table_p || !table_s || !bounds)
    return set_error(ADT_EINVAL, "locate: bad arguments");
  if (m < 2 || n < 2 || !(h > 0.0))
    return set_error(ADT_EINVAL, "locate: tables need m, n >= 2 and h > 0");
  const int64_t P = offs[n_events];
  if (offs[0] != 0 || P < 0) return set_error(ADT_EINVAL, "locate: bad pick offsets");
  for (int e = 0; e < n_events; ++e) {
    if (offs[e + 1] < offs[e]) return set_error(ADT_EINVAL, "locate: pick offsets decrease");
    if (gamma != 0.0 && offs[e + 1] - offs[e] > LOC_MAX_PICKS)
      return set_error(ADT_EINVAL, "locate: the pair term takes at most %d picks per event",
                       LOC_MAX_PICKS);
    if (!sta_xyz || !t_obs || !phase || !weight)
      if (offs[e + 1] > offs[e]) return set_error(ADT_EINVAL, "locate: null pick arrays");
  }
  for (int64_t q = 0; q < P; ++q)
    if (phase[q] != 0 && phase[q] != 1) return set_error(ADT_EINVAL, "locate: phase must be 0 or 1");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(ADT_ENODEV, "no CUDA device available");
  }
  const size_t T = (size_t)m * n;
  DevBuf dpar, doff, dsta, dobs, dph, dw, dtp, dts, db, dl, dg;
  ADT_CUDA(dpar.reserve(4 * n_events * sizeof(double)));
  ADT_CUDA(doff.reserve((n_events + 1) * sizeof(int64_t)));
  ADT_CUDA(dsta.reserve(std::max<int64_t>(1, 3 * P) * sizeof(double)));
  ADT_CUDA(dobs.reserve(std::max<int64_t>(1, P) * sizeof(double)));
  ADT_CUDA(dph.reserve(std::max<int64_t>(1, P) * sizeof(int32_t)));
  ADT_CUDA(dw.reserve(std::max<int64_t>(1, P) * sizeof(double)));
  ADT_CUDA(dtp.reserve(T * sizeof(double)));
  ADT_CUDA(dts.reserve(T * sizeof(double)));
  ADT_CUDA(db.reserve(6 * sizeof(double)));
  ADT_CUDA(dl.reserve(n_events * sizeof(double)));
  ADT_CUDA(dg.reserve(4 * n_events * sizeof(double)));
  ADT_CUDA(cudaMemcpy(dpar.p, params, 4 * n_events * sizeof(double), cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(doff.p, offs, (n_events + 1) * sizeof(int64_t), cudaMemcpyHostToDevice));
  if (P > 0) {
    ADT_CUDA(cudaMemcpy(dsta.p, sta_xyz, 3 * P * sizeof(double), cudaMemcpyHostToDevice));
    ADT_CUDA(cudaMemcpy(dobs.p, t_obs, P * sizeof(double), cudaMemcpyHostToDevice));
    ADT_CUDA(cudaMemcpy(dph.p, phase, P * sizeof(int32_t), cudaMemcpyHostToDevice));
    ADT_CUDA(cudaMemcpy(dw.p, weight, P * sizeof(double), cudaMemcpyHostToDevice));
  }
  ADT_CUDA(cudaMemcpy(dtp.p, table_p, T * sizeof(double), cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(dts.p, table_s, T * sizeof(double), cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(db.p, bounds, 6 * sizeof(double), cudaMemcpyHostToDevice));
  const LocTable tp{dtp.as<double>(), m, n, r0, z0, h}, ts{dts.as<double>(), m, n, r0, z0, h};
  const int wpb = 4;
  k_locate<<<(n_events + wpb - 1) / wpb, 32 * wpb>>>(
      n_events, dpar.as<double>(), doff.as<int64_t>(), dsta.as<double>(), dobs.as<double>(),
      dph.as<int32_t>(), dw.as<double>(), tp, ts, db.as<double>(), gamma, dl.as<double>(),
      dg.as<double>());
  ADT_CUDA(cudaGetLastError());
  ADT_CUDA(cudaMemcpy(loss, dl.p, n_events * sizeof(double), cudaMemcpyDeviceToHost));
  ADT_CUDA(cudaMemcpy(grad, dg.p, 4 * n_events * sizeof(double), cudaMemcpyDeviceToHost));
  return ADT_OK;
}
