// smooth.cu -- the smoothness penalty of the tomographic inversion.
//
// scripts/inversion.jl:107-121 adds lambda * sum |v - S v| to the misfit,
// where v is the velocity model (m x n x l) and S the mean over an
// sh x sh x sv box centred on each cell, with circular padding (the model is
// wrapped by the tf.concat lines before a VALID conv3d with weights
// 1/(sh sh sv)).  Its gradient is (I - S)^T sign(v - S v) = s - S s with
// s = sign(v - S v), because a centred box with wrap-around is symmetric.
//
// The box mean is separable: three passes of a 1D circular sum (k, then j,
// then i), each a coalesced FP64 stencil, then one division by sh sh sv.
// The L1 sum is a deterministic two-stage reduction (fixed grid, fixed
// order), so repeated calls give identical results.
#include <cmath>
#include <cstdio>
#include <vector>

#include "adt_common.cuh"
#include "eik3d_common_host.h"

namespace adt {
namespace {

constexpr int SM_THREADS = 256;
constexpr int SM_MAX_BLOCKS = 1024;

// out[c] = sum_{d=-r..r} in[c with its coordinate along the axis shifted by d, wrapped]
__global__ void k_box_pass(const double* __restrict__ in, double* __restrict__ out, int64_t ncell,
                           int64_t stride, int64_t ext, int r) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int64_t pos = (c / stride) % ext;
    const int64_t base = c - pos * stride;
    double acc = 0.0;
    for (int d = -r; d <= r; ++d) {
      int64_t q = pos + d;
      q = q < 0 ? q + ext : (q >= ext ? q - ext : q);
      acc = __dadd_rn(acc, in[base + q * stride]);
    }
    out[c] = acc;
  }
}

__device__ __forceinline__ double block_sum(double v, double* sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) sh[threadIdx.x] = __dadd_rn(sh[threadIdx.x], sh[threadIdx.x + o]);
    __syncthreads();
  }
  return sh[0];
}

// s = sign(v - box/N); partial[b] = sum over this block's cells of |v - box/N|
__global__ void k_resid_sign(const double* __restrict__ v, const double* __restrict__ box,
                             double inv_n, int64_t ncell, double* __restrict__ s,
                             double* __restrict__ partial) {
  __shared__ double sh[SM_THREADS];
  double acc = 0.0;
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
       c += (int64_t)gridDim.x * blockDim.x) {
    const double r = __dsub_rn(v[c], __dmul_rn(box[c], inv_n));
    s[c] = r > 0.0 ? 1.0 : (r < 0.0 ? -1.0 : 0.0);
    acc = __dadd_rn(acc, fabs(r));
  }
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

__global__ void k_sum_partials(const double* __restrict__ partial, int n, double scale,
                               double* __restrict__ out) {
  __shared__ double sh[SM_THREADS];
  double acc = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) acc = __dadd_rn(acc, partial[i]);
  const double t = block_sum(acc, sh);
  if (threadIdx.x == 0) *out = __dmul_rn(t, scale);
}

// grad = scale * (s - box/N)
__global__ void k_grad(const double* __restrict__ s, const double* __restrict__ box, double inv_n,
                       double scale, int64_t ncell, double* __restrict__ grad) {
  for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < ncell;
       c += (int64_t)gridDim.x * blockDim.x)
    grad[c] = __dmul_rn(scale, __dsub_rn(s[c], __dmul_rn(box[c], inv_n)));
}

int check_smooth(int64_t m, int64_t n, int64_t l, int sh, int sv, const void* v, const void* pen) {
  if (m < 1 || n < 1 || l < 1)
    return set_error(ADT_EINVAL, "smooth_l1: need m, n, l >= 1 (got %lld x %lld x %lld)",
                     (long long)m, (long long)n, (long long)l);
  if (sh < 1 || sv < 1 || sh % 2 == 0 || sv % 2 == 0)
    return set_error(ADT_EINVAL, "smooth_l1: box sizes must be odd and >= 1 (got %d, %d)", sh, sv);
  if ((sh - 1) / 2 > m || (sh - 1) / 2 > n || (sv - 1) / 2 > l)
    return set_error(ADT_EINVAL, "smooth_l1: box half-width exceeds the grid");
  if (!v || !pen) return set_error(ADT_EINVAL, "smooth_l1: null array");
  return ADT_OK;
}

// Enqueue the whole penalty on `st`; scratch: 2 * ncell + SM_MAX_BLOCKS doubles.
int enqueue_smooth(const double* v, int64_t m, int64_t n, int64_t l, int sh, int sv,
                   double lambda, double* pen, double* grad, double* scratch, cudaStream_t st) {
  const int64_t nc = m * n * l;
  double* A = scratch;
  double* B = scratch + nc;
  double* part = scratch + 2 * nc;
  const int blocks = (int)std::min<int64_t>((nc + SM_THREADS - 1) / SM_THREADS, SM_MAX_BLOCKS);
  const double inv_n = 1.0 / ((double)sh * sh * sv);
  const int rh = (sh - 1) / 2, rv = (sv - 1) / 2;
  // S v: k, j, i passes
  k_box_pass<<<blocks, SM_THREADS, 0, st>>>(v, A, nc, 1, l, rv);
  k_box_pass<<<blocks, SM_THREADS, 0, st>>>(A, B, nc, l, n, rh);
  k_box_pass<<<blocks, SM_THREADS, 0, st>>>(B, A, nc, n * l, m, rh);
  k_resid_sign<<<blocks, SM_THREADS, 0, st>>>(v, A, inv_n, nc, B, part);
  k_sum_partials<<<1, SM_THREADS, 0, st>>>(part, blocks, lambda, pen);
  if (grad) {
    // S s, into A, through `grad` as the middle buffer
    k_box_pass<<<blocks, SM_THREADS, 0, st>>>(B, A, nc, 1, l, rv);
    k_box_pass<<<blocks, SM_THREADS, 0, st>>>(A, grad, nc, l, n, rh);
    k_box_pass<<<blocks, SM_THREADS, 0, st>>>(grad, A, nc, n * l, m, rh);
    k_grad<<<blocks, SM_THREADS, 0, st>>>(B, A, inv_n, lambda, nc, grad);
  }
  ADT_CUDA(cudaGetLastError());
  return ADT_OK;
}

}  // namespace
}  // namespace adt

using namespace adt;

extern "C" int adt_smooth_l1_device(const double* v, int64_t m, int64_t n, int64_t l, int32_t sh,
                                    int32_t sv, double lambda, double* penalty, double* grad,
                                    void* stream) {
  int rc = check_smooth(m, n, l, sh, sv, v, penalty);
  if (rc) return rc;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(ADT_ENODEV, "no CUDA device available");
  }
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nc = m * n * l;
  void* scratch = nullptr;
  ADT_CUDA(cudaMallocAsync(&scratch, (2 * nc + SM_MAX_BLOCKS) * sizeof(double), st));
  rc = enqueue_smooth(v, m, n, l, sh, sv, lambda, penalty, grad, (double*)scratch, st);
  cudaError_t e = cudaFreeAsync(scratch, st);
  if (rc) return rc;
  if (e != cudaSuccess) return cuda_error(e, "cudaFreeAsync");
  return ADT_OK;
}

extern "C" int adt_smooth_l1(const double* v, int64_t m, int64_t n, int64_t l, int32_t sh,
                             int32_t sv, double lambda, double* penalty, double* grad) {
  int rc = check_smooth(m, n, l, sh, sv, v, penalty);
  if (rc) return rc;
  const int64_t nc = m * n * l;
  for (int64_t i = 0; i < nc; ++i)
    if (!std::isfinite(v[i])) return set_error(ADT_EINVAL, "smooth_l1: non-finite model value");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return set_error(ADT_ENODEV, "no CUDA device available");
  }
  DevBuf dv, dg, dp;
  ADT_CUDA(dv.reserve(nc * sizeof(double)));
  ADT_CUDA(dp.reserve(sizeof(double)));
  if (grad) ADT_CUDA(dg.reserve(nc * sizeof(double)));
  ADT_CUDA(cudaMemcpy(dv.p, v, nc * sizeof(double), cudaMemcpyHostToDevice));
  rc = adt_smooth_l1_device((const double*)dv.p, m, n, l, sh, sv, lambda, (double*)dp.p,
                            grad ? (double*)dg.p : nullptr, nullptr);
  if (rc) return rc;
  ADT_CUDA(cudaMemcpy(penalty, dp.p, sizeof(double), cudaMemcpyDeviceToHost));
  if (grad) ADT_CUDA(cudaMemcpy(grad, dg.p, nc * sizeof(double), cudaMemcpyDeviceToHost));
  return ADT_OK;
}
