// capi.cu -- the extern "C" entry points of libadtomo_gpu.so (include/adtomo_gpu.h).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "eik2d.h"
#include "eik3d_batch.h"
#include "eik3d_common_host.h"
#include "eik3d_single.h"

namespace adt {

static thread_local char g_err[512] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof g_err, fmt, ap);
  va_end(ap);
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation)
    return set_error(ADT_ENOMEM, "%s: %s", what, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return set_error(ADT_ENODEV, "%s: %s", what, cudaGetErrorString(e));
  return set_error(ADT_ECUDA, "%s: %s", what, cudaGetErrorString(e));
}

namespace {

int check_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) {
    cudaGetLastError();
    return set_error(ADT_ENODEV, "no CUDA device available");
  }
  return ADT_OK;
}

bool finite_positive(const double* a, int64_t n) {
  for (int64_t i = 0; i < n; ++i)
    if (!(a[i] > 0.0) || !std::isfinite(a[i])) return false;
  return true;
}

// Host <-> device staging for the host-pointer entry points: per device, the
// buffers are kept between calls (grown, never shrunk; one above 256 MiB is
// freed when its call ends), so a repeated call allocates nothing.  A call
// holds its device's lock while it uses them (recursive: the buffers of a
// nested call follow the outer call's); this lock is always taken before
// the solvers' own workspace locks.
struct StagingPool {
  std::recursive_mutex mu;
  std::vector<DevBuf*> bufs;
  size_t used = 0;
};
StagingPool& staging_pool(int dev) {
  static StagingPool* pools = new StagingPool[64];
  return pools[dev & 63];
}

struct Staging {
  StagingPool* P;
  std::unique_lock<std::recursive_mutex> lock;
  size_t first;
  Staging() {
    int dev = 0;
    cudaGetDevice(&dev);
    P = &staging_pool(dev);
    lock = std::unique_lock<std::recursive_mutex>(P->mu);
    first = P->used;
  }
  ~Staging() {
    for (size_t k = first; k < P->used; ++k)
      if (P->bufs[k]->bytes > ((size_t)256 << 20)) P->bufs[k]->release();
    P->used = first;
  }
  void* alloc_bytes(size_t bytes, int* rc) {
    if (P->used == P->bufs.size()) P->bufs.push_back(new DevBuf());
    DevBuf* b = P->bufs[P->used++];
    if (b->reserve(std::max<size_t>(bytes, 8)) != cudaSuccess) {
      cudaGetLastError();
      *rc = set_error(ADT_ENOMEM, "cudaMalloc of %zu bytes failed", bytes);
      return nullptr;
    }
    return b->p;
  }
  double* alloc(size_t n, int* rc) { return static_cast<double*>(alloc_bytes(n * sizeof(double), rc)); }
};

int check2d(int64_t m, int64_t n, int64_t srcx, int64_t srcy, double h) {
  if (m < 1 || n < 1 || (m + 1) * (n + 1) > (int64_t)1 << 31)
    return set_error(ADT_EINVAL, "eikonal: need m >= 1 and n >= 1 (a grid of at least 2 x 2 nodes)");
  if (srcx < 1 || srcx > m + 1 || srcy < 1 || srcy > n + 1)
    return set_error(ADT_EINVAL, "eikonal: source (%lld, %lld) outside 1..%lld x 1..%lld",
                     (long long)srcx, (long long)srcy, (long long)(m + 1), (long long)(n + 1));
  if (!(h > 0.0) || !std::isfinite(h)) return set_error(ADT_EINVAL, "eikonal: h must be finite and > 0");
  return ADT_OK;
}

int check3d(int64_t m, int64_t n, int64_t l, double h, double tol) {
  if (m < 2 || n < 2 || l < 2)
    return set_error(ADT_EINVAL, "eikonal3d: need m, n, l >= 2 (got %lld x %lld x %lld)", (long long)m,
                     (long long)n, (long long)l);
  if (m > BI * 2047 || n > BJ * 2047 || l > (1 << 20) || m * n * l > ((int64_t)1 << 34))
    return set_error(ADT_EINVAL, "eikonal3d: grid too large");
  // brick coordinates are packed in 11/11/10 bits (pack_brick): at most 1023
  // bricks along k
  if (make_geom((int)m, (int)n, (int)l, SBK).nbz > 1023)
    return set_error(ADT_EINVAL, "eikonal3d: l = %lld is too deep (at most %d)", (long long)l,
                     SBK * 1023);
  if (!(h > 0.0) || !std::isfinite(h)) return set_error(ADT_EINVAL, "eikonal3d: h must be finite and > 0");
  if (!(tol >= 0.0)) return set_error(ADT_EINVAL, "eikonal3d: tol must be >= 0");
  return ADT_OK;
}

}  // namespace
}  // namespace adt

using namespace adt;

extern "C" {

const char* adt_last_error(void) { return g_err; }

const char* adt_version(void) { return "adtomo-gb300 0.1 (sm_103a)"; }

int adt_tile_layout(int32_t bk, int32_t* out) {
  if (!out || (bk != 16 && bk != 32 && bk != 64))
    return set_error(ADT_EINVAL, "tile_layout: bk must be 16, 32 or 64");
  out[0] = adt::tile_row_stride(bk);
  out[1] = adt::itile_row_stride(bk);
  out[2] = adt::tile_col_stride(bk, true);
  out[3] = adt::tile_col_stride(bk, false);
  out[4] = adt::tile_elems(bk);
  out[5] = adt::itile_elems(bk);
  return ADT_OK;
}

int adt_abi_struct_sizes(int64_t* out, int n) {
  const int64_t sz[3] = {(int64_t)sizeof(adt_solve_status), (int64_t)sizeof(adt_batch_opts),
                         (int64_t)sizeof(adt_batch_stats)};
  for (int i = 0; out && i < n && i < 3; ++i) out[i] = sz[i];
  return 3;
}

int adt_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

int adt_eikonal(const double* f, int64_t m, int64_t n, int64_t srcx, int64_t srcy, double h,
                double* u, adt_solve_status* status) {
  int rc = check2d(m, n, srcx, srcy, h);
  if (rc) return rc;
  if (!f || !u) return set_error(ADT_EINVAL, "eikonal: null array");
  const int64_t N = (m + 1) * (n + 1);
  if (!finite_positive(f, N)) return set_error(ADT_EINVAL, "eikonal: slowness must be finite and > 0");
  if ((rc = check_device())) return rc;
  Staging S;
  double* df = S.alloc(N, &rc);
  double* du = df ? S.alloc(N, &rc) : nullptr;
  if (!du) return rc;
  int* dsrc = static_cast<int*>(S.alloc_bytes(2 * sizeof(int), &rc));
  if (!dsrc) return rc;
  const int hs[2] = {(int)srcx - 1, (int)srcy - 1};
  ADT_CUDA(cudaMemcpy(dsrc, hs, sizeof hs, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(df, f, N * 8, cudaMemcpyHostToDevice));
  adt_solve_status st;
  rc = eik2d_forward_batch(df, (int)m, (int)n, h, 1, dsrc, dsrc + 1, du, &st, 0);
  if (rc) return rc;
  ADT_CUDA(cudaMemcpy(u, du, N * 8, cudaMemcpyDeviceToHost));
  if (status) *status = st;
  return ADT_OK;
}

int adt_eikonal_batch(const double* f, int64_t m, int64_t n, int64_t count, const int64_t* srcx,
                      const int64_t* srcy, double h, double* u, adt_solve_status* status) {
  if (count < 1 || !srcx || !srcy || !f || !u) return set_error(ADT_EINVAL, "eikonal_batch: bad arguments");
  int rc;
  for (int64_t k = 0; k < count; ++k)
    if ((rc = check2d(m, n, srcx[k], srcy[k], h))) return rc;
  const int64_t N = (m + 1) * (n + 1);
  if (!finite_positive(f, N)) return set_error(ADT_EINVAL, "eikonal: slowness must be finite and > 0");
  if ((rc = check_device())) return rc;
  Staging S;
  double* df = S.alloc(N, &rc);
  double* du = df ? S.alloc(N * count, &rc) : nullptr;
  if (!du) return rc;
  std::vector<int> hs(2 * count);
  for (int64_t k = 0; k < count; ++k) {
    hs[k] = (int)srcx[k] - 1;
    hs[count + k] = (int)srcy[k] - 1;
  }
  int* dsrc = static_cast<int*>(S.alloc_bytes(hs.size() * sizeof(int), &rc));
  if (!dsrc) return rc;
  ADT_CUDA(cudaMemcpy(dsrc, hs.data(), hs.size() * sizeof(int), cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(df, f, N * 8, cudaMemcpyHostToDevice));
  std::vector<adt_solve_status> st(count);
  rc = eik2d_forward_batch(df, (int)m, (int)n, h, (int)count, dsrc, dsrc + count, du,
                           st.data(), 0);
  if (rc) return rc;
  ADT_CUDA(cudaMemcpy(u, du, N * count * 8, cudaMemcpyDeviceToHost));
  if (status) std::memcpy(status, st.data(), count * sizeof(adt_solve_status));
  return ADT_OK;
}

int adt_eikonal_grad(const double* grad_u, const double* u, const double* f, int64_t m, int64_t n,
                     int64_t srcx, int64_t srcy, double h, double* grad_f) {
  int rc = check2d(m, n, srcx, srcy, h);
  if (rc) return rc;
  if (!grad_u || !u || !f || !grad_f) return set_error(ADT_EINVAL, "eikonal_grad: null array");
  const int64_t N = (m + 1) * (n + 1);
  if ((rc = check_device())) return rc;
  Staging S;
  double* dg = S.alloc(N, &rc);
  double* du = dg ? S.alloc(N, &rc) : nullptr;
  double* df = du ? S.alloc(N, &rc) : nullptr;
  double* dgf = df ? S.alloc(N, &rc) : nullptr;
  if (!dgf) return rc;
  ADT_CUDA(cudaMemcpy(dg, grad_u, N * 8, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(du, u, N * 8, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(df, f, N * 8, cudaMemcpyHostToDevice));
  rc = eik2d_adjoint(dg, du, df, (int)m, (int)n, h, (int)srcx - 1, (int)srcy - 1, dgf, 0);
  if (rc) return rc;
  ADT_CUDA(cudaMemcpy(grad_f, dgf, N * 8, cudaMemcpyDeviceToHost));
  return ADT_OK;
}

int adt_eikonal_three_d_device(const double* u0, const double* f, double h, int64_t m, int64_t n,
                               int64_t l, double tol, int verbose, double* u,
                               adt_solve_status* status, void* stream) {
  int rc = check3d(m, n, l, h, tol);
  if (rc) return rc;
  if (!u0 || !f || !u) return set_error(ADT_EINVAL, "eikonal3d: null array");
  if ((rc = check_device())) return rc;
  rc = eik3d_single_forward(u0, f, h, (int)m, (int)n, (int)l, tol, 20, verbose, u, status,
                            (cudaStream_t)stream);
  return rc;
}

int adt_eikonal_three_d(const double* u0, const double* f, double h, int64_t m, int64_t n,
                        int64_t l, double tol, int verbose, double* u, adt_solve_status* status) {
  int rc = check3d(m, n, l, h, tol);
  if (rc) return rc;
  if (!u0 || !f || !u) return set_error(ADT_EINVAL, "eikonal3d: null array");
  const int64_t N = m * n * l;
  if (!finite_positive(f, N)) return set_error(ADT_EINVAL, "eikonal3d: slowness must be finite and > 0");
  for (int64_t i = 0; i < N; ++i)
    if (std::isnan(u0[i])) return set_error(ADT_EINVAL, "eikonal3d: u0 contains NaN");
  if ((rc = check_device())) return rc;
  Staging S;
  double* d0 = S.alloc(N, &rc);
  double* df = d0 ? S.alloc(N, &rc) : nullptr;
  double* du = df ? S.alloc(N, &rc) : nullptr;
  if (!du) return rc;
  ADT_CUDA(cudaMemcpy(d0, u0, N * 8, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(df, f, N * 8, cudaMemcpyHostToDevice));
  rc = eik3d_single_forward(d0, df, h, (int)m, (int)n, (int)l, tol, 20, verbose, du, status, 0);
  if (rc) return rc;
  ADT_CUDA(cudaMemcpy(u, du, N * 8, cudaMemcpyDeviceToHost));
  return ADT_OK;
}

int adt_eikonal_three_d_grad_device(const double* grad_u, const double* u, const double* u0,
                                    const double* f, double h, int64_t m, int64_t n, int64_t l,
                                    double* grad_u0, double* grad_f, void* stream) {
  int rc = check3d(m, n, l, h, 0.0);
  if (rc) return rc;
  if (!grad_u || !u || !u0 || !f || !grad_f) return set_error(ADT_EINVAL, "eikonal3d_grad: null array");
  if ((rc = check_device())) return rc;
  int iters = 0, conv = 0;
  rc = eik3d_single_adjoint(grad_u, u, u0, f, h, (int)m, (int)n, (int)l, 100000, grad_u0, grad_f, &iters,
                            &conv, (cudaStream_t)stream);
  if (rc) return rc;
  if (!conv) return set_error(ADT_ENOCONV, "eikonal3d_grad: the adjoint solve did not complete");
  return ADT_OK;
}

int adt_eikonal_three_d_grad(const double* grad_u, const double* u, const double* u0,
                             const double* f, double h, int64_t m, int64_t n, int64_t l,
                             double tol, int verbose, double* grad_u0, double* grad_f) {
  (void)tol;
  (void)verbose;
  int rc = check3d(m, n, l, h, 0.0);
  if (rc) return rc;
  if (!grad_u || !u || !u0 || !f || !grad_u0 || !grad_f)
    return set_error(ADT_EINVAL, "eikonal3d_grad: null array");
  const int64_t N = m * n * l;
  if ((rc = check_device())) return rc;
  Staging S;
  double* dg = S.alloc(N, &rc);
  double* du = dg ? S.alloc(N, &rc) : nullptr;
  double* d0 = du ? S.alloc(N, &rc) : nullptr;
  double* df = d0 ? S.alloc(N, &rc) : nullptr;
  double* dgu0 = df ? S.alloc(N, &rc) : nullptr;
  double* dgf = dgu0 ? S.alloc(N, &rc) : nullptr;
  if (!dgf) return rc;
  ADT_CUDA(cudaMemcpy(dg, grad_u, N * 8, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(du, u, N * 8, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(d0, u0, N * 8, cudaMemcpyHostToDevice));
  ADT_CUDA(cudaMemcpy(df, f, N * 8, cudaMemcpyHostToDevice));
  rc = adt_eikonal_three_d_grad_device(dg, du, d0, df, h, m, n, l, dgu0, dgf, nullptr);
  if (rc) return rc;
  ADT_CUDA(cudaMemcpy(grad_u0, dgu0, N * 8, cudaMemcpyDeviceToHost));
  ADT_CUDA(cudaMemcpy(grad_f, dgf, N * 8, cudaMemcpyDeviceToHost));
  return ADT_OK;
}

// ----------------------------------------------------------------- batch
struct adt_batch {
  BatchPlan* plan;
};

void adt_batch_opts_default(adt_batch_opts* opts) {
  if (opts) batch_opts_default(opts);
}

int adt_batch_create(adt_batch** out, int32_t n_fields, const int32_t* dims, const double* h,
                     const int32_t* nsta, const double* sta_xyz, int32_t n_solves,
                     const int32_t* solve_field, const double* src_xyz,
                     const adt_batch_opts* opts) {
  if (!out) return set_error(ADT_EINVAL, "batch: null output handle");
  *out = nullptr;
  int rc = batch_check_args(n_fields, dims, h, nsta, n_solves, solve_field, src_xyz, opts);
  if (rc) return rc;
  rc = check_device();
  if (rc) return rc;
  BatchPlan* p = nullptr;
  rc = batch_create(&p, n_fields, dims, h, nsta, sta_xyz, n_solves, solve_field, src_xyz, opts);
  if (rc) return rc;
  *out = new adt_batch{p};
  return ADT_OK;
}

int adt_batch_destroy(adt_batch* b) {
  if (!b) return ADT_OK;
  batch_destroy(b->plan);
  delete b;
  return ADT_OK;
}

int adt_batch_upload(adt_batch* b, const double* slowness, const double* t_obs,
                     const double* weight) {
  if (!b) return set_error(ADT_EINVAL, "batch: null handle");
  return batch_upload(b->plan, slowness, t_obs, weight);
}

int adt_batch_set_source_velocity(adt_batch* b, const double* vel0) {
  if (!b) return set_error(ADT_EINVAL, "batch: null handle");
  return batch_set_source_velocity(b->plan, vel0);
}

int adt_batch_autotune(adt_batch* b, int32_t reps) {
  if (!b) return set_error(ADT_EINVAL, "batch: null handle");
  return batch_autotune(b->plan, reps);
}

int adt_batch_run_resident(adt_batch* b) {
  if (!b) return set_error(ADT_EINVAL, "batch: null handle");
  return batch_run_resident(b->plan);
}

int adt_batch_download(adt_batch* b, double* misfit, double* t_pred, double* grad,
                       adt_solve_status* status) {
  if (!b) return set_error(ADT_EINVAL, "batch: null handle");
  return batch_download(b->plan, misfit, t_pred, grad, status);
}

int adt_batch_run(adt_batch* b, const double* slowness, const double* t_obs, const double* weight,
                  double* misfit, double* t_pred, double* grad, adt_solve_status* status) {
  if (!b) return set_error(ADT_EINVAL, "batch: null handle");
  if (!slowness || !t_obs || !weight) return set_error(ADT_EINVAL, "batch: null input");
  int rc = batch_upload(b->plan, slowness, t_obs, weight);
  if (rc) return rc;
  if ((rc = batch_run_resident(b->plan))) return rc;
  return batch_download(b->plan, misfit, t_pred, grad, status);
}

void* adt_batch_stream(adt_batch* b) { return b ? batch_stream(b->plan) : nullptr; }

void* adt_batch_device_buffer(adt_batch* b, int32_t which) {
  return b ? batch_device_buffer(b->plan, which) : nullptr;
}

int adt_batch_stats_get(adt_batch* b, adt_batch_stats* out) {
  if (!b || !out) return set_error(ADT_EINVAL, "batch: null handle");
  return batch_stats(b->plan, out);
}

}  // extern "C"
