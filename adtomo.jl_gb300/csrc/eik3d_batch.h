// eik3d_batch.h -- batched misfit + gradient plan (host side).
#pragma once
#include <cstddef>
#include <cstdint>
#include "../../include/adtomo_gpu.h"

namespace adt {

struct BatchPlan;

void batch_opts_default(adt_batch_opts* o);
// Host-only checks of the plan's arguments and options (no device work).
int batch_check_args(int32_t n_fields, const int32_t* dims, const double* h, const int32_t* nsta,
                     int32_t n_solves, const int32_t* solve_field, const double* src_xyz,
                     const adt_batch_opts* opts);
int batch_create(BatchPlan** out, int32_t n_fields, const int32_t* dims, const double* h,
                 const int32_t* nsta, const double* sta_xyz, int32_t n_solves,
                 const int32_t* solve_field, const double* src_xyz, const adt_batch_opts* opts);
void batch_destroy(BatchPlan* p);
int batch_upload(BatchPlan* p, const double* slowness, const double* t_obs, const double* weight);
int batch_run_resident(BatchPlan* p);
int batch_set_source_velocity(BatchPlan* p, const double* vel0);
int batch_autotune(BatchPlan* p, int reps);
int batch_download(BatchPlan* p, double* misfit, double* t_pred, double* grad,
                   adt_solve_status* status);
int batch_stats(BatchPlan* p, adt_batch_stats* s);
void* batch_stream(BatchPlan* p);
void* batch_device_buffer(BatchPlan* p, int which);

// The single-event 3D adjoint in causal order (k_single_adj_causal), for
// grids of fewer than 2^31 cells: lambda into rec (blk_slots(m, n, l) records
// of CAUSAL_REC64_BYTES bytes in the blocked layout, lambda first),
// *d_complete = 1 when every non-fixed cell was evaluated.  meta:
// blk_slots(m, n, l) words; queue: one word per cell.
constexpr size_t CAUSAL_REC64_BYTES = 32;
int causal_single_adjoint(const double* d_u, const double* d_u0, const double* d_grad_u, int m,
                          int n, int l, uint32_t* meta, void* rec, int* queue, int* d_complete,
                          void* stream);

}  // namespace adt
