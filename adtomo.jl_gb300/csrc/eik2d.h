// eik2d.h -- 2D fast sweeping and adjoint (device pointers).
#pragma once
#include <cuda_runtime.h>

#include "../../include/adtomo_gpu.h"

namespace adt {

// count solves on one slowness grid; sources are 0-based node indices.
int eik2d_forward_batch(const double* d_f, int m, int n, double h, int count, const int* d_srcx,
                        const int* d_srcy, double* d_u, adt_solve_status* st, cudaStream_t stream);

int eik2d_adjoint(const double* d_gu, const double* d_u, const double* d_f, int m, int n, double h,
                  int ix, int jx, double* d_gf, cudaStream_t stream);

}  // namespace adt
