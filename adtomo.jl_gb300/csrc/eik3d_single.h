// eik3d_single.h -- plain FP64 single-solve 3D path (device pointers).
#pragma once
#include <cuda_runtime.h>

#include "../../include/adtomo_gpu.h"

namespace adt {

int eik3d_single_forward(const double* d_u0, const double* d_f, double h, int m, int n, int l,
                         double tol, int max_iter, int verbose, double* d_u, adt_solve_status* st,
                         cudaStream_t stream);

int eik3d_single_adjoint(const double* d_gu, const double* d_u, const double* d_u0,
                         const double* d_f, double h, int m, int n, int l, int max_iter,
                         double* d_gu0, double* d_gf, int* iters_out, int* converged_out,
                         cudaStream_t stream);

}  // namespace adt
