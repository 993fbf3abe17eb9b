// C entry points around the reference's own Eikonal functions, compiled from
// the reference sources in place (deps/CustomOps/Eikonal/Eikonal.h,
// deps/CustomOps/Eikonal3D/Eikonal3D.cpp) by oracle/Makefile into
// oracle/_ref/libadtomo_ref.so.  The TF op glue (Eikonal.cpp, EikonalThreeD.cpp)
// is not compiled; these wrappers do what its Compute methods do
// (Eikonal.cpp:125,217-219; EikonalThreeD.cpp:136-138,245-248), taking the
// 2D source as 0-based node indices.
// TEST INFRASTRUCTURE ONLY: used to generate tests/golden fixtures.
#include "Eikonal.h"
#include "Eikonal3D.h"

extern "C" {

void ref_eik2d_forward(double* u, const double* f, int m, int n, double h, int ix, int jx) {
  forward(u, f, m, n, h, ix, jx);
}

void ref_eik2d_backward(double* grad_f, const double* grad_u, const double* u, const double* f,
                        int m, int n, double h, int ix, int jx) {
  backward(grad_f, grad_u, u, f, m, n, h, ix, jx);
}

void ref_eik3d_forward(double* u, const double* u0, const double* f, double h, int m, int n, int l,
                       double tol, int verbose) {
  Eikonal3D::forward(u, u0, f, h, m, n, l, tol, verbose != 0);
}

void ref_eik3d_backward(double* grad_u0, double* grad_f, const double* grad_u, const double* u,
                        const double* u0, const double* f, double h, int m, int n, int l) {
  Eikonal3D::backward(grad_u0, grad_f, grad_u, u, u0, f, h, m, n, l);
}
}
