// eik_local.cuh -- per-cell upwind updates.
//
// Two families:
//  * *_exact (FP64): the reference's operation sequence written with IEEE
//    round-to-nearest intrinsics (__dmul_rn, __dadd_rn, __ddiv_rn, __dsqrt_rn),
//    which the compiler never contracts into FMAs, so results are bit-identical
//    to the reference compiled for x86-64 (Eikonal.h:14-20, Eikonal3D.cpp:11-28).
//    A division by 2.0 is written as a multiplication by 0.5: both are the
//    correctly rounded value of the same exact quotient, so the bits are the
//    same, and the multiplication is one instruction where the division is a
//    long dependent sequence in FP64.  Square roots and the divisions by 3
//    run on the integer pipes (fi_sqrt, fi_div3 in fp64_int.cuh: the same
//    bits, a shorter chain and a fraction of the FP64 unit's time).
//  * upd3_stable<T>: the same roots written without the B^2 - 4C cancellation:
//      two-term:   x = a + (d2 + sqrt(2 F^2 - d2^2)) / 2,           d2 = b - a
//      three-term: x = a + (d2 + d3 + sqrt(3 F^2 - d2^2 - d3^2 - (d3-d2)^2)) / 3
//    with F = f h.  Every term is a small difference, so FP32 keeps ~1 ulp of
//    the travel time instead of losing digits to (a+b)^2 when u >> f h.
#pragma once
#include "adt_common.cuh"
#include "fp64_int.cuh"

namespace adt {

// Sorted three-term update, reference arithmetic (Eikonal3D.cpp:11-28), with
// fh = f h given and ffhh = f f h h formed by ffhh_of() when the two-axis
// root is needed.
template <class FF>
__device__ __forceinline__ double upd3_exact_core(double a1, double a2, double a3, double fh,
                                                  FF ffhh_of) {
  double t;
  if (lt_nn(a2, a1)) { t = a1; a1 = a2; a2 = t; }
  if (lt_nn(a3, a1)) { t = a1; a1 = a3; a3 = t; }
  if (lt_nn(a3, a2)) { t = a2; a2 = a3; a3 = t; }
  double x = __dadd_rn(a1, fh);
  if (le_nn(x, a2)) return x;
  const double ffhh = ffhh_of();
  double B = -__dadd_rn(a1, a2);
  double C = __dmul_rn(__dsub_rn(__dadd_rn(__dmul_rn(a1, a1), __dmul_rn(a2, a2)), ffhh), 0.5);
  x = __dmul_rn(__dadd_rn(-B, fi_sqrt(__dsub_rn(__dmul_rn(B, B), __dmul_rn(4.0, C)))), 0.5);
  if (le_nn(x, a3)) return x;
  B = fi_div3(__dmul_rn(-2.0, __dadd_rn(__dadd_rn(a1, a2), a3)));
  C = fi_div3(
      __dsub_rn(__dadd_rn(__dadd_rn(__dmul_rn(a1, a1), __dmul_rn(a2, a2)), __dmul_rn(a3, a3)), ffhh));
  return __dmul_rn(__dadd_rn(-B, fi_sqrt(__dsub_rn(__dmul_rn(B, B), __dmul_rn(4.0, C)))), 0.5);
}

// The update from the cell's slowness f and the spacing h.
__device__ __forceinline__ double upd3_exact(double a1, double a2, double a3, double f, double h) {
  return upd3_exact_core(a1, a2, a3, __dmul_rn(f, h),
                         [&] { return __dmul_rn(__dmul_rn(__dmul_rn(f, f), h), h); });
}

// The update from the cell's fh = f h and ffhh = f f h h, each formed once in
// the reference's order (the same bits as upd3_exact).
__device__ __forceinline__ double upd3_exact_fh(double a1, double a2, double a3, double fh,
                                                double ffhh) {
  return upd3_exact_core(a1, a2, a3, fh, [&] { return ffhh; });
}

// Two-term update, reference arithmetic (Eikonal.h:14-20), given the node's
// fh = f h and q2 = 2 f f h h (each formed in the reference's order).  The
// square root runs on the integer pipes (fp64_int.cuh; the same bits as
// __dsqrt_rn): the one-CTA 2D wavefront keeps four warps busy, where the FP64
// unit, shared by the SM, serialises every FP64 instruction of the four.
__device__ __forceinline__ double upd2_exact(double a, double b, double fh, double q2) {
  const double d = fabs(__dsub_rn(a, b));
  if (le_nn(fh, d)) return __dadd_rn(min_nn(a, b), fh);
  const double ab = __dsub_rn(a, b);
  const double disc = __dsub_rn(q2, __dmul_rn(ab, ab));
  return __dmul_rn(__dadd_rn(__dadd_rn(a, b), fi_sqrt(disc)), 0.5);
}

template <class T>
__device__ __forceinline__ T tsqrt(T x);
template <>
__device__ __forceinline__ float tsqrt<float>(float x) {
  return sqrtf(x);
}
template <>
__device__ __forceinline__ double tsqrt<double>(double x) {
  return sqrt(x);
}

// Cancellation-free sorted three-term update (same roots as upd3_exact).
template <class T>
__device__ __forceinline__ T upd3_stable(T a, T b, T c, T fh) {
  T t;
  if (a > b) { t = a; a = b; b = t; }
  if (a > c) { t = a; a = c; c = t; }
  if (b > c) { t = b; b = c; c = t; }
  T x = a + fh;
  if (x <= b) return x;
  const T d2 = b - a;
  const T F2 = fh * fh;
  x = a + T(0.5) * (d2 + tsqrt<T>(T(2) * F2 - d2 * d2));
  if (x <= c) return x;
  const T d3 = c - a;
  const T e = d3 - d2;
  T disc = T(3) * F2 - d2 * d2 - d3 * d3 - e * e;
  disc = disc > T(0) ? disc : T(0);
  return a + (d2 + d3 + tsqrt<T>(disc)) * T(1.0 / 3.0);
}

}  // namespace adt
