// fp64_int.cuh -- IEEE binary64 square roots and divisions evaluated on the
// integer and FP32 pipes, bit-identical to the correctly rounded
// (round-to-nearest-even) FP64 operations.
//
// GB300 executes FP64 at about 2 lanes per clock per SM: with one warp per
// sub-partition an FP64 addition takes about 77 cycles, and the FP64 unit's
// square root and division sequences about 650 and 600 cycles, while integer
// and FP32 instructions issue every one or two cycles.  The reference's local
// solves (Eikonal.h:14-20, Eikonal3D.cpp:11-28) and its adjoint rows take
// their square roots and divisions from here, and the exact local solves
// their compares (for values that are never NaN); additions and
// multiplications stay FP64 instructions, which measured faster than
// integer-pipe versions of them in these kernels.
//
// Every function returns exactly the IEEE result for every input.  The
// integer path covers finite normal operands (and zero where stated) with a
// normal result; anything else (subnormals, infinities, NaN, a result that
// would leave the normal range) takes the FP64 operation itself.
//
// Square root and division follow the classical scheme for correctly
// rounded results (Newton-Raphson iterations, then an exact remainder test
// for the last bit; e.g. J.-M. Muller et al., Handbook of Floating-Point
// Arithmetic, 2nd ed., Birkhauser 2018): an FP32 reciprocal (square root)
// seed with relative error up to 2^-19, one Newton step on the reciprocal
// (square root) in 64-bit fixed point, one correction of the quotient (root)
// from its residual, which leaves it within one unit of the truncated
// 53-bit result; the exact integer remainder then fixes the truncation and
// the rounding.  Binary division and square root never land exactly halfway
// between two doubles, so round-to-nearest needs no tie case; the division
// keeps the even rule anyway.  Division by 3 takes a shorter exact route
// (fi_div3).
//
// The header compiles for the host too (plain C++), where the FP32 seeds are
// exact IEEE operations and the fallbacks are the host's IEEE operations, so
// the integer algorithm can be checked on the CPU against IEEE arithmetic.
#pragma once
#include <stdint.h>

#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define FI_HD __host__ __device__ __forceinline__
#else
#define FI_HD inline
#endif

namespace adt {

constexpr uint64_t FI_SIGN = 0x8000000000000000ull;
constexpr uint64_t FI_FRAC = 0x000fffffffffffffull;
constexpr uint64_t FI_HID = 0x0010000000000000ull;

FI_HD uint64_t fi_bits(double x) {
#if defined(__CUDA_ARCH__)
  return (uint64_t)__double_as_longlong(x);
#else
  uint64_t b;
  std::memcpy(&b, &x, 8);
  return b;
#endif
}

FI_HD double fi_double(uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __longlong_as_double((long long)b);
#else
  double x;
  std::memcpy(&x, &b, 8);
  return x;
#endif
}

FI_HD uint64_t fi_mulhi(uint64_t a, uint64_t b) {
#if defined(__CUDA_ARCH__)
  return __umul64hi(a, b);
#else
  return (uint64_t)(((unsigned __int128)a * b) >> 64);
#endif
}

// FP32 seeds: 1/sqrt(x) and 1/x for x in [1/4, 1) and [1/2, 1).
FI_HD float fi_rsqrt_seed(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / std::sqrt(x);
#endif
}

FI_HD float fi_rcp_seed(float x) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
#else
  return 1.0f / x;
#endif
}

FI_HD double fi_hw_sqrt(double x) {
#if defined(__CUDA_ARCH__)
  return __dsqrt_rn(x);
#else
  return std::sqrt(x);
#endif
}

FI_HD double fi_hw_div(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __ddiv_rn(a, b);
#else
  return a / b;
#endif
}

// ------------------------------------------------ compares without NaN
// IEEE a < b, a <= b, a == b and the reference's min (b < a ? b : a) for
// doubles that are not NaN (travel times and their candidates never are):
// the bit patterns as two's complement keys (a negative value's magnitude
// bits flipped) compared as integers, with -0 and +0 kept equal.  A few
// integer instructions, where an FP64 compare is a trip through the FP64
// unit.
FI_HD int64_t fi_key(uint64_t b) {
  const int64_t x = (int64_t)b;
  return x ^ ((x >> 63) & (int64_t)0x7fffffffffffffffLL);
}
FI_HD bool fi_both_zero(uint64_t x, uint64_t y) { return ((x | y) << 1) == 0; }
FI_HD bool lt_nn(double a, double b) {
  const uint64_t x = fi_bits(a), y = fi_bits(b);
  return fi_key(x) < fi_key(y) && !fi_both_zero(x, y);
}
FI_HD bool le_nn(double a, double b) { return !lt_nn(b, a); }
FI_HD bool eq_nn(double a, double b) {
  const uint64_t x = fi_bits(a), y = fi_bits(b);
  return x == y || fi_both_zero(x, y);
}
FI_HD double min_nn(double a, double b) { return lt_nn(b, a) ? b : a; }

// -------------------------------------------------------------- square root
// Integer core for a positive normal x = m 2^E (m in [2^52, 2^54), E even)
// with v = m 2^10, V = v / 2^64 in [1/4, 1) and an FP32 seed r0f ~ 1/sqrt(V).
FI_HD double fi_sqrt_core(uint64_t m, int E, float r0f) {
  const uint64_t v = m << 10;
  r0f = r0f < 0x1.fffffep0f ? r0f : 0x1.fffffep0f;  // 1/sqrt(V) <= 2
  const uint64_t R0 = (uint64_t)(r0f * 0x1p30f);     // r0 2^30 (exact), < 2^31
  // r1 = r0 (3 - V r0^2) / 2
  const uint64_t t = fi_mulhi(v, R0 * R0);           // V r0^2 2^60
  const uint64_t e = (3ull << 60) - t;               // (3 - V r0^2) 2^60
  const uint64_t R1 = fi_mulhi(R0 << 32, e);         // r1 2^59
  // s0 = V r1 ~ sqrt(V); s1 = s0 + r1/2 (V - s0^2)
  const uint64_t S0 = fi_mulhi(v, R1);  // s0 2^59
  const uint64_t p_lo = S0 * S0, p_hi = fi_mulhi(S0, S0);
  const uint64_t a_lo = v << 54, a_hi = v >> 10;  // V 2^118
  const uint64_t d_lo = a_lo - p_lo;
  const uint64_t d_hi = a_hi - p_hi - (a_lo < p_lo ? 1u : 0u);
  const int64_t d = (int64_t)((d_hi << 42) | (d_lo >> 22));  // (V - s0^2) 2^96
  const uint64_t ad = d < 0 ? (uint64_t)0 - (uint64_t)d : (uint64_t)d;
  const uint64_t c = fi_mulhi(R1, ad) >> 33;                 // r1/2 (V - s0^2) 2^59
  const uint64_t S1 = d < 0 ? S0 - c : S0 + c;               // sqrt(V) 2^59
  // s = floor(sqrt(M)), M = m 2^52 = V 2^106; r = M - s^2
  // s is within one of floor(sqrt(M)); the corrections are selects, not
  // branches
  uint64_t s = S1 >> 6;
  int64_t r = (int64_t)((m << 52) - s * s);
  const bool lo = r < 0;
  r += lo ? (int64_t)(2 * s - 1) : 0;
  s -= lo ? 1u : 0u;
  const bool hi = r > (int64_t)(2 * s);
  r -= hi ? (int64_t)(2 * s + 1) : 0;
  s += hi ? 1u : 0u;
  s += (r > (int64_t)s) ? 1u : 0u;  // sqrt(M) >= s + 1/2  <=>  r > s
  // sqrt(x) = s 2^(E/2 - 26): exponent field E/2 + 1049 (s carries into it at 2^53)
  return fi_double(((uint64_t)((E >> 1) + 1048) << 52) + s);
}

FI_HD double fi_sqrt(double x) {
  const uint64_t b = fi_bits(x);
  const uint32_t ef = (uint32_t)(b >> 52);  // sign and exponent
  if (ef - 1u >= 2046u) return fi_hw_sqrt(x);  // zero, negative, subnormal, inf, NaN
  uint64_t m = (b & FI_FRAC) | FI_HID;
  int E = (int)ef - 1075;
  if (E & 1) {
    m <<= 1;
    --E;
  }
  const float vf = (float)(uint32_t)(m >> 22) * 0x1p-32f;  // V, rounded to FP32
  return fi_sqrt_core(m, E, fi_rsqrt_seed(vf));
}

// ----------------------------------------------------------------- division
// Integer core for normal a, b with an FP32 seed r0f ~ 1/B, B = mb / 2^53.
FI_HD double fi_div_core(uint64_t ab, uint64_t bb, float r0f) {
  const uint32_t ea = (uint32_t)(ab >> 52) & 0x7ffu, eb = (uint32_t)(bb >> 52) & 0x7ffu;
  const uint64_t sg = (ab ^ bb) & FI_SIGN;
  const uint64_t ma = (ab & FI_FRAC) | FI_HID, mb = (bb & FI_FRAC) | FI_HID;
  const uint64_t w = mb << 11;                        // B 2^64, B in [1/2, 1)
  r0f = r0f < 0x1.fffffep0f ? r0f : 0x1.fffffep0f;   // 1/B <= 2
  const uint64_t R0 = (uint64_t)(r0f * 0x1p31f);      // r0 2^31 (exact), < 2^32
  // r1 = r0 (2 - B r0)
  const uint64_t t = fi_mulhi(w, R0 << 32);           // B r0 2^63
  const uint64_t e = (uint64_t)0 - t;                 // (2 - B r0) 2^63
  const uint64_t R1 = fi_mulhi(R0 << 32, e);          // r1 2^62
  // q0 = A r1; q1 = q0 + r1 (A - B q0)
  const uint64_t wa = ma << 11;                       // A 2^64, A in [1/2, 1)
  const uint64_t Q0 = fi_mulhi(wa, R1);               // q0 2^62
  const uint64_t p_lo = w * Q0, p_hi = fi_mulhi(w, Q0);
  const uint64_t a_lo = wa << 62, a_hi = wa >> 2;     // A 2^126
  const uint64_t d_lo = a_lo - p_lo;
  const uint64_t d_hi = a_hi - p_hi - (a_lo < p_lo ? 1u : 0u);
  const int64_t d = (int64_t)((d_hi << 36) | (d_lo >> 28));  // (A - B q0) 2^98
  const uint64_t ad = d < 0 ? (uint64_t)0 - (uint64_t)d : (uint64_t)d;
  const uint64_t c = fi_mulhi(R1, ad) >> 34;                 // r1 (A - B q0) 2^62
  const uint64_t Q1 = d < 0 ? Q0 - c : Q0 + c;               // (A/B) 2^62
  // 53-bit quotient qi = floor(ma 2^k / mb), k = 52 when ma >= mb, else 53
  const bool big = ma >= mb;
  uint64_t qi = Q1 >> (big ? 10 : 9);
  // qi is within one of the truncated quotient; corrections by selects
  int64_t r = (int64_t)((ma << (big ? 52 : 53)) - qi * mb);
  const bool lo = r < 0;
  r += lo ? (int64_t)mb : 0;
  qi -= lo ? 1u : 0u;
  const bool hi = r >= (int64_t)mb;
  r -= hi ? (int64_t)mb : 0;
  qi += hi ? 1u : 0u;
  const int64_t r2 = 2 * r;
  qi += (r2 > (int64_t)mb || (r2 == (int64_t)mb && (qi & 1u))) ? 1u : 0u;
  const int biased = (int)ea - (int)eb + (big ? 1023 : 1022);
  if (biased < 1 || biased > 2045) return fi_hw_div(fi_double(ab), fi_double(bb));
  return fi_double(sg | (((uint64_t)(biased - 1) << 52) + qi));
}

// a / 3, correctly rounded.  For a = m 2^E (m the 53-bit significand) the
// 53-bit quotient is floor(m 2^k / 3), k = 1 when m >= 1.5 * 2^52, else 2:
// an exact integer division by 3 (multiply-high by ceil(2^65 / 3) =
// 0xAAAAAAAAAAAAAAAB, then a shift of one, exact for every 64-bit dividend:
// T. Granlund, P. Montgomery, Division by Invariant Integers using
// Multiplication, PLDI 1994), whose remainder (0, 1 or 2) decides the
// rounding: 2/3 of a unit rounds up, 1/3 down, no ties.
FI_HD double fi_div3(double a) {
  const uint64_t b = fi_bits(a);
  const uint32_t e = (uint32_t)(b >> 52) & 0x7ffu;
  const uint64_t m = (b & FI_FRAC) | FI_HID;
  const int k = m >= (3ull << 51) ? 1 : 2;
  if (e - 1u >= 2046u || (int)e - k < 1) {
    if ((b << 1) == 0) return a;  // +-0 / 3
    return fi_hw_div(a, 3.0);     // subnormal, inf, NaN, or a subnormal quotient
  }
  const uint64_t n = m << k;
  uint64_t q = fi_mulhi(n, 0xAAAAAAAAAAAAAAABull) >> 1;  // floor(n / 3)
  q += (n - 3 * q == 2) ? 1u : 0u;
  // a / 3 = q 2^(E - k): exponent field e - k (q carries into it at 2^53)
  return fi_double((b & FI_SIGN) | (((uint64_t)(e - k - 1) << 52) + q));
}

FI_HD double fi_div(double a, double b) {
  const uint64_t ab = fi_bits(a), bb = fi_bits(b);
  const uint32_t ea = (uint32_t)(ab >> 52) & 0x7ffu, eb = (uint32_t)(bb >> 52) & 0x7ffu;
  if (eb - 1u >= 2046u) return fi_hw_div(a, b);  // b zero, subnormal, inf or NaN
  if (ea - 1u >= 2046u) {
    if ((ab << 1) == 0) return fi_double((ab ^ bb) & FI_SIGN);  // +-0 / normal
    return fi_hw_div(a, b);
  }
  const float bf = (float)((uint32_t)((bb & FI_FRAC) >> 21) | 0x80000000u) * 0x1p-32f;  // B, rounded
  return fi_div_core(ab, bb, fi_rcp_seed(bf));
}

}  // namespace adt
