// Host driver for tests/test_fp64_int.py: runs the integer-pipe FP64 square
// roots, divisions and compares of fp64_int.cuh on arrays (plain C++ build of the
// header) so that they can be compared bit for bit with IEEE arithmetic.  perturb != 0
// scales each FP32 seed by 1 +- perturb (sign from the operand bits), which
// checks that the Newton steps and the remainder correction tolerate a seed
// far worse than the GPU's approximate reciprocal and square root.
#include <cstdint>

#include "fp64_int.cuh"

using namespace adt;

namespace {
float perturbed(float seed, uint64_t key, double perturb) {
  if (perturb == 0.0) return seed;
  const double s = ((key >> 17) ^ (key >> 3)) & 1 ? perturb : -perturb;
  return (float)((double)seed * (1.0 + s));
}

double sqrt_seeded(double x, double perturb) {
  const uint64_t b = fi_bits(x);
  const uint32_t ef = (uint32_t)(b >> 52);
  if (perturb == 0.0 || ef - 1u >= 2046u) return fi_sqrt(x);
  uint64_t m = (b & FI_FRAC) | FI_HID;
  int E = (int)ef - 1075;
  if (E & 1) {
    m <<= 1;
    --E;
  }
  const float vf = (float)(uint32_t)(m >> 22) * 0x1p-32f;
  return fi_sqrt_core(m, E, perturbed(fi_rsqrt_seed(vf), b, perturb));
}

double div_seeded(double a, double b, double perturb) {
  const uint64_t ab = fi_bits(a), bb = fi_bits(b);
  const uint32_t ea = (uint32_t)(ab >> 52) & 0x7ffu, eb = (uint32_t)(bb >> 52) & 0x7ffu;
  if (perturb == 0.0 || eb - 1u >= 2046u || ea - 1u >= 2046u) return fi_div(a, b);
  const float bf = (float)((uint32_t)((bb & FI_FRAC) >> 21) | 0x80000000u) * 0x1p-32f;
  return fi_div_core(ab, bb, perturbed(fi_rcp_seed(bf), ab ^ bb, perturb));
}
}  // namespace

// op: 0 sqrt(a), 1 a / b, 2 a / 3, 3 a < b, 4 a <= b, 5 a == b, 6 min(a, b)
extern "C" int fi_check_run(int op, const double* a, const double* b, double* out, int64_t n,
                            double perturb) {
  for (int64_t i = 0; i < n; ++i) {
    double r = 0.0;
    switch (op) {
      case 0: r = sqrt_seeded(a[i], perturb); break;
      case 1: r = div_seeded(a[i], b[i], perturb); break;
      case 2: r = fi_div3(a[i]); break;
      case 3: r = lt_nn(a[i], b[i]) ? 1.0 : 0.0; break;
      case 4: r = le_nn(a[i], b[i]) ? 1.0 : 0.0; break;
      case 5: r = eq_nn(a[i], b[i]) ? 1.0 : 0.0; break;
      case 6: r = min_nn(a[i], b[i]); break;
      default: return -1;
    }
    out[i] = r;
  }
  return 0;
}
