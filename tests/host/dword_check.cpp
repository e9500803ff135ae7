// Host check of the double-word primitives of csrc/dword.cuh against long
// double (x86: 64-bit significand; on targets where long double is FP64 the
// exactness checks use the FP64 sums of two FP32 values, which are exact).
// Prints one line per failed property and exits non-zero on any failure.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <limits>
#include <random>

#include "../../axia-fem_gb300/csrc/dword.cuh"

static int fails = 0;
#define CHECK(cond, ...)              \
  do {                                \
    if (!(cond)) {                    \
      ++fails;                        \
      std::printf(__VA_ARGS__);       \
      std::printf("\n");              \
    }                                 \
  } while (0)

typedef long double R;
static R val(dw a) { return (R)a.h + (R)a.l; }

int main() {
  std::mt19937_64 rng(20261204);
  std::uniform_real_distribution<double> U(-1.0, 1.0);
  std::uniform_int_distribution<int> X(-30, 30);
  auto rf = [&]() { return (float)std::ldexp(U(rng), X(rng)); };
  for (int i = 0; i < 200000; ++i) {
    const float a = rf(), b = rf();
    float s, e;
    dwop::two_sum(a, b, s, e);
    CHECK((double)s + (double)e == (double)a + (double)b && s == a + b, "two_sum %a %a", a, b);
    dwop::two_prod(a, b, s, e);
    CHECK((double)s + (double)e == (double)a * (double)b, "two_prod %a %a", a, b);
  }
  // f32 -> f64 re-encoding: every class of FP32 number
  const float specials[] = {0.f, -0.f, 1.f, -2.5f, 3.4e38f, -1.2e-38f, 1e-40f, -1e-45f,
                            std::numeric_limits<float>::infinity(), -std::numeric_limits<float>::infinity()};
  for (float f : specials) {
    const double d = f32_to_f64_exact(f);
    CHECK(d == (double)f && std::signbit(d) == std::signbit(f), "f32_to_f64_exact %a", f);
  }
  CHECK(std::isnan(f32_to_f64_exact(std::numeric_limits<float>::quiet_NaN())), "f32_to_f64_exact nan");
  for (int i = 0; i < 100000; ++i) {
    const float f = rf();
    CHECK(f32_to_f64_exact(f) == (double)f, "f32_to_f64_exact %a", f);
  }
  // double <-> double word: 48 significant bits
  const double u48 = std::ldexp(1.0, -48);
  double worst_rt = 0, worst_mul = 0, worst_div = 0, worst_dot = 0;
  for (int i = 0; i < 100000; ++i) {
    const double x = std::ldexp(U(rng), X(rng)), y = std::ldexp(U(rng), X(rng));
    if (x == 0.0 || y == 0.0) continue;
    const dw a = dw_from_double(x), b = dw_from_double(y);
    worst_rt = std::fmax(worst_rt, std::fabs(dw_to_double(a) - x) / std::fabs(x));
    CHECK(std::fabs(a.l) <= std::ldexp(std::fabs((double)a.h), -24), "dw_from_double not normalised %a", x);
    const dw p = dw_mul(a, b), q = dw_div(a, b);
    worst_mul = std::fmax(worst_mul, (double)(std::fabs(val(p) - (R)x * (R)y) / std::fabs((R)x * (R)y)));
    worst_div = std::fmax(worst_div, (double)(std::fabs(val(q) - (R)x / (R)y) / std::fabs((R)x / (R)y)));
  }
  CHECK(worst_rt <= u48, "dw round trip error %.3e", worst_rt);
  CHECK(worst_mul <= 4 * u48, "dw_mul error %.3e", worst_mul);
  CHECK(worst_div <= 8 * u48, "dw_div error %.3e", worst_div);
  // compensated dot products of 8 .. 64 terms with cancellation: error
  // relative to sum |a_i b_i|
  for (int n : {8, 27, 64})
    for (int rep = 0; rep < 2000; ++rep) {
      dw_acc acc;
      R exact = 0, mag = 0;
      for (int j = 0; j < n; ++j) {
        const double x = U(rng) * 3.0, y = std::ldexp(U(rng), X(rng) / 6);
        const dw a = dw_from_double(x), b = dw_from_double(y);
        dw_fma(acc, a, b);
        exact += val(a) * val(b);
        mag += std::fabs(val(a) * val(b));
      }
      const dw r = dw_value(acc);
      worst_dot = std::fmax(worst_dot, (double)(std::fabs(val(r) - exact) / mag));
    }
  CHECK(worst_dot <= 16 * u48, "compensated dot error %.3e", worst_dot);
  std::printf("round trip %.2e  mul %.2e  div %.2e  dot %.2e  (2^-48 = %.2e)\n", worst_rt, worst_mul, worst_div,
              worst_dot, u48);
  return fails ? 1 : 0;
}
