// dword.cuh -- double-word arithmetic: a value held as an unevaluated sum of
// two FP32 numbers h + l (|l| <= ulp(h) / 2 once normalised), computed on
// the FP32 pipe.
//
// GB300 executes FP64 at about 1/75 of its FP32 rate (measured: 1.05 against
// 78 TFLOP/s), so FP64-accurate work that is compute bound runs faster as
// error-free transformations of FP32 operations:
//   * TwoSum (Knuth, TAOCP vol. 2, 4.2.2): s + e = a + b exactly, 6 adds;
//   * TwoProduct with a fused multiply-add (the FMA form of Dekker's 1971
//     product): p + e = a * b exactly, 2 operations;
//   * compensated dot products (Ogita, Rump and Oishi, "Accurate sum and dot
//     product", SIAM J. Sci. Comput. 26, 2005, algorithm Dot2), extended to
//     double-word inputs by the two cross products a.h b.l + a.l b.h (the
//     dropped a.l b.l is below 2^-48 |a b|): the result is as accurate as if
//     computed in twice the FP32 precision and rounded, error about
//     n^2 2^-48 sum |a_i b_i| in the worst case, ~2^-48 in practice.
// Double-word values carry 48 significant bits against FP64's 53; the FP32
// exponent range bounds them (|x| < 3.4e38; parts below 1.2e-38 lose
// precision gradually), which every stiffness and geometry value here
// respects by many orders of magnitude.
//
// Every operation is an explicit round-to-nearest intrinsic on the device so
// the compiler cannot contract or reorder the transformations; host builds
// (the tests' emulation) compile with -ffp-contract=off.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef __CUDACC__
#define DW_FN __host__ __device__ __forceinline__
#else
#define DW_FN inline
#endif

struct alignas(8) dw {
  float h, l;
};

namespace dwop {

DW_FN float add(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fadd_rn(a, b);
#else
  return a + b;
#endif
}
DW_FN float sub(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fsub_rn(a, b);
#else
  return a - b;
#endif
}
DW_FN float mul(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fmul_rn(a, b);
#else
  return a * b;
#endif
}
DW_FN float fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
DW_FN float div(float a, float b) {
#ifdef __CUDA_ARCH__
  return __fdiv_rn(a, b);
#else
  return a / b;
#endif
}

// s + e = a + b exactly
DW_FN void two_sum(float a, float b, float& s, float& e) {
  s = add(a, b);
  const float bb = sub(s, a);
  e = add(sub(a, sub(s, bb)), sub(b, bb));
}

// s + e = a + b exactly, provided |a| >= |b| or a == 0
DW_FN void fast_two_sum(float a, float b, float& s, float& e) {
  s = add(a, b);
  e = sub(b, sub(s, a));
}

// p + e = a * b exactly (barring underflow)
DW_FN void two_prod(float a, float b, float& p, float& e) {
  p = mul(a, b);
  e = fma(a, b, -p);
}

}  // namespace dwop

DW_FN dw dw_neg(dw a) { return dw{-a.h, -a.l}; }

// An FP32 number as the FP64 number of the same value, by re-encoding its
// bits with integer operations only (no conversion instruction, which runs on
// the FP64 pipe; a branch to one for the rare classes is if-converted by the
// compiler and then executes on every call): normal numbers rebase the
// exponent by 1023 - 127 and shift the significand into place, subnormals are
// normalised from the position of their top bit, zero keeps its sign, and
// inf / NaN keep the payload.
DW_FN double f32_to_f64_exact(float f) {
  uint32_t u;
#ifdef __CUDA_ARCH__
  u = __float_as_uint(f);
#else
  std::memcpy(&u, &f, 4);
#endif
  const uint32_t sign = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  uint32_t hi = sign | ((e + (1023u - 127u)) << 20) | (m >> 3), lo = m << 29;  // normal
  if (e == 0xffu) hi = sign | 0x7ff00000u | (m >> 3);                          // inf, NaN
  if (e == 0) {
    if (m == 0) {  // zero
      hi = sign;
      lo = 0;
    } else {       // subnormal: m 2^-149 with its top bit at p
#ifdef __CUDA_ARCH__
      const int p = 31 - __clz((int)m);
#else
      int p = 31;
      while (!((m >> p) & 1u)) --p;
#endif
      const uint64_t frac = ((uint64_t)m << (52 - p)) & 0xfffffffffffffull;
      hi = sign | ((uint32_t)(p + 874) << 20) | (uint32_t)(frac >> 32);
      lo = (uint32_t)frac;
    }
  }
#ifdef __CUDA_ARCH__
  return __hiloint2double((int)hi, (int)lo);
#else
  const uint64_t bits = ((uint64_t)hi << 32) | lo;
  double d;
  std::memcpy(&d, &bits, 8);
  return d;
#endif
}

// FP64 -> double word: h = fl32(x), l = fl32(x - h); x - h is exact in FP64.
DW_FN dw dw_from_double(double x) {
  const float h = (float)x;
  return dw{h, (float)(x - f32_to_f64_exact(h))};
}

// Double word -> FP64: one FP64 add of two exactly re-encoded parts.
DW_FN double dw_to_double(dw a) { return f32_to_f64_exact(a.h) + f32_to_f64_exact(a.l); }

// a * b for double words (Dekker's product with the cross terms), normalised
DW_FN dw dw_mul(dw a, dw b) {
  float p, e;
  dwop::two_prod(a.h, b.h, p, e);
  e = dwop::fma(a.l, b.h, dwop::fma(a.h, b.l, e));
  dw r;
  dwop::fast_two_sum(p, e, r.h, r.l);
  return r;
}

// a / b for double words: FP32 quotient, one correction from the remainder
DW_FN dw dw_div(dw a, dw b) {
  const float q1 = dwop::div(a.h, b.h);
  float p, e;
  dwop::two_prod(q1, b.h, p, e);
  // a - q1 b = (a.h - p) - e + a.l - q1 b.l; a.h - p is exact (Sterbenz)
  float r = dwop::sub(a.h, p);
  r = dwop::sub(r, e);
  r = dwop::add(r, a.l);
  r = dwop::fma(-q1, b.l, r);
  const float q2 = dwop::div(r, b.h);
  dw q;
  dwop::fast_two_sum(q1, q2, q.h, q.l);
  return q;
}

// Compensated accumulator (Dot2): running FP32 sum s, every rounding error
// and low-order part collected in c.
struct dw_acc {
  float s = 0.f, c = 0.f;
};

// acc += a * b
DW_FN void dw_fma(dw_acc& acc, dw a, dw b) {
  float p, e, s, t;
  dwop::two_prod(a.h, b.h, p, e);
  e = dwop::fma(a.l, b.h, dwop::fma(a.h, b.l, e));
  dwop::two_sum(acc.s, p, s, t);
  acc.s = s;
  acc.c = dwop::add(acc.c, dwop::add(t, e));
}

// acc += a
DW_FN void dw_add(dw_acc& acc, dw a) {
  float s, t;
  dwop::two_sum(acc.s, a.h, s, t);
  acc.s = s;
  acc.c = dwop::add(acc.c, dwop::add(t, a.l));
}

// a += b for two accumulators (the same result whichever is a: the exact
// rounding error of the sum is unique and the addition of the c parts commutes)
DW_FN void dw_acc_add(dw_acc& a, const dw_acc& b) {
  float s, t;
  dwop::two_sum(a.s, b.s, s, t);
  a.s = s;
  a.c = dwop::add(dwop::add(a.c, b.c), t);
}

DW_FN dw dw_value(const dw_acc& acc) {
  dw r;
  dwop::two_sum(acc.s, acc.c, r.h, r.l);
  return r;
}

#ifdef __CUDACC__
// Device helpers on the bits of FP64 numbers (integer operations, no FP64
// instruction).

// 2^e as an FP64 number, e in [-1022, 1023]
__device__ __forceinline__ double pow2(int e) {
  return __longlong_as_double((long long)(1023 + e) << 52);
}

// x 2^-k as a double word from the bits of x with integer operations only:
// h = its leading 24 significant bits, l = the next 24 (both truncated, so
// |x 2^-k - h - l| < 2^-47 |x 2^-k|); zero keeps its sign.  Subnormal,
// non-finite and out-of-range values (|x 2^-k| outside [2^-74, 2^127)) go
// through the FP64 conversion.
// the rare classes of dw_split_scaled, out of line so that the FP64
// instructions of this path are not executed speculatively on the common one
static __device__ __noinline__ dw dw_split_scaled_slow(double x, int k) { return dw_from_double(x * pow2(-k)); }

__device__ __forceinline__ dw dw_split_scaled(double x, int k) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  if ((b << 1) == 0) return dw{__uint_as_float((unsigned)(b >> 32)), 0.f};  // +-0
  const int e = (int)((b >> 52) & 0x7ff) - k;  // biased exponent of x 2^-k
  if ((unsigned)(e - 949) > (unsigned)(1150 - 949) || ((b >> 52) & 0x7ff) == 0 || ((b >> 52) & 0x7ff) == 0x7ff)
    return dw_split_scaled_slow(x, k);
  const unsigned sign = (unsigned)(b >> 32) & 0x80000000u;
  const unsigned long long m = b & 0xfffffffffffffull;
  const float h = __uint_as_float(sign | ((unsigned)(e - 896) << 23) | (unsigned)(m >> 29));
  const unsigned r = (unsigned)(m & 0x1fffffffu);  // value r 2^(e - 1075)
  float l = 0.f;
  if (r) {
    const int p = 31 - __clz(r);                   // top bit of r, 0..28
    const unsigned frac = p >= 23 ? (r >> (p - 23)) & 0x7fffffu : (r << (23 - p)) & 0x7fffffu;
    l = __uint_as_float(sign | ((unsigned)(p + e - 948) << 23) | frac);
  }
  return dw{h, l};
}

// a 2^k for a double word, |k| <= 100 (exact: a power-of-two product of each part)
__device__ __forceinline__ dw dw_scale(dw a, int k) {
  const float s = __uint_as_float((unsigned)(127 + k) << 23);
  return dw{__fmul_rn(a.h, s), __fmul_rn(a.l, s)};
}

// FP64 finiteness and positivity from the bits (no FP64 instruction)
__device__ __forceinline__ bool finite_bits(double x) {
  return ((__double_as_longlong(x) >> 52) & 0x7ff) != 0x7ff;
}
#endif  // __CUDACC__
