// Double-word ("float-float") arithmetic on the FP32 pipes.
//
// GB300 issues FP64 at about 1/60 of its FP32 rate (measured here: 1.20 vs 70
// TFLOP/s of FMA), so the FP64-accurate assembly path carries each value as an
// unevaluated sum hi + lo of two floats (|lo| <= ulp(hi)/2, ~48 significant bits,
// relative error of one operation ~2^-47) and runs on the FP32 units.
//
// Building blocks (published error-free transformations):
//   two_sum        Knuth (TAOCP vol. 2): s + e = a + b exactly, any order of |a|, |b|
//   fast_two_sum   Dekker (1971): s + e = a + b exactly when |a| >= |b|
//   two_prod       with a fused multiply-add: p + e = a * b exactly
//   add / mul / div  the double-word algorithms analysed by Joldes, Muller and
//                  Popescu, "Tight and rigorous error bounds for basic building
//                  blocks of double-word arithmetic", ACM TOMS 44(2), 2017
//                  (AccurateDWPlusDW, DWTimesDW with FMA, and a Newton-corrected
//                  DW division).
// Everything here is plain IEEE float arithmetic; the compiler must not
// re-associate it (nvcc does not without --use_fast_math, which is not used).
#pragma once

#include <cstdint>

namespace mg {

struct ff {
  float hi, lo;
};

__device__ __forceinline__ ff ff_make(float hi) { return ff{hi, 0.0f}; }

__device__ __forceinline__ ff two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return ff{s, e};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return ff{s, e};
}

__device__ __forceinline__ ff two_prod(float a, float b)
{
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  return ff{p, e};
}

// AccurateDWPlusDW (relative error <= 3u^2 + 13u^3, u = 2^-24)
__device__ __forceinline__ ff ff_add(ff a, ff b)
{
  ff s = two_sum(a.hi, b.hi);
  const ff t = two_sum(a.lo, b.lo);
  s.lo = __fadd_rn(s.lo, t.hi);
  s = fast_two_sum(s.hi, s.lo);
  s.lo = __fadd_rn(s.lo, t.lo);
  return fast_two_sum(s.hi, s.lo);
}

// SloppyDWPlusDW: two_sum of the high parts, low parts added in float.  Its
// error is bounded relative to max(|a|, |b|) (not to |a + b|), which is what a
// sum of element contributions or a cofactor needs; 11 operations instead of 20.
__device__ __forceinline__ ff ff_add_s(ff a, ff b)
{
  ff s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}

// a.b of two 3-vectors: error-free products of the high parts chained with
// two_sum, every low-order term collected in one float, one renormalisation.
// The renormalisation is fast_two_sum although the dot may cancel below its low
// part (|hi| < |lo|): the result is then still within ~2^-48 of the terms'
// magnitudes, which is the accuracy every caller needs (entries are compared
// row-scaled; a cancelling determinant is caught by det_cancels).
__device__ __forceinline__ ff ff_dot3(const ff* a, const ff* b)
{
  ff p = two_prod(a[0].hi, b[0].hi);
  float lo = __fmaf_rn(a[0].hi, b[0].lo, __fmaf_rn(a[0].lo, b[0].hi, p.lo));
  float hi = p.hi;
#pragma unroll
  for (int k = 1; k < 3; ++k) {
    const ff q = two_prod(a[k].hi, b[k].hi);
    const ff s = two_sum(hi, q.hi);
    hi = s.hi;
    lo = __fadd_rn(lo, __fadd_rn(s.lo, __fmaf_rn(a[k].hi, b[k].lo, __fmaf_rn(a[k].lo, b[k].hi, q.lo))));
  }
  return fast_two_sum(hi, lo);
}

// a * b - c * d in the same style (the cofactor pattern), absolute error
// ~2^-48 (|a b| + |c d|) also when the difference cancels (see ff_dot3).
__device__ __forceinline__ ff ff_cross(ff a, ff b, ff c, ff d)
{
  const ff p = two_prod(a.hi, b.hi), q = two_prod(-c.hi, d.hi);
  const ff s = two_sum(p.hi, q.hi);
  float lo = __fadd_rn(s.lo, __fadd_rn(p.lo, q.lo));
  lo = __fadd_rn(lo, __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, 0.0f)));
  lo = __fsub_rn(lo, __fmaf_rn(c.hi, d.lo, __fmaf_rn(c.lo, d.hi, 0.0f)));
  return fast_two_sum(s.hi, lo);
}

__device__ __forceinline__ ff ff_neg(ff a) { return ff{-a.hi, -a.lo}; }
__device__ __forceinline__ ff ff_sub(ff a, ff b) { return ff_add(a, ff_neg(b)); }

// DWTimesDW with FMA (relative error <= 5u^2)
__device__ __forceinline__ ff ff_mul(ff a, ff b)
{
  ff p = two_prod(a.hi, b.hi);
  float t = __fmul_rn(a.hi, b.lo);
  t = __fmaf_rn(a.lo, b.hi, t);
  p.lo = __fadd_rn(p.lo, t);
  return fast_two_sum(p.hi, p.lo);
}

// Division: q1 = a.hi * rcp(b.hi), remainder r = a - q1 b in double-word, one
// correction q2 = r.hi * rcp(b.hi) (a Newton step on the quotient); relative
// error ~2^-45 with the correctly rounded reciprocal.
__device__ __forceinline__ ff ff_div(ff a, ff b)
{
  const float rb = __frcp_rn(b.hi);
  const float q1 = __fmul_rn(a.hi, rb);
  const ff r = ff_sub(a, ff_mul(b, ff_make(q1)));
  const float q2 = __fmul_rn(r.hi, rb);
  return fast_two_sum(q1, q2);
}

// Exact split of a double into hi + lo floats with |lo| <= ulp(hi)/2 (to the
// rounding of lo, relative 2^-48), done with FP64 conversions: only used off the
// hot loop (one coefficient per element).
__device__ __forceinline__ ff ff_from_double(double x)
{
  const float hi = __double2float_rn(x);
  const float lo = __double2float_rn(x - (double)hi);
  return ff{hi, lo};
}

// Rare-case paths of the integer conversions below, kept out of line: inlined,
// the compiler if-converts them into the hot path, and their predicated FP64
// instructions still occupy GB300's narrow FP64 pipe (measured: ~20 FP64-pipe
// instructions per element instead of ~5 in the element kernels).
static __device__ __noinline__ ff ff_from_double_slow(double x) { return ff_from_double(x); }
static __device__ __noinline__ double f2d_slow(float f) { return (double)f; }

// The same two conversions with integer operations, for hot loops: GB300 runs
// FP32<->FP64 conversions on its FP64 pipe (~1/60 of the FP32 rate).
// float -> double by re-biasing the exponent (exact for normal floats; zero
// and subnormals map to zero, Inf/NaN fall back to the conversion).
__device__ __forceinline__ double f2d_bits(float f)
{
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  if (e == 0u) return 0.0;
  if (e == 0xffu) return f2d_slow(f);
  const uint64_t d = ((uint64_t)(u >> 31) << 63) | ((uint64_t)(e + (1023u - 127u)) << 52) |
                     ((uint64_t)(u & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}

// hi + lo as a double: both parts exact, one FP64 addition.
__device__ __forceinline__ double ff_to_double_bits(ff a) { return f2d_bits(a.hi) + f2d_bits(a.lo); }
static __device__ __noinline__ double ff_to_double_slow(ff a) { return ff_to_double_bits(a); }

// hi + lo as a double without FP64 arithmetic: after renormalisation
// (|lo| <= ulp(hi)/2), lo is expressed in units of the double ulp of the
// binade hi + lo lies in (a power-of-two scaling, exact) and rounded to an
// integer k, which is added to the bit pattern of double(hi).  That binade is
// hi's own, except when |hi| is a power of two and lo points towards zero: then
// hi + lo lies in the binade below, whose ulp is half as large (counting in
// hi's ulp there would move the result by only half of lo).  The result is
// within half a double ulp of hi + lo.  Outside the range where the scaling
// stays a normal float (|hi| below ~2^-74 or above ~2^126), and for Inf or NaN,
// it falls back to ff_to_double_bits (zero gives +0).
__device__ __forceinline__ double ff_to_double_int(ff a)
{
  const ff n = fast_two_sum(a.hi, a.lo);
  const uint32_t u = __float_as_uint(n.hi);
  const int e = (int)((u >> 23) & 0xffu) - 127;  // unbiased exponent of hi
  if (n.hi == 0.0f) return 0.0;
  if (e < -74 || e > 126) return ff_to_double_slow(n);
  // one binade down when hi = +-2^e and lo has the opposite sign
  const int down = ((u & 0x7fffffu) == 0u && n.lo != 0.0f && ((__float_as_uint(n.lo) ^ u) >> 31)) ? 1 : 0;
  const float scale = __uint_as_float((uint32_t)(52 - e + down + 127) << 23);  // 1 / ulp_double of hi + lo
  int k = __float2int_rn(__fmul_rn(n.lo, scale));                           // lo in those units
  if (u >> 31) k = -k;  // magnitudes: the bit pattern grows with |x|
  const long long bits = __double_as_longlong(f2d_bits(n.hi)) + (long long)k;
  return __longlong_as_double(bits);
}

// double -> hi + lo: hi keeps the top 24 bits of the significand (truncated,
// exact), lo the next 29 bits rounded to nearest -- |x - hi - lo| <= 2^-48 |x|.
// lo is built without an integer-to-float conversion (which GB300 issues at a
// small fraction of the FP32 rate): with mlo the low 29 significand bits, lo =
// RN(mlo 2^(e-52)) is the float sum of two exact terms, the top 23 and the low 6
// bits of mlo, each obtained as (2^k (1 + bits 2^-23)) - 2^k from a float built
// with that exponent.  For |x| in about 2^-74 .. 2^127 and x = 0; other values
// fall back to the FP64 conversions.
__device__ __forceinline__ ff ff_from_double_bits(double x)
{
  const uint64_t u = (uint64_t)__double_as_longlong(x);
  const uint32_t H = (uint32_t)(u >> 32), L = (uint32_t)u;
  const uint32_t E = (H >> 20) & 0x7ffu;  // biased exponent
  if (E == 0u && (u << 1) == 0u) return ff{0.0f, 0.0f};
  if (E < 949u || E > 1150u) return ff_from_double_slow(x);
  const uint32_t sign = H & 0x80000000u;
  // top 24 significand bits with the exponent re-biased from 1023 to 127
  const uint32_t t = __funnelshift_l(L, H, 3);
  const float hi = __uint_as_float(((t - (384u << 23)) & 0x7fffffffu) | sign);
  const uint32_t k1 = (E - 919u) << 23;  // 2^(e - 23): unit of bit 6 of mlo is 2^(e - 46)
  const uint32_t k2 = (E - 925u) << 23;  // 2^(e - 29): unit of bit 0 is 2^(e - 52)
  const float f1 = __fsub_rn(__uint_as_float(k1 | ((L >> 6) & 0x7fffffu)), __uint_as_float(k1));
  const float f2 = __fsub_rn(__uint_as_float(k2 | (L & 63u)), __uint_as_float(k2));
  const float lo = __uint_as_float(__float_as_uint(__fadd_rn(f1, f2)) ^ sign);
  return ff{hi, lo};
}

}  // namespace mg
