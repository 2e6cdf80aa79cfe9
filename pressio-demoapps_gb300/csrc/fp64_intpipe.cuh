// Correctly rounded FP64 division and square root on the integer pipe.
//
// GB300 executes one FP64 warp instruction per ~64 cycles per SM
// sub-partition, while its integer and FP32 pipes accept a warp instruction
// every cycle or two.  An IEEE double division costs about nine FP64
// instructions (a reciprocal seed refined by Newton steps in FP64 plus the
// rounding correction), so the FP64-bound face kernels spend about half of
// their FP64 pipe time in divisions.  Here the quotient is computed exactly
// in 64-bit integer arithmetic instead:
//
//   * a, b normal: a / b = (MA / MB) * 2^(ea - eb) with 53-bit integer
//     mantissas MA, MB.  With d = MB * 2^11 (top bit set) and
//     U = MA * 2^63 (MA >= MB) or MA * 2^64 (MA < MB), the 53-bit quotient
//     mantissa is Q = floor(U / d) and the remainder R = U - Q d.
//   * Q is estimated with a 64-bit fixed-point reciprocal 2^64 + v of d
//     (v ~ 2^128 / d - 2^64): seeded by the FP32 reciprocal of d's top 24
//     bits and refined by two Newton-Raphson steps X' = X + X (2^128 - X d)
//     / 2^128 in integer arithmetic, the method of division by invariant
//     integers (T. Granlund, P. Montgomery, PLDI 1994; N. Moller,
//     T. Granlund, IEEE Trans. Computers 60(2), 2011).
//   * the remainder of the estimate is formed exactly in 128 bits and the
//     estimate corrected until 0 <= R < d, so Q is exact whatever the
//     accuracy of the reciprocal; rounding to nearest, ties to even, then
//     compares R with d - R (the schoolbook rule: the quotient is exact, so
//     no rounding-error analysis is involved).
//
// Results are therefore the IEEE round-to-nearest quotients, bit for bit.
// Operands outside the fast path (zero, subnormal, infinite or NaN divisor,
// subnormal, infinite or NaN dividend, a quotient outside the normal range)
// take the ordinary division, which gives the IEEE result for them too.
//
// A divisor used with several dividends is prepared once (den_prep) and each
// quotient then costs one 64x64 high product, one 128-bit product and a few
// integer operations (quot).
//
// The same file holds the integer forms of the correctly rounded products by
// constants (small integers, powers of two, literals such as 1/6) and of the
// density guard r + 1e-30; they are described beside their code.
//
// The square root follows the same pattern: for normal x > 0 with 53-bit
// mantissa MX and unbiased exponent E, N = MX * 2^(52 + (E & 1)) lies in
// [2^104, 2^106) and sqrt(x) = sqrt(N) * 2^(floor(E / 2) - 52).  The integer
// square root Q = floor(sqrt(N)) is estimated from a 64-bit fixed-point
// inverse square root (FP32 seed, two Newton-Raphson steps
// r' = r (3 - m r^2) / 2), then made exact with the remainder N - Q^2
// (0 <= N - Q^2 <= 2Q); sqrt(N) is never a rounding midpoint (N is an
// integer), so it rounds up exactly when N - Q^2 > Q.
#pragma once

#include <stdint.h>

namespace pda {

// several quotients by one divisor (the divisor's reciprocal formed once)
struct Quot2 {
  double q0, q1;
};
struct Quot3 {
  double q0, q1, q2;
};
struct Quot4 {
  double q0, q1, q2, q3;
};

namespace ip {

#if defined(__CUDACC__)

__device__ __forceinline__ float rcp_seed_f32(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// 2^64 + v approximates 2^128 / d for d in [2^63, 2^64), within a few units
// of the last place (the exact correction of each quotient absorbs the
// remaining error).
__device__ __forceinline__ uint64_t recip_v(uint64_t d) {
  const uint32_t frac = (uint32_t)(d >> 40) & 0x7FFFFFu;  // 23 bits below d's leading one
  const uint32_t rb = __float_as_uint(rcp_seed_f32(__uint_as_float(0x3F800000u | frac)));
  // r in (1/2, 1]: 2^65 r = 2^64 + (r's 23 fraction bits << 41); r = 1 only for d = 2^63
  uint64_t v = rb >= 0x3F800000u ? ~0ull : (uint64_t)(rb & 0x7FFFFFu) << 41;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    // E = 2^128 - (2^64 + v) d, a small signed 128-bit number; eh = floor(E / 2^64)
    const uint64_t plo = v * d;
    const uint64_t phi = d + __umul64hi(v, d);
    const int64_t eh = (int64_t)(~phi + (plo == 0 ? 1ull : 0ull));
    const uint64_t ae = eh < 0 ? (uint64_t)(-eh) : (uint64_t)eh;
    const uint64_t c = ae + __umul64hi(v, ae);  // (2^64 + v) |eh| / 2^64
    if (eh < 0) {
      v = c > v ? 0ull : v - c;
    } else {
      const uint64_t nv = v + c;
      v = nv < v ? ~0ull : nv;
    }
  }
  return v;
}

// a prepared divisor
struct Den {
  double b;
  uint64_t d;     // (b's 53-bit mantissa) << 11
  uint64_t v;     // 2^64 + v ~ 2^128 / d
  uint64_t sign;  // b's sign bit
  int e;          // b's biased exponent
  bool ok;        // b normal (finite, nonzero, not subnormal)
};

__device__ __forceinline__ Den den_prep(double b) {
  Den D;
  const uint64_t ub = (uint64_t)__double_as_longlong(b);
  D.b = b;
  D.e = (int)((ub >> 52) & 0x7FF);
  D.ok = D.e != 0 && D.e != 0x7FF;
  D.sign = ub & 0x8000000000000000ull;
  D.d = ((ub & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull) << 11;
  D.v = recip_v(D.d);
  return D;
}

// RN(a / b) for a prepared divisor
__device__ __forceinline__ double quot(double a, const Den &D) {
  const uint64_t ua = (uint64_t)__double_as_longlong(a);
  const int ea = (int)((ua >> 52) & 0x7FF);
  const uint64_t sign = (ua & 0x8000000000000000ull) ^ D.sign;
  const uint64_t fa = ua & 0x000FFFFFFFFFFFFFull;
  if (ea == 0 && fa == 0 && D.ok) return __longlong_as_double((long long)sign);  // +-0 / normal
  const uint64_t ma = fa | 0x0010000000000000ull;
  const bool ge = (ma << 11) >= D.d;
  const int er = ea - D.e + 1022 + (ge ? 1 : 0);
  if (!D.ok || ea == 0 || ea == 0x7FF || er < 1 || er > 2045) return a / D.b;
  const uint64_t u1 = ge ? ma >> 1 : ma;
  const uint64_t u0 = ge ? ma << 63 : 0ull;
  // estimate: the exact quotient minus 0, 1 or 2 (rarely plus one)
  uint64_t q = u1 + __umul64hi(u1, D.v);
  // exact remainder R = U - q d in 128 bits (rhi:rlo, two's complement)
  const uint64_t plo = q * D.d;
  const uint64_t phi = __umul64hi(q, D.d);
  uint64_t rlo = u0 - plo;
  uint64_t rhi = u1 - phi - (u0 < plo ? 1ull : 0ull);
  if ((int64_t)rhi < 0) {
    q -= 1;
    const uint64_t t = rlo + D.d;
    rhi += t < rlo ? 1ull : 0ull;
    rlo = t;
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    if (rhi != 0 || rlo >= D.d) {
      q += 1;
      rhi -= rlo < D.d ? 1ull : 0ull;
      rlo -= D.d;
    }
  }
  if (rhi != 0 || rlo >= D.d) return a / D.b;  // estimate out of range: not expected
  // round to nearest, ties to even: compare R with d - R
  const uint64_t rest = D.d - rlo;
  q += (rlo > rest || (rlo == rest && (q & 1ull))) ? 1ull : 0ull;
  uint64_t e = (uint64_t)er;
  if (q >> 53) {  // rounded up to 2^53
    q >>= 1;
    e += 1;
  }
  return __longlong_as_double((long long)(sign | (e << 52) | (q & 0x000FFFFFFFFFFFFFull)));
}

__device__ __forceinline__ double div(double a, double b) { return quot(a, den_prep(b)); }
__device__ __forceinline__ Quot2 div2(double a0, double a1, double b) {
  const Den D = den_prep(b);
  return {quot(a0, D), quot(a1, D)};
}
__device__ __forceinline__ Quot3 div3(double a0, double a1, double a2, double b) {
  const Den D = den_prep(b);
  return {quot(a0, D), quot(a1, D), quot(a2, D)};
}
__device__ __forceinline__ Quot4 div4(double a0, double a1, double a2, double a3, double b) {
  const Den D = den_prep(b);
  return {quot(a0, D), quot(a1, D), quot(a2, D), quot(a3, D)};
}

__device__ __forceinline__ float rsqrt_seed_f32(float x) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

// RN(sqrt(x))
__device__ __forceinline__ double sqrt(double x) {
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((ux >> 52) & 0x7FF);
  if ((ux << 1) == 0) return x;  // +-0
  if (ex == 0 || ex == 0x7FF || (ux >> 63)) return ::sqrt(x);
  const uint64_t mx = (ux & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;
  const int E = ex - 1023;
  const bool odd = (E & 1) != 0;
  // N = mx * 2^(52 + odd) = n1:n0
  const uint64_t n1 = odd ? mx >> 11 : mx >> 12;
  const uint64_t n0 = odd ? mx << 53 : mx << 52;
  const uint64_t m64 = (n1 << 22) | (n0 >> 42);  // m = N / 2^104 in [1, 4), as m * 2^62
  // FP32 seed of 1/sqrt(m) from m's top 24 bits t = m * 2^22 in [2^22, 2^24)
  const uint32_t t = (uint32_t)(m64 >> 40);
  const uint32_t lead = t >> 23;
  const uint32_t fb = ((127u + lead) << 23) | ((lead ? t : t << 1) & 0x7FFFFFu);
  const uint32_t rb = __float_as_uint(rsqrt_seed_f32(__uint_as_float(fb)));
  // r in (1/2, 1]: R = r * 2^64 (r = 1 only for m = 1)
  uint64_t R = rb >= 0x3F800000u ? ~0ull : (uint64_t)((rb & 0x7FFFFFu) | 0x800000u) << 40;
#pragma unroll
  for (int it = 0; it < 2; ++it) {
    const uint64_t mr2 = __umul64hi(m64, __umul64hi(R, R));  // m r^2 * 2^62
    R = __umul64hi(R, 3ull * (1ull << 62) - mr2) << 1;     // r (3 - m r^2) / 2
  }
  uint64_t q = __umul64hi(m64, R) >> 10;  // sqrt(N) = m r 2^52, off by a unit or two
  const uint64_t plo = q * q, phi = __umul64hi(q, q);
  uint64_t rlo = n0 - plo;
  uint64_t rhi = n1 - phi - (n0 < plo ? 1ull : 0ull);
  if ((int64_t)rhi < 0) {  // (q - 1)^2 = q^2 - (2q - 1)
    const uint64_t add = 2 * q - 1;
    q -= 1;
    const uint64_t s = rlo + add;
    rhi += s < rlo ? 1ull : 0ull;
    rlo = s;
  }
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const uint64_t s = 2 * q + 1;  // (q + 1)^2 = q^2 + 2q + 1
    if (rhi != 0 || rlo >= s) {
      q += 1;
      rhi -= rlo < s ? 1ull : 0ull;
      rlo -= s;
    }
  }
  if (rhi != 0 || rlo > 2 * q) return ::sqrt(x);  // estimate out of range: not expected
  q += rlo > q ? 1ull : 0ull;
  uint64_t e = (uint64_t)((E >> 1) + 1023);
  if (q >> 53) {
    q >>= 1;
    e += 1;
  }
  return __longlong_as_double((long long)((e << 52) | (q & 0x000FFFFFFFFFFFFFull)));
}

// Out-of-line forms for kernels where code size and compile time matter more
// than the last cycles (row tables, Jacobians, reduced-order model): a call
// costs a few integer and move instructions, which do not touch the FP64 pipe.
static __device__ __noinline__ double div_call(double a, double b) { return div(a, b); }
static __device__ __noinline__ double sqrt_call(double x) { return sqrt(x); }
// Several quotients by one divisor, out of line: one division call per
// quotient.  A call that returns one double keeps its result in registers;
// sharing the reciprocal through a call that returns two or more quotients
// (or stores them) measured slower in the face kernels, and so did forming
// the reciprocal out of line with the quotients in place (more code).
__device__ __forceinline__ Quot2 div2_call(double a0, double a1, double b) { return {div_call(a0, b), div_call(a1, b)}; }
__device__ __forceinline__ Quot3 div3_call(double a0, double a1, double a2, double b) {
  return {div_call(a0, b), div_call(a1, b), div_call(a2, b)};
}
__device__ __forceinline__ Quot4 div4_call(double a0, double a1, double a2, double a3, double b) {
  return {div_call(a0, b), div_call(a1, b), div_call(a2, b), div_call(a3, b)};
}

// ---------------------------------------------------------------------------
// Exact-by-construction products and sums on the integer pipe.
//
// The WENO and Rusanov expressions multiply by small integers (3, 5, 7, 11),
// by 1/2 and 1/4, by constants (1/6, 13/12, 2e-6), and add 1e-30 to a
// density.  Each of these has an IEEE round-to-nearest result that integer
// arithmetic forms from the bit pattern at a fraction of an FP64
// instruction's cost on GB300, so they leave the FP64 pipe to the products
// and sums of two variables:
//   * RN(K x), K a small integer: the 53-bit mantissa times K fits 57 bits;
//     it is shifted back to 53 bits with round to nearest, ties to even
//     (adding half a unit minus one, plus the kept part's last bit, before
//     the shift), and a carry into bit 53 moves into the exponent field by
//     adding the mantissa (implicit bit included) to the exponent minus one;
//   * x * 2^-S is exact while the result stays normal: S is subtracted from
//     the exponent field;
//   * RN(r + 1e-30) = r whenever 1e-30 is below half a unit in the last place
//     of r: for |r| >= 2^-44 the nearest neighbour of r lies at least 2^-97
//     (about 6.3e-30) away on either side.
// Operands outside these fast paths (zeros aside: zero, subnormal, huge,
// infinite or NaN) take the ordinary FP64 operation out of line, so every
// result is the IEEE one bit for bit.
static __device__ __noinline__ double mul_call(double a, double b) { return a * b; }
static __device__ __noinline__ double add_call(double a, double b) { return a + b; }

// RN(K x) for an integer constant 2 < K < 16 that is not a power of two
template <int K>
__device__ __forceinline__ double mul_small(double x) {
  static_assert(K > 2 && K < 16 && (K & (K - 1)) != 0, "K: a small integer that is not a power of two");
  constexpr int KB = K >= 8 ? 3 : (K >= 4 ? 2 : 1);  // floor(log2 K)
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  const uint32_t ex = (uint32_t)(ux >> 52) & 0x7FFu;
  // fast path: normal x with K x (rounded) below 2^1023 * 2: ex in [1, 0x7F9]
  if (ex - 1u >= 0x7F9u) {
    if ((ux << 1) == 0) return x;  // K * (+-0) = +-0
    return mul_call(x, (double)K);
  }
  // P = m K in [2^(52+KB), 2^(54+KB)); s = KB or KB + 1 puts P >> s in [2^52, 2^53)
  const uint64_t P = ((ux & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull) * (uint64_t)K;
  const int s = (P >> (53 + KB)) != 0 ? KB + 1 : KB;
  const uint64_t q = (P + ((1ull << (s - 1)) - 1ull) + ((P >> s) & 1ull)) >> s;  // in [2^52, 2^53]
  return __longlong_as_double(
      (long long)((ux & 0x8000000000000000ull) + ((uint64_t)(ex + (uint32_t)s - 1u) << 52) + q));
}

// RN(x c) for a positive normal constant c (a literal: its mantissa and
// exponent fold at compile time).  With 53-bit mantissas MX, MC, the product
// P = MX MC lies in [2^104, 2^106); a = MX 2^11 and b = MC 2^11 give
// hi = floor(a b / 2^64) = floor(P / 2^42) exactly, the low word a b mod 2^64
// is zero exactly when P mod 2^42 is, so the 53 kept bits, the bits below
// them and the sticky bit are all known: round to nearest, ties to even.
__device__ __forceinline__ double mul_const(double x, const double c) {
  const uint64_t uc = (uint64_t)__double_as_longlong(c);
  const int ec = (int)((uc >> 52) & 0x7FF);
  const uint64_t b = ((uc & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull) << 11;
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  const int ex = (int)((ux >> 52) & 0x7FF);
  const int er = ex + ec - 1023;  // biased exponent of the result when P < 2^105
  // fast path: x normal and the result normal and finite: er in [1, 0x7FC]
  if (ex == 0 || ex == 0x7FF || er < 1 || er > 0x7FC) {
    if ((ux << 1) == 0) return x;  // +-0 * c = +-0 for c > 0
    return mul_call(x, c);
  }
  const uint64_t a = ((ux & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull) << 11;
  const uint64_t hi = __umul64hi(a, b);  // in [2^62, 2^64)
  const uint64_t lo = a * b;
  const int top = (int)(hi >> 63);  // P >= 2^105
  const int sh = 10 + top;
  const uint64_t m = hi >> sh;                      // the 53 kept bits
  const uint64_t rest = hi & ((1ull << sh) - 1ull);  // the bits of hi below them
  const uint64_t half = 1ull << (sh - 1);
  const bool up = rest > half || (rest == half && (lo != 0 || (m & 1ull)));
  const uint64_t q = m + (up ? 1ull : 0ull);  // in [2^52, 2^53]
  return __longlong_as_double(
      (long long)((ux & 0x8000000000000000ull) + ((uint64_t)(er + top - 1) << 52) + q));
}

// x * 2^-S (S = 1, 2): exact for a normal result
template <int S>
__device__ __forceinline__ double mul_pow2_neg(double x) {
  static_assert(S >= 1 && S <= 8, "S");
  const uint64_t ux = (uint64_t)__double_as_longlong(x);
  const uint32_t ex = (uint32_t)(ux >> 52) & 0x7FFu;
  // fast path: ex in [S + 1, 0x7FE]
  if (ex - (uint32_t)(S + 1) >= (uint32_t)(0x7FF - (S + 1))) {
    if ((ux << 1) == 0) return x;  // +-0 * 2^-S = +-0
    return mul_call(x, 1.0 / (double)(1 << S));
  }
  return __longlong_as_double((long long)(ux - ((uint64_t)S << 52)));
}

// RN(r + 1e-30)
__device__ __forceinline__ double add_1em30(double r) {
  const uint32_t ex = (uint32_t)((uint64_t)__double_as_longlong(r) >> 52) & 0x7FFu;
  if (ex - 979u < 0x7FFu - 979u) return r;  // 2^-44 <= |r| < infinity
  return add_call(r, 1.e-30);
}

#endif  // __CUDACC__

}  // namespace ip
}  // namespace pda
