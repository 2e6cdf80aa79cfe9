// Point-wise numerics of the cell-centered finite-volume hot path, shared by
// every kernel of this library: WENO3/WENO5 face reconstruction (with and
// without the analytic gradient), the Rusanov flux for the Euler and
// shallow-water equations and its analytic Jacobians.
//
// Every expression below keeps the operand order and association of the
// reference implementation so that, compiled without FMA contraction
// (nvcc -fmad=false), each value is bit-identical to the reference's
// double-precision result.  The few places that cannot be bit-identical are
// marked "deviation" and are within the stated parity tolerance.
//
// The gradient and flux-Jacobian functions are templates on the scalar type:
// T = double is the reference's arithmetic (every literal is a T, so the
// double instantiation is the same expression tree); T = float serves the
// reduced-order model's approximate Jacobians.
//
// Reference (pressio-demoapps, include/pressiodemoapps/...):
//   impl/weno5.hpp:56-178   weno5           -> weno5_face
//   impl/weno5.hpp:180-434  weno5WithGrad   -> weno5_face_grad
//   impl/weno3.hpp:56-132   weno3           -> weno3_face
//   impl/weno3.hpp:134-246  weno3WithGrad   -> weno3_face_grad
//   impl/euler_rusanov_flux_values_function.hpp:54-208   -> euler*_flux
//   impl/euler_rusanov_flux_jacobian_function.hpp:54-406 -> euler*_flux_jac
//   impl/swe_rusanov_flux_values_function.hpp:54-97      -> swe_flux
//   impl/swe_rusanov_flux_jacobian_function.hpp:54-137   -> swe_flux_jac
#pragma once

#include <math.h>

#include "fp64_intpipe.cuh"

#if defined(__CUDACC__)
#define PDA_HD __host__ __device__ __forceinline__
#else
#define PDA_HD inline
#endif

namespace pda {

enum Scheme : int { FirstOrder = 0, Weno3 = 1, Weno5 = 2 };

// half-width of the reconstruction stencil: 1, 2, 3
template <int S> struct SchemeTraits;
template <> struct SchemeTraits<FirstOrder> { static constexpr int h = 1; };
template <> struct SchemeTraits<Weno3> { static constexpr int h = 2; };
template <> struct SchemeTraits<Weno5> { static constexpr int h = 3; };

// Division and square root of runtime operands.  Device code computes them
// on the integer pipe (fp64_intpipe.cuh): the IEEE round-to-nearest results,
// bit for bit, without occupying GB300's FP64 pipe (one warp instruction per
// ~64 cycles per SM sub-partition), which is left to the multiplications and
// additions.  INL = true expands them in place; otherwise (every kernel of
// the library) they are calls: inlined, the face kernels outgrew the
// instruction cache and ran slower.  Host code uses the operators.  Compiling with
// -DPDA_FP64_PIPE_DIVSQRT selects the FP64-pipe operations on the device too
// (the same results), for comparison.
template <bool INL = false>
PDA_HD double div_rn(double a, double b) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (INL) return ip::div(a, b);
  else return ip::div_call(a, b);
#else
  return a / b;
#endif
}
template <bool INL = false>
PDA_HD double sqrt_rn(double x) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (INL) return ip::sqrt(x);
  else return ip::sqrt_call(x);
#else
  return sqrt(x);
#endif
}
// Several quotients by one divisor: the same IEEE quotients as div_rn, with
// the divisor's reciprocal formed once on the device.
template <bool INL = false>
PDA_HD Quot2 div2_rn(double a0, double a1, double b) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (INL) return ip::div2(a0, a1, b);
  else return ip::div2_call(a0, a1, b);
#else
  return {a0 / b, a1 / b};
#endif
}
template <bool INL = false>
PDA_HD Quot3 div3_rn(double a0, double a1, double a2, double b) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (INL) return ip::div3(a0, a1, a2, b);
  else return ip::div3_call(a0, a1, a2, b);
#else
  return {a0 / b, a1 / b, a2 / b};
#endif
}
template <bool INL = false>
PDA_HD Quot4 div4_rn(double a0, double a1, double a2, double a3, double b) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (INL) return ip::div4(a0, a1, a2, a3, b);
  else return ip::div4_call(a0, a1, a2, a3, b);
#else
  return {a0 / b, a1 / b, a2 / b, a3 / b};
#endif
}
template <bool INL = false>
PDA_HD float div_rn(float a, float b) { return a / b; }
template <bool INL = false>
PDA_HD float sqrt_rn(float x) { return sqrtf(x); }

// The reference's products by small integers (K x), by 1/2 and 1/4, by
// constants, and its density guard r + 1e-30.  Device code forms the double results on the
// integer pipe (fp64_intpipe.cuh: the IEEE round-to-nearest values, bit for
// bit); host code and single precision use the operators.
template <int K, typename T>
PDA_HD T mul_k(T x) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (sizeof(T) == 8) return ip::mul_small<K>(x);
#endif
  return T(K) * x;
}
template <typename T>
PDA_HD T half_of(T x) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (sizeof(T) == 8) return ip::mul_pow2_neg<1>(x);
#endif
  return T(1. / 2.) * x;
}
template <typename T>
PDA_HD T quarter_of(T x) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  if constexpr (sizeof(T) == 8) return ip::mul_pow2_neg<2>(x);
#endif
  return T(1. / 4.) * x;
}
// RN(c x) for a positive literal constant c (1/6, 13/12, 2e-6)
PDA_HD double mul_c(double x, double c) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  return ip::mul_const(x, c);
#else
  return c * x;
#endif
}
PDA_HD double plus_es(double r) {
#if defined(__CUDA_ARCH__) && !defined(PDA_FP64_PIPE_DIVSQRT)
  return ip::add_1em30(r);
#else
  return r + 1.e-30;
#endif
}
// Selectable forms of the above: IP = true forms the exact products on the
// integer pipe (the tile kernels of the residual, where that pays); IP = false
// keeps the FP64 operations (row, Jacobian and reduced-order kernels, where
// the extra integer code measured slower).  Both give the same bits.
template <bool IP, int K, typename T>
PDA_HD T kx(T x) {
  if constexpr (IP) return mul_k<K>(x);
  else return T(K) * x;
}
template <bool IP, typename T>
PDA_HD T halfx(T x) {
  if constexpr (IP) return half_of(x);
  else return T(1. / 2.) * x;
}
template <bool IP>
PDA_HD double esx(double r) {
  if constexpr (IP) return plus_es(r);
  else return r + 1.e-30;
}


template <typename T> PDA_HD T sq(T x) { return x * x; }
// x^3 for the reference's std::pow(x, 3.) (glibc pow, correctly rounded in
// all but pathological near-midpoint cases).  Computed with Dekker's exact
// two-product: x*x = p + e and p*x = c + ce exactly, so x^3 = c + ce + e*x
// with an error of order 2^-106 before the final rounding; the result is the
// correctly rounded cube except when x^3 lies within that distance of a
// rounding midpoint.  Used only on the Jacobian path.
PDA_HD double cube(double x) {
  const double p = x * x;
  const double e = fma(x, x, -p);
  const double c = p * x;
  const double ce = fma(p, x, -c);
  return c + (ce + e * x);
}

// x / d for a constant d with its reciprocal r = RN(1/d), correctly rounded
// (Markstein's correction step, P. Markstein, IBM J. Res. Dev. 34(1), 1990:
// with r within half an ulp of 1/d and q0 = RN(x r) within one ulp of x/d, the
// remainder x - q0 d is exact in one FMA and RN(q0 + r (x - q0 d)) is the
// correctly rounded quotient).  Three FP64 instructions instead of a full
// division; equal to the division for results in the normal range.
PDA_HD double div_const(double x, double d, double r) {
  const double q0 = x * r;
  const double e = fma(-q0, d, x);
  return fma(e, r, q0);
}

// Single precision, for the approximate (inexact Gauss-Newton) Jacobians of
// the reduced-order model: no exact-rounding constructions are needed there.
PDA_HD float cube(float x) { return x * x * x; }
PDA_HD float div_const(float x, float, float r) { return x * r; }

// k x + c rounded once, for k a power of two.  k x is then exact (for
// |x| >= 2^-1020, far below any state or gradient value here), so the result
// equals RN(RN(k x) + c), the separately rounded product and sum of the
// reference's source, in one FP64 instruction instead of two.
template <typename T>
PDA_HD T fma_p2(T k, T x, T c) { return fma(k, x, c); }

// x + k w for a tabulated constant k: a zero k makes the product exact (a
// signed zero, or NaN for an infinite or NaN w, exactly as RN(k w)), so one
// rounding; otherwise the two separate roundings of the source
template <typename T>
PDA_HD T add_table_prod(T x, T k, T w) { return k == T(0.) ? fma(k, w, x) : x + k * w; }

// The reference's WENO5 stencil expressions (impl/weno5.hpp), evaluated left
// to right as in its source, with the power-of-two products fused:
//   w5_curv(a, m, c)   = a - 2 m + c
//   w5_slopeL(a, m, c) = a - 4 m + 3 c
//   w5_slopeR(a, m, c) = 3 a - 4 m + c
//   w5_pFarL(a, b, c)  = 2 a - 7 b + 11 c     (6 x a candidate polynomial)
//   w5_pMidL(a, b, c)  = -a + 5 b + 2 c
//   w5_pMidR(a, b, c)  = 2 a + 5 b - c
//   w5_pFarR(a, b, c)  = 11 a - 7 b + 2 c
template <bool IP = false, typename T>
PDA_HD T w5_curv(T a, T m, T c) { return fma_p2(-T(2.), m, a) + c; }
template <bool IP = false, typename T>
PDA_HD T w5_slopeL(T a, T m, T c) { return fma_p2(-T(4.), m, a) + kx<IP, 3>(c); }
template <bool IP = false, typename T>
PDA_HD T w5_slopeR(T a, T m, T c) { return fma_p2(-T(4.), m, kx<IP, 3>(a)) + c; }
template <bool IP = false, typename T>
PDA_HD T w5_pFarL(T a, T b, T c) { return fma_p2(T(2.), a, -kx<IP, 7>(b)) + kx<IP, 11>(c); }
template <bool IP = false, typename T>
PDA_HD T w5_pMidL(T a, T b, T c) { return fma_p2(T(2.), c, -a + kx<IP, 5>(b)); }
template <bool IP = false, typename T>
PDA_HD T w5_pMidR(T a, T b, T c) { return fma_p2(T(2.), a, kx<IP, 5>(b)) - c; }
template <bool IP = false, typename T>
PDA_HD T w5_pFarR(T a, T b, T c) { return fma_p2(T(2.), c, kx<IP, 11>(a) - kx<IP, 7>(b)); }

// ---------------------------------------------------------------------------
// WENO5, one face i+1/2: uNeg from q_{i-2..i+2}, uPos from q_{i-1..i+3}.
// ---------------------------------------------------------------------------
// one side of weno5_face: uNeg (left-biased, q_{i-2..i+2})
PDA_HD double weno5_neg(double qim2, double qim1, double qi, double qip1, double qip2) {
  constexpr double epsilon = 1e-6;
  constexpr double two = 2., three = 3., four = 4., five = 5., seven = 7.,
                   eleven = 11.;
  constexpr double oneOvfour = 1. / 4., oneOvsix = 1. / 6.,
                   oneOvten = 1. / 10., threeOvten = 3. / 10.,
                   sixOvten = 6. / 10., thirteenOvtwelve = 13. / 12.;
  double uNeg;
  {
    const double p0 = w5_pFarL(qim2, qim1, qi) * oneOvsix;
    const double p1 = w5_pMidL(qim1, qi, qip1) * oneOvsix;
    const double p2 = w5_pMidR(qi, qip1, qip2) * oneOvsix;
    const double X0 = w5_curv(qim2, qim1, qi), Y0 = w5_slopeL(qim2, qim1, qi);
    const double X1 = w5_curv(qim1, qi, qip1), Y1 = qim1 - qip1;
    const double X2 = w5_curv(qi, qip1, qip2), Y2 = w5_slopeR(qi, qip1, qip2);
    const double B0 = thirteenOvtwelve * X0 * X0 + oneOvfour * Y0 * Y0;
    const double B1 = thirteenOvtwelve * X1 * X1 + oneOvfour * Y1 * Y1;
    const double B2 = thirteenOvtwelve * X2 * X2 + oneOvfour * Y2 * Y2;
    const double alpha0 = div_rn(oneOvten, (epsilon * epsilon + 2. * epsilon * B0 + B0 * B0));
    const double alpha1 = div_rn(sixOvten, (epsilon * epsilon + 2. * epsilon * B1 + B1 * B1));
    const double alpha2 = div_rn(threeOvten, (epsilon * epsilon + 2. * epsilon * B2 + B2 * B2));
    const double alphaSInv = div_rn(1., (alpha0 + alpha1 + alpha2));
    const double w0 = alpha0 * alphaSInv;
    const double w1 = alpha1 * alphaSInv;
    const double w2 = alpha2 * alphaSInv;
    uNeg = w0 * p0 + w1 * p1 + w2 * p2;
  }
  return uNeg;
}

// one side of weno5_face: uPos (right-biased, q_{i-1..i+3})
PDA_HD double weno5_pos(double qim1, double qi, double qip1, double qip2, double qip3) {
  constexpr double epsilon = 1e-6;
  constexpr double two = 2., three = 3., four = 4., five = 5., seven = 7.,
                   eleven = 11.;
  constexpr double oneOvfour = 1. / 4., oneOvsix = 1. / 6.,
                   oneOvten = 1. / 10., threeOvten = 3. / 10.,
                   sixOvten = 6. / 10., thirteenOvtwelve = 13. / 12.;
  double uPos;
  {
    const double p0 = w5_pMidL(qim1, qi, qip1) * oneOvsix;
    const double p1 = w5_pMidR(qi, qip1, qip2) * oneOvsix;
    const double p2 = w5_pFarR(qip1, qip2, qip3) * oneOvsix;
    const double X0 = w5_curv(qim1, qi, qip1), Y0 = w5_slopeL(qim1, qi, qip1);
    const double X1 = w5_curv(qi, qip1, qip2), Y1 = qi - qip2;
    const double X2 = w5_curv(qip1, qip2, qip3), Y2 = w5_slopeR(qip1, qip2, qip3);
    const double B0 = thirteenOvtwelve * X0 * X0 + oneOvfour * Y0 * Y0;
    const double B1 = thirteenOvtwelve * X1 * X1 + oneOvfour * Y1 * Y1;
    const double B2 = thirteenOvtwelve * X2 * X2 + oneOvfour * Y2 * Y2;
    const double alpha0 = div_rn(threeOvten, (epsilon * epsilon + 2. * epsilon * B0 + B0 * B0));
    const double alpha1 = div_rn(sixOvten, (epsilon * epsilon + 2. * epsilon * B1 + B1 * B1));
    const double alpha2 = div_rn(oneOvten, (epsilon * epsilon + 2. * epsilon * B2 + B2 * B2));
    const double alphaSInv = div_rn(1., (alpha0 + alpha1 + alpha2));
    const double w0 = alpha0 * alphaSInv;
    const double w1 = alpha1 * alphaSInv;
    const double w2 = alpha2 * alphaSInv;
    uPos = w0 * p0 + w1 * p1 + w2 * p2;
  }
  return uPos;
}

PDA_HD void weno5_face(double &uNeg, double &uPos, double qim2, double qim1,
                       double qi, double qip1, double qip2, double qip3) {
  uNeg = weno5_neg(qim2, qim1, qi, qip1, qip2);
  uPos = weno5_pos(qim1, qi, qip1, qip2, qip3);
}

// WENO5 with the gradient of the two face values with respect to the six
// stencil values q_{i-2..i+3}: gNeg[5] == 0, gPos[0] == 0.
// one side of weno5_face_grad: uNeg and its gradient
template <typename T>
PDA_HD void weno5_neg_grad(T &uNeg, T gNeg[6], T qim2, T qim1, T qi, T qip1, T qip2, T qip3) {
  constexpr T epsilon = T(1e-6);
  constexpr T two = T(2.), three = T(3.), four = T(4.), five = T(5.), seven = T(7.),
                   eleven = T(11.);
  constexpr T oneOvfour = T(1.) / T(4.), oneOvsix = T(1.) / T(6.),
                   oneOvten = T(1.) / T(10.), threeOvten = T(3.) / T(10.),
                   sixOvten = T(6.) / T(10.), thirteenOvtwelve = T(13.) / T(12.);
  {
    const T p0 = w5_pFarL(qim2, qim1, qi) * oneOvsix;
    const T p1 = w5_pMidL(qim1, qi, qip1) * oneOvsix;
    const T p2 = w5_pMidR(qi, qip1, qip2) * oneOvsix;
    const T dp0[5] = {T(1.) / T(3.), -T(7.) / T(6.), T(11.) / T(6.), T(0.), T(0.)};
    const T dp1[5] = {T(0.), -T(1.) / T(6.), T(5.) / T(6.), T(1.) / T(3.), T(0.)};
    const T dp2[5] = {T(0.), T(0.), T(1.) / T(3.), T(5.) / T(6.), -T(1.) / T(6.)};
    const T B0 = thirteenOvtwelve * sq(w5_curv(qim2, qim1, qi)) +
                      oneOvfour * sq(w5_slopeL(qim2, qim1, qi));
    const T B1 = thirteenOvtwelve * sq(w5_curv(qim1, qi, qip1)) +
                      oneOvfour * sq(qim1 - qip1);
    const T B2 = thirteenOvtwelve * sq(w5_curv(qi, qip1, qip2)) +
                      oneOvfour * sq(w5_slopeR(qi, qip1, qip2));
    // derivative terms (impl/weno5.hpp:294-310), the products by 2 and 1/2 fused
    const T X0 = T(13.) * w5_curv(qim2, qim1, qi), Y0 = w5_slopeL(qim2, qim1, qi);
    const T X1 = T(13.) * fma_p2(-T(2.), qi, qip1 + qim1), Y1 = qim1 - qip1;
    const T X2 = T(13.) * w5_curv(qip2, qip1, qi), Y2 = w5_slopeL(qip2, qip1, qi);
    T dB0[5], dB1[5], dB2[5];
    dB0[0] = fma_p2(T(0.5), Y0, div_const(X0, T(6.), T(1.) / T(6.)));
    dB0[1] = fma_p2(-T(2.), Y0, div_const(-X0, T(3.), T(1.) / T(3.)));
    dB0[2] = fma_p2(T(0.5), T(3.) * Y0, div_const(X0, T(6.), T(1.) / T(6.)));
    dB0[3] = T(0.);
    dB0[4] = T(0.);
    dB1[0] = T(0.);
    dB1[1] = fma_p2(T(0.5), Y1, div_const(X1, T(6.), T(1.) / T(6.)));
    dB1[2] = div_const(-X1, T(3.), T(1.) / T(3.));
    dB1[3] = fma_p2(-T(0.5), Y1, div_const(X1, T(6.), T(1.) / T(6.)));
    dB1[4] = T(0.);
    dB2[0] = T(0.);
    dB2[1] = T(0.);
    dB2[2] = fma_p2(T(0.5), T(3.) * Y2, div_const(X2, T(6.), T(1.) / T(6.)));
    dB2[3] = fma_p2(-T(2.), Y2, div_const(-X2, T(3.), T(1.) / T(3.)));
    dB2[4] = fma_p2(T(0.5), Y2, div_const(X2, T(6.), T(1.) / T(6.)));
    const T alpha0 = div_rn(oneOvten, sq(epsilon + B0));
    const T alpha1 = div_rn(sixOvten, sq(epsilon + B1));
    const T alpha2 = div_rn(threeOvten, sq(epsilon + B2));
    const T alphaSInv = div_rn(T(1.), (alpha0 + alpha1 + alpha2));
    const T c0 = div_rn(-T(1.), (T(5.) * cube(B0 + epsilon)));
    const T c1 = div_rn(-T(6.), (T(5.) * cube(B1 + epsilon)));
    const T c2 = div_rn(-T(3.), (T(5.) * cube(B2 + epsilon)));
    const T cS = div_rn(-T(1.), sq(alpha2 + alpha1 + alpha0));
    const T w0 = alpha0 * alphaSInv;
    const T w1 = alpha1 * alphaSInv;
    const T w2 = alpha2 * alphaSInv;
    for (int i = 0; i < 5; i++) {
      const T da0 = c0 * dB0[i];
      const T da1 = c1 * dB1[i];
      const T da2 = c2 * dB2[i];
      const T daS = cS * (da0 + da1 + da2);
      T g = add_table_prod((da0 * alphaSInv + daS * alpha0) * p0, dp0[i], w0);
      g += add_table_prod((da1 * alphaSInv + daS * alpha1) * p1, dp1[i], w1);
      g += add_table_prod((da2 * alphaSInv + daS * alpha2) * p2, dp2[i], w2);
      gNeg[i] = g;
    }
    gNeg[5] = T(0.);
    uNeg = w0 * p0 + w1 * p1 + w2 * p2;
  }
}

// one side of weno5_face_grad: uPos and its gradient
template <typename T>
PDA_HD void weno5_pos_grad(T &uPos, T gPos[6], T qim2, T qim1, T qi, T qip1, T qip2, T qip3) {
  constexpr T epsilon = T(1e-6);
  constexpr T two = T(2.), three = T(3.), four = T(4.), five = T(5.), seven = T(7.),
                   eleven = T(11.);
  constexpr T oneOvfour = T(1.) / T(4.), oneOvsix = T(1.) / T(6.),
                   oneOvten = T(1.) / T(10.), threeOvten = T(3.) / T(10.),
                   sixOvten = T(6.) / T(10.), thirteenOvtwelve = T(13.) / T(12.);
  {
    const T p0 = w5_pMidL(qim1, qi, qip1) * oneOvsix;
    const T p1 = w5_pMidR(qi, qip1, qip2) * oneOvsix;
    const T p2 = w5_pFarR(qip1, qip2, qip3) * oneOvsix;
    const T dp0[5] = {-T(1.) / T(6.), T(5.) / T(6.), T(1.) / T(3.), T(0.), T(0.)};
    const T dp1[5] = {T(0.), T(1.) / T(3.), T(5.) / T(6.), -T(1.) / T(6.), T(0.)};
    const T dp2[5] = {T(0.), T(0.), T(11.) / T(6.), -T(7.) / T(6.), T(1.) / T(3.)};
    const T B0 = thirteenOvtwelve * sq(w5_curv(qim1, qi, qip1)) +
                      oneOvfour * sq(w5_slopeL(qim1, qi, qip1));
    const T B1 = thirteenOvtwelve * sq(w5_curv(qi, qip1, qip2)) +
                      oneOvfour * sq(qi - qip2);
    const T B2 = thirteenOvtwelve * sq(w5_curv(qip1, qip2, qip3)) +
                      oneOvfour * sq(w5_slopeR(qip1, qip2, qip3));
    // derivative terms (impl/weno5.hpp:385-401), the products by 2, 4 and 1/2 fused
    const T X0 = T(13.) * fma_p2(-T(2.), qi, qip1 + qim1), Y0 = fma_p2(-T(4.), qi, T(3.) * qip1 + qim1);
    const T X1 = T(13.) * w5_curv(qip2, qip1, qi), Y1 = qi - qip2;
    const T X2 = T(13.) * w5_curv(qip3, qip2, qip1), Y2 = w5_slopeL(qip3, qip2, qip1);
    T dB0[5], dB1[5], dB2[5];
    dB0[0] = fma_p2(T(0.5), Y0, div_const(X0, T(6.), T(1.) / T(6.)));
    dB0[1] = fma_p2(-T(2.), Y0, -div_const(X0, T(3.), T(1.) / T(3.)));
    dB0[2] = fma_p2(T(0.5), T(3.) * Y0, div_const(X0, T(6.), T(1.) / T(6.)));
    dB0[3] = T(0.);
    dB0[4] = T(0.);
    dB1[0] = T(0.);
    dB1[1] = fma_p2(T(0.5), Y1, div_const(X1, T(6.), T(1.) / T(6.)));
    dB1[2] = div_const(-X1, T(3.), T(1.) / T(3.));
    dB1[3] = fma_p2(-T(0.5), Y1, div_const(X1, T(6.), T(1.) / T(6.)));
    dB1[4] = T(0.);
    dB2[0] = T(0.);
    dB2[1] = T(0.);
    dB2[2] = fma_p2(T(0.5), T(3.) * Y2, div_const(X2, T(6.), T(1.) / T(6.)));
    dB2[3] = fma_p2(-T(2.), Y2, div_const(-X2, T(3.), T(1.) / T(3.)));
    dB2[4] = fma_p2(T(0.5), Y2, div_const(X2, T(6.), T(1.) / T(6.)));
    const T alpha0 = div_rn(threeOvten, sq(epsilon + B0));
    const T alpha1 = div_rn(sixOvten, sq(epsilon + B1));
    const T alpha2 = div_rn(oneOvten, sq(epsilon + B2));
    const T alphaSInv = div_rn(T(1.), (alpha0 + alpha1 + alpha2));
    const T c0 = div_rn(-T(3.), (T(5.) * cube(B0 + epsilon)));
    const T c1 = div_rn(-T(6.), (T(5.) * cube(B1 + epsilon)));
    const T c2 = div_rn(-T(1.), (T(5.) * cube(B2 + epsilon)));
    const T cS = div_rn(-T(1.), sq(alpha2 + alpha1 + alpha0));
    const T w0 = alpha0 * alphaSInv;
    const T w1 = alpha1 * alphaSInv;
    const T w2 = alpha2 * alphaSInv;
    for (int i = 0; i < 5; i++) {
      const T da0 = c0 * dB0[i];
      const T da1 = c1 * dB1[i];
      const T da2 = c2 * dB2[i];
      const T daS = cS * (da0 + da1 + da2);
      T g = add_table_prod((da0 * alphaSInv + daS * alpha0) * p0, dp0[i], w0);
      g += add_table_prod((da1 * alphaSInv + daS * alpha1) * p1, dp1[i], w1);
      g += add_table_prod((da2 * alphaSInv + daS * alpha2) * p2, dp2[i], w2);
      gPos[i + 1] = g;
    }
    gPos[0] = T(0.);
    uPos = w0 * p0 + w1 * p1 + w2 * p2;
  }
}

PDA_HD void weno5_face_grad(double &uNeg, double &uPos, double gNeg[6],
                            double gPos[6], double qim2, double qim1, double qi,
                            double qip1, double qip2, double qip3) {
  weno5_neg_grad(uNeg, gNeg, qim2, qim1, qi, qip1, qip2, qip3);
  weno5_pos_grad(uPos, gPos, qim2, qim1, qi, qip1, qip2, qip3);
}

// ---------------------------------------------------------------------------
// WENO3, one face i+1/2: uNeg from q_{i-1..i+1}, uPos from q_{i..i+2}.
// ---------------------------------------------------------------------------
// one side of weno3_face: uNeg (q_{i-1..i+1})
PDA_HD double weno3_neg(double qim1, double qi, double qip1) {
  constexpr double epsilon = 1.e-6;
  constexpr double two = 2., three = 3.;
  constexpr double oneOvtwo = 1. / 2., oneOvthree = 1. / 3., twoOvthree = 2. / 3.;
  double uNeg;
  {
    const double p0 = (-qim1 + three * qi) * oneOvtwo;
    const double p1 = (qi + qip1) * oneOvtwo;
    const double B0 = (qim1 - qi) * (qim1 - qi);
    const double B1 = (qi - qip1) * (qi - qip1);
    const double alpha0 = div_rn(oneOvthree, (epsilon * epsilon + two * epsilon * B0 + B0 * B0));
    const double alpha1 = div_rn(twoOvthree, (epsilon * epsilon + two * epsilon * B1 + B1 * B1));
    const double alphaSInv = div_rn(1., (alpha0 + alpha1));
    const double w0 = alpha0 * alphaSInv;
    const double w1 = alpha1 * alphaSInv;
    uNeg = w0 * p0 + w1 * p1;
  }
  return uNeg;
}

// one side of weno3_face: uPos (q_{i..i+2})
PDA_HD double weno3_pos(double qi, double qip1, double qip2) {
  constexpr double epsilon = 1.e-6;
  constexpr double two = 2., three = 3.;
  constexpr double oneOvtwo = 1. / 2., oneOvthree = 1. / 3., twoOvthree = 2. / 3.;
  double uPos;
  {
    const double p0 = (qi + qip1) * oneOvtwo;
    const double p1 = (three * qip1 - qip2) * oneOvtwo;
    const double B0 = (qi - qip1) * (qi - qip1);
    const double B1 = (qip1 - qip2) * (qip1 - qip2);
    const double alpha0 = div_rn(twoOvthree, (epsilon * epsilon + two * epsilon * B0 + B0 * B0));
    const double alpha1 = div_rn(oneOvthree, (epsilon * epsilon + two * epsilon * B1 + B1 * B1));
    const double alphaSInv = div_rn(1., (alpha0 + alpha1));
    const double w0 = alpha0 * alphaSInv;
    const double w1 = alpha1 * alphaSInv;
    uPos = w0 * p0 + w1 * p1;
  }
  return uPos;
}

PDA_HD void weno3_face(double &uNeg, double &uPos, double qim1, double qi,
                       double qip1, double qip2) {
  uNeg = weno3_neg(qim1, qi, qip1);
  uPos = weno3_pos(qi, qip1, qip2);
}

// WENO3 with gradients with respect to q_{i-1..i+2}: gNeg[3] == 0, gPos[0] == 0.
// one side of weno3_face_grad: uNeg and its gradient
template <typename T>
PDA_HD void weno3_neg_grad(T &uNeg, T gNeg[4], T qim1, T qi, T qip1, T qip2) {
  constexpr T epsilon = T(1e-6);
  constexpr T two = T(2.), three = T(3.);
  constexpr T oneOvtwo = T(1.) / T(2.), oneOvthree = T(1.) / T(3.), twoOvthree = T(2.) / T(3.);
  {
    const T p0 = (-qim1 + three * qi) * oneOvtwo;
    const T p1 = (qi + qip1) * oneOvtwo;
    const T dp0[3] = {-T(1.) / T(2.), T(3.) / T(2.), T(0.)};
    const T dp1[3] = {T(0.), T(1.) / T(2.), T(1.) / T(2.)};
    const T B0 = (qim1 - qi) * (qim1 - qi);
    const T B1 = (qi - qip1) * (qi - qip1);
    const T alpha0 = div_rn(oneOvthree, (epsilon * epsilon + two * epsilon * B0 + B0 * B0));
    const T alpha1 = div_rn(twoOvthree, (epsilon * epsilon + two * epsilon * B1 + B1 * B1));
    const T alphaSInv = div_rn(T(1.), (alpha0 + alpha1));
    const T e0 = sq(qim1 - qi) + epsilon;  // pow(pow(qim1-qi,2.)+eps, .)
    const T e1 = sq(qi - qip1) + epsilon;
    const T A = div_rn(T(2.), (T(3.) * sq(e1))) + div_rn(T(1.), (T(3.) * sq(e0)));
    T da0[3], da1[3], daS[3];
    da0[0] = div_rn(-T(4.) * (qim1 - qi), (T(3.) * cube(e0)));
    da0[1] = div_rn(T(4.) * (qim1 - qi), (T(3.) * cube(e0)));
    da0[2] = T(0.);
    da1[0] = T(0.);
    da1[1] = div_rn(-T(8.) * (qi - qip1), (T(3.) * cube(e1)));
    da1[2] = div_rn(T(8.) * (qi - qip1), (T(3.) * cube(e1)));
    daS[0] = div_rn((T(4.) * (qim1 - qi)), (T(3.) * cube(e0) * sq(A)));
    daS[1] = div_rn(-(div_rn((T(4.) * (qim1 - qi)), (T(3.) * cube(e0))) - div_rn((T(8.) * (qi - qip1)), (T(3.) * cube(e1)))), sq(A));
    daS[2] = div_rn(-(T(8.) * (qi - qip1)), (T(3.) * sq(A) * cube(e1)));
    const T w0 = alpha0 * alphaSInv;
    const T w1 = alpha1 * alphaSInv;
    for (int i = 0; i < 3; i++) {
      T g = (da0[i] * alphaSInv + daS[i] * alpha0) * p0 + dp0[i] * w0;
      g += (da1[i] * alphaSInv + daS[i] * alpha1) * p1 + dp1[i] * w1;
      gNeg[i] = g;
    }
    gNeg[3] = T(0.);
    uNeg = w0 * p0 + w1 * p1;
  }
}

// one side of weno3_face_grad: uPos and its gradient
template <typename T>
PDA_HD void weno3_pos_grad(T &uPos, T gPos[4], T qim1, T qi, T qip1, T qip2) {
  constexpr T epsilon = T(1e-6);
  constexpr T two = T(2.), three = T(3.);
  constexpr T oneOvtwo = T(1.) / T(2.), oneOvthree = T(1.) / T(3.), twoOvthree = T(2.) / T(3.);
  {
    const T p0 = (qi + qip1) * oneOvtwo;
    const T p1 = (three * qip1 - qip2) * oneOvtwo;
    const T B0 = (qi - qip1) * (qi - qip1);
    const T B1 = (qip1 - qip2) * (qip1 - qip2);
    const T alpha0 = div_rn(twoOvthree, (epsilon * epsilon + two * epsilon * B0 + B0 * B0));
    const T alpha1 = div_rn(oneOvthree, (epsilon * epsilon + two * epsilon * B1 + B1 * B1));
    const T alphaSInv = div_rn(T(1.), (alpha0 + alpha1));
    const T w0 = alpha0 * alphaSInv;
    const T w1 = alpha1 * alphaSInv;
    const T dp0[3] = {T(1.) / T(2.), 1 / T(2.), T(0.)};
    const T dp1[3] = {T(0.), T(3.) / T(2.), -T(1.) / T(2.)};
    const T e0 = sq(qi - qip1) + epsilon;
    const T e1 = sq(qip1 - qip2) + epsilon;
    const T A = div_rn(T(1.), (T(3.) * sq(e1))) + div_rn(T(2.), (T(3.) * sq(e0)));
    T da0[3], da1[3], daS[3];
    da0[0] = div_rn(-T(8.) * (qi - qip1), (T(3.) * cube(e0)));
    da0[1] = div_rn(T(8.) * (qi - qip1), (T(3.) * cube(e0)));
    da0[2] = T(0.);
    da1[0] = T(0.);
    da1[1] = div_rn(-T(4.) * (qip1 - qip2), (T(3.) * cube(e1)));
    da1[2] = div_rn(T(4.) * (qip1 - qip2), (T(3.) * cube(e1)));
    daS[0] = div_rn(T(8.) * (qi - qip1), (T(3.) * cube(e0) * sq(A)));
    daS[1] = div_rn(-(div_rn(T(8.) * (qi - qip1), (3 * cube(e0))) - div_rn(T(4.) * (qip1 - qip2), (T(3.) * cube(e1)))), sq(A));
    daS[2] = div_rn(-T(4.) * (qip1 - qip2), (T(3.) * sq(A) * cube(e1)));
    for (int i = 0; i < 3; i++) {
      T g = (da0[i] * alphaSInv + daS[i] * alpha0) * p0 + dp0[i] * w0;
      g += (da1[i] * alphaSInv + daS[i] * alpha1) * p1 + dp1[i] * w1;
      gPos[i + 1] = g;
    }
    gPos[0] = T(0.);
    uPos = w0 * p0 + w1 * p1;
  }
}

PDA_HD void weno3_face_grad(double &uNeg, double &uPos, double gNeg[4],
                            double gPos[4], double qim1, double qi, double qip1,
                            double qip2) {
  weno3_neg_grad(uNeg, gNeg, qim1, qi, qip1, qip2);
  weno3_pos_grad(uPos, gPos, qim1, qi, qip1, qip2);
}

// ---------------------------------------------------------------------------
// Rusanov flux for the Euler equations.  The 2D/3D versions are specialised on
// the face normal (axis-aligned unit vectors); products with 0 and 1 are
// elided, which changes no value other than the sign of an exact zero.
// ---------------------------------------------------------------------------
template <bool INL = false, bool IP = false>
PDA_HD void euler3_flux(double F[3], const double qL[3], const double qR[3],
                        double gamma) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double rL = qL[0];
  const double uL = div_rn<INL>(qL[1], esx<IP>(rL));
  const double pL = (gamma - 1) * (qL[2] - halfx<IP>(rL) * (uL * uL));
  const Quot2 hl = div2_rn<INL>((qL[2] + pL), qR[0], rL);  // HL and rR / rL
  const double HL = hl.q0;
  const double FL0 = rL * uL, FL1 = rL * uL * uL + pL, FL2 = rL * uL * HL;
  const double rR = qR[0];
  const double uR = div_rn<INL>(qR[1], esx<IP>(rR));
  const double pR = (gamma - 1) * (qR[2] - halfx<IP>(rR) * (uR * uR));
  const double HR = div_rn<INL>((qR[2] + pR), rR);
  const double FR0 = rR * uR, FR1 = rR * uR * uR + pR, FR2 = rR * uR * HR;
  const double RT = sqrt_rn<INL>(hl.q1);
  const Quot2 roe = div2_rn<INL>((uL + RT * uR), (HL + RT * HR), (1. + RT));
  const double u = roe.q0, H = roe.q1;
  const double a = sqrt_rn<INL>((gamma - 1.) * (H - halfx<IP>(u * u)));
  const double smax = fabs(u) + a;
  F[0] = halfx<IP>(FL0 + FR0 + smax * (qL[0] - qR[0]));
  F[1] = halfx<IP>(FL1 + FR1 + smax * (qL[1] - qR[1]));
  F[2] = halfx<IP>(FL2 + FR2 + smax * (qL[2] - qR[2]));
}

template <int AXIS, bool INL = false, bool IP = false>
PDA_HD void euler4_flux(double F[4], const double qL[4], const double qR[4],
                        double gamma) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double rL = qL[0];
  const Quot2 vl = div2_rn<INL>(qL[1], qL[2], esx<IP>(rL));
  const double uL = vl.q0, vL = vl.q1;
  const double unL = AXIS == 0 ? uL : vL;
  const double pL = (gamma - 1) * (qL[3] - halfx<IP>(rL) * (uL * uL + vL * vL));
  const Quot2 hl = div2_rn<INL>((qL[3] + pL), qR[0], rL);  // HL and rR / rL
  const double HL = hl.q0;
  double FL[4];
  FL[0] = rL * unL;
  FL[1] = AXIS == 0 ? rL * unL * uL + pL : rL * unL * uL;
  FL[2] = AXIS == 1 ? rL * unL * vL + pL : rL * unL * vL;
  FL[3] = rL * unL * HL;
  const double rR = qR[0];
  const Quot2 vr = div2_rn<INL>(qR[1], qR[2], esx<IP>(rR));
  const double uR = vr.q0, vR = vr.q1;
  const double unR = AXIS == 0 ? uR : vR;
  const double pR = (gamma - 1) * (qR[3] - halfx<IP>(rR) * (uR * uR + vR * vR));
  const double HR = div_rn<INL>((qR[3] + pR), rR);
  double FR[4];
  FR[0] = rR * unR;
  FR[1] = AXIS == 0 ? rR * unR * uR + pR : rR * unR * uR;
  FR[2] = AXIS == 1 ? rR * unR * vR + pR : rR * unR * vR;
  FR[3] = rR * unR * HR;
  const double RT = sqrt_rn<INL>(hl.q1);
  const Quot3 roe = div3_rn<INL>((uL + RT * uR), (vL + RT * vR), (HL + RT * HR), (1. + RT));
  const double u = roe.q0, v = roe.q1, H = roe.q2;
  const double a = sqrt_rn<INL>((gamma - 1.) * (H - halfx<IP>(u * u + v * v)));
  const double smax = sqrt_rn<INL>(u * u + v * v) + a;
#pragma unroll
  for (int d = 0; d < 4; ++d) F[d] = halfx<IP>(FL[d] + FR[d] + smax * (qL[d] - qR[d]));
}

template <int AXIS, bool INL = false, bool IP = false>
PDA_HD void euler5_flux(double F[5], const double qL[5], const double qR[5],
                        double gamma) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double rL = qL[0];
  const Quot3 vl = div3_rn<INL>(qL[1], qL[2], qL[3], esx<IP>(rL));
  const double uL = vl.q0, vL = vl.q1, wL = vl.q2;
  const double unL = AXIS == 0 ? uL : (AXIS == 1 ? vL : wL);
  const double pL = (gamma - 1) * (qL[4] - halfx<IP>(rL) * (uL * uL + vL * vL + wL * wL));
  const Quot2 hl = div2_rn<INL>((qL[4] + pL), qR[0], rL);  // HL and rR / rL
  const double HL = hl.q0;
  double FL[5];
  FL[0] = rL * unL;
  FL[1] = AXIS == 0 ? rL * unL * uL + pL : rL * unL * uL;
  FL[2] = AXIS == 1 ? rL * unL * vL + pL : rL * unL * vL;
  FL[3] = AXIS == 2 ? rL * unL * wL + pL : rL * unL * wL;
  FL[4] = rL * unL * HL;
  const double rR = qR[0];
  const Quot3 vr = div3_rn<INL>(qR[1], qR[2], qR[3], esx<IP>(rR));
  const double uR = vr.q0, vR = vr.q1, wR = vr.q2;
  const double unR = AXIS == 0 ? uR : (AXIS == 1 ? vR : wR);
  const double pR = (gamma - 1) * (qR[4] - halfx<IP>(rR) * (uR * uR + vR * vR + wR * wR));
  const double HR = div_rn<INL>((qR[4] + pR), rR);
  double FR[5];
  FR[0] = rR * unR;
  FR[1] = AXIS == 0 ? rR * unR * uR + pR : rR * unR * uR;
  FR[2] = AXIS == 1 ? rR * unR * vR + pR : rR * unR * vR;
  FR[3] = AXIS == 2 ? rR * unR * wR + pR : rR * unR * wR;
  FR[4] = rR * unR * HR;
  const double RT = sqrt_rn<INL>(hl.q1);
  const Quot4 roe = div4_rn<INL>((uL + RT * uR), (vL + RT * vR), (wL + RT * wR), (HL + RT * HR), (1. + RT));
  const double u = roe.q0, v = roe.q1, w = roe.q2, H = roe.q3;
  const double a = sqrt_rn<INL>((gamma - 1.) * (H - halfx<IP>(u * u + v * v + w * w)));
  const double smax = sqrt_rn<INL>(u * u + v * v + w * w) + a;
#pragma unroll
  for (int d = 0; d < 5; ++d) F[d] = halfx<IP>(FL[d] + FR[d] + smax * (qL[d] - qR[d]));
}

// Shallow-water Rusanov flux.  deviation: the reference's std::pow(h, 0.5) is
// evaluated as sqrt(h) (correctly rounded; glibc pow agrees except in rare
// near-midpoint cases, a 1-ulp difference).
template <int AXIS, bool INL = false, bool IP = false>
PDA_HD void swe_flux(double F[3], const double qL[3], const double qR[3],
                     double gravity) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double hL = qL[0];
  const Quot2 vl = div2_rn<INL>(qL[1], qL[2], esx<IP>(hL));
  const double uL = vl.q0, vL = vl.q1;
  const double unL = AXIS == 0 ? uL : vL;
  const double pL = halfx<IP>(gravity) * hL * hL;
  double FL[3];
  FL[0] = hL * unL;
  FL[1] = AXIS == 0 ? hL * unL * uL + pL : hL * unL * uL;
  FL[2] = AXIS == 1 ? hL * unL * vL + pL : hL * unL * vL;
  const double hR = qR[0];
  const Quot2 vr = div2_rn<INL>(qR[1], qR[2], esx<IP>(hR));
  const double uR = vr.q0, vR = vr.q1;
  const double unR = AXIS == 0 ? uR : vR;
  const double pR = halfx<IP>(gravity) * hR * hR;
  double FR[3];
  FR[0] = hR * unR;
  FR[1] = AXIS == 0 ? hR * unR * uR + pR : hR * unR * uR;
  FR[2] = AXIS == 1 ? hR * unR * vR + pR : hR * unR * vR;
  const double hm = halfx<IP>(hL + hR);
  const double sL = sqrt_rn<INL>(hL), sR = sqrt_rn<INL>(hR);
  const double um = div_rn<INL>((unL * sL + unR * sR), esx<IP>(sL + sR));
  const double sg = sqrt_rn<INL>(gravity * hm);
  const double smax = sqrt_rn<INL>(um * um) + sqrt_rn<INL>(sg * sg);
#pragma unroll
  for (int d = 0; d < 3; ++d) F[d] = halfx<IP>(FL[d] + FR[d] + smax * (qL[d] - qR[d]));
}

// ---------------------------------------------------------------------------
// The Rusanov fluxes above in two halves: flux_side (the quantities of one
// face state: its velocities, enthalpy or sqrt(h), and physical flux) and
// flux_combine (the Roe / wave-speed average and the Rusanov sum).  The side
// takes the face normal as a runtime axis (*_side_ax; the templated form
// passes its constant), so threads of one warp that hold faces of different
// axes run one instruction stream; the combination does not depend on the
// axis at all.
// combine(side(qL), side(qR)) evaluates every expression of the *_flux
// function above unchanged, so it is bit-identical; the halves let a kernel
// compute the two states of a face on different warps.
// ---------------------------------------------------------------------------
template <int N> struct FluxSide {
  double F[N];  // the state's physical flux along the axis
  double u, v, w, H;  // Euler: velocities and total enthalpy; shallow water: u = normal velocity, H = sqrt(h)
};

PDA_HD void euler3_side(FluxSide<3> &o, const double q[3], double gamma) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double r = q[0];
  const double u = div_rn(q[1], (r + es));
  const double p = (gamma - 1) * (q[2] - half * r * (u * u));
  const double H = div_rn((q[2] + p), r);
  o.F[0] = r * u;
  o.F[1] = r * u * u + p;
  o.F[2] = r * u * H;
  o.u = u;
  o.H = H;
}
PDA_HD void euler3_combine(double F[3], const double qL[3], const double qR[3], const FluxSide<3> &L,
                           const FluxSide<3> &R, double gamma) {
  constexpr double half = 1. / 2.;
  const double RT = sqrt_rn(div_rn(qR[0], (qL[0])));
  const double u = div_rn((L.u + RT * R.u), (1. + RT));
  const double H = div_rn((L.H + RT * R.H), (1. + RT));
  const double a = sqrt_rn((gamma - 1.) * (H - half * (u * u)));
  const double smax = fabs(u) + a;
#pragma unroll
  for (int d = 0; d < 3; ++d) F[d] = half * (L.F[d] + R.F[d] + smax * (qL[d] - qR[d]));
}

PDA_HD void euler4_side_ax(FluxSide<4> &o, const double q[4], double gamma, int ax) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double r = q[0];
  const double u = div_rn(q[1], (r + es));
  const double v = div_rn(q[2], (r + es));
  const double un = ax == 0 ? u : v;
  const double p = (gamma - 1) * (q[3] - half * r * (u * u + v * v));
  const double H = div_rn((q[3] + p), r);
  o.F[0] = r * un;
  o.F[1] = ax == 0 ? r * un * u + p : r * un * u;
  o.F[2] = ax == 1 ? r * un * v + p : r * un * v;
  o.F[3] = r * un * H;
  o.u = u;
  o.v = v;
  o.H = H;
}
template <int AXIS>
PDA_HD void euler4_side(FluxSide<4> &o, const double q[4], double gamma) {
  euler4_side_ax(o, q, gamma, AXIS);
}
template <int AXIS>
PDA_HD void euler4_combine(double F[4], const double qL[4], const double qR[4], const FluxSide<4> &L,
                           const FluxSide<4> &R, double gamma) {
  constexpr double half = 1. / 2.;
  const double RT = sqrt_rn(div_rn(qR[0], (qL[0])));
  const double u = div_rn((L.u + RT * R.u), (1. + RT));
  const double v = div_rn((L.v + RT * R.v), (1. + RT));
  const double H = div_rn((L.H + RT * R.H), (1. + RT));
  const double a = sqrt_rn((gamma - 1.) * (H - half * (u * u + v * v)));
  const double smax = sqrt_rn(u * u + v * v) + a;
#pragma unroll
  for (int d = 0; d < 4; ++d) F[d] = half * (L.F[d] + R.F[d] + smax * (qL[d] - qR[d]));
}

PDA_HD void euler5_side_ax(FluxSide<5> &o, const double q[5], double gamma, int ax) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double r = q[0];
  const double u = div_rn(q[1], (r + es));
  const double v = div_rn(q[2], (r + es));
  const double w = div_rn(q[3], (r + es));
  const double un = ax == 0 ? u : (ax == 1 ? v : w);
  const double p = (gamma - 1) * (q[4] - half * r * (u * u + v * v + w * w));
  const double H = div_rn((q[4] + p), r);
  o.F[0] = r * un;
  o.F[1] = ax == 0 ? r * un * u + p : r * un * u;
  o.F[2] = ax == 1 ? r * un * v + p : r * un * v;
  o.F[3] = ax == 2 ? r * un * w + p : r * un * w;
  o.F[4] = r * un * H;
  o.u = u;
  o.v = v;
  o.w = w;
  o.H = H;
}
template <int AXIS>
PDA_HD void euler5_side(FluxSide<5> &o, const double q[5], double gamma) {
  euler5_side_ax(o, q, gamma, AXIS);
}
template <int AXIS>
PDA_HD void euler5_combine(double F[5], const double qL[5], const double qR[5], const FluxSide<5> &L,
                           const FluxSide<5> &R, double gamma) {
  constexpr double half = 1. / 2.;
  const double RT = sqrt_rn(div_rn(qR[0], (qL[0])));
  const double u = div_rn((L.u + RT * R.u), (1. + RT));
  const double v = div_rn((L.v + RT * R.v), (1. + RT));
  const double w = div_rn((L.w + RT * R.w), (1. + RT));
  const double H = div_rn((L.H + RT * R.H), (1. + RT));
  const double a = sqrt_rn((gamma - 1.) * (H - half * (u * u + v * v + w * w)));
  const double smax = sqrt_rn(u * u + v * v + w * w) + a;
#pragma unroll
  for (int d = 0; d < 5; ++d) F[d] = half * (L.F[d] + R.F[d] + smax * (qL[d] - qR[d]));
}

PDA_HD void swe_side_ax(FluxSide<3> &o, const double q[3], double gravity, int ax) {
  constexpr double es = 1.e-30;
  const double h = q[0];
  const double u = div_rn(q[1], (h + es));
  const double v = div_rn(q[2], (h + es));
  const double un = ax == 0 ? u : v;
  const double p = 0.5 * gravity * h * h;
  o.F[0] = h * un;
  o.F[1] = ax == 0 ? h * un * u + p : h * un * u;
  o.F[2] = ax == 1 ? h * un * v + p : h * un * v;
  o.u = un;
  o.H = sqrt_rn(h);
}
template <int AXIS>
PDA_HD void swe_side(FluxSide<3> &o, const double q[3], double gravity) {
  swe_side_ax(o, q, gravity, AXIS);
}
template <int AXIS>
PDA_HD void swe_combine(double F[3], const double qL[3], const double qR[3], const FluxSide<3> &L,
                        const FluxSide<3> &R, double gravity) {
  constexpr double half = 1. / 2.;
  constexpr double es = 1.e-30;
  const double hm = 0.5 * (qL[0] + qR[0]);
  const double um = div_rn((L.u * L.H + R.u * R.H), (L.H + R.H + es));
  const double sg = sqrt_rn(gravity * hm);
  const double smax = sqrt_rn(um * um) + sqrt_rn(sg * sg);
#pragma unroll
  for (int d = 0; d < 3; ++d) F[d] = half * (L.F[d] + R.F[d] + smax * (qL[d] - qR[d]));
}

// ---------------------------------------------------------------------------
// Analytic Rusanov flux Jacobians JL = dF/dqL, JR = dF/dqR (row-major n x n).
// These keep the reference's generic normal vector n, built from a runtime
// axis (*_flux_jac_ax; the templated form passes its constant), so threads
// of one warp that hold faces of different axes run one instruction stream.
// ---------------------------------------------------------------------------
template <typename T>
PDA_HD void euler3_flux_jac(T JL[9], T JR[9], const T qL[3],
                            const T qR[3], T gamma) {
  constexpr T one = T(1.), two = T(2.), three = T(3.), half = T(1.) / T(2.);
  constexpr T es = T(1.e-30);
  const T gm1 = gamma - one;
  const T rL = qL[0];
  const T uL = div_rn(qL[1], (rL + es));
  const T pL = gm1 * (qL[2] - half * rL * (uL * uL));
  const T HL = div_rn((qL[2] + pL), rL);
  const T aL = sqrt_rn(gm1 * (HL - half * (uL * uL)));
  const T rR = qR[0];
  const T uR = div_rn(qR[1], (rR + es));
  const T pR = gm1 * (qR[2] - half * rR * (uR * uR));
  const T HR = div_rn((qR[2] + pR), rR);
  const T aR = sqrt_rn(gm1 * (HR - half * (uR * uR)));
  const T r = sqrt_rn(rR * rL);
  const T RT = sqrt_rn(div_rn(rR, (rL)));
  const T u = div_rn((uL + RT * uR), (one + RT));
  const T H = div_rn((HL + RT * HR), (one + RT));
  const T a = sqrt_rn(gm1 * (H - half * (u * u)));
  const T smax = fabs(u) + a;
  const T VMagSqrRoe = u * u + es;
  const T VMagSqrL = uL * uL;
  const T VVRoeL = uL * u;
  const T VMagSqrR = uR * uR;
  const T VVRoeR = uR * u;
  const T uRelRoe = div_rn(u, sqrt_rn(VMagSqrRoe));
  T gL[3], gR[3];
  gL[0] = div_rn(one, (rL + r)) * (-half * (uL + u) * uRelRoe + div_rn(half * gm1, a) * (fma_p2(half, VMagSqrRoe + VVRoeL, half * (HL - H)) - div_rn(aL * aL, gm1) + half * (gamma - two) * VMagSqrL));
  gL[1] = div_rn(one, (rL + r)) * (uRelRoe - div_rn(half * (gm1 * (u + gm1 * uL)), (a)));
  gL[2] = div_rn(div_rn(half, (rL + r)) * gamma * gm1, (a));
  gR[0] = div_rn(one, (rR + r)) * (-half * (uR + u) * uRelRoe + div_rn(half * gm1, a) * (fma_p2(half, VMagSqrRoe + VVRoeR, half * (HR - H)) - div_rn(aR * aR, gm1) + half * (gamma - two) * VMagSqrR));
  gR[1] = div_rn(one, (rR + r)) * (uRelRoe - div_rn(half * (gm1 * (u + gm1 * uR)), (a)));
  gR[2] = div_rn(div_rn(half, (rR + r)) * gamma * gm1, (a));
  JL[0] = 0;
  JL[1] = half;
  JL[2] = 0;
  JL[3] = half * (half * gm1 * uL * uL - uL * uL);
  JL[4] = half * ((three - gamma) * uL);
  JL[5] = half * gm1;
  JL[6] = half * ((half * gm1 * uL * uL - HL) * uL);
  JL[7] = half * (HL - gm1 * uL * uL);
  JL[8] = half * gamma * uL;
  for (int i = 0; i < 3; i++) {
    JL[i * 3 + i] = fma_p2(half, smax, JL[i * 3 + i]);
    for (int j = 0; j < 3; j++) JL[i * 3 + j] += half * gL[j] * (qL[i] - qR[i]);
  }
  JR[0] = 0;
  JR[1] = half;
  JR[2] = 0;
  JR[3] = half * (half * gm1 * uR * uR - uR * uR);
  JR[4] = half * ((three - gamma) * uR);
  JR[5] = half * gm1;
  JR[6] = half * ((half * gm1 * uR * uR - HR) * uR);
  JR[7] = half * (HR - gm1 * uR * uR);
  JR[8] = half * gamma * uR;
  for (int i = 0; i < 3; i++) {
    JR[i * 3 + i] = fma_p2(-half, smax, JR[i * 3 + i]);
    for (int j = 0; j < 3; j++) JR[i * 3 + j] += half * gR[j] * (qL[i] - qR[i]);
  }
}

template <typename T>
PDA_HD void euler4_flux_jac_ax(T JL[16], T JR[16], const T qL[4],
                            const T qR[4], T gamma, int ax) {
  constexpr T one = T(1.), two = T(2.), half = T(1.) / T(2.);
  constexpr T es = T(1.e-30);
  const T n[2] = {ax == 0 ? T(1.) : T(0.), ax == 1 ? T(1.) : T(0.)};
  const T gm1 = gamma - one;
  const T rL = qL[0];
  const T uL = div_rn(qL[1], (rL + es));
  const T vL = div_rn(qL[2], (rL + es));
  const T unL = uL * n[0] + vL * n[1];
  const T pL = gm1 * (qL[3] - half * rL * (uL * uL + vL * vL));
  const T HL = div_rn((qL[3] + pL), rL);
  const T aL = sqrt_rn(gm1 * (HL - half * (uL * uL + vL * vL)));
  const T rR = qR[0];
  const T uR = div_rn(qR[1], (rR + es));
  const T vR = div_rn(qR[2], (rR + es));
  const T unR = uR * n[0] + vR * n[1];
  const T pR = gm1 * (qR[3] - half * rR * (uR * uR + vR * vR));
  const T HR = div_rn((qR[3] + pR), rR);
  const T aR = sqrt_rn(gm1 * (HR - half * (uR * uR + vR * vR)));
  const T r = sqrt_rn(rR * rL);
  const T RT = sqrt_rn(div_rn(rR, (rL)));
  const T u = div_rn((uL + RT * uR), (one + RT));
  const T v = div_rn((vL + RT * vR), (one + RT));
  const T H = div_rn((HL + RT * HR), (one + RT));
  const T a = sqrt_rn(gm1 * (H - half * (u * u + v * v)));
  const T smax = sqrt_rn(u * u + v * v) + a;
  const T VMagSqrRoe = u * u + v * v + es;
  const T VMagSqrL = uL * uL + vL * vL;
  const T VVRoeL = uL * u + vL * v;
  const T VMagSqrR = uR * uR + vR * vR;
  const T VVRoeR = uR * u + vR * v;
  const T uRelRoe = div_rn(u, sqrt_rn(VMagSqrRoe));
  const T vRelRoe = div_rn(v, sqrt_rn(VMagSqrRoe));
  T gL[4], gR[4];
  gL[0] = div_rn(one, (rL + r)) * (-half * (uL + u) * uRelRoe - half * (vL + v) * vRelRoe + div_rn(half * gm1, a) * (fma_p2(half, VMagSqrRoe + VVRoeL, half * (HL - H)) - div_rn(aL * aL, gm1) + half * (gamma - two) * VMagSqrL));
  gL[1] = div_rn(one, (rL + r)) * (uRelRoe - div_rn(half * (gm1 * (u + gm1 * uL)), (a)));
  gL[2] = div_rn(one, (rL + r)) * (vRelRoe - div_rn(half * (gm1 * (v + gm1 * vL)), (a)));
  gL[3] = div_rn(div_rn(half, (rL + r)) * gamma * gm1, (a));
  gR[0] = div_rn(one, (rR + r)) * (-half * (uR + u) * uRelRoe - half * (vR + v) * vRelRoe + div_rn(half * gm1, a) * (fma_p2(half, VMagSqrRoe + VVRoeR, half * (HR - H)) - div_rn(aR * aR, gm1) + half * (gamma - two) * VMagSqrR));
  gR[1] = div_rn(one, (rR + r)) * (uRelRoe - div_rn(half * (gm1 * (u + gm1 * uR)), (a)));
  gR[2] = div_rn(one, (rR + r)) * (vRelRoe - div_rn(half * (gm1 * (v + gm1 * vR)), (a)));
  gR[3] = div_rn(div_rn(half, (rR + r)) * gamma * gm1, (a));
  // left
  JL[0] = 0;
  JL[1] = half * n[0];
  JL[2] = half * n[1];
  JL[3] = 0;
  JL[4] = half * (half * gm1 * VMagSqrL * n[0] - uL * unL);
  JL[5] = half * (uL * n[0] - gm1 * uL * n[0] + unL);
  JL[6] = half * (uL * n[1] - gm1 * vL * n[0]);
  JL[7] = half * gm1 * n[0];
  JL[8] = half * (half * gm1 * VMagSqrL * n[1] - vL * unL);
  JL[9] = half * (vL * n[0] - gm1 * uL * n[1]);
  JL[10] = half * (vL * n[1] - gm1 * vL * n[1] + unL);
  JL[11] = half * gm1 * n[1];
  JL[12] = half * ((half * gm1 * VMagSqrL - HL) * unL);
  JL[13] = half * (HL * n[0] - gm1 * uL * unL);
  JL[14] = half * (HL * n[1] - gm1 * vL * unL);
  JL[15] = half * gamma * unL;
  for (int i = 0; i < 4; i++) {
    JL[i * 4 + i] = fma_p2(half, smax, JL[i * 4 + i]);
    for (int j = 0; j < 4; j++) JL[i * 4 + j] += half * gL[j] * (qL[i] - qR[i]);
  }
  // right
  JR[0] = 0;
  JR[1] = half * n[0];
  JR[2] = half * n[1];
  JR[3] = 0;
  JR[4] = half * (half * gm1 * VMagSqrR * n[0] - uR * unR);
  JR[5] = half * (uR * n[0] - gm1 * uR * n[0] + unR);
  JR[6] = half * (uR * n[1] - gm1 * vR * n[0]);
  JR[7] = half * gm1 * n[0];
  JR[8] = half * (half * gm1 * VMagSqrR * n[1] - vR * unR);
  JR[9] = half * (vR * n[0] - gm1 * uR * n[1]);
  JR[10] = half * (vR * n[1] - gm1 * vR * n[1] + unR);
  JR[11] = half * gm1 * n[1];
  JR[12] = half * ((half * gm1 * VMagSqrR - HR) * unR);
  JR[13] = half * (HR * n[0] - gm1 * uR * unR);
  JR[14] = half * (HR * n[1] - gm1 * vR * unR);
  JR[15] = half * gamma * unR;
  for (int i = 0; i < 4; i++) {
    JR[i * 4 + i] = fma_p2(-half, smax, JR[i * 4 + i]);
    for (int j = 0; j < 4; j++) JR[i * 4 + j] += half * gR[j] * (qL[i] - qR[i]);
  }
}
template <int AXIS, typename T>
PDA_HD void euler4_flux_jac(T JL[16], T JR[16], const T qL[4],
                            const T qR[4], T gamma) {
  euler4_flux_jac_ax(JL, JR, qL, qR, gamma, AXIS);
}

template <typename T>
PDA_HD void euler5_flux_jac_ax(T JL[25], T JR[25], const T qL[5],
                            const T qR[5], T gamma, int ax) {
  constexpr T one = T(1.), two = T(2.), half = T(1.) / T(2.);
  constexpr T es = T(1.e-30);
  const T n[3] = {ax == 0 ? T(1.) : T(0.), ax == 1 ? T(1.) : T(0.), ax == 2 ? T(1.) : T(0.)};
  const T gm1 = gamma - one;
  const T rL = qL[0];
  const T uL = div_rn(qL[1], (rL + es));
  const T vL = div_rn(qL[2], (rL + es));
  const T wL = div_rn(qL[3], (rL + es));
  const T unL = uL * n[0] + vL * n[1] + wL * n[2];
  const T pL = gm1 * (qL[4] - half * rL * (uL * uL + vL * vL + wL * wL));
  const T HL = div_rn((qL[4] + pL), rL);
  const T aL = sqrt_rn(gm1 * (HL - half * (uL * uL + vL * vL + wL * wL)));
  const T rR = qR[0];
  const T uR = div_rn(qR[1], (rR + es));
  const T vR = div_rn(qR[2], (rR + es));
  const T wR = div_rn(qR[3], (rR + es));
  const T unR = uR * n[0] + vR * n[1] + wR * n[2];
  const T pR = gm1 * (qR[4] - half * rR * (uR * uR + vR * vR + wR * wR));
  const T HR = div_rn((qR[4] + pR), rR);
  const T aR = sqrt_rn(gm1 * (HR - half * (uR * uR + vR * vR + wR * wR)));
  const T r = sqrt_rn(rR * rL);
  const T RT = sqrt_rn(div_rn(rR, (rL)));
  const T u = div_rn((uL + RT * uR), (one + RT));
  const T v = div_rn((vL + RT * vR), (one + RT));
  const T w = div_rn((wL + RT * wR), (one + RT));
  const T H = div_rn((HL + RT * HR), (one + RT));
  const T a = sqrt_rn(gm1 * (H - half * (u * u + v * v + w * w)));
  const T smax = sqrt_rn(u * u + v * v + w * w) + a;
  const T VMagSqrRoe = u * u + v * v + w * w + es;
  const T VMagSqrL = uL * uL + vL * vL + wL * wL;
  const T VVRoeL = uL * u + vL * v + wL * w;
  const T VMagSqrR = uR * uR + vR * vR + wR * wR;
  const T VVRoeR = uR * u + vR * v + wR * w;
  const T uRelRoe = div_rn(u, sqrt_rn(VMagSqrRoe));
  const T vRelRoe = div_rn(v, sqrt_rn(VMagSqrRoe));
  const T wRelRoe = div_rn(w, sqrt_rn(VMagSqrRoe));
  T gL[5], gR[5];
  gL[0] = div_rn(one, (rL + r)) * (-half * (uL + u) * uRelRoe - half * (vL + v) * vRelRoe - half * (wL + w) * wRelRoe + div_rn(half * gm1, a) * (fma_p2(half, VMagSqrRoe + VVRoeL, half * (HL - H)) - div_rn(aL * aL, gm1) + half * (gamma - two) * VMagSqrL));
  gL[1] = div_rn(one, (rL + r)) * (uRelRoe - div_rn(half * (gm1 * (u + gm1 * uL)), (a)));
  gL[2] = div_rn(one, (rL + r)) * (vRelRoe - div_rn(half * (gm1 * (v + gm1 * vL)), (a)));
  gL[3] = div_rn(one, (rL + r)) * (wRelRoe - div_rn(half * (gm1 * (w + gm1 * wL)), (a)));
  gL[4] = div_rn(div_rn(half, (rL + r)) * gamma * gm1, (a));
  gR[0] = div_rn(one, (rR + r)) * (-half * (uR + u) * uRelRoe - half * (vR + v) * vRelRoe - half * (wR + w) * wRelRoe + div_rn(half * gm1, a) * (fma_p2(half, VMagSqrRoe + VVRoeR, half * (HR - H)) - div_rn(aR * aR, gm1) + half * (gamma - two) * VMagSqrR));
  gR[1] = div_rn(one, (rR + r)) * (uRelRoe - div_rn(half * (gm1 * (u + gm1 * uR)), (a)));
  gR[2] = div_rn(one, (rR + r)) * (vRelRoe - div_rn(half * (gm1 * (v + gm1 * vR)), (a)));
  gR[3] = div_rn(one, (rR + r)) * (wRelRoe - div_rn(half * (gm1 * (w + gm1 * wR)), (a)));
  gR[4] = div_rn(div_rn(half, (rR + r)) * gamma * gm1, (a));
  // left and right use the same template; X = L or R
#define PDA_FILL_J5(J, uX, vX, wX, unX, HX, VMagSqrX)                 \
  J[0] = 0;                                                           \
  J[1] = half * n[0];                                                 \
  J[2] = half * n[1];                                                 \
  J[3] = half * n[2];                                                 \
  J[4] = 0;                                                           \
  J[5] = half * (half * gm1 * VMagSqrX * n[0] - uX * unX);            \
  J[6] = half * (uX * n[0] - gm1 * uX * n[0] + unX);                  \
  J[7] = half * (uX * n[1] - gm1 * vX * n[0]);                        \
  J[8] = half * (uX * n[2] - gm1 * wX * n[0]);                        \
  J[9] = half * gm1 * n[0];                                           \
  J[10] = half * (half * gm1 * VMagSqrX * n[1] - vX * unX);           \
  J[11] = half * (vX * n[0] - gm1 * uX * n[1]);                       \
  J[12] = half * (vX * n[1] - gm1 * vX * n[1] + unX);                 \
  J[13] = half * (vX * n[2] - gm1 * wX * n[1]);                       \
  J[14] = half * gm1 * n[1];                                          \
  J[15] = half * (half * gm1 * VMagSqrX * n[2] - wX * unX);           \
  J[16] = half * (wX * n[0] - gm1 * uX * n[2]);                       \
  J[17] = half * (wX * n[1] - gm1 * vX * n[2]);                       \
  J[18] = half * (wX * n[2] - gm1 * wX * n[2] + unX);                 \
  J[19] = half * gm1 * n[2];                                          \
  J[20] = half * ((half * gm1 * VMagSqrX - HX) * unX);                \
  J[21] = half * (HX * n[0] - gm1 * uX * unX);                        \
  J[22] = half * (HX * n[1] - gm1 * vX * unX);                        \
  J[23] = half * (HX * n[2] - gm1 * wX * unX);                        \
  J[24] = half * gamma * unX;
  PDA_FILL_J5(JL, uL, vL, wL, unL, HL, VMagSqrL)
  for (int i = 0; i < 5; i++) {
    JL[i * 5 + i] = fma_p2(half, smax, JL[i * 5 + i]);
    for (int j = 0; j < 5; j++) JL[i * 5 + j] += half * gL[j] * (qL[i] - qR[i]);
  }
  PDA_FILL_J5(JR, uR, vR, wR, unR, HR, VMagSqrR)
#undef PDA_FILL_J5
  for (int i = 0; i < 5; i++) {
    JR[i * 5 + i] = fma_p2(-half, smax, JR[i * 5 + i]);
    for (int j = 0; j < 5; j++) JR[i * 5 + j] += half * gR[j] * (qL[i] - qR[i]);
  }
}
template <int AXIS, typename T>
PDA_HD void euler5_flux_jac(T JL[25], T JR[25], const T qL[5],
                            const T qR[5], T gamma) {
  euler5_flux_jac_ax(JL, JR, qL, qR, gamma, AXIS);
}

// Shallow-water Rusanov flux Jacobian (generic normal).  deviation: pow(x,0.5)
// -> sqrt(x); pow(2,3/2) is the correctly rounded constant 2*sqrt(2).
template <typename T>
PDA_HD void swe_flux_jac_ax(T JL[9], T JR[9], const T qL[3],
                         const T qR[3], T g, int ax) {
  constexpr T es = T(1.e-30);
  const T n[2] = {ax == 0 ? T(1.) : T(0.), ax == 1 ? T(1.) : T(0.)};
  const T hL = qL[0];
  const T uL = div_rn(qL[1], (hL + es));
  const T vL = div_rn(qL[2], (hL + es));
  const T unL = uL * n[0] + vL * n[1];
  const T hR = qR[0];
  const T uR = div_rn(qR[1], (hR + es));
  const T vR = div_rn(qR[2], (hR + es));
  const T unR = uR * n[0] + vR * n[1];
  const T hm = T(0.5) * (hL + hR);
  const T hL_sqrt = sqrt_rn(hL);
  const T hR_sqrt = sqrt_rn(hR);
  const T um = div_rn((unL * hL_sqrt + unR * hR_sqrt), (hL_sqrt + hR_sqrt + es));
  const T smax = fabs(um) + fabs(sqrt_rn(g * hm));
  const T termL = div_rn((n[0] * qL[1] + n[1] * qL[2]), sq(qL[0]));
  const T termR = div_rn((n[0] * qR[1] + n[1] * qR[2]), sq(qR[0]));
  const T hsqrt_un = hL_sqrt * unL + hR_sqrt * unR + es;
  const T two_pow_1p5 = T(2.) * sqrt(T(2.));
  T dL[3], dR[3];
  dL[0] = div_rn(-fabs(hsqrt_un), (T(2.) * hL_sqrt * sq(hL_sqrt + hR_sqrt))) +
          div_rn((div_rn(T(0.5) * unL, hL_sqrt) - hL_sqrt * termL) * hsqrt_un, ((hL_sqrt + hR_sqrt) * fabs(hsqrt_un))) +
          div_rn(g, (two_pow_1p5 * sqrt_rn(g * (hL + hR))));
  dL[1] = div_rn(n[0] * hsqrt_un, (hL_sqrt * (hL_sqrt + hR_sqrt) * fabs(hsqrt_un)));
  dL[2] = div_rn(n[1] * hsqrt_un, (hL_sqrt * (hL_sqrt + hR_sqrt) * fabs(hsqrt_un)));
  dR[0] = div_rn(-fabs(hsqrt_un), (T(2.) * hR_sqrt * sq(hL_sqrt + hR_sqrt))) +
          div_rn((div_rn(T(0.5) * unR, hR_sqrt) - hR_sqrt * termR) * hsqrt_un, ((hL_sqrt + hR_sqrt) * fabs(hsqrt_un))) +
          div_rn(g, (two_pow_1p5 * sqrt_rn(g * (hL + hR))));
  dR[1] = div_rn(n[0] * hsqrt_un, (hR_sqrt * (hL_sqrt + hR_sqrt) * fabs(hsqrt_un)));
  dR[2] = div_rn(n[1] * hsqrt_un, (hR_sqrt * (hL_sqrt + hR_sqrt) * fabs(hsqrt_un)));
  JL[0] = -T(0.5) * dL[0] * (qR[0] - qL[0]) + T(0.5) * (n[0] * uL + n[1] * vL - qL[0] * termL) + T(0.5) * smax;
  JL[1] = T(0.5) * n[0] - T(0.5) * dL[1] * (qR[0] - qL[0]);
  JL[2] = T(0.5) * n[1] - T(0.5) * dL[2] * (qR[0] - qL[0]);
  JL[3] = T(0.5) * (g * n[0] * qL[0] - qL[1] * termL) - T(0.5) * dL[0] * (qR[1] - qL[1]);
  JL[4] = n[0] * uL + T(0.5) * n[1] * vL + T(0.5) * smax - T(0.5) * dL[1] * (qR[1] - qL[1]);
  JL[5] = T(0.5) * n[1] * uL - T(0.5) * dL[2] * (qR[1] - qL[1]);
  JL[6] = T(0.5) * (g * n[1] * qL[0] - qL[2] * termL) - T(0.5) * dL[0] * (qR[2] - qL[2]);
  JL[7] = T(0.5) * n[0] * vL - T(0.5) * dL[1] * (qR[2] - qL[2]);
  JL[8] = n[1] * vL + T(0.5) * n[0] * uL + T(0.5) * smax - T(0.5) * dL[2] * (qR[2] - qL[2]);
  JR[0] = -T(0.5) * dR[0] * (qR[0] - qL[0]) + T(0.5) * (n[0] * uR + n[1] * vR - qR[0] * termR) - T(0.5) * smax;
  JR[1] = T(0.5) * n[0] - T(0.5) * dR[1] * (qR[0] - qL[0]);
  JR[2] = T(0.5) * n[1] - T(0.5) * dR[2] * (qR[0] - qL[0]);
  JR[3] = T(0.5) * (g * n[0] * qR[0] - qR[1] * termR) - T(0.5) * dR[0] * (qR[1] - qL[1]);
  JR[4] = n[0] * uR + T(0.5) * n[1] * vR - T(0.5) * smax - T(0.5) * dR[1] * (qR[1] - qL[1]);
  JR[5] = T(0.5) * n[1] * uR - T(0.5) * dR[2] * (qR[1] - qL[1]);
  JR[6] = T(0.5) * (g * n[1] * qR[0] - qR[2] * termR) - T(0.5) * dR[0] * (qR[2] - qL[2]);
  JR[7] = T(0.5) * n[0] * vR - T(0.5) * dR[1] * (qR[2] - qL[2]);
  JR[8] = n[1] * vR + T(0.5) * n[0] * uR - T(0.5) * smax - T(0.5) * dR[2] * (qR[2] - qL[2]);
}
template <int AXIS, typename T>
PDA_HD void swe_flux_jac(T JL[9], T JR[9], const T qL[3],
                         const T qR[3], T g) {
  swe_flux_jac_ax(JL, JR, qL, qR, g, AXIS);
}

}  // namespace pda
