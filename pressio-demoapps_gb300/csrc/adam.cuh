// One Adam update (Kingma & Ba 2015, in the form with the bias corrections
// folded into the step size and the denominator), written with explicitly
// rounded operations so that the stand-alone optimizer kernels and the GEMM
// epilogue that fuses the update give the same bits whatever the compiler's
// contraction settings:
//   m = b1 m + (1 - b1) g,   v = b2 v + ((1 - b2) g) g,
//   w = w - ss (m / (sqrt(v) rs2 + eps)),
// with ss = lr / (1 - b1^t) and rs2 = 1 / sqrt(1 - b2^t) formed on the host
// once per step (adam_coef).  One square root and one division per weight.
#pragma once

#include <cmath>

namespace pda {

struct AdamCoef {
  float b1, omb1, b2, omb2;  // b1, 1 - b1, b2, 1 - b2
  float ss, rs2, eps;
};

// coefficients of step t (t >= 1) with step size lr
inline AdamCoef adam_coef(float lr, long t, float b1 = 0.9f, float b2 = 0.999f, float eps = 1e-8f) {
  const double c1 = 1.0 - std::pow((double)b1, (double)t), c2 = 1.0 - std::pow((double)b2, (double)t);
  return AdamCoef{b1, 1.f - b1, b2, 1.f - b2, (float)(lr / c1), (float)(1.0 / std::sqrt(c2)), eps};
}

#if defined(__CUDACC__)
__device__ __forceinline__ float adam_update(float w, float &m, float &v, float g, const AdamCoef &c) {
  m = __fadd_rn(__fmul_rn(c.b1, m), __fmul_rn(c.omb1, g));
  v = __fadd_rn(__fmul_rn(c.b2, v), __fmul_rn(__fmul_rn(c.omb2, g), g));
  const float denom = __fadd_rn(__fmul_rn(__fsqrt_rn(v), c.rs2), c.eps);
  return __fsub_rn(w, __fmul_rn(c.ss, __fdiv_rn(m, denom)));
}
#endif

}  // namespace pda
