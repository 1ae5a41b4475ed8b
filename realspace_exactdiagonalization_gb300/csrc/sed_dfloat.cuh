// sed_dfloat.cuh -- double-float arithmetic on the FP32 pipe.
#pragma once

#include "sed_internal.cuh"

namespace sed {

// ------------------------------------------------------- double-float vectors
// GB300 executes FP64 at 1/64 of its FP32 rate, so the mixed-precision solvers
// (batched and device-wide) keep their Lanczos vectors as double-float
// numbers: a value is the unevaluated sum
// hi + lo of two floats (48-bit significand, unit roundoff 2^-48 ~ 3.6e-15),
// and products and sums go through the error-free transformations TwoProd
// (via FMA) and TwoSum (Knuth 1969; Dekker 1971; Ogita, Rump & Oishi 2005).
// The recurrence, the reorthogonalisation and the restart rotations thus keep
// FP64-class accuracy (basis orthogonal to ~1e-14) while running on the FP32
// pipe.  A complex element is a float4 (re_hi, im_hi, re_lo, im_lo).  The
// rounding intrinsics keep the compiler from contracting the operations the
// transformations depend on.
__device__ __forceinline__ void df_two_sum(float a, float b, float& s, float& e) {
  s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}
// (h, l) += (xh + xl) (yh + yl), dropping xl yl
__device__ __forceinline__ void df_mac(float& h, float& l, float xh, float xl, float yh, float yl) {
  const float p = __fmul_rn(xh, yh);
  const float pe = __fmaf_rn(xh, yh, -p);
  float sh, e;
  df_two_sum(h, p, sh, e);
  h = sh;
  l = __fadd_rn(l, __fadd_rn(e, __fmaf_rn(xh, yl, __fmaf_rn(xl, yh, pe))));
}
// (h, l) += (h2, l2)
__device__ __forceinline__ void df_add(float& h, float& l, float h2, float l2) {
  float sh, e;
  df_two_sum(h, h2, sh, e);
  h = sh;
  l = __fadd_rn(l, __fadd_rn(l2, e));
}
__device__ __forceinline__ void df_renorm(float& h, float& l) {
  const float sh = __fadd_rn(h, l);
  l = __fsub_rn(l, __fsub_rn(sh, h));
  h = sh;
}
__device__ __forceinline__ double df_to_d(float h, float l) { return (double)h + (double)l; }
__device__ __forceinline__ void d_to_df(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

}  // namespace sed
