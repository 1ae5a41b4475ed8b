// sed_dfloat.cuh -- double-float arithmetic on the FP32 pipe.
#pragma once

#include "sed_internal.cuh"

namespace sed {

// ------------------------------------------------------- double-float arithmetic
// GB300 executes FP64 at 1/64 of its FP32 rate, so the solvers do their
// FP64-class arithmetic in double-float numbers on the FP32 pipe: a value is
// the unevaluated sum hi + lo of two floats (48-bit significand, unit
// roundoff 2^-48 ~ 3.6e-15), and products and sums go through the error-free
// transformations TwoProd (via FMA) and TwoSum (Knuth 1969; Dekker 1971;
// Ogita, Rump & Oishi 2005).  The FP64 batched kernel keeps its Lanczos
// vectors in double-float (a complex element is a float4: re_hi, im_hi,
// re_lo, im_lo); the mixed-precision paths keep complex64 vectors and use
// these helpers where a stored value must come out of an accurate sum
// (restart rotations, hi + lo coefficients, norms, reductions, the
// Rayleigh-Ritz check).  The rounding intrinsics keep the compiler from
// contracting the operations the transformations depend on.
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
// (h, l) += x (zh + zl) for a float x: TwoProd of the leading product, the
// rest folded into the low word (restart rotations of complex64 vectors)
__device__ __forceinline__ void df_mac1(float& h, float& l, float x, float zh, float zl) {
  const float p = __fmul_rn(x, zh);
  const float pe = __fmaf_rn(x, zl, __fmaf_rn(x, zh, -p));
  float sh, e;
  df_two_sum(h, p, sh, e);
  h = sh;
  l = __fadd_rn(l, __fadd_rn(e, pe));
}
// x -= c v for one complex64 element, the FP64 coefficient c given as
// (re_hi, im_hi, re_lo, im_lo): the hi parts first, then the lo parts, so a
// large coefficient cancels without losing its low bits
__device__ __forceinline__ void cf_sub(float& xr, float& xi, float4 c, float2 v) {
  xr = __fmaf_rn(-c.x, v.x, xr);
  xr = __fmaf_rn(c.y, v.y, xr);
  xi = __fmaf_rn(-c.x, v.y, xi);
  xi = __fmaf_rn(-c.y, v.x, xi);
  xr = __fmaf_rn(-c.z, v.x, xr);
  xr = __fmaf_rn(c.w, v.y, xr);
  xi = __fmaf_rn(-c.z, v.y, xi);
  xi = __fmaf_rn(-c.w, v.x, xi);
}
__device__ __forceinline__ double df_to_d(float h, float l) { return (double)h + (double)l; }
__device__ __forceinline__ void d_to_df(double v, float& h, float& l) {
  h = (float)v;
  l = (float)(v - (double)h);
}

}  // namespace sed
