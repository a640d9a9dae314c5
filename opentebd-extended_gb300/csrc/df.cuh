// df.cuh -- double-float arithmetic for the precision forms (bidiag.cu, dense.cu).
#pragma once
#include <cuda_runtime.h>

namespace tebd {
namespace {

// A real number is an unevaluated sum hi + lo of two floats (48 significant
// bits); products by Dekker's method with the FMA giving the exact error of
// hi*hi, sums by Knuth's two-sum; __fadd_rn/__fmul_rn keep the compiler from
// fusing the error-free steps.  A complex element is float4 (re_hi, re_lo,
// im_hi, im_lo), the same 16 bytes as a double2.
__device__ __forceinline__ float4 dfs(double2 v) {  // double2 -> double-float
  const float rh = (float)v.x, ih = (float)v.y;
  return make_float4(rh, (float)(v.x - (double)rh), ih, (float)(v.y - (double)ih));
}
__device__ __forceinline__ double2 dfd(float4 v) {
  return make_double2((double)v.x + (double)v.y, (double)v.z + (double)v.w);
}
__device__ __forceinline__ double2 dfl(const float4 *p) { return dfd(__ldcg(p)); }

// (sh, sl) += (xh, xl) * (yh, yl)
__device__ __forceinline__ void df_mac(float &sh, float &sl, float xh, float xl, float yh, float yl) {
  const float pr = __fmul_rn(xh, yh);
  float e = fmaf(xh, yh, -pr);
  e = fmaf(xh, yl, e);
  e = fmaf(xl, yh, e);
  const float t = __fadd_rn(sh, pr);
  const float bp = __fadd_rn(t, -sh);
  const float err = __fadd_rn(__fadd_rn(sh, -__fadd_rn(t, -bp)), __fadd_rn(pr, -bp));
  sl = __fadd_rn(sl, __fadd_rn(err, e));
  sh = t;
}
// acc += conj(a) v (real and imaginary double-float accumulators)
__device__ __forceinline__ void df_cmac_ca(float &rh, float &rl, float &ih, float &il, float4 a, float4 v) {
  df_mac(rh, rl, a.x, a.y, v.x, v.y);   // + ar vr
  df_mac(rh, rl, a.z, a.w, v.z, v.w);   // + ai vi
  df_mac(ih, il, a.x, a.y, v.z, v.w);   // + ar vi
  df_mac(ih, il, -a.z, -a.w, v.x, v.y); // - ai vr
}
// acc += a v
__device__ __forceinline__ void df_cmac(float &rh, float &rl, float &ih, float &il, float4 a, float4 v) {
  df_mac(rh, rl, a.x, a.y, v.x, v.y);
  df_mac(rh, rl, -a.z, -a.w, v.z, v.w);
  df_mac(ih, il, a.x, a.y, v.z, v.w);
  df_mac(ih, il, a.z, a.w, v.x, v.y);
}
// acc -= l conj(g)
__device__ __forceinline__ void df_cmsub_cb(float4 &acc, float4 l, float4 g) {
  df_mac(acc.x, acc.y, -l.x, -l.y, g.x, g.y);  // - lr gr
  df_mac(acc.x, acc.y, -l.z, -l.w, g.z, g.w);  // - li gi
  df_mac(acc.z, acc.w, l.x, l.y, g.z, g.w);    // + lr gi
  df_mac(acc.z, acc.w, -l.z, -l.w, g.x, g.y);  // - li gr
}
__device__ __forceinline__ float4 df_norm4(float4 v) {  // renormalise hi + lo (fast two-sum)
  const float rh = __fadd_rn(v.x, v.y), ih = __fadd_rn(v.z, v.w);
  return make_float4(rh, __fadd_rn(v.y, -__fadd_rn(rh, -v.x)), ih, __fadd_rn(v.w, -__fadd_rn(ih, -v.z)));
}
}  // namespace
}  // namespace tebd
