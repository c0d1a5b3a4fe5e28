// grx_df.cuh -- double-float ("float-float") arithmetic on the FP32 pipe.
//
// A value is an unevaluated sum hi + lo of two floats (about 48 significant bits).
// The error-free transformations are the classical ones: TwoSum (Knuth, TAOCP
// vol. 2, 4.2.2), FastTwoSum (Dekker 1971) and TwoProduct via fused multiply-add
// (the fma residual a*b - fl(a*b) is exact). Products and sums follow the
// double-double algorithms of Hida, Li and Bailey (QD library, 2001), restated
// here for float pairs. On GB300 one FP64 instruction issues at 1/64 of the FP32
// rate, so these 7-11 FP32 instructions per operation are several times cheaper
// than FP64 while keeping ~1e-14 relative accuracy.
#pragma once

namespace grx {

struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_from(double x) {
  const float h = __double2float_rn(x);
  return {h, __double2float_rn(x - (double)h)};
}

__device__ __forceinline__ double df_to(df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = __fadd_rn(a, b);
  const float e = __fsub_rn(b, __fsub_rn(s, a));
  return {s, e};
}

__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

// a + b with the error bound relative to |a| + |b| (no cancellation guarantee)
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo));
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_add_f(df a, float b) {
  df s = two_sum(a.hi, b);
  s.lo = __fadd_rn(s.lo, a.lo);
  return fast_two_sum(s.hi, s.lo);
}

__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  p.lo = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
  return fast_two_sum(p.hi, p.lo);
}

__device__ __forceinline__ df df_mul_f(df a, float b) {
  df p = two_prod(a.hi, b);
  p.lo = __fmaf_rn(a.lo, b, p.lo);
  return fast_two_sum(p.hi, p.lo);
}

// x^2 + y^2 + z^2 for x = xh + xl etc., where xh carries few significant bits and
// |xl| is tiny: exact squares of the hi parts via TwoProduct, cross terms in FP32.
__device__ __forceinline__ df df_norm2_split(float3 h, float3 l) {
  df sx = two_prod(h.x, h.x), sy = two_prod(h.y, h.y), sz = two_prod(h.z, h.z);
  const float cross = __fmaf_rn(2.0f * h.x, l.x, __fmaf_rn(2.0f * h.y, l.y, __fmul_rn(2.0f * h.z, l.z)));
  const float small = __fmaf_rn(l.x, l.x, __fmaf_rn(l.y, l.y, __fmul_rn(l.z, l.z)));
  df s = two_sum(sx.hi, sy.hi);
  df t = two_sum(s.hi, sz.hi);
  const float lo = __fadd_rn(__fadd_rn(__fadd_rn(s.lo, t.lo), __fadd_rn(sx.lo, __fadd_rn(sy.lo, sz.lo))),
                             __fadd_rn(cross, small));
  return fast_two_sum(t.hi, lo);
}

// a < b for double-float values (b normalised)
__device__ __forceinline__ bool df_lt(df a, df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }

// 1 / a to double-float accuracy (one Newton step on the FP32 reciprocal)
__device__ __forceinline__ df df_recip(df a) {
  const float r = __frcp_rn(a.hi);
  // e = 1 - a*r computed in double-float, then r + r*e
  df ar = df_mul_f(a, r);
  const float e = __fsub_rn(__fsub_rn(1.0f, ar.hi), ar.lo);
  return fast_two_sum(r, __fmul_rn(r, e));
}

}  // namespace grx
