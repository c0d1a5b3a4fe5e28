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

#include <cstdint>

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

// ------------------------------------------------------------------ elementary functions
// sqrt(a): the FP32 root r refined by one Newton step, r + (a - r^2) / (2 r), with a - r^2
// formed exactly (TwoProduct); ~1e-14 relative. a >= 0.
__device__ __forceinline__ df df_sqrt(df a) {
  if (!(a.hi > 0.0f)) return {0.0f, 0.0f};
  const float r = __fsqrt_rn(a.hi);
  const df rr = two_prod(r, r);
  const float e = __fadd_rn(__fsub_rn(__fsub_rn(a.hi, rr.hi), rr.lo), a.lo);
  return fast_two_sum(r, __fdiv_rn(e, __fmul_rn(2.0f, r)));
}

// Exact double-float of a Philox uniform w * 2^-32: the top 24 and the low 8 bits of w, then
// normalised (the low part below half an ulp of the high one; for w < 2^8 the high part is 0
// and the value moves into it, which df_sqrt and the products need).
__device__ __forceinline__ df df_u01(uint32_t w) {
  return fast_two_sum(__fmul_rn((float)(w & 0xffffff00u), 2.3283064365386963e-10f),
                      __fmul_rn((float)(w & 0xffu), 2.3283064365386963e-10f));
}

// sin(2 pi v) and cos(2 pi v) for any v of moderate size (|4 v| < 2^22), ~1e-14 absolute:
// v = q/4 + r with q = nearest integer to 4v, so x = 2 pi r lies in [-pi/4, pi/4] (r exact);
// sin x and cos x from their Taylor series in Horner form, the orders up to x^9 / x^8 in
// double-float, the smaller tail (below 3e-8 of the result) in FP32; the quadrant q mod 4
// then swaps and negates (sin(x + q pi/2), cos(x + q pi/2)).
__device__ __forceinline__ float4 df_sincos_2pi_inl(float vhi, float vlo) {
  const df v = {vhi, vlo};
  const float q = rintf(4.0f * v.hi);
  const df r = df_add_f(v, -0.25f * q);
  const df x = df_mul(r, df{6.2831855f, -1.7484555e-07f});
  const df x2 = df_mul(x, x);
  const float t = x2.hi;
  // sin x / x = 1 - x2/3! + x2^2/5! - x2^3/7! + x2^4/9! - x2^5/11! + x2^6/13! - x2^7/15!
  const float st = t * (-2.5052108e-08f + t * (1.6059044e-10f - t * 7.6471636e-13f));
  df ps = df_add_f(df{2.7557319e-06f, 3.7935712e-14f}, st);
  ps = df_add(df_mul(x2, ps), df{-0.0001984127f, 2.7255969e-12f});
  ps = df_add(df_mul(x2, ps), df{0.008333334f, -4.346172e-10f});
  ps = df_add(df_mul(x2, ps), df{-0.16666667f, 4.967054e-09f});
  ps = df_add_f(df_mul(x2, ps), 1.0f);
  const df sx = df_mul(x, ps);
  // cos x = 1 - x2/2! + x2^2/4! - x2^3/6! + x2^4/8! - x2^5/10! + x2^6/12! - x2^7/14! + x2^8/16!
  const float ct = t * (-2.755732e-07f + t * (2.0876756e-09f + t * (-1.1470745e-11f + t * 4.7794773e-14f)));
  df pc = df_add_f(df{2.4801588e-05f, -3.406996e-13f}, ct);
  pc = df_add(df_mul(x2, pc), df{-0.0013888889f, 3.3631094e-11f});
  pc = df_add(df_mul(x2, pc), df{0.041666668f, -1.2417635e-09f});
  pc = df_add_f(df_mul(x2, pc), -0.5f);
  pc = df_add_f(df_mul(x2, pc), 1.0f);
  const int quad = ((int)q) & 3;
  const df ns = {-sx.hi, -sx.lo}, nc = {-pc.hi, -pc.lo};
  const df s = quad == 0 ? sx : (quad == 1 ? pc : (quad == 2 ? ns : nc));
  const df c = quad == 0 ? pc : (quad == 1 ? ns : (quad == 2 ? nc : sx));
  return make_float4(s.hi, s.lo, c.hi, c.lo);
}

// The same out of line (one copy per kernel for the orientation, rotation and eik call
// sites: these run once per move on few lanes, where instruction fetch, not arithmetic,
// sets the time), the result returned in registers.
static __device__ __noinline__ float4 df_sincos_2pi_out(float vhi, float vlo) { return df_sincos_2pi_inl(vhi, vlo); }

__device__ __forceinline__ void df_sincos_2pi(df v, df& s, df& c) {
  const float4 r = df_sincos_2pi_out(v.hi, v.lo);
  s = df{r.x, r.y};
  c = df{r.z, r.w};
}

// e^{i 2 pi k f} for k = 0..km as double-float complex {re hi, re lo, im hi, im lo} in
// tab[k * stride]: the k = 1 factor from df_sincos_2pi, the higher ones by complex products
// (the kx / ky / kz recurrence of Initialize_Vectors_thread, Ewald_Energy_Functions.h:162-185).
__device__ __forceinline__ void df_eik_row(double f, int km, float4* tab, int stride) {
  tab[0] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  if (km < 1) return;
  df er, ei;
  df_sincos_2pi(df_from(f), ei, er);
  df r = er, i = ei;
  tab[stride] = make_float4(r.hi, r.lo, i.hi, i.lo);
#pragma unroll 1
  for (int k = 2; k <= km; ++k) {
    const df nr = df_add(df_mul(r, er), df_mul(df{-i.hi, -i.lo}, ei));
    const df ni = df_add(df_mul(r, ei), df_mul(i, er));
    r = nr;
    i = ni;
    tab[k * stride] = make_float4(r.hi, r.lo, i.hi, i.lo);
  }
}

// (x, y, z) rotated by the quaternion of Rotate_Quaternions (mc_utilities.h:423-457, uniform
// rotation from three uniforms) with the uniforms given as Philox words, in double-float on
// the FP32 pipe: the same rotation as the FP64 form to ~1e-13 relative.
__device__ __forceinline__ void df_rotate_quaternion_inl(double& x, double& y, double& z, uint32_t wu, uint32_t wv,
                                                         uint32_t ww) {
  const df u = df_u01(wu);
  df s1, c1, s2, c2;
  df_sincos_2pi(df_u01(wv), s1, c1);
  df_sincos_2pi(df_u01(ww), s2, c2);
  const df a = df_sqrt(df_add_f(df{-u.hi, -u.lo}, 1.0f)), b = df_sqrt(u);
  const df q0 = df_mul(a, s1), q1 = df_mul(a, c1), q2 = df_mul(b, s2), q3 = df_mul(b, c2);
  const df a01 = df_mul(q0, q1), a02 = df_mul(q0, q2), a03 = df_mul(q0, q3);
  const df a11 = df_mul(q1, q1), a12 = df_mul(q1, q2), a13 = df_mul(q1, q3);
  const df a22 = df_mul(q2, q2), a23 = df_mul(q2, q3), a33 = df_mul(q3, q3);
  auto two = [](df p) { return df{2.0f * p.hi, 2.0f * p.lo}; };
  auto neg = [](df p) { return df{-p.hi, -p.lo}; };
  auto one_minus_2 = [&](df p, df q) { return df_add_f(neg(two(df_add(p, q))), 1.0f); };
  const df r0 = one_minus_2(a22, a33), r1 = two(df_add(a12, neg(a03))), r2 = two(df_add(a13, a02));
  const df r3 = two(df_add(a12, a03)), r4 = one_minus_2(a11, a33), r5 = two(df_add(a23, neg(a01)));
  const df r6 = two(df_add(a13, neg(a02))), r7 = two(df_add(a23, a01)), r8 = one_minus_2(a11, a22);
  const df X = df_from(x), Y = df_from(y), Z = df_from(z);
  const df nx = df_add(df_add(df_mul(X, r0), df_mul(Y, r1)), df_mul(Z, r2));
  const df ny = df_add(df_add(df_mul(X, r3), df_mul(Y, r4)), df_mul(Z, r5));
  const df nz = df_add(df_add(df_mul(X, r6), df_mul(Y, r7)), df_mul(Z, r8));
  x = df_to(nx);
  y = df_to(ny);
  z = df_to(nz);
}

// Out of line (the orientation stages run it once per trial on few lanes; a smaller kernel
// fetches fewer instructions), the result returned in registers.
static __device__ __noinline__ double4 df_rotate_quaternion_out(double x, double y, double z, uint32_t wu,
                                                                uint32_t wv, uint32_t ww) {
  df_rotate_quaternion_inl(x, y, z, wu, wv, ww);
  return make_double4(x, y, z, 0.0);
}

__device__ __forceinline__ void df_rotate_quaternion(double& x, double& y, double& z, uint32_t wu, uint32_t wv,
                                                     uint32_t ww) {
  const double4 r = df_rotate_quaternion_out(x, y, z, wu, wv, ww);
  x = r.x;
  y = r.y;
  z = r.z;
}

}  // namespace grx
