// ff.cuh -- float-float ("double-single") arithmetic for FP64-scarce GPUs.
//
// GB300 issues FP32 FMAs about 66 times faster than FP64 FMAs, and its
// FP64 <-> FP32 conversion instructions run at the FP64 rate.  A value here
// is an unevaluated sum hi + lo of two floats (about 48 significant bits);
// sums use Knuth's error-free two-sum, products split the high product
// exactly with an FMA (Dekker / Kahan), both renormalised with a fast
// two-sum.  Every operation is an explicitly rounded intrinsic, so the
// compiler cannot contract the error terms away.  Doubles enter and leave
// through integer bit operations (and one FP64 add on the way out), never
// through conversion instructions.
//
// Range: magnitudes between about 1e-38 and 3e38; the split flushes the
// low part to zero where it would be subnormal (below 2^-126).
#pragma once
#include <cuda_runtime.h>

namespace vpmg {
namespace ff {

// d = hi + lo + r with |r| <= 2^-47 |d|: hi is d truncated to 24
// significant bits, lo the next 24 (truncated).  Integer operations only.
__device__ __forceinline__ float2 split(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned s = (unsigned)(b >> 32) & 0x80000000u;
  const int e = (int)((b >> 52) & 0x7FF) - 1023;
  if (e < -126) return make_float2(0.0f, 0.0f);                       // zero, subnormal, tiny
  if (e > 127) return make_float2(__uint_as_float(s | 0x7F800000u), 0.0f);  // beyond float range
  const unsigned long long M = b & 0xFFFFFFFFFFFFFull;
  const float hi = __uint_as_float(s | ((unsigned)(e + 127) << 23) | (unsigned)(M >> 29));
  const unsigned m = (unsigned)(M & 0x1FFFFFFFull);  // the rest: m * 2^(e-52)
  float lo = 0.0f;
  if (m) {
    const int p = 32 - __clz(m);  // its significant bits, 1..29
    const unsigned mant = (p > 24) ? (m >> (p - 24)) : (m << (24 - p));
    const int el = e - 52 + (p - 1);
    if (el >= -126) lo = __uint_as_float(s | ((unsigned)(el + 127) << 23) | (mant & 0x7FFFFFu));
  }
  return make_float2(hi, lo);
}

// Exact float -> double by bit operations (normal floats; zero and
// subnormals give zero).
__device__ __forceinline__ double widen(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned ex = (u >> 23) & 0xFFu;
  if (ex == 0) return 0.0;
  const unsigned long long b = ((unsigned long long)(u & 0x80000000u) << 32) |
                               ((unsigned long long)(ex - 127 + 1023) << 52) |
                               ((unsigned long long)(u & 0x7FFFFFu) << 29);
  return __longlong_as_double((long long)b);
}

__device__ __forceinline__ double to_double(float2 a) { return __dadd_rn(widen(a.x), widen(a.y)); }

__device__ __forceinline__ float2 renorm(float s, float e) {  // fast two-sum, |s| >= |e|
  const float h = __fadd_rn(s, e);
  return make_float2(h, __fsub_rn(e, __fsub_rn(h, s)));
}

__device__ __forceinline__ float2 add(float2 a, float2 b) {
  const float s = __fadd_rn(a.x, b.x);
  const float bb = __fsub_rn(s, a.x);
  float e = __fadd_rn(__fsub_rn(a.x, __fsub_rn(s, bb)), __fsub_rn(b.x, bb));
  e = __fadd_rn(e, __fadd_rn(a.y, b.y));
  return renorm(s, e);
}

__device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return add(a, neg(b)); }

__device__ __forceinline__ float2 mul(float2 a, float2 b) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  return renorm(p, e);
}

// a * b + c
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) {
  const float p = __fmul_rn(a.x, b.x);
  float e = __fmaf_rn(a.x, b.x, -p);
  e = __fmaf_rn(a.x, b.y, e);
  e = __fmaf_rn(a.y, b.x, e);
  const float s = __fadd_rn(p, c.x);
  const float bb = __fsub_rn(s, p);
  const float t = __fadd_rn(__fsub_rn(p, __fsub_rn(s, bb)), __fsub_rn(c.x, bb));
  e = __fadd_rn(__fadd_rn(e, c.y), t);
  return renorm(s, e);
}

// Multiplication by 2^k (exact)
__device__ __forceinline__ float2 scale(float2 a, float f) { return make_float2(__fmul_rn(a.x, f), __fmul_rn(a.y, f)); }

// ---- complex values: float4 = (re.hi, re.lo, im.hi, im.lo) --------------
__device__ __forceinline__ float2 re(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 im(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 cplx(float2 r, float2 i) { return make_float4(r.x, r.y, i.x, i.y); }
__device__ __forceinline__ float4 cadd(float4 a, float4 b) { return cplx(add(re(a), re(b)), add(im(a), im(b))); }
__device__ __forceinline__ float4 csub(float4 a, float4 b) { return cplx(sub(re(a), re(b)), sub(im(a), im(b))); }
__device__ __forceinline__ float4 cmul(float4 a, float4 b) {
  return cplx(fma(re(a), re(b), neg(mul(im(a), im(b)))), fma(re(a), im(b), mul(im(a), re(b))));
}
__device__ __forceinline__ float4 from_double2(double2 v) {
  const float2 r = split(v.x), i = split(v.y);
  return make_float4(r.x, r.y, i.x, i.y);
}
__device__ __forceinline__ double2 to_double2(float4 v) { return make_double2(to_double(re(v)), to_double(im(v))); }

}  // namespace ff
}  // namespace vpmg
