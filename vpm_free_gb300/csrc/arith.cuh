// arith.cuh -- the two arithmetics of the heavy kernels, as policies.
//
// F64 is IEEE double precision throughout: the reference's arithmetic
// (source/pmsolve.f90:351-354 MKL d_Helmholtz_3D, pmbound.f90:1225-1240,
// pmproject.f90:74-90 are all REAL(8)).  It is the library's default.
// FF is float-float (ff.cuh): about 48 significant bits and FP32's exponent
// range, computed on the FP32 pipes, which GB300 issues about 60 times
// faster than FP64.  A kernel templated on a policy A sees
//   A::R  a real value   (double  | float2 hi+lo)
//   A::C  a complex value (double2 | float4)
// Both types have the same size in either policy (8 and 16 bytes), so every
// array and shared-memory layout is the same for both.
#pragma once
#include <cuda_runtime.h>

#include "ff.cuh"

namespace vpmg {

struct F64 {
  using R = double;
  using C = double2;
  static constexpr bool kFF = false;
  __device__ __forceinline__ static R zero() { return 0.0; }
  __device__ __forceinline__ static R from(double d) { return d; }
  __device__ __forceinline__ static double to(R r) { return r; }
  __device__ __forceinline__ static R add(R a, R b) { return a + b; }
  __device__ __forceinline__ static R sub(R a, R b) { return a - b; }
  __device__ __forceinline__ static R mul(R a, R b) { return a * b; }
  __device__ __forceinline__ static R fma(R a, R b, R c) { return ::fma(a, b, c); }
  __device__ __forceinline__ static R neg(R a) { return -a; }
  // a * f for f = +-0.5 (the transforms' only scalings) by integer
  // operations on the bits, exactly the IEEE product and without an FP64
  // pipe slot: the exponent field is decremented when the result stays
  // normal; below that the significand (with its implicit bit) is halved,
  // rounding half to even; inf and nan pass through.
  __device__ __forceinline__ static R scale(R a, float f) {
    if (f != 0.5f && f != -0.5f) return a * (double)f;
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    const unsigned long long sgn = (b & 0x8000000000000000ull) ^ (f < 0.0f ? 0x8000000000000000ull : 0ull);
    const unsigned long long u = b & 0x7FFFFFFFFFFFFFFFull;
    unsigned long long r;
    if (u >= 0x7FF0000000000000ull) r = u;                           // inf, nan
    else if (u >= 0x0020000000000000ull) r = u - 0x0010000000000000ull;  // biased exponent >= 2
    else r = (u >> 1) + (u & (u >> 1) & 1ull);                         // subnormal result
    return __longlong_as_double((long long)(sgn | r));
  }
  __device__ __forceinline__ static R re(C v) { return v.x; }
  __device__ __forceinline__ static R im(C v) { return v.y; }
  __device__ __forceinline__ static C cplx(R r, R i) { return make_double2(r, i); }
  __device__ __forceinline__ static C cadd(C a, C b) { return make_double2(a.x + b.x, a.y + b.y); }
  __device__ __forceinline__ static C csub(C a, C b) { return make_double2(a.x - b.x, a.y - b.y); }
  __device__ __forceinline__ static C cmul(C a, C b) {
    return make_double2(::fma(a.x, b.x, -a.y * b.y), ::fma(a.x, b.y, a.y * b.x));
  }
  __device__ __forceinline__ static C from2(double2 v) { return v; }
  __device__ __forceinline__ static double2 to2(C v) { return v; }
  __device__ __forceinline__ static C mul_mi(C t) { return make_double2(t.y, -t.x); }  // -i t
  __device__ __forceinline__ static C mul_pi(C t) { return make_double2(-t.y, t.x); }  // +i t
  __device__ __forceinline__ static R rsqrt2() { return 0.70710678118654752440; }
};

struct FF {
  using R = float2;
  using C = float4;
  static constexpr bool kFF = true;
  __device__ __forceinline__ static R zero() { return make_float2(0.0f, 0.0f); }
  __device__ __forceinline__ static R from(double d) { return ff::split(d); }
  __device__ __forceinline__ static double to(R r) { return ff::to_double(r); }
  __device__ __forceinline__ static R add(R a, R b) { return ff::add(a, b); }
  __device__ __forceinline__ static R sub(R a, R b) { return ff::sub(a, b); }
  __device__ __forceinline__ static R mul(R a, R b) { return ff::mul(a, b); }
  __device__ __forceinline__ static R fma(R a, R b, R c) { return ff::fma(a, b, c); }
  __device__ __forceinline__ static R neg(R a) { return ff::neg(a); }
  __device__ __forceinline__ static R scale(R a, float f) { return ff::scale(a, f); }
  __device__ __forceinline__ static R re(C v) { return ff::re(v); }
  __device__ __forceinline__ static R im(C v) { return ff::im(v); }
  __device__ __forceinline__ static C cplx(R r, R i) { return ff::cplx(r, i); }
  __device__ __forceinline__ static C cadd(C a, C b) { return ff::cadd(a, b); }
  __device__ __forceinline__ static C csub(C a, C b) { return ff::csub(a, b); }
  __device__ __forceinline__ static C cmul(C a, C b) { return ff::cmul(a, b); }
  __device__ __forceinline__ static C from2(double2 v) { return ff::from_double2(v); }
  __device__ __forceinline__ static double2 to2(C v) { return ff::to_double2(v); }
  __device__ __forceinline__ static C mul_mi(C t) { return make_float4(t.z, t.w, -t.x, -t.y); }
  __device__ __forceinline__ static C mul_pi(C t) { return make_float4(-t.z, -t.w, t.x, t.y); }
  __device__ __forceinline__ static R rsqrt2() { return make_float2(0.7071067690849304f, 1.2101617485882343e-08f); }
};

}  // namespace vpmg
