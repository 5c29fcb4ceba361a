// fft_stages.cuh -- radix-2/3/4/8 Stockham stages of complex FFTs held in
// shared memory, templated on an arithmetic policy (arith.cuh).  Used by the
// Dirichlet solver's DST passes (poisson.cu) and by the far-field
// convolutions of the boundary operator (farfield.cu).
#pragma once
#include "arith.cuh"

namespace vpmg {
namespace {

// ---- FFT stages in the policy's arithmetic (arith.cuh) -------------------
// F64: IEEE double, the reference's arithmetic.  FF: float-float on the FP32
// pipes (48-bit significand, error-free sums and products), entered and
// left by bit operations.
template <class A, int R>
struct DFT;

template <class A>
struct DFT<A, 2> {
  using C = typename A::C;
  __device__ __forceinline__ static void run(C (&v)[2]) {
    const C a = v[0], b = v[1];
    v[0] = A::cadd(a, b);
    v[1] = A::csub(a, b);
  }
};

template <class A>
__device__ __forceinline__ void dft4(typename A::C& v0, typename A::C& v1, typename A::C& v2, typename A::C& v3) {
  using C = typename A::C;
  const C t0 = A::cadd(v0, v2), t1 = A::csub(v0, v2), t2 = A::cadd(v1, v3), t3 = A::csub(v1, v3);
  v0 = A::cadd(t0, t2);
  v2 = A::csub(t0, t2);
  v1 = A::cadd(t1, A::mul_mi(t3));  // t1 - i t3
  v3 = A::cadd(t1, A::mul_pi(t3));  // t1 + i t3
}

template <class A>
struct DFT<A, 4> {
  using C = typename A::C;
  __device__ __forceinline__ static void run(C (&v)[4]) { dft4<A>(v[0], v[1], v[2], v[3]); }
};

template <class A>
struct DFT<A, 8> {
  using C = typename A::C;
  using R = typename A::R;
  __device__ __forceinline__ static void run(C (&v)[8]) {
    C e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    C o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4<A>(e0, e1, e2, e3);
    dft4<A>(o0, o1, o2, o3);
    const R r = A::rsqrt2();
    // W8^1 o1 = ((x+y) + i(y-x))/sqrt2 ; W8^2 o2 = -i o2 ; W8^3 o3 = ((y-x) - i(x+y))/sqrt2
    const R s1 = A::add(A::re(o1), A::im(o1)), d1 = A::sub(A::im(o1), A::re(o1));
    const R s3 = A::add(A::re(o3), A::im(o3)), d3 = A::sub(A::im(o3), A::re(o3));
    const C w1 = A::cplx(A::mul(s1, r), A::mul(d1, r));
    const C w2 = A::mul_mi(o2);
    const C w3 = A::cplx(A::mul(d3, r), A::neg(A::mul(s3, r)));
    v[0] = A::cadd(e0, o0);
    v[4] = A::csub(e0, o0);
    v[1] = A::cadd(e1, w1);
    v[5] = A::csub(e1, w1);
    v[2] = A::cadd(e2, w2);
    v[6] = A::csub(e2, w2);
    v[3] = A::cadd(e3, w3);
    v[7] = A::csub(e3, w3);
  }
};

// One Stockham radix-R stage over npair transforms of length M held back
// to back in shared memory.
template <class A, int R>
__device__ __forceinline__ void stage(const typename A::C* __restrict__ in, typename A::C* __restrict__ out, int M,
                                      int Ns, const typename A::C* __restrict__ tw, int npair) {
  using C = typename A::C;
  const int nbf = M / R;
  const int tws = M / (Ns * R);
  for (int t = threadIdx.x; t < npair * nbf; t += blockDim.x) {
    const int pr = t / nbf;
    const int j = t - pr * nbf;
    const C* src = in + pr * M;
    C* dst = out + pr * M;
    C v[R];
#pragma unroll
    for (int m = 0; m < R; ++m) v[m] = src[j + m * nbf];
    const int k = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int m = 1; m < R; ++m) v[m] = A::cmul(v[m], __ldg(&tw[k * m * tws]));
    }
    DFT<A, R>::run(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int m = 0; m < R; ++m) dst[base + m * Ns] = v[m];
  }
}

// Radix 3, forward (W = e^{-2 pi i / 3}): X_0 = a + (b + c),
// X_{1,2} = (a - (b + c)/2) -/+ i (sqrt(3)/2) (b - c).
template <class A>
struct DFT<A, 3> {
  using C = typename A::C;
  __device__ __forceinline__ static void run(C (&v)[3]) {
    const C t = A::cadd(v[1], v[2]), d = A::csub(v[1], v[2]);
    const C m = A::csub(v[0], A::cplx(A::scale(A::re(t), 0.5f), A::scale(A::im(t), 0.5f)));
    const typename A::R k = A::from(0.86602540378443864676);
    const C e = A::cplx(A::mul(k, A::re(d)), A::mul(k, A::im(d)));
    v[0] = A::cadd(v[0], t);
    v[1] = A::cadd(m, A::mul_mi(e));
    v[2] = A::cadd(m, A::mul_pi(e));
  }
};

}  // namespace
}  // namespace vpmg
