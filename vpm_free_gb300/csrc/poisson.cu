// poisson.cu -- batched FP64 Dirichlet solver for the 7-point Laplacian.
//
// Replaces the MKL Poisson Library calls of source/pmsolve.f90:284-432
// (d_Helmholtz_3D with 'DDDDDD' boundaries, q = 0, f = -RHS): the exact
// discrete solution of  Lap_h u = RHS  on a node box with Dirichlet values.
//
// Method (GB300-first: FP64 is the scarce resource, ~1.2 TFLOP/s):
//   1. x pass: fold the boundary values into the RHS of the first/last
//      interior layers, DST-I along x, scaled for the later inverse.  For
//      even N = n+1 the DST-I is computed in its real-symmetric form: the
//      line is pre-twiddled, y_j = sin(pi j/N)(x_j + x_{N-j}) + (x_j - x_{N-j})/2,
//      two lines share one complex FFT of length N, and the outputs come
//      from the split spectrum, X_{2m} = -Im F_m and X_{2m+1} = X_{2m-1} + Re F_m
//      (a prefix sum, X_1 = Re F_0 / 2).  Odd N falls back to the odd
//      extension (two lines in one complex FFT of length 2N);
//   2. y pass: the same DST-I along y, in place;
//   3. z pass: per (p,q) mode the constant-coefficient tridiagonal system
//      -u[k-1] + d_pq u[k] - u[k+1] = r[k] by a Thomas sweep whose
//      reciprocal pivots come from a table built once per grid (no FP64
//      divisions per step);
//   4. inverse y and x passes (DST-I is its own inverse up to 2/N).
// FFTs run in shared memory as mixed-radix Stockham stages (radix 2,4,8
// and odd primes up to 17 through the symmetric direct DFT), instantiated
// twice: power-of-two radices only, and with the odd radices.
#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "ff.cuh"
#include "vpmg_internal.h"

namespace vpmg {

namespace {

// Tile shape: a CTA of kThreads transforms PAIRS line pairs (2 * PAIRS real
// lines).  PAIRS is 2, 4 or 8, chosen per plan by timing (tune_pairs); the
// values computed do not depend on it.
constexpr int kThreads = 128;
constexpr int kDefaultPairs = 4;
constexpr int kMaxOddRadix = 17;  // largest odd prime radix (2*(cells) must factor into 2..17)

__constant__ float2 c_rcos_f[(kMaxOddRadix + 1) * (kMaxOddRadix + 1)];  // cos(2 pi i/R), float-float
__constant__ float2 c_rsin_f[(kMaxOddRadix + 1) * (kMaxOddRadix + 1)];
bool g_tables_ready = false;

struct FFTDev {
  int n, N, M, nst;
  int odd;    // 1 if a stage has an odd radix
  int rs;     // 1: real-symmetric DST-I (M = N), 0: odd extension (M = 2N)
  int pairs;  // line pairs per CTA
  int radix[24];
  const float4* tw;  // e^{-2 pi i t / M} as float-float (re.hi, re.lo, im.hi, im.lo)
  const double* sn;  // sin(pi j / N) (rs only)
};

// ---- FFT stages in float-float arithmetic (ff.cuh) ----------------------
// The stages are the FP64-heaviest part of the solve; on GB300 they run
// about as fast again in float-float on the FP32 pipes (48-bit significand,
// error-free sums and products), entered and left by bit operations.
using ff::cadd;
using ff::csub;
using ff::cmul;

template <int R>
struct DFT;

template <>
struct DFT<2> {
  __device__ __forceinline__ static void run(float4 (&v)[2]) {
    const float4 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

__device__ __forceinline__ float4 mul_mi(float4 t) { return make_float4(t.z, t.w, -t.x, -t.y); }  // -i t
__device__ __forceinline__ float4 mul_pi(float4 t) { return make_float4(-t.z, -t.w, t.x, t.y); }  // +i t

__device__ __forceinline__ void dft4(float4& v0, float4& v1, float4& v2, float4& v3) {
  const float4 t0 = cadd(v0, v2), t1 = csub(v0, v2), t2 = cadd(v1, v3), t3 = csub(v1, v3);
  v0 = cadd(t0, t2);
  v2 = csub(t0, t2);
  v1 = cadd(t1, mul_mi(t3));  // t1 - i t3
  v3 = cadd(t1, mul_pi(t3));  // t1 + i t3
}

template <>
struct DFT<4> {
  __device__ __forceinline__ static void run(float4 (&v)[4]) { dft4(v[0], v[1], v[2], v[3]); }
};

template <>
struct DFT<8> {
  __device__ __forceinline__ static void run(float4 (&v)[8]) {
    float4 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    float4 o0 = v[1], o1 = v[3], o2 = v[5], o3 = v[7];
    dft4(e0, e1, e2, e3);
    dft4(o0, o1, o2, o3);
    const float2 r = make_float2(0.7071067690849304f, 1.2101617485882343e-08f);  // 1/sqrt(2) as hi + lo
    // W8^1 o1 = ((x+y) + i(y-x))/sqrt2 ; W8^2 o2 = -i o2 ; W8^3 o3 = ((y-x) - i(x+y))/sqrt2
    const float2 s1 = ff::add(ff::re(o1), ff::im(o1)), d1 = ff::sub(ff::im(o1), ff::re(o1));
    const float2 s3 = ff::add(ff::re(o3), ff::im(o3)), d3 = ff::sub(ff::im(o3), ff::re(o3));
    const float4 w1 = ff::cplx(ff::mul(s1, r), ff::mul(d1, r));
    const float4 w2 = mul_mi(o2);
    const float4 w3 = ff::cplx(ff::mul(d3, r), ff::neg(ff::mul(s3, r)));
    v[0] = cadd(e0, o0);
    v[4] = csub(e0, o0);
    v[1] = cadd(e1, w1);
    v[5] = csub(e1, w1);
    v[2] = cadd(e2, w2);
    v[6] = csub(e2, w2);
    v[3] = cadd(e3, w3);
    v[7] = csub(e3, w3);
  }
};

// Odd radix: X_k = x0 + sum_m [(v_m + v_{R-m}) cos(2 pi mk/R) - i (v_m - v_{R-m}) sin(2 pi mk/R)].
template <int R>
struct DFT {
  __device__ __forceinline__ static void run(float4 (&v)[R]) {
    constexpr int H = (R - 1) / 2;
    float4 s[H], d[H];
    const float4 x0 = v[0];
    float4 sum = x0;
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      s[m - 1] = cadd(v[m], v[R - m]);
      d[m - 1] = csub(v[m], v[R - m]);
      sum = cadd(sum, s[m - 1]);
    }
    v[0] = sum;
#pragma unroll
    for (int k = 1; k <= H; ++k) {
      float2 ar = ff::re(x0), ai = ff::im(x0), br = make_float2(0.0f, 0.0f), bi = make_float2(0.0f, 0.0f);
#pragma unroll
      for (int m = 1; m <= H; ++m) {
        const int idx = (m * k) % R;
        const float2 c = c_rcos_f[R * (kMaxOddRadix + 1) + idx];
        const float2 sn = c_rsin_f[R * (kMaxOddRadix + 1) + idx];
        ar = ff::fma(c, ff::re(s[m - 1]), ar);
        ai = ff::fma(c, ff::im(s[m - 1]), ai);
        br = ff::fma(sn, ff::re(d[m - 1]), br);
        bi = ff::fma(sn, ff::im(d[m - 1]), bi);
      }
      v[k] = ff::cplx(ff::add(ar, bi), ff::sub(ai, br));
      v[R - k] = ff::cplx(ff::sub(ar, bi), ff::add(ai, br));
    }
  }
};

// One Stockham radix-R stage over npair transforms of length M held back
// to back in shared memory.
template <int R>
__device__ __forceinline__ void stage(const float4* __restrict__ in, float4* __restrict__ out, int M, int Ns,
                                      const float4* __restrict__ tw, int npair) {
  const int nbf = M / R;
  const int tws = M / (Ns * R);
  for (int t = threadIdx.x; t < npair * nbf; t += blockDim.x) {
    const int pr = t / nbf;
    const int j = t - pr * nbf;
    const float4* src = in + pr * M;
    float4* dst = out + pr * M;
    float4 v[R];
#pragma unroll
    for (int m = 0; m < R; ++m) v[m] = src[j + m * nbf];
    const int k = j % Ns;
    if (Ns > 1) {
#pragma unroll
      for (int m = 1; m < R; ++m) v[m] = cmul(v[m], __ldg(&tw[k * m * tws]));
    }
    DFT<R>::run(v);
    const int base = (j - k) * R + k;
#pragma unroll
    for (int m = 0; m < R; ++m) dst[base + m * Ns] = v[m];
  }
}

// Odd-radix stage in two phases, so that a transform's few butterflies
// (16 per radix-17 stage of a 272-point line) do not leave most threads
// idle: (A) one thread per butterfly folds its twiddled inputs into
// s_m = v_m + v_{R-m} and d_m = v_m - v_{R-m}, in place in the stage's input
// buffer (free after the stage), and writes X_0 = v_0 + sum s_m; (B) one
// thread per output pair q = 1..H reads x0, s_m, d_m back from shared
// memory and writes X_q and X_{R-q}.  The arithmetic and its order per
// output are DFT<R>'s.
template <int R>
__device__ __forceinline__ void stage_odd(float4* __restrict__ in, float4* __restrict__ out, int M, int Ns,
                                          const float4* __restrict__ tw, int npair) {
  constexpr int H = (R - 1) / 2;
  const int nbf = M / R;
  const int tws = M / (Ns * R);
  for (int t = threadIdx.x; t < npair * nbf; t += blockDim.x) {
    const int pr = t / nbf;
    const int j = t - pr * nbf;
    float4* src = in + pr * M;
    const int k = j % Ns;
    const int base = (j - k) * R + k;
    float4 sum = src[j];
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      float4 a = src[j + m * nbf], b = src[j + (R - m) * nbf];
      if (Ns > 1) {
        a = cmul(a, __ldg(&tw[k * m * tws]));
        b = cmul(b, __ldg(&tw[k * (R - m) * tws]));
      }
      const float4 sm = cadd(a, b);
      src[j + m * nbf] = sm;
      src[j + (R - m) * nbf] = csub(a, b);
      sum = cadd(sum, sm);
    }
    out[pr * M + base] = sum;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < npair * nbf * H; t += blockDim.x) {
    const int q = t % H + 1;
    const int bf = t / H;
    const int pr = bf / nbf;
    const int j = bf - pr * nbf;
    const float4* src = in + pr * M;
    const int k = j % Ns;
    const int base = (j - k) * R + k;
    const float4 x0 = src[j];
    float2 ar = ff::re(x0), ai = ff::im(x0), br = make_float2(0.0f, 0.0f), bi = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      const float4 sm = src[j + m * nbf], dm = src[j + (R - m) * nbf];
      const int idx = (m * q) % R;
      const float2 c = c_rcos_f[R * (kMaxOddRadix + 1) + idx];
      const float2 sn = c_rsin_f[R * (kMaxOddRadix + 1) + idx];
      ar = ff::fma(c, ff::re(sm), ar);
      ai = ff::fma(c, ff::im(sm), ai);
      br = ff::fma(sn, ff::re(dm), br);
      bi = ff::fma(sn, ff::im(dm), bi);
    }
    float4* dst = out + pr * M;
    dst[base + q * Ns] = ff::cplx(ff::add(ar, bi), ff::sub(ai, br));
    dst[base + (R - q) * Ns] = ff::cplx(ff::sub(ar, bi), ff::add(ai, br));
  }
}

// Runs all stages; returns the buffer holding the result.  ODD = false
// instantiates only the power-of-two radices, which keeps the register
// count (and so the occupancy) of those kernels independent of the large
// odd-radix butterflies.
template <bool ODD>
__device__ float4* fft_all(float4* A, float4* B, const FFTDev& p, int npair) {
  int Ns = 1;
  for (int s = 0; s < p.nst; ++s) {
    const int r = p.radix[s];
    switch (r) {
      case 2: stage<2>(A, B, p.M, Ns, p.tw, npair); break;
      case 4: stage<4>(A, B, p.M, Ns, p.tw, npair); break;
      case 8: stage<8>(A, B, p.M, Ns, p.tw, npair); break;
      default:
        if constexpr (ODD) {
          switch (r) {
            case 3: stage_odd<3>(A, B, p.M, Ns, p.tw, npair); break;
            case 5: stage_odd<5>(A, B, p.M, Ns, p.tw, npair); break;
            case 7: stage_odd<7>(A, B, p.M, Ns, p.tw, npair); break;
            case 11: stage_odd<11>(A, B, p.M, Ns, p.tw, npair); break;
            case 13: stage_odd<13>(A, B, p.M, Ns, p.tw, npair); break;
            case 17: stage_odd<17>(A, B, p.M, Ns, p.tw, npair); break;
            default: break;
          }
        }
        break;
    }
    __syncthreads();
    Ns *= r;
    float4* t = A;
    A = B;
    B = t;
  }
  return A;
}

// In place, the npair * M complex values of a buffer: FP64 -> float-float
// (same 16 bytes per value).
__device__ __forceinline__ void to_ff(double2* z, int n) {
  for (int t = threadIdx.x; t < n; t += blockDim.x) {
    const double2 v = z[t];
    reinterpret_cast<float4*>(z)[t] = ff::from_double2(v);
  }
}

// Odd extension of the loaded real pairs: z[0] = z[N] = 0, z[M-j] = -z[j].
__device__ __forceinline__ void odd_extend(double2* z, const FFTDev& p, int npair) {
  for (int t = threadIdx.x; t < npair * p.N; t += blockDim.x) {
    const int pr = t / p.N, j = t - pr * p.N;
    double2* zz = z + pr * p.M;
    if (j == 0) {
      zz[0] = make_double2(0.0, 0.0);
      zz[p.N] = make_double2(0.0, 0.0);
    } else {
      const double2 v = zz[j];
      zz[p.M - j] = make_double2(-v.x, -v.y);
    }
  }
}

// Real-symmetric DST-I, input side: the pair's lines sit in L at 1..n;
// Z_0 = 0, Z_j = s_j (L_j + L_{N-j}) + (L_j - L_{N-j}) / 2, s_j = sin(pi j / N).
// The doubles are split into float-float here and Z is float-float.
__device__ __forceinline__ void rs_pre(const double2* __restrict__ L, float4* __restrict__ Z, const FFTDev& p,
                                       int npair) {
  for (int t = threadIdx.x; t < npair * p.N; t += blockDim.x) {
    const int pr = t / p.N, j = t - pr * p.N;
    float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (j > 0) {
      const float4 a = ff::from_double2(L[pr * p.M + j]), b = ff::from_double2(L[pr * p.M + p.N - j]);
      const float2 sj = ff::split(__ldg(&p.sn[j]));
      z = ff::cplx(ff::fma(sj, ff::add(ff::re(a), ff::re(b)), ff::scale(ff::sub(ff::re(a), ff::re(b)), 0.5f)),
                   ff::fma(sj, ff::add(ff::im(a), ff::im(b)), ff::scale(ff::sub(ff::im(a), ff::im(b)), 0.5f)));
    }
    Z[pr * p.M + j] = z;
  }
}

// Output side: Z is the length-N FFT of a packed pair.  With Z_m = a + ib,
// Z_{N-m} = c + id the two lines' spectra are F = ((a+c) + i(b-d))/2 and
// G = ((b+d) - i(a-c))/2, so X_{2m} = (d-b)/2 and (a-c)/2, and the odd
// outputs are the prefix sums of r_0 = Z_0 / 2, r_m = ((a+c)/2, (b+d)/2).
// O[pair * M + k] receives X_k of both lines, k = 1..n, in float-float.
// The prefix sum runs over kScanSegs fixed segments of each line in a
// fixed order, so the result does not depend on the tile shape; Z is its
// scratch afterwards.
constexpr int kScanSegs = 32;
__device__ __forceinline__ void rs_post(float4* __restrict__ Z, float4* __restrict__ O, const FFTDev& p,
                                        int npair) {
  const int H = p.N >> 1;
  for (int t = threadIdx.x; t < npair * H; t += blockDim.x) {
    const int pr = t / H, m = t - pr * H;
    const float4 u = Z[pr * p.M + m];
    if (m == 0) {
      O[pr * p.M + 1] = ff::cplx(ff::scale(ff::re(u), 0.5f), ff::scale(ff::im(u), 0.5f));
    } else {
      const float4 v = Z[pr * p.M + p.N - m];
      O[pr * p.M + 2 * m] = ff::cplx(ff::scale(ff::sub(ff::im(v), ff::im(u)), 0.5f),
                                     ff::scale(ff::sub(ff::re(u), ff::re(v)), 0.5f));
      O[pr * p.M + 2 * m + 1] = ff::cplx(ff::scale(ff::add(ff::re(u), ff::re(v)), 0.5f),
                                         ff::scale(ff::add(ff::im(u), ff::im(v)), 0.5f));
    }
  }
  __syncthreads();
  // segments per line: min(kScanSegs, H) -- a function of N only; the
  // scratch (2 npair S float-float values) fits in Z (npair M complex, M >= 2H >= 2S)
  const int S = min(kScanSegs, H);
  float2* seg = reinterpret_cast<float2*>(Z);  // [line][S]
  const int C = (H + S - 1) / S;
  const int nls = 2 * npair * S;
  for (int t = threadIdx.x; t < nls; t += blockDim.x) {  // segment sums
    const int line = t / S, g = t - line * S;
    const float2* o = reinterpret_cast<const float2*>(O + (line >> 1) * p.M) + (line & 1);  // X_k at o[2k]
    const int m0 = min(H, g * C), m1 = min(H, m0 + C);
    float2 sum = make_float2(0.0f, 0.0f);
    for (int m = m0; m < m1; ++m) sum = ff::add(sum, o[2 * (2 * m + 1)]);
    seg[t] = sum;
  }
  __syncthreads();
  for (int line = threadIdx.x; line < 2 * npair; line += blockDim.x) {  // exclusive scan of the segment sums
    float2 run = make_float2(0.0f, 0.0f);
    for (int g = 0; g < S; ++g) {
      const float2 v = seg[line * S + g];
      seg[line * S + g] = run;
      run = ff::add(run, v);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nls; t += blockDim.x) {  // inclusive values inside each segment
    const int line = t / S, g = t - line * S;
    float2* o = reinterpret_cast<float2*>(O + (line >> 1) * p.M) + (line & 1);
    const int m0 = min(H, g * C), m1 = min(H, m0 + C);
    float2 run = seg[t];
    for (int m = m0; m < m1; ++m) {
      run = ff::add(run, o[2 * (2 * m + 1)]);
      o[2 * (2 * m + 1)] = run;
    }
  }
}

// The transform of the 2*npair lines loaded into `L` (the staging buffer
// of the plan's mode, see staging()): returns the buffer holding X_k of
// line (pair, c) at index pair * M + k (k = 1..n) as component c (rs), or
// the raw odd-extension spectrum (X_k = -W.y / 2 and W.x / 2).
// The values in shared memory are float-float from the pre-twiddle (or the
// odd extension) to the output; dst_out joins them back into doubles.
template <bool ODD, int PAIRS>
__device__ __forceinline__ float4* dst_pairs(double2* A, double2* B, const FFTDev& p) {
  constexpr int npair = PAIRS;
  float4* Af = reinterpret_cast<float4*>(A);
  float4* Bf = reinterpret_cast<float4*>(B);
  if (p.rs) {
    rs_pre(B, Af, p, npair);
  } else {
    odd_extend(A, p, npair);
    __syncthreads();
    to_ff(A, npair * p.M);
  }
  __syncthreads();
  float4* R = fft_all<ODD>(Af, Bf, p, npair);
  if (!p.rs) return R;
  float4* O = (R == Af) ? Bf : Af;
  rs_post(R, O, p, npair);
  __syncthreads();
  return O;
}
__device__ __forceinline__ double2* staging(double2* A, double2* B, const FFTDev& p) { return p.rs ? B : A; }
__device__ __forceinline__ double dst_out(const float4* O, const FFTDev& p, int li, int k) {
  const float4 W = O[(li >> 1) * p.M + (k + 1)];
  if (p.rs) return ff::to_double((li & 1) ? ff::im(W) : ff::re(W));
  return ff::to_double((li & 1) ? ff::scale(ff::re(W), 0.5f) : ff::scale(ff::im(W), -0.5f));
}

// ------------------------------------------------------------ passes ----
struct Box {
  int dims[3];  // node array dims
  int o[3];     // node offset of interior (a,b,c) = (0,0,0)
  int m[3];     // interior counts
};

// x pass, forward: rhs (+ folded boundary values) -> work, scaled.
template <bool ODD, int PAIRS>
__global__ void __launch_bounds__(kThreads) k_dst_x_fwd(const double* __restrict__ rhs, const double* __restrict__ sol,
                                                        int zero_bc, double* __restrict__ work, Box b, FFTDev p,
                                                        double ihx2, double ihy2, double ihz2, double scale) {
  extern __shared__ double2 smem[];
  double2* A = smem;
  double2* B = smem + PAIRS * p.M;
  const int nlines = b.m[1] * b.m[2];
  const int l0 = blockIdx.x * (2 * PAIRS);
  const int n = p.n;
  const size_t sy = b.dims[0], sz = (size_t)b.dims[0] * b.dims[1];
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, a = t - li * n;
    const int l = l0 + li;
    double v = 0.0;
    if (l < nlines) {
      const int q = l % b.m[1], c = l / b.m[1];
      const size_t node = (size_t)(b.o[0] + a) + sy * (b.o[1] + q) + sz * (b.o[2] + c);
      v = rhs[node];
      if (!zero_bc) {
        if (a == 0) v -= sol[node - 1] * ihx2;
        if (a == b.m[0] - 1) v -= sol[node + 1] * ihx2;
        if (q == 0) v -= sol[node - sy] * ihy2;
        if (q == b.m[1] - 1) v -= sol[node + sy] * ihy2;
        if (c == 0) v -= sol[node - sz] * ihz2;
        if (c == b.m[2] - 1) v -= sol[node + sz] * ihz2;
      }
      v *= scale;
    }
    double* zp = reinterpret_cast<double*>(staging(A, B, p) + (li >> 1) * p.M + (a + 1));
    zp[li & 1] = v;
  }
  __syncthreads();
  const float4* R = dst_pairs<ODD, PAIRS>(A, B, p);
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, k = t - li * n;
    const int l = l0 + li;
    if (l >= nlines) continue;
    work[(size_t)l * n + k] = dst_out(R, p, li, k);
  }
}

// y pass (forward or inverse): in place on work (m0 x m1 x m2, x fastest).
template <bool ODD, int PAIRS>
__global__ void __launch_bounds__(kThreads) k_dst_y(double* __restrict__ work, int m0, int m1, int m2, FFTDev p) {
  extern __shared__ double2 smem[];
  double2* A = smem;
  double2* B = smem + PAIRS * p.M;
  const int nlines = m0 * m2;
  const int l0 = blockIdx.x * (2 * PAIRS);
  const int n = p.n;  // == m1
  const size_t plane = (size_t)m0 * m1;
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t % (2 * PAIRS), e = t / (2 * PAIRS);
    const int l = l0 + li;
    double v = 0.0;
    if (l < nlines) {
      const int a = l % m0, c = l / m0;
      v = work[(size_t)a + (size_t)m0 * e + plane * c];
    }
    double* zp = reinterpret_cast<double*>(staging(A, B, p) + (li >> 1) * p.M + (e + 1));
    zp[li & 1] = v;
  }
  __syncthreads();
  const float4* R = dst_pairs<ODD, PAIRS>(A, B, p);
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t % (2 * PAIRS), k = t / (2 * PAIRS);
    const int l = l0 + li;
    if (l >= nlines) continue;
    const int a = l % m0, c = l / m0;
    work[(size_t)a + (size_t)m0 * k + plane * c] = dst_out(R, p, li, k);
  }
}

// x pass, inverse: work -> interior of sol.
template <bool ODD, int PAIRS>
__global__ void __launch_bounds__(kThreads) k_dst_x_inv(const double* __restrict__ work, double* __restrict__ sol, Box b,
                                                        FFTDev p) {
  extern __shared__ double2 smem[];
  double2* A = smem;
  double2* B = smem + PAIRS * p.M;
  const int nlines = b.m[1] * b.m[2];
  const int l0 = blockIdx.x * (2 * PAIRS);
  const int n = p.n;
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, a = t - li * n;
    const int l = l0 + li;
    const double v = (l < nlines) ? work[(size_t)l * n + a] : 0.0;
    double* zp = reinterpret_cast<double*>(staging(A, B, p) + (li >> 1) * p.M + (a + 1));
    zp[li & 1] = v;
  }
  __syncthreads();
  const float4* R = dst_pairs<ODD, PAIRS>(A, B, p);
  const size_t sy = b.dims[0], sz = (size_t)b.dims[0] * b.dims[1];
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, k = t - li * n;
    const int l = l0 + li;
    if (l >= nlines) continue;
    const int q = l % b.m[1], c = l / b.m[1];
    sol[(size_t)(b.o[0] + k) + sy * (b.o[1] + q) + sz * (b.o[2] + c)] = dst_out(R, p, li, k);
  }
}

// z pass: Thomas sweep per (p,q) with the reciprocal pivot table, in
// float-float arithmetic (ff.cuh): the forward sweep leaves its values in
// place as float-float pairs, the backward sweep writes the doubles.  The
// column's loads are issued four planes ahead of the dependent chain (the
// sweep is latency-bound otherwise).
__global__ void k_thomas(double* __restrict__ g, const float2* __restrict__ rinv, int m0, int m1, int m2) {
  const int pq = blockIdx.x * blockDim.x + threadIdx.x;
  if (pq >= m0 * m1) return;
  const size_t plane = (size_t)m0 * m1;
  float2* gf = reinterpret_cast<float2*>(g);
  float2 y = ff::split(g[pq]);
  gf[pq] = y;
  float2 ri = rinv[pq];
  int c = 1;
  for (; c + 3 < m2; c += 4) {
    const size_t id = pq + plane * c;
    const double g0 = g[id], g1 = g[id + plane], g2 = g[id + 2 * plane], g3 = g[id + 3 * plane];
    const float2 r0 = rinv[id], r1 = rinv[id + plane], r2 = rinv[id + 2 * plane], r3 = rinv[id + 3 * plane];
    y = ff::fma(y, ri, ff::split(g0));
    gf[id] = y;
    y = ff::fma(y, r0, ff::split(g1));
    gf[id + plane] = y;
    y = ff::fma(y, r1, ff::split(g2));
    gf[id + 2 * plane] = y;
    y = ff::fma(y, r2, ff::split(g3));
    gf[id + 3 * plane] = y;
    ri = r3;
  }
  for (; c < m2; ++c) {
    const size_t id = pq + plane * c;
    y = ff::fma(y, ri, ff::split(g[id]));
    gf[id] = y;
    ri = rinv[id];
  }
  float2 u = ff::mul(y, ri);
  g[pq + plane * (m2 - 1)] = ff::to_double(u);
  c = m2 - 2;
  for (; c - 3 >= 0; c -= 4) {
    const size_t id = pq + plane * c;
    const float2 g0 = gf[id], g1 = gf[id - plane], g2 = gf[id - 2 * plane], g3 = gf[id - 3 * plane];
    const float2 r0 = rinv[id], r1 = rinv[id - plane], r2 = rinv[id - 2 * plane], r3 = rinv[id - 3 * plane];
    u = ff::mul(ff::add(g0, u), r0);
    g[id] = ff::to_double(u);
    u = ff::mul(ff::add(g1, u), r1);
    g[id - plane] = ff::to_double(u);
    u = ff::mul(ff::add(g2, u), r2);
    g[id - 2 * plane] = ff::to_double(u);
    u = ff::mul(ff::add(g3, u), r3);
    g[id - 3 * plane] = ff::to_double(u);
  }
  for (; c >= 0; --c) {
    const size_t id = pq + plane * c;
    u = ff::mul(ff::add(gf[id], u), rinv[id]);
    g[id] = ff::to_double(u);
  }
}

// Reciprocal pivots 1/d, 1/(d - r), ... in FP64, stored as float-float
// pairs (and as doubles when rinvd is given).
__global__ void k_pivots(float2* __restrict__ rinv, double* __restrict__ rinvd, const double* __restrict__ mux,
                         const double* __restrict__ muy, int m0, int m1, int m2, double cx, double cy) {
  const int pq = blockIdx.x * blockDim.x + threadIdx.x;
  if (pq >= m0 * m1) return;
  const int p = pq % m0, q = pq / m0;
  const double d = 2.0 + (mux[p] * cx + muy[q] * cy);
  const size_t plane = (size_t)m0 * m1;
  double r = 1.0 / d;
  rinv[pq] = ff::split(r);
  if (rinvd) rinvd[pq] = r;
  for (int c = 1; c < m2; ++c) {
    r = 1.0 / (d - r);
    rinv[pq + plane * c] = ff::split(r);
    if (rinvd) rinvd[pq + plane * c] = r;
  }
}

__global__ void k_zero_box_faces(double* __restrict__ sol, Box b) {
  // faces of the box [o-1, o+m] in each direction
  const int ex = b.m[0] + 2, ey = b.m[1] + 2, ez = b.m[2] + 2;
  const long total = 2L * ey * ez + 2L * ex * ez + 2L * ex * ey;
  const size_t sy = b.dims[0], sz = (size_t)b.dims[0] * b.dims[1];
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    int i, j, k;
    long r = t;
    if (r < 2L * ey * ez) {
      const int f = (int)(r / ((long)ey * ez));
      r -= (long)f * ey * ez;
      j = (int)(r % ey); k = (int)(r / ey); i = f ? ex - 1 : 0;
    } else if ((r -= 2L * ey * ez) < 2L * ex * ez) {
      const int f = (int)(r / ((long)ex * ez));
      r -= (long)f * ex * ez;
      i = (int)(r % ex); k = (int)(r / ex); j = f ? ey - 1 : 0;
    } else {
      r -= 2L * ex * ez;
      const int f = (int)(r / ((long)ex * ey));
      r -= (long)f * ex * ey;
      i = (int)(r % ex); j = (int)(r / ex); k = f ? ez - 1 : 0;
    }
    sol[(size_t)(b.o[0] - 1 + i) + sy * (b.o[1] - 1 + j) + sz * (b.o[2] - 1 + k)] = 0.0;
  }
}

// Launches picking the instantiation of the plan's radices and tile shape;
// grid and shared memory follow from the plan.
size_t tile_smem(const FFTDev& p) { return (size_t)2 * p.pairs * p.M * sizeof(double2); }
unsigned tile_grid(int lines, const FFTDev& p) { return (unsigned)((lines + 2 * p.pairs - 1) / (2 * p.pairs)); }

template <int PAIRS>
void x_fwd_t(cudaStream_t s, const double* rhs, const double* sol, int zbc, double* work, Box b, FFTDev p,
             double ihx2, double ihy2, double ihz2, double scale) {
  const unsigned g = tile_grid(b.m[1] * b.m[2], p);
  if (p.odd) k_dst_x_fwd<true, PAIRS><<<g, kThreads, tile_smem(p), s>>>(rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else k_dst_x_fwd<false, PAIRS><<<g, kThreads, tile_smem(p), s>>>(rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
}
template <int PAIRS>
void y_t(cudaStream_t s, double* work, int m0, int m1, int m2, FFTDev p) {
  const unsigned g = tile_grid(m0 * m2, p);
  if (p.odd) k_dst_y<true, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, m0, m1, m2, p);
  else k_dst_y<false, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, m0, m1, m2, p);
}
template <int PAIRS>
void x_inv_t(cudaStream_t s, const double* work, double* sol, Box b, FFTDev p) {
  const unsigned g = tile_grid(b.m[1] * b.m[2], p);
  if (p.odd) k_dst_x_inv<true, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, sol, b, p);
  else k_dst_x_inv<false, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, sol, b, p);
}
void launch_x_fwd(cudaStream_t s, const double* rhs, const double* sol, int zbc, double* work, Box b, FFTDev p,
                  double ihx2, double ihy2, double ihz2, double scale) {
  if (p.pairs == 2) x_fwd_t<2>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else if (p.pairs == 8) x_fwd_t<8>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else x_fwd_t<4>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
}
void launch_y(cudaStream_t s, double* work, int m0, int m1, int m2, FFTDev p) {
  if (p.pairs == 2) y_t<2>(s, work, m0, m1, m2, p);
  else if (p.pairs == 8) y_t<8>(s, work, m0, m1, m2, p);
  else y_t<4>(s, work, m0, m1, m2, p);
}
void launch_x_inv(cudaStream_t s, const double* work, double* sol, Box b, FFTDev p) {
  if (p.pairs == 2) x_inv_t<2>(s, work, sol, b, p);
  else if (p.pairs == 8) x_inv_t<8>(s, work, sol, b, p);
  else x_inv_t<4>(s, work, sol, b, p);
}
template <int PAIRS>
cudaError_t set_smem_t(int smax) {
  cudaError_t e = cudaSuccess;
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_fwd<true, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_fwd<false, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_y<true, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_y<false, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_inv<true, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_inv<false, PAIRS>, a, smax);
  return e;
}
cudaError_t set_dst_smem(int smax) {
  cudaError_t e = set_smem_t<2>(smax);
  if (e == cudaSuccess) e = set_smem_t<4>(smax);
  if (e == cudaSuccess) e = set_smem_t<8>(smax);
  return e;
}

FFTDev dev_plan(const FFTPlan& p) {
  FFTDev d;
  d.n = p.n; d.N = p.N; d.M = p.M; d.nst = p.nst;
  d.rs = p.rs;
  d.pairs = p.pairs;
  d.sn = p.sn.p;
  d.odd = 0;
  for (int i = 0; i < 24; ++i) {
    d.radix[i] = p.radix[i];
    if (i < p.nst && (p.radix[i] & 1)) d.odd = 1;
  }
  d.tw = p.tw.p;
  return d;
}

// A double as a float-float pair (hi = v rounded to float, lo = the rest).
float2 host_split(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

// cos / sin (2 pi i / R) of the odd radices, float-float.
void odd_radix_tables(float2* hc, float2* hs) {
  for (int R = 1; R <= kMaxOddRadix; ++R)
    for (int i = 0; i < R; ++i) {
      hc[R * (kMaxOddRadix + 1) + i] = host_split(std::cos(2.0 * kPI * i / R));
      hs[R * (kMaxOddRadix + 1) + i] = host_split(std::sin(2.0 * kPI * i / R));
    }
}

void ensure_tables() {
  if (g_tables_ready) return;
  static float2 hc[(kMaxOddRadix + 1) * (kMaxOddRadix + 1)], hs[(kMaxOddRadix + 1) * (kMaxOddRadix + 1)];
  odd_radix_tables(hc, hs);
  VPMG_CUDA(cudaMemcpyToSymbol(c_rcos_f, hc, sizeof(hc)));
  VPMG_CUDA(cudaMemcpyToSymbol(c_rsin_f, hs, sizeof(hs)));
  g_tables_ready = true;
}

size_t smem_bytes(const FFTPlan& p, int pairs) { return (size_t)2 * pairs * p.M * sizeof(double2); }
constexpr size_t kMaxDstSmem = 227 * 1024;

// The DST kernels' shared-memory limit is an attribute of each kernel on
// each device, shared by every plan and by the allocation-free entry
// point: it is only ever raised (set-up time, outside any stream capture).
constexpr int kMaxDevices = 64;
size_t g_dst_smem[kMaxDevices] = {0};
cudaError_t raise_dst_smem_status(size_t need) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (need <= g_dst_smem[dev]) return cudaSuccess;
  e = set_dst_smem((int)need);
  if (e == cudaSuccess) g_dst_smem[dev] = need;
  return e;
}
void raise_dst_smem(size_t need) { VPMG_CUDA(raise_dst_smem_status(need)); }

// Tile-shape autotuner: times the DST pass of this plan with 2, 4 and 8
// line pairs per CTA on a scratch array shaped like the solve's lines
// (m0 x n x m2, lines along the middle axis; m0 = 1 gives contiguous rows as
// in the x passes) and keeps the fastest.  The transform of a line does not
// depend on the tile, so neither do the results.  Set VPMG_DST_PAIRS=2|4|8
// to fix the choice.
void tune_pairs(FFTPlan& p, int lines, int m0, int n, int m2, cudaStream_t s) {
  static const char* fixed = std::getenv("VPMG_DST_PAIRS");
  int cand[3] = {2, 4, 8}, ncand = 0, ok[3];
  for (int c : cand)
    if (smem_bytes(p, c) <= kMaxDstSmem) ok[ncand++] = c;
  raise_dst_smem(smem_bytes(p, ok[ncand - 1]));
  if (fixed) {
    const int f = std::atoi(fixed);
    for (int i = 0; i < ncand; ++i)
      if (ok[i] == f) { p.pairs = f; return; }
  }
  if (lines < 64 || ncand == 1) {  // too few lines to time; keep the smallest tile that fits
    p.pairs = std::min(kDefaultPairs, ok[ncand - 1]);
    return;
  }
  DBuf<double> scratch;
  scratch.ensure((size_t)m0 * n * m2);
  fill_zero(scratch.p, scratch.n, s);
  cudaEvent_t e0, e1;
  VPMG_CUDA(cudaEventCreate(&e0));
  VPMG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  int pick = ok[0];
  for (int i = 0; i < ncand; ++i) {
    p.pairs = ok[i];
    const FFTDev d = dev_plan(p);
    launch_y(s, scratch.p, m0, n, m2, d);  // warm-up
    VPMG_CUDA(cudaEventRecord(e0, s));
    for (int r = 0; r < 3; ++r) launch_y(s, scratch.p, m0, n, m2, d);
    VPMG_CUDA(cudaEventRecord(e1, s));
    VPMG_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    VPMG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    count_launch(4);
    if (ms < best) { best = ms; pick = ok[i]; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  VPMG_CUDA(cudaGetLastError());
  p.pairs = pick;
}

}  // namespace

void make_fft_plan(FFTPlan& p, int n) {
  ensure_tables();
  p.n = n;
  p.N = n + 1;
  p.pairs = kDefaultPairs;
  p.rs = (p.N % 2 == 0) ? 1 : 0;
  p.M = p.rs ? p.N : 2 * p.N;
  // factor M: odd primes first (largest first), then 8s, a 4, a 2
  int m = p.M, twos = 0;
  std::vector<int> odd;
  while (m % 2 == 0) { m /= 2; ++twos; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) { odd.push_back(f); m /= f; }
  std::sort(odd.begin(), odd.end(), [](int a, int b) { return a > b; });
  p.nst = 0;
  for (int f : odd) {
    VPMG_CHECK(f <= kMaxOddRadix, VPMG_ERR_UNSUPPORTED, "mesh size has a prime factor > 17 in 2*(cells)");
    p.radix[p.nst++] = f;
  }
  while (twos >= 3) { p.radix[p.nst++] = 8; twos -= 3; }
  if (twos == 2) p.radix[p.nst++] = 4;
  if (twos == 1) p.radix[p.nst++] = 2;
  VPMG_CHECK(p.nst <= 24, VPMG_ERR_UNSUPPORTED, "too many FFT stages");
  std::vector<double2> h(p.M);
  for (int t = 0; t < p.M; ++t) {
    const double a = -2.0 * kPI * (double)t / (double)p.M;
    h[t] = make_double2(std::cos(a), std::sin(a));
  }
  std::vector<float4> hf(p.M);
  for (int t = 0; t < p.M; ++t) {
    const float2 r = host_split(h[t].x), i = host_split(h[t].y);
    hf[t] = make_float4(r.x, r.y, i.x, i.y);
  }
  p.tw.ensure(p.M);
  VPMG_CUDA(cudaMemcpy(p.tw.p, hf.data(), sizeof(float4) * p.M, cudaMemcpyHostToDevice));
  if (p.rs) {
    std::vector<double> sn(p.N);
    for (int j = 0; j < p.N; ++j) sn[j] = std::sin(kPI * (double)j / (double)p.N);
    p.sn.ensure(p.N);
    VPMG_CUDA(cudaMemcpy(p.sn.p, sn.data(), sizeof(double) * p.N, cudaMemcpyHostToDevice));
  }
}

void dirichlet_prepare(DirichletPlan& P, const int dims[3], const int box[6], const double h[3], cudaStream_t s) {
  bool same = P.ready;
  for (int d = 0; d < 3; ++d) same = same && P.dims[d] == dims[d] && P.h[d] == h[d];
  for (int d = 0; d < 6; ++d) same = same && P.box[d] == box[d];
  if (same) return;
  for (int d = 0; d < 3; ++d) { P.dims[d] = dims[d]; P.h[d] = h[d]; }
  for (int d = 0; d < 6; ++d) P.box[d] = box[d];
  for (int d = 0; d < 3; ++d) {
    P.m[d] = box[d + 3] - box[d] - 1;
    VPMG_CHECK(P.m[d] >= 1, VPMG_ERR_ARG, "Dirichlet box without interior");
  }
  make_fft_plan(P.fx, P.m[0]);
  make_fft_plan(P.fy, P.m[1]);
  VPMG_CHECK(std::max(smem_bytes(P.fx, 2), smem_bytes(P.fy, 2)) <= kMaxDstSmem, VPMG_ERR_UNSUPPORTED,
             "mesh too large for the shared-memory DST");
  tune_pairs(P.fx, P.m[1] * P.m[2], 1, P.m[0], P.m[1] * P.m[2], s);  // rows along x
  tune_pairs(P.fy, P.m[0] * P.m[2], P.m[0], P.m[1], P.m[2], s);      // columns along y
  // eigenvalues mu_p = 4 sin^2(pi p / 2N), pivots for d = 2 + hz^2 (mu_p/hx^2 + mu_q/hy^2)
  std::vector<double> mux(P.m[0]), muy(P.m[1]);
  for (int p = 0; p < P.m[0]; ++p) { const double sn = std::sin(kPI * (p + 1) / (2.0 * (P.m[0] + 1))); mux[p] = 4.0 * sn * sn; }
  for (int q = 0; q < P.m[1]; ++q) { const double sn = std::sin(kPI * (q + 1) / (2.0 * (P.m[1] + 1))); muy[q] = 4.0 * sn * sn; }
  DBuf<double> dmx, dmy;
  dmx.ensure(P.m[0]);
  dmy.ensure(P.m[1]);
  VPMG_CUDA(cudaMemcpy(dmx.p, mux.data(), sizeof(double) * P.m[0], cudaMemcpyHostToDevice));
  VPMG_CUDA(cudaMemcpy(dmy.p, muy.data(), sizeof(double) * P.m[1], cudaMemcpyHostToDevice));
  P.rinv.ensure((size_t)P.m[0] * P.m[1] * P.m[2]);
  P.rinvd.ensure((size_t)P.m[0] * P.m[1] * P.m[2]);
  const double hz2 = h[2] * h[2];
  const int nl = P.m[0] * P.m[1];
  k_pivots<<<(nl + 255) / 256, 256, 0, s>>>(P.rinv.p, P.rinvd.p, dmx.p, dmy.p, P.m[0], P.m[1], P.m[2], hz2 / (h[0] * h[0]),
                                            hz2 / (h[1] * h[1]));
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
  VPMG_CUDA(cudaStreamSynchronize(s));
  P.ready = true;
}

void dirichlet_solve(DirichletPlan& P, const double* rhs, double* sol, bool zero_bc, double* work, cudaStream_t s) {
  Box b;
  for (int d = 0; d < 3; ++d) { b.dims[d] = P.dims[d]; b.o[d] = P.box[d] + 1; b.m[d] = P.m[d]; }
  const FFTDev px = dev_plan(P.fx), py = dev_plan(P.fy);
  const double hx2 = P.h[0] * P.h[0], hy2 = P.h[1] * P.h[1], hz2 = P.h[2] * P.h[2];
  // Thomas RHS r = -hz^2 * ghat, with the inverse DST normalisation 4/(Nx Ny).
  const double scale = -hz2 * 4.0 / ((double)(P.m[0] + 1) * (double)(P.m[1] + 1));
  launch_x_fwd(s, rhs, sol, zero_bc ? 1 : 0, work, b, px, 1.0 / hx2, 1.0 / hy2, 1.0 / hz2, scale);
  launch_y(s, work, P.m[0], P.m[1], P.m[2], py);
  const int nl = P.m[0] * P.m[1];
  k_thomas<<<(nl + 127) / 128, 128, 0, s>>>(work, P.rinv.p, P.m[0], P.m[1], P.m[2]);
  launch_y(s, work, P.m[0], P.m[1], P.m[2], py);
  launch_x_inv(s, work, sol, b, px);
  count_launch(5);
  if (zero_bc) {
    k_zero_box_faces<<<256, 256, 0, s>>>(sol, b);
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}

// ----------------------------- pieces of a partially evaluated solve ----
// Forward x and y passes only: ghat = scale * DST_y DST_x (rhs - folded
// boundary values), the input of the Thomas sweep.
void dst_forward_xy(DirichletPlan& P, const double* rhs, const double* sol, bool zero_bc, double* ghat,
                    cudaStream_t s) {
  Box b;
  for (int d = 0; d < 3; ++d) { b.dims[d] = P.dims[d]; b.o[d] = P.box[d] + 1; b.m[d] = P.m[d]; }
  const FFTDev px = dev_plan(P.fx), py = dev_plan(P.fy);
  const double hx2 = P.h[0] * P.h[0], hy2 = P.h[1] * P.h[1], hz2 = P.h[2] * P.h[2];
  const double scale = dirichlet_scale(P);
  launch_x_fwd(s, rhs, sol, zero_bc ? 1 : 0, ghat, b, px, 1.0 / hx2, 1.0 / hy2, 1.0 / hz2, scale);
  launch_y(s, ghat, P.m[0], P.m[1], P.m[2], py);
  count_launch(2);
  VPMG_CUDA(cudaGetLastError());
}

double dirichlet_scale(const DirichletPlan& P) {
  const double hz2 = P.h[2] * P.h[2];
  return -hz2 * 4.0 / ((double)(P.m[0] + 1) * (double)(P.m[1] + 1));
}

// In-place DST-I along the middle axis of an m0 x m1 x m2 array (m1 = p.n).
// With m0 = 1 it transforms contiguous rows.
void dst_lines_y(const FFTPlan& p, double* data, int m0, int m1, int m2, cudaStream_t s) {
  if (m0 <= 0 || m2 <= 0) return;
  VPMG_CHECK(m1 == p.n, VPMG_ERR_ARG, "dst_lines_y: line length differs from the plan");
  launch_y(s, data, m0, m1, m2, dev_plan(p));
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

// Inverse DST-I along x of the m[0] x m[1] x m[2] array `data`; line (q, c)
// lands on nodes (o0 + k, o1 + q, o2 + c) of the node array sol (dims).
void dst_x_inv_to_box(const FFTPlan& p, const double* data, double* sol, const int dims[3], const int o[3],
                      const int m[3], cudaStream_t s) {
  if (m[1] <= 0 || m[2] <= 0) return;
  VPMG_CHECK(m[0] == p.n, VPMG_ERR_ARG, "dst_x_inv_to_box: line length differs from the plan");
  Box b;
  for (int d = 0; d < 3; ++d) { b.dims[d] = dims[d]; b.o[d] = o[d]; b.m[d] = m[d]; }
  launch_x_inv(s, data, sol, b, dev_plan(p));
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

// ------------------------------------------ allocation-free variant -----
// vpmg_dirichlet_static: the same five-kernel solve, with every temporary
// (DST work array, reciprocal pivot table, twiddles, eigenvalues) carved
// out of one file-scope device array instead of cudaMalloc'd buffers.
namespace {

constexpr size_t kStaticMaxInterior = (size_t)1 << 21;  // interior nodes (e.g. 128 x 128 x 128)
constexpr int kStaticMaxLine = 900;                     // interior nodes along x and along y
constexpr size_t kStaticTw = 2 * (kStaticMaxLine + 1);  // complex FFT length bound
constexpr size_t kStaticSn = kStaticMaxLine + 1;         // sin(pi j / N) table bound
// doubles: work | pivots | twiddles x (2 per complex) | twiddles y | mu x | mu y | sin x | sin y
constexpr size_t kStaticDoubles = 2 * kStaticMaxInterior + 4 * kStaticTw + 2 * kStaticMaxLine + 2 * kStaticSn;

// 33.6 MB per GPU that loads the library, held until the process exits.
__device__ __align__(256) double g_static_scratch[kStaticDoubles];

constexpr int kStaticMaxDevices = 64;
double* g_static_base[kStaticMaxDevices] = {nullptr};
bool g_static_consts[kStaticMaxDevices] = {false};

__global__ void k_static_tables(float4* __restrict__ twx, int mx, float4* __restrict__ twy, int my,
                                double* __restrict__ mux, int nx, double* __restrict__ muy, int ny,
                                double* __restrict__ snx, int sx, double* __restrict__ sny, int sy) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double sn, cs;
  if (t < sx) snx[t] = sinpi((double)t / sx);
  if (t < sy) sny[t] = sinpi((double)t / sy);
  if (t < mx) {
    sincospi(-2.0 * t / mx, &sn, &cs);
    twx[t] = ff::from_double2(make_double2(cs, sn));
  }
  if (t < my) {
    sincospi(-2.0 * t / my, &sn, &cs);
    twy[t] = ff::from_double2(make_double2(cs, sn));
  }
  if (t < nx) {
    sn = sinpi((t + 1) / (2.0 * (nx + 1)));
    mux[t] = 4.0 * sn * sn;
  }
  if (t < ny) {
    sn = sinpi((t + 1) / (2.0 * (ny + 1)));
    muy[t] = 4.0 * sn * sn;
  }
}

// Radix list of the DST-I of n points (no allocation), in the same form
// as make_fft_plan (real-symmetric for even N).
bool static_plan(int n, const float4* tw, const double* sn, FFTDev& d) {
  d.n = n;
  d.N = n + 1;
  d.rs = (d.N % 2 == 0) ? 1 : 0;
  d.M = d.rs ? d.N : 2 * d.N;
  d.tw = tw;
  d.sn = sn;
  int m = d.M, twos = 0, odd[24], no = 0;
  while (m % 2 == 0) { m /= 2; ++twos; }
  for (int f = 3; m > 1; f += 2)
    while (m % f == 0) {
      if (f > kMaxOddRadix || no >= 24) return false;
      odd[no++] = f;
      m /= f;
    }
  d.nst = 0;
  d.odd = no > 0 ? 1 : 0;
  for (int i = no - 1; i >= 0; --i) d.radix[d.nst++] = odd[i];  // largest first
  while (twos >= 3) { if (d.nst >= 24) return false; d.radix[d.nst++] = 8; twos -= 3; }
  if (twos == 2 && d.nst < 24) d.radix[d.nst++] = 4;
  if (twos == 1 && d.nst < 24) d.radix[d.nst++] = 2;
  return d.nst <= 24;
}

}  // namespace

}  // namespace vpmg

extern "C" int vpmg_dirichlet_static(const double* rhs, double* sol, const int dims[3], const int box[6],
                                     const double h[3], int zero_bc, void* stream) {
  using namespace vpmg;
  if (!rhs || !sol || !dims || !box || !h) return VPMG_ERR_ARG;
  int m[3];
  for (int d = 0; d < 3; ++d) {
    m[d] = box[d + 3] - box[d] - 1;
    if (box[d] < 0 || box[d + 3] >= dims[d] || m[d] < 1 || !(h[d] > 0.0)) return VPMG_ERR_ARG;
  }
  // sizes beyond the static scratch are refused, never truncated
  if (m[0] > kStaticMaxLine || m[1] > kStaticMaxLine || (size_t)m[0] * m[1] * m[2] > kStaticMaxInterior)
    return VPMG_ERR_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kStaticMaxDevices) {
    cudaGetLastError();
    return VPMG_ERR_CUDA;
  }
  // once per device, with that device current: the scratch's device address
  // and the odd-radix DFT constants
  if (!g_static_base[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return VPMG_ERR_CUDA;
    }
    g_static_base[dev] = static_cast<double*>(p);
  }
  if (!g_static_consts[dev]) {
    static float2 hc[(kMaxOddRadix + 1) * (kMaxOddRadix + 1)], hs[(kMaxOddRadix + 1) * (kMaxOddRadix + 1)];
    odd_radix_tables(hc, hs);
    if (cudaMemcpyToSymbol(c_rcos_f, hc, sizeof(hc)) != cudaSuccess ||
        cudaMemcpyToSymbol(c_rsin_f, hs, sizeof(hs)) != cudaSuccess) {
      cudaGetLastError();
      return VPMG_ERR_CUDA;
    }
    g_static_consts[dev] = true;
  }
  double* base = g_static_base[dev];
  double* work = base;
  float2* rinv = reinterpret_cast<float2*>(base + kStaticMaxInterior);  // 8 bytes per pivot
  float4* twx = reinterpret_cast<float4*>(base + 2 * kStaticMaxInterior);  // float-float twiddles, 16 B each
  float4* twy = twx + kStaticTw;
  double* mux = reinterpret_cast<double*>(twy + kStaticTw);
  double* muy = mux + kStaticMaxLine;
  double* snx = muy + kStaticMaxLine;
  double* sny = snx + kStaticSn;
  FFTDev px, py;
  if (!static_plan(m[0], twx, snx, px) || !static_plan(m[1], twy, sny, py)) return VPMG_ERR_UNSUPPORTED;
  px.pairs = py.pairs = kDefaultPairs;
  const int smax = 2 * kDefaultPairs * std::max(px.M, py.M) * (int)sizeof(double2);
  if (smax > 227 * 1024) return VPMG_ERR_UNSUPPORTED;
  if (raise_dst_smem_status((size_t)smax) != cudaSuccess) {
    cudaGetLastError();
    return VPMG_ERR_CUDA;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // tables and pivots are rebuilt on every call: the array keeps whatever the
  // previous call (possibly another grid) left in it
  const int nt = std::max(std::max(px.M, py.M), std::max(px.N, py.N));
  k_static_tables<<<(nt + 255) / 256, 256, 0, s>>>(twx, px.M, twy, py.M, mux, m[0], muy, m[1], snx,
                                                   px.rs ? px.N : 0, sny, py.rs ? py.N : 0);
  const double hz2 = h[2] * h[2], hx2 = h[0] * h[0], hy2 = h[1] * h[1];
  const int nl = m[0] * m[1];
  k_pivots<<<(nl + 255) / 256, 256, 0, s>>>(rinv, nullptr, mux, muy, m[0], m[1], m[2], hz2 / hx2, hz2 / hy2);
  Box b;
  for (int d = 0; d < 3; ++d) { b.dims[d] = dims[d]; b.o[d] = box[d] + 1; b.m[d] = m[d]; }
  const double scale = -hz2 * 4.0 / ((double)(m[0] + 1) * (double)(m[1] + 1));
  launch_x_fwd(s, rhs, sol, zero_bc ? 1 : 0, work, b, px, 1.0 / hx2, 1.0 / hy2, 1.0 / hz2, scale);
  launch_y(s, work, m[0], m[1], m[2], py);
  k_thomas<<<(nl + 127) / 128, 128, 0, s>>>(work, rinv, m[0], m[1], m[2]);
  launch_y(s, work, m[0], m[1], m[2], py);
  launch_x_inv(s, work, sol, b, px);
  if (zero_bc) k_zero_box_faces<<<256, 256, 0, s>>>(sol, b);
  if (cudaGetLastError() != cudaSuccess) return VPMG_ERR_CUDA;
  return VPMG_OK;
}
