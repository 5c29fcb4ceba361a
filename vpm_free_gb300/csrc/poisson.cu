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

#include "arith.cuh"
#include "fft_stages.cuh"
#include "vpmg_internal.h"

namespace vpmg {

namespace {

// Tile shape: a CTA of kThreads transforms PAIRS line pairs (2 * PAIRS real
// lines).  PAIRS is 2, 4 or 8, chosen per plan by timing (tune_pairs); the
// values computed do not depend on it.
constexpr int kThreads = 128;
constexpr int kDefaultPairs = 4;
constexpr int kMaxOddRadix = 17;  // largest odd prime with a specialised stage (larger: stage_generic)
constexpr int kRadixTab = (kMaxOddRadix + 1) * (kMaxOddRadix + 1);

// cos / sin (2 pi i / R) of the odd radices: FP64 and float-float copies
__constant__ double c_rcos_d[kRadixTab];
__constant__ double c_rsin_d[kRadixTab];
__constant__ float2 c_rcos_f[kRadixTab];
__constant__ float2 c_rsin_f[kRadixTab];

template <class A>
__device__ __forceinline__ typename A::R rcos(int i);
template <class A>
__device__ __forceinline__ typename A::R rsin(int i);
template <>
__device__ __forceinline__ double rcos<F64>(int i) { return c_rcos_d[i]; }
template <>
__device__ __forceinline__ double rsin<F64>(int i) { return c_rsin_d[i]; }
template <>
__device__ __forceinline__ float2 rcos<FF>(int i) { return c_rcos_f[i]; }
template <>
__device__ __forceinline__ float2 rsin<FF>(int i) { return c_rsin_f[i]; }

struct FFTDev {
  int n, N, M, nst;
  int odd;    // 1 if a stage has an odd radix
  int rs;     // 1: real-symmetric DST-I (M = N), 0: odd extension (M = 2N)
  int pairs;  // line pairs per CTA
  int arith;  // VPMG_ARITH_FP64 or VPMG_ARITH_FF48
  int radix[24];
  const double2* twd;  // e^{-2 pi i t / M}, FP64
  const float4* twf;   // the same as float-float (re.hi, re.lo, im.hi, im.lo)
  const double* sn;    // sin(pi j / N) (rs only)
};
template <class A>
__device__ __forceinline__ const typename A::C* twiddles(const FFTDev& p);
template <>
__device__ __forceinline__ const double2* twiddles<F64>(const FFTDev& p) { return p.twd; }
template <>
__device__ __forceinline__ const float4* twiddles<FF>(const FFTDev& p) { return p.twf; }

// Odd-radix stage in two phases, so that a transform's few butterflies
// (16 per radix-17 stage of a 272-point line) do not leave most threads
// idle: (A) one thread per butterfly folds its twiddled inputs into
// s_m = v_m + v_{R-m} and d_m = v_m - v_{R-m}, in place in the stage's input
// buffer (free after the stage), and writes X_0 = v_0 + sum s_m; (B) one
// thread per output pair q = 1..H reads x0, s_m, d_m back from shared
// memory and writes X_q and X_{R-q}:
//   X_q = x0 + sum_m [s_m cos(2 pi mq/R) - i d_m sin(2 pi mq/R)].
template <class A, int R>
__device__ __forceinline__ void stage_odd(typename A::C* __restrict__ in, typename A::C* __restrict__ out, int M,
                                          int Ns, const typename A::C* __restrict__ tw, int npair) {
  using C = typename A::C;
  using Re = typename A::R;
  constexpr int H = (R - 1) / 2;
  const int nbf = M / R;
  const int tws = M / (Ns * R);
  for (int t = threadIdx.x; t < npair * nbf; t += blockDim.x) {
    const int pr = t / nbf;
    const int j = t - pr * nbf;
    C* src = in + pr * M;
    const int k = j % Ns;
    const int base = (j - k) * R + k;
    C sum = src[j];
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      C a = src[j + m * nbf], b = src[j + (R - m) * nbf];
      if (Ns > 1) {
        a = A::cmul(a, __ldg(&tw[k * m * tws]));
        b = A::cmul(b, __ldg(&tw[k * (R - m) * tws]));
      }
      const C sm = A::cadd(a, b);
      src[j + m * nbf] = sm;
      src[j + (R - m) * nbf] = A::csub(a, b);
      sum = A::cadd(sum, sm);
    }
    out[pr * M + base] = sum;
  }
  __syncthreads();
  for (int t = threadIdx.x; t < npair * nbf * H; t += blockDim.x) {
    const int q = t % H + 1;
    const int bf = t / H;
    const int pr = bf / nbf;
    const int j = bf - pr * nbf;
    const C* src = in + pr * M;
    const int k = j % Ns;
    const int base = (j - k) * R + k;
    const C x0 = src[j];
    Re ar = A::re(x0), ai = A::im(x0), br = A::zero(), bi = A::zero();
#pragma unroll
    for (int m = 1; m <= H; ++m) {
      const C sm = src[j + m * nbf], dm = src[j + (R - m) * nbf];
      const int idx = (m * q) % R;
      const Re c = rcos<A>(R * (kMaxOddRadix + 1) + idx);
      const Re sn = rsin<A>(R * (kMaxOddRadix + 1) + idx);
      ar = A::fma(c, A::re(sm), ar);
      ai = A::fma(c, A::im(sm), ai);
      br = A::fma(sn, A::re(dm), br);
      bi = A::fma(sn, A::im(dm), bi);
    }
    C* dst = out + pr * M;
    dst[base + q * Ns] = A::cplx(A::add(ar, bi), A::sub(ai, br));
    dst[base + (R - q) * Ns] = A::cplx(A::sub(ar, bi), A::add(ai, br));
  }
}

// Radix-R stage for any odd prime R above kMaxOddRadix (the coarse grids
// of some meshes, e.g. 58 = 2 x 29 points): one thread per output, the
// direct DFT X_q = sum_m (w^{km} v_m) W_R^{mq}, its roots read from the
// plan's twiddles (W_R^s = tw[s M / R]).  R^2 products per butterfly; used
// only where no specialised stage exists.
template <class A>
__device__ __forceinline__ void stage_generic(const typename A::C* __restrict__ in, typename A::C* __restrict__ out,
                                              int M, int Ns, int R, const typename A::C* __restrict__ tw,
                                              int npair) {
  using C = typename A::C;
  const int nbf = M / R;
  const int tws = M / (Ns * R);
  const int rs = M / R;
  for (int t = threadIdx.x; t < npair * nbf * R; t += blockDim.x) {
    const int q = t % R;
    const int bf = t / R;
    const int pr = bf / nbf;
    const int j = bf - pr * nbf;
    const C* src = in + pr * M;
    const int k = j % Ns;
    C acc = src[j];
    for (int m = 1; m < R; ++m) {
      C v = src[j + m * nbf];
      if (Ns > 1) v = A::cmul(v, __ldg(&tw[k * m * tws]));
      acc = A::cadd(acc, A::cmul(v, __ldg(&tw[((m * q) % R) * rs])));
    }
    out[pr * M + (j - k) * R + k + q * Ns] = acc;
  }
}

// Runs all stages; returns the buffer holding the result.  ODD = false
// instantiates only the power-of-two radices, which keeps the register
// count (and so the occupancy) of those kernels independent of the large
// odd-radix butterflies.
template <class A, bool ODD>
__device__ typename A::C* fft_all(typename A::C* Abuf, typename A::C* Bbuf, const FFTDev& p, int npair) {
  using C = typename A::C;
  const C* tw = twiddles<A>(p);
  int Ns = 1;
  for (int s = 0; s < p.nst; ++s) {
    const int r = p.radix[s];
    switch (r) {
      case 2: stage<A, 2>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
      case 4: stage<A, 4>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
      case 8: stage<A, 8>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
      default:
        if constexpr (ODD) {
          switch (r) {
            case 3: stage_odd<A, 3>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
            case 5: stage_odd<A, 5>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
            case 7: stage_odd<A, 7>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
            case 11: stage_odd<A, 11>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
            case 13: stage_odd<A, 13>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
            case 17: stage_odd<A, 17>(Abuf, Bbuf, p.M, Ns, tw, npair); break;
            default: stage_generic<A>(Abuf, Bbuf, p.M, Ns, r, tw, npair); break;
          }
        }
        break;
    }
    __syncthreads();
    Ns *= r;
    C* t = Abuf;
    Abuf = Bbuf;
    Bbuf = t;
  }
  return Abuf;
}

// In place, the npair * M complex values of a buffer: FP64 -> the policy's
// complex type (same 16 bytes per value; nothing to do for F64).
template <class A>
__device__ __forceinline__ void to_arith(double2* z, int n) {
  if constexpr (A::kFF) {
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const double2 v = z[t];
      reinterpret_cast<typename A::C*>(z)[t] = A::from2(v);
    }
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
// The doubles enter the policy's arithmetic here.
template <class A>
__device__ __forceinline__ void rs_pre(const double2* __restrict__ L, typename A::C* __restrict__ Z, const FFTDev& p,
                                       int npair) {
  using C = typename A::C;
  using R = typename A::R;
  for (int t = threadIdx.x; t < npair * p.N; t += blockDim.x) {
    const int pr = t / p.N, j = t - pr * p.N;
    C z = A::cplx(A::zero(), A::zero());
    if (j > 0) {
      const C a = A::from2(L[pr * p.M + j]), b = A::from2(L[pr * p.M + p.N - j]);
      const R sj = A::from(__ldg(&p.sn[j]));
      z = A::cplx(A::fma(sj, A::add(A::re(a), A::re(b)), A::scale(A::sub(A::re(a), A::re(b)), 0.5f)),
                  A::fma(sj, A::add(A::im(a), A::im(b)), A::scale(A::sub(A::im(a), A::im(b)), 0.5f)));
    }
    Z[pr * p.M + j] = z;
  }
}

// Output side: Z is the length-N FFT of a packed pair.  With Z_m = a + ib,
// Z_{N-m} = c + id the two lines' spectra are F = ((a+c) + i(b-d))/2 and
// G = ((b+d) - i(a-c))/2, so X_{2m} = (d-b)/2 and (a-c)/2, and the odd
// outputs are the prefix sums of r_0 = Z_0 / 2, r_m = ((a+c)/2, (b+d)/2).
// O[pair * M + k] receives X_k of both lines, k = 1..n.
// The prefix sum runs over kScanSegs fixed segments of each line in a
// fixed order, so the result does not depend on the tile shape; Z is its
// scratch afterwards.
constexpr int kScanSegs = 32;
template <class A>
__device__ __forceinline__ void rs_post(typename A::C* __restrict__ Z, typename A::C* __restrict__ O, const FFTDev& p,
                                        int npair) {
  using C = typename A::C;
  using R = typename A::R;
  const int H = p.N >> 1;
  for (int t = threadIdx.x; t < npair * H; t += blockDim.x) {
    const int pr = t / H, m = t - pr * H;
    const C u = Z[pr * p.M + m];
    if (m == 0) {
      O[pr * p.M + 1] = A::cplx(A::scale(A::re(u), 0.5f), A::scale(A::im(u), 0.5f));
    } else {
      const C v = Z[pr * p.M + p.N - m];
      O[pr * p.M + 2 * m] = A::cplx(A::scale(A::sub(A::im(v), A::im(u)), 0.5f),
                                    A::scale(A::sub(A::re(u), A::re(v)), 0.5f));
      O[pr * p.M + 2 * m + 1] = A::cplx(A::scale(A::add(A::re(u), A::re(v)), 0.5f),
                                        A::scale(A::add(A::im(u), A::im(v)), 0.5f));
    }
  }
  __syncthreads();
  // segments per line: min(kScanSegs, H) -- a function of N only; the
  // scratch (2 npair S real values) fits in Z (npair M complex, M >= 2H >= 2S)
  const int S = min(kScanSegs, H);
  R* seg = reinterpret_cast<R*>(Z);  // [line][S]
  const int Cn = (H + S - 1) / S;
  const int nls = 2 * npair * S;
  for (int t = threadIdx.x; t < nls; t += blockDim.x) {  // segment sums
    const int line = t / S, g = t - line * S;
    const R* o = reinterpret_cast<const R*>(O + (line >> 1) * p.M) + (line & 1);  // X_k at o[2k]
    const int m0 = min(H, g * Cn), m1 = min(H, m0 + Cn);
    R sum = A::zero();
    for (int m = m0; m < m1; ++m) sum = A::add(sum, o[2 * (2 * m + 1)]);
    seg[t] = sum;
  }
  __syncthreads();
  for (int line = threadIdx.x; line < 2 * npair; line += blockDim.x) {  // exclusive scan of the segment sums
    R run = A::zero();
    for (int g = 0; g < S; ++g) {
      const R v = seg[line * S + g];
      seg[line * S + g] = run;
      run = A::add(run, v);
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nls; t += blockDim.x) {  // inclusive values inside each segment
    const int line = t / S, g = t - line * S;
    R* o = reinterpret_cast<R*>(O + (line >> 1) * p.M) + (line & 1);
    const int m0 = min(H, g * Cn), m1 = min(H, m0 + Cn);
    R run = seg[t];
    for (int m = m0; m < m1; ++m) {
      run = A::add(run, o[2 * (2 * m + 1)]);
      o[2 * (2 * m + 1)] = run;
    }
  }
}

// The transform of the 2*npair lines loaded into `L` (the staging buffer
// of the plan's mode, see staging()): returns the buffer holding X_k of
// line (pair, c) at index pair * M + k (k = 1..n) as component c (rs), or
// the raw odd-extension spectrum (X_k = -W.y / 2 and W.x / 2).
// The values in shared memory are in the policy's arithmetic from the
// pre-twiddle (or the odd extension) to the output; dst_out joins them
// back into doubles.
template <class A, bool ODD, int PAIRS>
__device__ __forceinline__ typename A::C* dst_pairs(double2* Ab, double2* Bb, const FFTDev& p) {
  using C = typename A::C;
  constexpr int npair = PAIRS;
  C* Af = reinterpret_cast<C*>(Ab);
  C* Bf = reinterpret_cast<C*>(Bb);
  if (p.rs) {
    rs_pre<A>(Bb, Af, p, npair);
  } else {
    odd_extend(Ab, p, npair);
    __syncthreads();
    to_arith<A>(Ab, npair * p.M);
  }
  __syncthreads();
  C* R = fft_all<A, ODD>(Af, Bf, p, npair);
  if (!p.rs) return R;
  C* O = (R == Af) ? Bf : Af;
  rs_post<A>(R, O, p, npair);
  __syncthreads();
  return O;
}
__device__ __forceinline__ double2* staging(double2* A, double2* B, const FFTDev& p) { return p.rs ? B : A; }
template <class A>
__device__ __forceinline__ double dst_out(const typename A::C* O, const FFTDev& p, int li, int k) {
  const typename A::C W = O[(li >> 1) * p.M + (k + 1)];
  if (p.rs) return A::to((li & 1) ? A::im(W) : A::re(W));
  return A::to((li & 1) ? A::scale(A::re(W), 0.5f) : A::scale(A::im(W), -0.5f));
}

// ------------------------------------------------------------ passes ----
struct Box {
  int dims[3];  // node array dims
  int o[3];     // node offset of interior (a,b,c) = (0,0,0)
  int m[3];     // interior counts
};

// x pass, forward: rhs (+ folded boundary values) -> work, scaled.
template <class Ar, bool ODD, int PAIRS>
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
  int nz = 0;
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
    nz |= v != 0.0;
    double* zp = reinterpret_cast<double*>(staging(A, B, p) + (li >> 1) * p.M + (a + 1));
    zp[li & 1] = v;
  }
  if (!__syncthreads_or(nz)) {
    // a tile of zero lines (a vorticity-free part of the box): its
    // transform is zero, no FFT needed
    for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
      const int l = l0 + t / n;
      if (l < nlines) work[(size_t)l * n + (t - (t / n) * n)] = 0.0;
    }
    return;
  }
  const typename Ar::C* R = dst_pairs<Ar, ODD, PAIRS>(A, B, p);
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, k = t - li * n;
    const int l = l0 + li;
    if (l >= nlines) continue;
    work[(size_t)l * n + k] = dst_out<Ar>(R, p, li, k);
  }
}

// y pass (forward or inverse): in place on work (m0 x m1 x m2, x fastest);
// `tile` = which 2 * PAIRS lines.
template <class Ar, bool ODD, int PAIRS>
__device__ __forceinline__ void y_body(double* __restrict__ work, int m0, int m1, int m2, const FFTDev& p,
                                       int tile) {
  extern __shared__ double2 smem[];
  double2* A = smem;
  double2* B = smem + PAIRS * p.M;
  const int nlines = m0 * m2;
  const int l0 = tile * (2 * PAIRS);
  const int n = p.n;  // == m1
  const size_t plane = (size_t)m0 * m1;
  int nz = 0;
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t % (2 * PAIRS), e = t / (2 * PAIRS);
    const int l = l0 + li;
    double v = 0.0;
    if (l < nlines) {
      const int a = l % m0, c = l / m0;
      v = work[(size_t)a + (size_t)m0 * e + plane * c];
    }
    nz |= v != 0.0;
    double* zp = reinterpret_cast<double*>(staging(A, B, p) + (li >> 1) * p.M + (e + 1));
    zp[li & 1] = v;
  }
  // zero lines (planes of the box without vorticity) transform to zero,
  // and the pass is in place: nothing to do
  if (!__syncthreads_or(nz)) return;
  const typename Ar::C* R = dst_pairs<Ar, ODD, PAIRS>(A, B, p);
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t % (2 * PAIRS), k = t / (2 * PAIRS);
    const int l = l0 + li;
    if (l >= nlines) continue;
    const int a = l % m0, c = l / m0;
    work[(size_t)a + (size_t)m0 * k + plane * c] = dst_out<Ar>(R, p, li, k);
  }
}
template <class Ar, bool ODD, int PAIRS>
__global__ void __launch_bounds__(kThreads) k_dst_y(double* __restrict__ work, int m0, int m1, int m2, FFTDev p) {
  y_body<Ar, ODD, PAIRS>(work, m0, m1, m2, p, blockIdx.x);
}

// x pass, inverse: work -> interior of sol.
template <class Ar, bool ODD, int PAIRS>
__device__ __forceinline__ void xinv_body(const double* __restrict__ work, double* __restrict__ sol, const Box& b,
                                          const FFTDev& p, int tile) {
  extern __shared__ double2 smem[];
  double2* A = smem;
  double2* B = smem + PAIRS * p.M;
  const int nlines = b.m[1] * b.m[2];
  const int l0 = tile * (2 * PAIRS);
  const int n = p.n;
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, a = t - li * n;
    const int l = l0 + li;
    const double v = (l < nlines) ? work[(size_t)l * n + a] : 0.0;
    double* zp = reinterpret_cast<double*>(staging(A, B, p) + (li >> 1) * p.M + (a + 1));
    zp[li & 1] = v;
  }
  __syncthreads();
  const typename Ar::C* R = dst_pairs<Ar, ODD, PAIRS>(A, B, p);
  const size_t sy = b.dims[0], sz = (size_t)b.dims[0] * b.dims[1];
  for (int t = threadIdx.x; t < 2 * PAIRS * n; t += blockDim.x) {
    const int li = t / n, k = t - li * n;
    const int l = l0 + li;
    if (l >= nlines) continue;
    const int q = l % b.m[1], c = l / b.m[1];
    sol[(size_t)(b.o[0] + k) + sy * (b.o[1] + q) + sz * (b.o[2] + c)] = dst_out<Ar>(R, p, li, k);
  }
}
template <class Ar, bool ODD, int PAIRS>
__global__ void __launch_bounds__(kThreads) k_dst_x_inv(const double* __restrict__ work, double* __restrict__ sol, Box b,
                                                        FFTDev p) {
  xinv_body<Ar, ODD, PAIRS>(work, sol, b, p, blockIdx.x);
}

// Several small transforms of one solve in one launch (the partially
// evaluated block solves have many of a few hundred lines each, too few to
// fill the GPU one launch at a time).  CTA blockIdx.x serves job j with
// tile0[j] <= blockIdx.x < tile0[j + 1].  The transform of a line does not
// depend on the launch it belongs to, so neither do the results.
constexpr int kMaxJobs = 8;
constexpr int kJobPairs = 2;
struct YJobs {
  int n;
  int tile0[kMaxJobs + 1];
  double* data[kMaxJobs];
  int m0[kMaxJobs], m1[kMaxJobs], m2[kMaxJobs];
  FFTDev p[kMaxJobs];
};
struct XJobs {
  int n;
  int tile0[kMaxJobs + 1];
  const double* work[kMaxJobs];
  double* sol[kMaxJobs];
  Box b[kMaxJobs];
  FFTDev p[kMaxJobs];
};
__device__ __forceinline__ int job_of(const int* tile0, int n) {
  int j = 0;
  while (j + 1 < n && (int)blockIdx.x >= tile0[j + 1]) ++j;
  return j;
}
template <class Ar, bool ODD>
__global__ void __launch_bounds__(kThreads) k_dst_y_jobs(const __grid_constant__ YJobs J) {
  const int j = job_of(J.tile0, J.n);
  y_body<Ar, ODD, kJobPairs>(J.data[j], J.m0[j], J.m1[j], J.m2[j], J.p[j], blockIdx.x - J.tile0[j]);
}
template <class Ar, bool ODD>
__global__ void __launch_bounds__(kThreads) k_dst_x_inv_jobs(const __grid_constant__ XJobs J) {
  const int j = job_of(J.tile0, J.n);
  xinv_body<Ar, ODD, kJobPairs>(J.work[j], J.sol[j], J.b[j], J.p[j], blockIdx.x - J.tile0[j]);
}

// z pass: Thomas sweep per (p,q) with the reciprocal pivot table (FP64:
// rinvd, float-float: rinvf), in the policy's arithmetic: the forward
// sweep leaves its values in place in that arithmetic, the backward sweep
// writes the doubles.  The column's loads are issued four planes ahead of
// the dependent chain (the sweep is latency-bound otherwise).
template <class A>
__global__ void k_thomas(double* __restrict__ g, const typename A::R* __restrict__ rinv, int m0, int m1, int m2) {
  using R = typename A::R;
  const int pq = blockIdx.x * blockDim.x + threadIdx.x;
  if (pq >= m0 * m1) return;
  const size_t plane = (size_t)m0 * m1;
  R* gf = reinterpret_cast<R*>(g);
  R y = A::from(g[pq]);
  gf[pq] = y;
  R ri = rinv[pq];
  int c = 1;
  for (; c + 3 < m2; c += 4) {
    const size_t id = pq + plane * c;
    const double g0 = g[id], g1 = g[id + plane], g2 = g[id + 2 * plane], g3 = g[id + 3 * plane];
    const R r0 = rinv[id], r1 = rinv[id + plane], r2 = rinv[id + 2 * plane], r3 = rinv[id + 3 * plane];
    y = A::fma(y, ri, A::from(g0));
    gf[id] = y;
    y = A::fma(y, r0, A::from(g1));
    gf[id + plane] = y;
    y = A::fma(y, r1, A::from(g2));
    gf[id + 2 * plane] = y;
    y = A::fma(y, r2, A::from(g3));
    gf[id + 3 * plane] = y;
    ri = r3;
  }
  for (; c < m2; ++c) {
    const size_t id = pq + plane * c;
    y = A::fma(y, ri, A::from(g[id]));
    gf[id] = y;
    ri = rinv[id];
  }
  R u = A::mul(y, ri);
  g[pq + plane * (m2 - 1)] = A::to(u);
  c = m2 - 2;
  for (; c - 3 >= 0; c -= 4) {
    const size_t id = pq + plane * c;
    const R g0 = gf[id], g1 = gf[id - plane], g2 = gf[id - 2 * plane], g3 = gf[id - 3 * plane];
    const R r0 = rinv[id], r1 = rinv[id - plane], r2 = rinv[id - 2 * plane], r3 = rinv[id - 3 * plane];
    u = A::mul(A::add(g0, u), r0);
    g[id] = A::to(u);
    u = A::mul(A::add(g1, u), r1);
    g[id - plane] = A::to(u);
    u = A::mul(A::add(g2, u), r2);
    g[id - 2 * plane] = A::to(u);
    u = A::mul(A::add(g3, u), r3);
    g[id - 3 * plane] = A::to(u);
  }
  for (; c >= 0; --c) {
    const size_t id = pq + plane * c;
    u = A::mul(A::add(gf[id], u), rinv[id]);
    g[id] = A::to(u);
  }
}

// Reciprocal pivots 1/d, 1/(d - r), ... in FP64, stored as doubles (rinvd)
// and as float-float pairs (rinvf); either may be null.
__global__ void k_pivots(float2* __restrict__ rinvf, double* __restrict__ rinvd, const double* __restrict__ mux,
                         const double* __restrict__ muy, int m0, int m1, int m2, double cx, double cy) {
  const int pq = blockIdx.x * blockDim.x + threadIdx.x;
  if (pq >= m0 * m1) return;
  const int p = pq % m0, q = pq / m0;
  const double d = 2.0 + (mux[p] * cx + muy[q] * cy);
  const size_t plane = (size_t)m0 * m1;
  double r = 1.0 / d;
  if (rinvf) rinvf[pq] = ff::split(r);
  if (rinvd) rinvd[pq] = r;
  for (int c = 1; c < m2; ++c) {
    r = 1.0 / (d - r);
    if (rinvf) rinvf[pq + plane * c] = ff::split(r);
    if (rinvd) rinvd[pq + plane * c] = r;
  }
}

void launch_thomas(cudaStream_t s, double* work, const DirichletPlan& P, int arith) {
  const int nl = P.m[0] * P.m[1];
  if (arith == VPMG_ARITH_FF48)
    k_thomas<FF><<<(nl + 127) / 128, 128, 0, s>>>(work, P.rinv.p, P.m[0], P.m[1], P.m[2]);
  else
    k_thomas<F64><<<(nl + 127) / 128, 128, 0, s>>>(work, P.rinvd.p, P.m[0], P.m[1], P.m[2]);
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

template <class A, int PAIRS>
void x_fwd_t(cudaStream_t s, const double* rhs, const double* sol, int zbc, double* work, Box b, FFTDev p,
             double ihx2, double ihy2, double ihz2, double scale) {
  const unsigned g = tile_grid(b.m[1] * b.m[2], p);
  if (p.odd)
    k_dst_x_fwd<A, true, PAIRS><<<g, kThreads, tile_smem(p), s>>>(rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else
    k_dst_x_fwd<A, false, PAIRS><<<g, kThreads, tile_smem(p), s>>>(rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
}
template <class A, int PAIRS>
void y_t(cudaStream_t s, double* work, int m0, int m1, int m2, FFTDev p) {
  const unsigned g = tile_grid(m0 * m2, p);
  if (p.odd) k_dst_y<A, true, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, m0, m1, m2, p);
  else k_dst_y<A, false, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, m0, m1, m2, p);
}
template <class A, int PAIRS>
void x_inv_t(cudaStream_t s, const double* work, double* sol, Box b, FFTDev p) {
  const unsigned g = tile_grid(b.m[1] * b.m[2], p);
  if (p.odd) k_dst_x_inv<A, true, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, sol, b, p);
  else k_dst_x_inv<A, false, PAIRS><<<g, kThreads, tile_smem(p), s>>>(work, sol, b, p);
}
template <class A>
void launch_x_fwd_a(cudaStream_t s, const double* rhs, const double* sol, int zbc, double* work, Box b, FFTDev p,
                    double ihx2, double ihy2, double ihz2, double scale) {
  if (p.pairs == 2) x_fwd_t<A, 2>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else if (p.pairs == 8) x_fwd_t<A, 8>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else x_fwd_t<A, 4>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
}
template <class A>
void launch_y_a(cudaStream_t s, double* work, int m0, int m1, int m2, FFTDev p) {
  if (p.pairs == 2) y_t<A, 2>(s, work, m0, m1, m2, p);
  else if (p.pairs == 8) y_t<A, 8>(s, work, m0, m1, m2, p);
  else y_t<A, 4>(s, work, m0, m1, m2, p);
}
template <class A>
void launch_x_inv_a(cudaStream_t s, const double* work, double* sol, Box b, FFTDev p) {
  if (p.pairs == 2) x_inv_t<A, 2>(s, work, sol, b, p);
  else if (p.pairs == 8) x_inv_t<A, 8>(s, work, sol, b, p);
  else x_inv_t<A, 4>(s, work, sol, b, p);
}
void launch_x_fwd(cudaStream_t s, const double* rhs, const double* sol, int zbc, double* work, Box b, FFTDev p,
                  double ihx2, double ihy2, double ihz2, double scale) {
  if (p.arith == VPMG_ARITH_FF48) launch_x_fwd_a<FF>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
  else launch_x_fwd_a<F64>(s, rhs, sol, zbc, work, b, p, ihx2, ihy2, ihz2, scale);
}
void launch_y(cudaStream_t s, double* work, int m0, int m1, int m2, FFTDev p) {
  if (p.arith == VPMG_ARITH_FF48) launch_y_a<FF>(s, work, m0, m1, m2, p);
  else launch_y_a<F64>(s, work, m0, m1, m2, p);
}
void launch_x_inv(cudaStream_t s, const double* work, double* sol, Box b, FFTDev p) {
  if (p.arith == VPMG_ARITH_FF48) launch_x_inv_a<FF>(s, work, sol, b, p);
  else launch_x_inv_a<F64>(s, work, sol, b, p);
}
template <class A, int PAIRS>
cudaError_t set_smem_t(int smax) {
  cudaError_t e = cudaSuccess;
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_fwd<A, true, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_fwd<A, false, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_y<A, true, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_y<A, false, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_inv<A, true, PAIRS>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_inv<A, false, PAIRS>, a, smax);
  return e;
}
template <class A>
cudaError_t set_jobs_smem(int smax) {
  cudaError_t e = cudaSuccess;
  const cudaFuncAttribute a = cudaFuncAttributeMaxDynamicSharedMemorySize;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_y_jobs<A, true>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_y_jobs<A, false>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_inv_jobs<A, true>, a, smax);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(k_dst_x_inv_jobs<A, false>, a, smax);
  return e;
}
cudaError_t set_dst_smem(int smax) {
  cudaError_t e = set_jobs_smem<F64>(smax);
  if (e == cudaSuccess) e = set_jobs_smem<FF>(smax);
  if (e == cudaSuccess) e = set_smem_t<F64, 2>(smax);
  if (e == cudaSuccess) e = set_smem_t<F64, 4>(smax);
  if (e == cudaSuccess) e = set_smem_t<F64, 8>(smax);
  if (e == cudaSuccess) e = set_smem_t<FF, 2>(smax);
  if (e == cudaSuccess) e = set_smem_t<FF, 4>(smax);
  if (e == cudaSuccess) e = set_smem_t<FF, 8>(smax);
  return e;
}

FFTDev dev_plan(const FFTPlan& p) {
  FFTDev d;
  d.n = p.n; d.N = p.N; d.M = p.M; d.nst = p.nst;
  d.rs = p.rs;
  d.pairs = p.pairs;
  d.arith = p.arith;
  d.sn = p.sn.p;
  d.odd = 0;
  for (int i = 0; i < 24; ++i) {
    d.radix[i] = p.radix[i];
    if (i < p.nst && (p.radix[i] & 1)) d.odd = 1;
  }
  d.twd = p.twd.p;
  d.twf = p.tw.p;
  return d;
}

// A double as a float-float pair (hi = v rounded to float, lo = the rest).
float2 host_split(double v) {
  const float hi = (float)v;
  return make_float2(hi, (float)(v - (double)hi));
}

// cos / sin (2 pi i / R) of the odd radices, in FP64 and as float-float.
void odd_radix_tables(double* dc, double* ds, float2* hc, float2* hs) {
  for (int R = 1; R <= kMaxOddRadix; ++R)
    for (int i = 0; i < R; ++i) {
      const int k = R * (kMaxOddRadix + 1) + i;
      dc[k] = std::cos(2.0 * kPI * i / R);
      ds[k] = std::sin(2.0 * kPI * i / R);
      hc[k] = host_split(dc[k]);
      hs[k] = host_split(ds[k]);
    }
}

// The odd-radix constants live in __constant__ memory, held separately on
// every device: uploaded once per device, with that device current, by the
// plans and by the allocation-free entry point alike.  The copies come from
// pageable host memory, so the device is synchronised before the tables
// are marked ready: kernels on any stream then see the whole tables.
constexpr int kMaxDevices = 64;
bool g_tables_ready[kMaxDevices] = {false};
cudaError_t ensure_tables_status() {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  if (g_tables_ready[dev]) return cudaSuccess;
  static double dc[kRadixTab], ds[kRadixTab];
  static float2 hc[kRadixTab], hs[kRadixTab];
  odd_radix_tables(dc, ds, hc, hs);
  if ((e = cudaMemcpyToSymbol(c_rcos_d, dc, sizeof(dc))) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_rsin_d, ds, sizeof(ds))) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_rcos_f, hc, sizeof(hc))) != cudaSuccess) return e;
  if ((e = cudaMemcpyToSymbol(c_rsin_f, hs, sizeof(hs))) != cudaSuccess) return e;
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return e;
  g_tables_ready[dev] = true;
  return cudaSuccess;
}
void ensure_tables() { VPMG_CUDA(ensure_tables_status()); }

size_t smem_bytes(const FFTPlan& p, int pairs) { return (size_t)2 * pairs * p.M * sizeof(double2); }
constexpr size_t kMaxDstSmem = 227 * 1024;

// The DST kernels' shared-memory limit is an attribute of each kernel on
// each device, shared by every plan and by the allocation-free entry
// point: it is only ever raised (set-up time, outside any stream capture).
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

void make_fft_plan(FFTPlan& p, int n, int arith) {
  ensure_tables();
  p.arith = arith;
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
  for (int f : odd) p.radix[p.nst++] = f;  // primes above 17 take the generic direct-DFT stage
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
  p.twd.ensure(p.M);
  VPMG_CUDA(cudaMemcpy(p.twd.p, h.data(), sizeof(double2) * p.M, cudaMemcpyHostToDevice));
  if (p.rs) {
    std::vector<double> sn(p.N);
    for (int j = 0; j < p.N; ++j) sn[j] = std::sin(kPI * (double)j / (double)p.N);
    p.sn.ensure(p.N);
    VPMG_CUDA(cudaMemcpy(p.sn.p, sn.data(), sizeof(double) * p.N, cudaMemcpyHostToDevice));
  }
}

void dirichlet_prepare(DirichletPlan& P, const int dims[3], const int box[6], const double h[3], cudaStream_t s,
                       int arith) {
  VPMG_CHECK(arith == VPMG_ARITH_FP64 || arith == VPMG_ARITH_FF48, VPMG_ERR_ARG, "unknown arithmetic");
  bool same = P.ready && P.arith == arith;
  for (int d = 0; d < 3; ++d) same = same && P.dims[d] == dims[d] && P.h[d] == h[d];
  for (int d = 0; d < 6; ++d) same = same && P.box[d] == box[d];
  if (same) return;
  for (int d = 0; d < 3; ++d) { P.dims[d] = dims[d]; P.h[d] = h[d]; }
  for (int d = 0; d < 6; ++d) P.box[d] = box[d];
  P.arith = arith;
  for (int d = 0; d < 3; ++d) {
    P.m[d] = box[d + 3] - box[d] - 1;
    VPMG_CHECK(P.m[d] >= 1, VPMG_ERR_ARG, "Dirichlet box without interior");
  }
  make_fft_plan(P.fx, P.m[0], arith);
  make_fft_plan(P.fy, P.m[1], arith);
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
  launch_thomas(s, work, P, P.arith);
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

// Job lists: several small transforms in one launch (tiles of kJobPairs line
// pairs; all jobs in the plans' common arithmetic).
void dst_lines_y_jobs(const DstYLines* jobs, int n, cudaStream_t s) {
  VPMG_CHECK(n >= 1 && n <= kMaxJobs, VPMG_ERR_ARG, "dst_lines_y_jobs: 1..8 jobs");
  YJobs J{};
  J.n = n;
  int tiles = 0, odd = 0, arith = jobs[0].plan->arith;
  size_t smem = 0;
  for (int j = 0; j < n; ++j) {
    const DstYLines& q = jobs[j];
    VPMG_CHECK(q.m1 == q.plan->n && q.plan->arith == arith, VPMG_ERR_ARG, "dst_lines_y_jobs: plan mismatch");
    J.tile0[j] = tiles;
    J.data[j] = q.data; J.m0[j] = q.m0; J.m1[j] = q.m1; J.m2[j] = q.m2;
    J.p[j] = dev_plan(*q.plan);
    J.p[j].pairs = kJobPairs;
    odd |= J.p[j].odd;
    tiles += (q.m0 * q.m2 + 2 * kJobPairs - 1) / (2 * kJobPairs);
    smem = std::max(smem, (size_t)2 * kJobPairs * J.p[j].M * sizeof(double2));
  }
  J.tile0[n] = tiles;
  if (tiles == 0) return;
  if (arith == VPMG_ARITH_FF48) {
    if (odd) k_dst_y_jobs<FF, true><<<tiles, kThreads, smem, s>>>(J);
    else k_dst_y_jobs<FF, false><<<tiles, kThreads, smem, s>>>(J);
  } else {
    if (odd) k_dst_y_jobs<F64, true><<<tiles, kThreads, smem, s>>>(J);
    else k_dst_y_jobs<F64, false><<<tiles, kThreads, smem, s>>>(J);
  }
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void dst_x_inv_jobs(const DstXInvLines* jobs, int n, cudaStream_t s) {
  VPMG_CHECK(n >= 1 && n <= kMaxJobs, VPMG_ERR_ARG, "dst_x_inv_jobs: 1..8 jobs");
  XJobs J{};
  J.n = n;
  int tiles = 0, odd = 0, arith = jobs[0].plan->arith;
  size_t smem = 0;
  for (int j = 0; j < n; ++j) {
    const DstXInvLines& q = jobs[j];
    VPMG_CHECK(q.m[0] == q.plan->n && q.plan->arith == arith, VPMG_ERR_ARG, "dst_x_inv_jobs: plan mismatch");
    J.tile0[j] = tiles;
    J.work[j] = q.data;
    J.sol[j] = q.sol;
    for (int d = 0; d < 3; ++d) { J.b[j].dims[d] = q.dims[d]; J.b[j].o[d] = q.o[d]; J.b[j].m[d] = q.m[d]; }
    J.p[j] = dev_plan(*q.plan);
    J.p[j].pairs = kJobPairs;
    odd |= J.p[j].odd;
    tiles += (q.m[1] * q.m[2] + 2 * kJobPairs - 1) / (2 * kJobPairs);
    smem = std::max(smem, (size_t)2 * kJobPairs * J.p[j].M * sizeof(double2));
  }
  J.tile0[n] = tiles;
  if (tiles == 0) return;
  if (arith == VPMG_ARITH_FF48) {
    if (odd) k_dst_x_inv_jobs<FF, true><<<tiles, kThreads, smem, s>>>(J);
    else k_dst_x_inv_jobs<FF, false><<<tiles, kThreads, smem, s>>>(J);
  } else {
    if (odd) k_dst_x_inv_jobs<F64, true><<<tiles, kThreads, smem, s>>>(J);
    else k_dst_x_inv_jobs<F64, false><<<tiles, kThreads, smem, s>>>(J);
  }
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

__global__ void k_static_tables(double2* __restrict__ twx, int mx, double2* __restrict__ twy, int my,
                                double* __restrict__ mux, int nx, double* __restrict__ muy, int ny,
                                double* __restrict__ snx, int sx, double* __restrict__ sny, int sy) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  double sn, cs;
  if (t < sx) snx[t] = sinpi((double)t / sx);
  if (t < sy) sny[t] = sinpi((double)t / sy);
  if (t < mx) {
    sincospi(-2.0 * t / mx, &sn, &cs);
    twx[t] = make_double2(cs, sn);
  }
  if (t < my) {
    sincospi(-2.0 * t / my, &sn, &cs);
    twy[t] = make_double2(cs, sn);
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
bool static_plan(int n, const double2* tw, const double* sn, FFTDev& d) {
  d.n = n;
  d.N = n + 1;
  d.rs = (d.N % 2 == 0) ? 1 : 0;
  d.M = d.rs ? d.N : 2 * d.N;
  d.arith = VPMG_ARITH_FP64;
  d.twd = tw;
  d.twf = nullptr;
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
  if (ensure_tables_status() != cudaSuccess) {
    cudaGetLastError();
    return VPMG_ERR_CUDA;
  }
  // FP64 throughout, as the handle-based solves by default
  double* base = g_static_base[dev];
  double* work = base;
  double* rinv = base + kStaticMaxInterior;                                  // reciprocal pivots
  double2* twx = reinterpret_cast<double2*>(base + 2 * kStaticMaxInterior);  // twiddles, 16 B each
  double2* twy = twx + kStaticTw;
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
  k_pivots<<<(nl + 255) / 256, 256, 0, s>>>(nullptr, rinv, mux, muy, m[0], m[1], m[2], hz2 / hx2, hz2 / hy2);
  Box b;
  for (int d = 0; d < 3; ++d) { b.dims[d] = dims[d]; b.o[d] = box[d] + 1; b.m[d] = m[d]; }
  const double scale = -hz2 * 4.0 / ((double)(m[0] + 1) * (double)(m[1] + 1));
  launch_x_fwd(s, rhs, sol, zero_bc ? 1 : 0, work, b, px, 1.0 / hx2, 1.0 / hy2, 1.0 / hz2, scale);
  launch_y(s, work, m[0], m[1], m[2], py);
  k_thomas<F64><<<(nl + 127) / 128, 128, 0, s>>>(work, rinv, m[0], m[1], m[2]);
  launch_y(s, work, m[0], m[1], m[2], py);
  launch_x_inv(s, work, sol, b, px);
  if (zero_bc) k_zero_box_faces<<<256, 256, 0, s>>>(sol, b);
  if (cudaGetLastError() != cudaSuccess) return VPMG_ERR_CUDA;
  return VPMG_OK;
}
