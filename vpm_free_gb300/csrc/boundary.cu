// boundary.cu -- infinite-domain boundary values on the GPU.
//
// Replaces infdomain_3d after its zero-BC solve (source/pinfdomain.f90:86-158):
//   * calc_normalderiv_3d (pinfdomain.f90:294-547): 4th-order one-sided
//     normal derivative at the 4 corners of every boundary cell -> panel
//     source strengths;
//   * build_level_nbound_3d (pinfdomain.f90:875-1530): area-weighted source
//     of every quadtree cell (topology and geometry come from the host);
//   * Bounds3d_lev / tree_calc_3d (pmbound.f90:980-1249): for every
//     boundary node, sum of -s dS / r over the tree with the opening test
//     r < 10 sqrt(dS), then SOL += sum / (4 pi)  (ibctyp = 2);
//   * ibctyp = 3, constant-source panels: tree_calc_3d_s
//     (pmbound.f90:1379-1501) and the untreed calc_boundinf_3d_s
//     (pmbound.f90:520-648), whose unopened cells contribute the panel
//     potential FSOUR_A4 (pmbound.f90:1540-1620) where the reference calls it.
// The walk is evaluated with explicitly rounded operations so its opening
// decisions are those of the reference's expressions.  Because the mesh is
// frozen after the first step, the walk's interaction list (cell, dS/r) is
// the same every step: when it fits the memory budget it is recorded once
// (count + fill passes) and each step is a CSR product with the three
// source components.  The product runs in float-float arithmetic: weights
// and sources are stored as pairs of floats (hi + lo, a 48-bit mantissa),
// products are split exactly with an FMA and sums are error-free
// (two-sum), so the FP32 pipes, about thirty times GB300's FP64 rate, do
// the work; each lane's partial sum is converted to FP64 before the warp
// reduction.  The relative error stays near 1e-14, and the product is
// bound by the 12 bytes per interaction it streams from HBM.
#include <algorithm>
#include <cmath>

#include "ff.cuh"
#include "tree_host.h"
#include "vpmg_internal.h"

namespace vpmg {

namespace {

constexpr int kMaxLev = 16;

struct WalkDev {
  const double *cx, *cy, *cz, *cds, *cthr;
  const int* child;
  const int* flags;
  const double* s0;
  const double* s1;
  const double* s2;
  const int* tgt_node;
  const double *tx, *ty, *tz;
  int top0, ntop, levmax, ntarget;
  double lg;      // log((sqrt2-1)/(sqrt2+1))
  double inv_pi4, pi4;
  int bctype;     // 2 or 3
  int tree;       // 1: Bounds3d_lev walk; 0: untreed sum (levmax = 0)
  int dense;      // 1: the coarsest level goes to the dense block (count / fill)
  int ff;         // 1: recorded weights as float-float pairs, 0: as doubles
  const int* tgt_frame;
  PanelFrame frame[6];
};

// FSOUR_A4 (source/pmbound.f90:1540-1620) with NSIDE = 0, ISING = 0,
// EPSS = 1e-14: potential at XO of a flat quadrilateral of unit constant
// source centred at RG, corners (S, T) in the frame (E1, E2, E3) of the
// target's plane.  Sums and products are explicitly rounded in the
// reference's order so the RATIO > 10 branch and the near-edge
// |A1*A2| < TINY cut decide as its expressions do.
__device__ double fsour_a4(const double XO[3], const double RG[3], const PanelFrame& F, double AREA, double PI4) {
  const double COSB[4] = {0.0, 1.0, 0.0, -1.0}, SINB[4] = {1.0, 0.0, -1.0, 0.0};
  const double TINY = 1e-10, EPSS = 1e-14;
  const double d0 = __dsub_rn(XO[0], RG[0]), d1 = __dsub_rn(XO[1], RG[1]), d2 = __dsub_rn(XO[2], RG[2]);
  const double X = __dadd_rn(__dadd_rn(__dmul_rn(d0, F.E1[0]), __dmul_rn(d1, F.E1[1])), __dmul_rn(d2, F.E1[2]));
  const double Y = __dadd_rn(__dadd_rn(__dmul_rn(d0, F.E2[0]), __dmul_rn(d1, F.E2[1])), __dmul_rn(d2, F.E2[2]));
  double Z = __dadd_rn(__dadd_rn(__dmul_rn(d0, F.E3[0]), __dmul_rn(d1, F.E3[1])), __dmul_rn(d2, F.E3[2]));
  const double RO = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(X, X), __dmul_rn(Y, Y)), __dmul_rn(Z, Z)));
  if (__ddiv_rn(RO, F.diag) > 10.0) return -__ddiv_rn(__ddiv_rn(AREA, PI4), RO);
  const double ZP = (Z < 0.0) ? -1.0 : 1.0;
  double AZ = fmax(EPSS, fabs(Z));
  Z = __dmul_rn(AZ, ZP);
  const double ZK = __dmul_rn(Z, Z);
  double R[4], E[4], H[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const double xs = __dsub_rn(X, F.S[k]), yt = __dsub_rn(Y, F.T[k]);
    const double XK = __dmul_rn(xs, xs), YK = __dmul_rn(yt, yt);
    H[k] = __dmul_rn(xs, yt);
    R[k] = __dsqrt_rn(__dadd_rn(__dadd_rn(XK, YK), ZK));
    E[k] = __dadd_rn(ZK, XK);
  }
  double FIL = 0.0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int k2 = (k == 3) ? 0 : k + 1;
    const double rr = __dadd_rn(R[k], R[k2]);
    const double A2 = __dadd_rn(rr, F.D[k]), A1 = __dsub_rn(rr, F.D[k]);
    if (fabs(__dmul_rn(A1, A2)) < TINY) continue;
    const double AK = log(__ddiv_rn(A1, A2));
    const double TOO = __dadd_rn(__dmul_rn(-__dsub_rn(X, F.S[k]), SINB[k]), __dmul_rn(__dsub_rn(Y, F.T[k]), COSB[k]));
    FIL = __dsub_rn(FIL, __dmul_rn(TOO, AK));
  }
  AZ = fmax(TINY, AZ);
  Z = __dmul_rn(AZ, ZP);
  double UL3 = 0.0;
#pragma unroll
  for (int k = 1; k < 4; k += 2) {  // COSB != 0 on sides 2 and 4 only
    const int k2 = (k == 3) ? 0 : k + 1;
    const double zc = __dmul_rn(Z, COSB[k]);
    const double t1 = atan(__ddiv_rn(__dsub_rn(__dmul_rn(SINB[k], E[k]), __dmul_rn(COSB[k], H[k])), __dmul_rn(zc, R[k])));
    const double t2 =
        atan(__ddiv_rn(__dsub_rn(__dmul_rn(SINB[k], E[k2]), __dmul_rn(COSB[k], H[k2])), __dmul_rn(zc, R[k2])));
    UL3 = __dsub_rn(__dadd_rn(UL3, t1), t2);
  }
  return __ddiv_rn(__dadd_rn(FIL, __dmul_rn(Z, UL3)), PI4);
}

enum { kAccum = 0, kCount = 1, kFill = 2, kTranspose = 3 };

// With W.dense, kCount counts only the finer levels (and adds the coarsest
// level's accepted cells to *dcount) and kFill writes the coarsest level
// into the dense block wtop.
template <int MODE>
__global__ void k_walk(WalkDev W, double* __restrict__ o0, double* __restrict__ o1, double* __restrict__ o2,
                       int* __restrict__ counts, const long long* __restrict__ rowptr, int* __restrict__ col,
                       float2* __restrict__ wgt, float2* __restrict__ wtop = nullptr,
                       unsigned long long* __restrict__ dcount = nullptr) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= W.ntarget) return;
  const double X = W.tx[t], Y = W.ty[t], Z = W.tz[t];
  int parent[kMaxLev], pos[kMaxLev], cnt[kMaxLev];
  int L = W.levmax;
  pos[L] = 0;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  int ni = 0, nd = 0;
  long long out = 0;
  if (MODE == kFill) out = rowptr[t];
  double bcv = 0.0;  // transpose: o1 is the adjoint of the boundary values, o0 the cell adjoints
  if (MODE == kTranspose) bcv = -W.inv_pi4 * o1[W.tgt_node[t]];
  while (true) {
    int c;
    if (L == W.levmax) {
      if (pos[L] >= W.ntop) break;
      c = W.top0 + pos[L]++;
    } else {
      if (pos[L] >= cnt[L]) {
        ++L;
        continue;
      }
      c = W.child[4 * parent[L] + pos[L]++];
    }
    const double XR = __dsub_rn(W.cx[c], X), YR = __dsub_rn(W.cy[c], Y), ZR = __dsub_rn(W.cz[c], Z);
    const double r = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(XR, XR), __dmul_rn(YR, YR)), __dmul_rn(ZR, ZR)));
    const int fl = W.flags[c];
    // ibctyp 3 (tree_calc_3d_s) tests r / sqrt(dS) < 10 and always opens
    // only the -1 dummies; a -2 dummy has dS = 0 and is never opened.
    const bool open = (W.bctype == 3) ? ((__ddiv_rn(r, __dsqrt_rn(W.cds[c])) < 10.0 && L > 0) || fl == -1)
                                      : ((r < W.cthr[c] && L > 0) || fl < 0);
    if (open) {
      parent[L - 1] = c;
      cnt[L - 1] = (fl < 0) ? 2 : 4;
      pos[L - 1] = 0;
      --L;
      continue;
    }
    if (MODE == kCount) {
      if (W.dense && L == W.levmax) ++nd;
      else ++ni;
      continue;
    }
    const double DS = W.cds[c];
    double w;
    int cc = c;
    if (W.bctype == 3) {
      if (L == W.levmax) {
        // coarsest level: FSOUR_A4 of the cell (area dS in the tree, the
        // target plane's cell area in the untreed sum), weighting the
        // source of the walk's start cell nv = 1 in the tree
        // (pmbound.f90:1492-1496) and the cell's own in the untreed sum
        const PanelFrame& F = W.frame[W.tgt_frame[t]];
        const double XO[3] = {X, Y, Z}, RG[3] = {W.cx[c], W.cy[c], W.cz[c]};
        const double fis = fsour_a4(XO, RG, F, W.tree ? DS : F.area, W.pi4);
        w = -fis * W.pi4;
        if (W.tree) cc = W.top0;
      } else {
        w = __ddiv_rn(DS, r);
      }
    } else {
      w = (r > 1e-05) ? __ddiv_rn(DS, r) : -2.0 * __dsqrt_rn(DS) * W.lg;
    }
    if (MODE == kFill) {
      // the weight word: the double itself, or its float-float pair
      const float hi = __double2float_rn(w);
      const float2 wf = make_float2(hi, __double2float_rn(w - (double)hi));
      const double word = W.ff ? *reinterpret_cast<const double*>(&wf) : w;
      if (W.dense && L == W.levmax) {
        const int cc2 = c - W.top0;  // [chunk][cell pair][lane][2]
        reinterpret_cast<double*>(wtop)[(((size_t)(t >> 5) * ((W.ntop + 1) >> 1) + (cc2 >> 1)) * 32 + (t & 31)) * 2 +
                                         (cc2 & 1)] = word;
      } else {
        col[out] = cc;
        reinterpret_cast<double*>(wgt)[out] = word;
        ++out;
      }
    } else if (MODE == kTranspose) {
      if (bcv != 0.0) atomicAdd(&o0[cc], w * bcv);
    } else {
      a0 = fma(-W.s0[cc], w, a0);
      a1 = fma(-W.s1[cc], w, a1);
      a2 = fma(-W.s2[cc], w, a2);
    }
  }
  if (MODE == kCount) {
    counts[t] = ni;
    if (nd) atomicAdd(dcount, (unsigned long long)nd);
  } else if (MODE == kAccum) {
    const int node = W.tgt_node[t];
    o0[node] += a0 * W.inv_pi4;
    o1[node] += a1 * W.inv_pi4;
    o2[node] += a2 * W.inv_pi4;
  }
}

// Float-float accumulate acc += w * s: the hi product and its exact error
// (FMA), the cross terms, an error-free two-sum into acc.hi and the errors
// into acc.lo.  Explicitly rounded intrinsics keep the compiler from
// fusing the two-sum's operations.
struct FF {
  float hi = 0.0f, lo = 0.0f;
};
__device__ __forceinline__ void ff_mac(FF& a, float2 w, float2 s) {
  const float ph = __fmul_rn(w.x, s.x);
  float pe = __fmaf_rn(w.x, s.x, -ph);
  pe = __fmaf_rn(w.x, s.y, pe);
  pe = __fmaf_rn(w.y, s.x, pe);
  const float t = __fadd_rn(a.hi, ph);
  const float bp = __fsub_rn(t, a.hi);
  const float er = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(t, bp)), __fsub_rn(ph, bp));
  a.lo = __fadd_rn(a.lo, __fadd_rn(er, pe));
  a.hi = t;
}

// Multiply-accumulate policies of the recorded operator's kernels.  A
// weight is 8 bytes (W), a cell's packed sources (s0, s1, s2, 0) are 32
// bytes read as two 16-byte halves (H), each holding two values (V).
//   MacFF: float-float pairs, products and sums on the FP32 pipes;
//   Mac64: IEEE FP64, one DFMA per product (the reference's arithmetic).
struct MacFF {
  using W = float2;
  using V = float2;
  using H = float4;
  using W2 = float4;  // two weights (cells 2i, 2i+1 of the dense block)
  using Acc = FF;
  static constexpr bool kFF = true;
  __device__ __forceinline__ static V v0(H h) { return make_float2(h.x, h.y); }
  __device__ __forceinline__ static V v1(H h) { return make_float2(h.z, h.w); }
  __device__ __forceinline__ static W wa(W2 w) { return make_float2(w.x, w.y); }
  __device__ __forceinline__ static W wb(W2 w) { return make_float2(w.z, w.w); }
  __device__ __forceinline__ static void mac(Acc& a, W w, V x) { ff_mac(a, w, x); }
  __device__ __forceinline__ static double fin(const Acc& a) { return (double)a.hi + (double)a.lo; }
  __device__ __forceinline__ static V vmake(double d) {  // rounded hi, then the rest
    const float hi = __double2float_rn(d);
    return make_float2(hi, __double2float_rn(d - (double)hi));
  }
  __device__ __forceinline__ static V vsplit(double d) { return ff::split(d); }
};
struct Acc64 {
  double v = 0.0;
};
struct Mac64 {
  using W = double;
  using V = double;
  using H = double2;
  using W2 = double2;
  using Acc = Acc64;
  static constexpr bool kFF = false;
  __device__ __forceinline__ static V v0(H h) { return h.x; }
  __device__ __forceinline__ static V v1(H h) { return h.y; }
  __device__ __forceinline__ static W wa(W2 w) { return w.x; }
  __device__ __forceinline__ static W wb(W2 w) { return w.y; }
  __device__ __forceinline__ static void mac(Acc& a, W w, V x) { a.v = fma(w, x, a.v); }
  __device__ __forceinline__ static double fin(const Acc& a) { return a.v; }
  __device__ __forceinline__ static V vmake(double d) { return d; }
  __device__ __forceinline__ static V vsplit(double d) { return d; }
};

// Sources in the policy's arithmetic, once per apply, packed per cell as
// (s0, s1, s2, 0): one 32-byte sector serves a gather of all components.
template <class M>
__global__ void k_split(const double* __restrict__ x, int ncell, typename M::V* __restrict__ out) {
  const size_t n = 4 * (size_t)ncell;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cell = (int)(i >> 2), comp = (int)(i & 3);
    out[i] = M::vmake(comp < 3 ? x[(size_t)comp * ncell + cell] : 0.0);
  }
}

// The coarsest level's dense block: a warp per 32 targets walks the level's
// cells in order.  Each lane's weights for cells (2i, 2i+1) sit together
// (one 16-byte load per lane, 512 coalesced bytes per warp load), and the
// block stages the cells' packed sources in shared memory a tile at a
// time, so the warps read them as broadcasts.
constexpr int kDenseTile = 512;  // cells per staged tile (16 KB of sources)
// blockIdx.y = segment of cseg (even) cells; its partial sums go to
// dsum[segment][component][node] (more, shorter warps: a fuller last wave).
template <class M>
__global__ void __launch_bounds__(256) k_apply_dense(const typename M::W2* __restrict__ wtop,
                                                     const typename M::H* __restrict__ src, int top0, int ntop,
                                                     int ntop2, int ntarget, int cseg, double* __restrict__ dsum) {
  using H = typename M::H;
  using W2 = typename M::W2;
  __shared__ H ss[2 * kDenseTile];
  const int lane = threadIdx.x & 31;
  const int g = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const bool active = g < (ntarget + 31) / 32;
  const int cb = blockIdx.y * cseg, ce = min(ntop, cb + cseg);
  dsum += (size_t)blockIdx.y * 3 * ntarget;
  typename M::Acc f0, f1, f2, g0, g1, g2;
  for (int c0 = cb; c0 < ce; c0 += kDenseTile) {
    const int nc = min(kDenseTile, ce - c0);
    __syncthreads();
    for (int i = threadIdx.x; i < 2 * nc; i += blockDim.x) ss[i] = __ldg(&src[2 * (size_t)(top0 + c0) + i]);
    __syncthreads();
    if (!active) continue;
    const W2* wp = wtop + ((size_t)g * ntop2 + (c0 >> 1)) * 32 + lane;
    int c = 0;
    for (; c + 7 < nc; c += 8) {
      W2 w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) w[u] = __ldg(&wp[(size_t)((c >> 1) + u) * 32]);
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const H a = ss[2 * (c + 2 * u)], z = ss[2 * (c + 2 * u) + 1];
        const H a2 = ss[2 * (c + 2 * u + 1)], z2 = ss[2 * (c + 2 * u + 1) + 1];
        M::mac(f0, M::wa(w[u]), M::v0(a));
        M::mac(f1, M::wa(w[u]), M::v1(a));
        M::mac(f2, M::wa(w[u]), M::v0(z));
        M::mac(g0, M::wb(w[u]), M::v0(a2));
        M::mac(g1, M::wb(w[u]), M::v1(a2));
        M::mac(g2, M::wb(w[u]), M::v0(z2));
      }
    }
    for (; c < nc; c += 2) {
      const W2 w = __ldg(&wp[(size_t)(c >> 1) * 32]);
      const H a = ss[2 * c], z = ss[2 * c + 1];
      M::mac(f0, M::wa(w), M::v0(a));
      M::mac(f1, M::wa(w), M::v1(a));
      M::mac(f2, M::wa(w), M::v0(z));
      if (c + 1 < nc) {
        const H a2 = ss[2 * (c + 1)], z2 = ss[2 * (c + 1) + 1];
        M::mac(g0, M::wb(w), M::v0(a2));
        M::mac(g1, M::wb(w), M::v1(a2));
        M::mac(g2, M::wb(w), M::v0(z2));
      }
    }
  }
  const int t = g * 32 + lane;
  if (active && t < ntarget) {
    dsum[t] = M::fin(f0) + M::fin(g0);
    dsum[ntarget + t] = M::fin(f1) + M::fin(g1);
    dsum[2 * (size_t)ntarget + t] = M::fin(f2) + M::fin(g2);
  }
}

// One warp per boundary node: lanes stride over the node's interaction
// list (coalesced), fixed-shape shuffle reduction (deterministic); with
// dsum, the dense block's partial sums join the warp's before the store.
template <class M>
__global__ void __launch_bounds__(256) k_apply_csr(const long long* __restrict__ rowptr, const int* __restrict__ col,
                                                   const typename M::W* __restrict__ wgt,
                                                   const typename M::H* __restrict__ src,
                                                   const int* __restrict__ tgt_node, int ntarget, double inv_pi4,
                                                   double* __restrict__ o0, double* __restrict__ o1,
                                                   double* __restrict__ o2, const double* __restrict__ dsum,
                                                   int nseg) {
  using H = typename M::H;
  using W = typename M::W;
  using V = typename M::V;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntarget) return;
  const long long b = rowptr[warp], e = rowptr[warp + 1];
  // Four interactions per lane per trip: their ids and weights are loaded
  // before any gather so the loads overlap; two accumulator sets break the
  // dependency chain.
  typename M::Acc f0, f1, f2, g0, g1, g2;
  long long k = b + lane;
  for (; k + 96 < e; k += 128) {
    int c[4];
    W w[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) c[u] = __ldg(&col[k + 32 * u]);
#pragma unroll
    for (int u = 0; u < 4; ++u) w[u] = __ldg(&wgt[k + 32 * u]);
    V x0[4], x1[4], x2[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const H a = __ldg(&src[2 * (size_t)c[u]]), z = __ldg(&src[2 * (size_t)c[u] + 1]);
      x0[u] = M::v0(a);
      x1[u] = M::v1(a);
      x2[u] = M::v0(z);
    }
#pragma unroll
    for (int u = 0; u < 4; u += 2) {
      M::mac(f0, w[u], x0[u]);
      M::mac(f1, w[u], x1[u]);
      M::mac(f2, w[u], x2[u]);
      M::mac(g0, w[u + 1], x0[u + 1]);
      M::mac(g1, w[u + 1], x1[u + 1]);
      M::mac(g2, w[u + 1], x2[u + 1]);
    }
  }
  for (; k < e; k += 32) {
    const int c = __ldg(&col[k]);
    const W w = __ldg(&wgt[k]);
    const H a = __ldg(&src[2 * (size_t)c]), z = __ldg(&src[2 * (size_t)c + 1]);
    M::mac(f0, w, M::v0(a));
    M::mac(f1, w, M::v1(a));
    M::mac(f2, w, M::v0(z));
  }
  double a0 = M::fin(f0) + M::fin(g0);
  double a1 = M::fin(f1) + M::fin(g1);
  double a2 = M::fin(f2) + M::fin(g2);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
  }
  if (lane == 0) {
    for (int q = 0; dsum && q < nseg; ++q) {
      const double* d = dsum + (size_t)q * 3 * ntarget;
      a0 += d[warp];
      a1 += d[ntarget + warp];
      a2 += d[2 * (size_t)ntarget + warp];
    }
    const int node = tgt_node[warp];
    o0[node] += -a0 * inv_pi4;
    o1[node] += -a1 * inv_pi4;
    o2[node] += -a2 * inv_pi4;
  }
}

// Group sources: problem `slot` of a group writes its records (policy
// values) into slot `slot` of [cell][slot][s0 s1 s2 0], so that the
// problems' records of one cell are adjacent (one coalesced load per warp).
template <class M>
__global__ void k_split_slot(const double* __restrict__ x, int ncell, int slot, int lanes,
                             typename M::V* __restrict__ out) {
  const size_t n = 4 * (size_t)ncell;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const int cell = (int)(i >> 2), comp = (int)(i & 3);
    out[((size_t)cell * lanes + slot) * 4 + comp] = M::vmake(comp < 3 ? x[(size_t)comp * ncell + cell] : 0.0);
  }
}

template <class M>
__device__ __forceinline__ void mac3(typename M::Acc& a0, typename M::Acc& a1, typename M::Acc& a2,
                                     typename M::W w, const typename M::H* __restrict__ rec) {
  const typename M::H a = __ldg(rec), z = __ldg(rec + 1);
  M::mac(a0, w, M::v0(a));
  M::mac(a1, w, M::v1(a));
  M::mac(a2, w, M::v0(z));
}

// The dense block (coarsest level) of a shared operator against a group's
// sources: a register-tiled product.  Lane = boundary node of a 32-node
// chunk (its weights are one coalesced row), warp = a quad of problems
// (4 problems x 3 components of accumulators), CTA = 8 warps over
// 8 / nquad chunks; a tile of kGroupTile cells of every problem's sources
// is staged in shared memory and read as broadcasts.  Each weight feeds
// twelve independent chains.  blockIdx.y = segment of the coarsest cells;
// partial sums go to part[segment][problem][comp][node].
constexpr int kGroupTile = 64;
template <class M>
__global__ void __launch_bounds__(256) k_group_dense(const typename M::W2* __restrict__ wtop,
                                                     const typename M::H* __restrict__ gsrc, int top0, int ntop,
                                                     int ntop2, int ntarget, int nprob, int nquad, int cseg,
                                                     double* __restrict__ part) {
  using H = typename M::H;
  using W2 = typename M::W2;
  extern __shared__ double2 gsm[];
  H* gs = reinterpret_cast<H*>(gsm);  // [cell][problem][2]
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int per = 8 / nquad;  // chunks per CTA
  const int q = wid % nquad;  // problem quad
  const int chunk = blockIdx.x * per + wid / nquad;
  const bool active = chunk < (ntarget + 31) / 32 && wid < per * nquad;
  const int p0 = 4 * q;
  const int np = active ? max(0, min(4, nprob - p0)) : 0;
  const int cb = blockIdx.y * cseg, ce = min(ntop, cb + cseg);
  typename M::Acc a[4][3];
  for (int c0 = cb; c0 < ce; c0 += kGroupTile) {
    const int nc = min(kGroupTile, ce - c0);
    __syncthreads();
    const H* src = gsrc + 2 * (size_t)(top0 + c0) * nprob;
    for (int i = threadIdx.x; i < 2 * nc * nprob; i += blockDim.x) gs[i] = __ldg(&src[i]);
    __syncthreads();
    if (!np) continue;
    const W2* wp = wtop + ((size_t)chunk * ntop2 + (c0 >> 1)) * 32 + lane;
    for (int c = 0; c < nc; c += 2) {
      const W2 w = __ldg(&wp[(size_t)(c >> 1) * 32]);
      const typename M::W wa = M::wa(w), wb = M::wb(w);
      const bool two = c + 1 < nc;
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (j < np) {
          const H* r = gs + 2 * ((size_t)c * nprob + p0 + j);
          const H x = r[0], z = r[1];
          M::mac(a[j][0], wa, M::v0(x));
          M::mac(a[j][1], wa, M::v1(x));
          M::mac(a[j][2], wa, M::v0(z));
          if (two) {
            const H* r2 = r + 2 * nprob;
            const H x2 = r2[0], z2 = r2[1];
            M::mac(a[j][0], wb, M::v0(x2));
            M::mac(a[j][1], wb, M::v1(x2));
            M::mac(a[j][2], wb, M::v0(z2));
          }
        }
      }
    }
  }
  const int t = chunk * 32 + lane;
  if (!np || t >= ntarget) return;
  double* out = part + (size_t)blockIdx.y * nprob * 3 * ntarget;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (j < np) {
#pragma unroll
      for (int cc = 0; cc < 3; ++cc) out[((size_t)(p0 + j) * 3 + cc) * ntarget + t] = M::fin(a[j][cc]);
    }
  }
}

// One recorded operator applied to the sources of up to kGroupMax problems
// with the same index geometry (their weights differ by the factor of the
// mesh spacing, folded into G.scale).  A warp per boundary node; lane
// p + LG * grp serves problem p (LG = nprob lanes per problem set, NG =
// 32 / LG sets) and every NG-th interaction from grp, so the weight and
// cell id are read once for all problems and the problems' source records
// of a cell are one contiguous load.  The row holds the finer levels; the
// NG partial sums are added in set order, then the dense block's partial
// sums (k_group_dense) in segment order.
template <class M>
__global__ void __launch_bounds__(256) k_apply_group(const long long* __restrict__ rowptr, const int* __restrict__ col,
                                                     const typename M::W* __restrict__ wgt,
                                                     const typename M::H* __restrict__ gsrc,
                                                     const int* __restrict__ tgt_node, int ntarget, int nprob,
                                                     const double* __restrict__ part, int nseg, GroupOut G) {
  using H = typename M::H;
  using W = typename M::W;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntarget) return;
  const int LG = nprob, NG = 32 / nprob;
  const int p = lane % LG, grp = lane / LG;
  const bool act = grp < NG;
  const H* sp = gsrc + 2 * (size_t)p;
  const size_t cstride = 2 * (size_t)LG;  // halves per cell
  typename M::Acc f0, f1, f2, g0, g1, g2;
  const long long b = rowptr[warp], e = rowptr[warp + 1];
  if (act) {
    long long k = b + grp;
    for (; k + 3 * NG < e; k += 4 * NG) {
      int c[4];
      W w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) c[u] = __ldg(&col[k + u * NG]);
#pragma unroll
      for (int u = 0; u < 4; ++u) w[u] = __ldg(&wgt[k + u * NG]);
#pragma unroll
      for (int u = 0; u < 4; u += 2) {
        mac3<M>(f0, f1, f2, w[u], sp + (size_t)c[u] * cstride);
        mac3<M>(g0, g1, g2, w[u + 1], sp + (size_t)c[u + 1] * cstride);
      }
    }
    for (; k < e; k += NG) mac3<M>(f0, f1, f2, __ldg(&wgt[k]), sp + (size_t)__ldg(&col[k]) * cstride);
  }
  double a0 = M::fin(f0) + M::fin(g0);
  double a1 = M::fin(f1) + M::fin(g1);
  double a2 = M::fin(f2) + M::fin(g2);
  const double b0 = a0, b1 = a1, b2 = a2;
  for (int g = 1; g < NG; ++g) {
    const int src = min(p + g * LG, 31);
    a0 += __shfl_sync(0xffffffffu, b0, src);
    a1 += __shfl_sync(0xffffffffu, b1, src);
    a2 += __shfl_sync(0xffffffffu, b2, src);
  }
  if (grp == 0) {
#pragma unroll 1
    for (int q = 0; part && q < nseg; ++q) {  // the dense block's partial sums, in segment order
      const double* d = part + ((size_t)q * nprob + p) * 3 * ntarget;
      a0 += d[warp];
      a1 += d[ntarget + warp];
      a2 += d[2 * (size_t)ntarget + warp];
    }
    const int node = tgt_node[warp];
    const double sc = G.scale[p];
    G.o[p][0][node] += a0 * sc;
    G.o[p][1][node] += a1 * sc;
    G.o[p][2][node] += a2 * sc;
  }
}

// Set-up comparison of a follower's recorded operator F with the leader's
// L scaled by `ratio`.  Their rows differ where a cell lies exactly on the
// opening radius of the tree walk in index units (each problem's rounding
// decides the tie): one accepted the cell, the other its children.  A walk
// visits cells in the tree's preorder, so both rows are sorted by pre[cell]
// and a merge gives their difference: F's cells missing from L (weight
// +wF) and L's missing from F (weight -ratio wL); for the dense block, the
// coarsest cells accepted by one of them.  Shared cells must agree within
// `tol` (relative), else *bad is set.
// A recorded weight word as a double: an FP64 weight, or a float-float pair.
__device__ __forceinline__ double wval(const double* w, size_t i, int ff) {
  if (!ff) return w[i];
  const float2 v = reinterpret_cast<const float2*>(w)[i];
  return (double)v.x + (double)v.y;
}
__device__ __forceinline__ bool w_close(double va, double vb, double ratio, double tol) {
  if (va == 0.0 || vb == 0.0) return va == 0.0 && vb == 0.0;
  return fabs(vb - ratio * va) <= tol * fabs(vb);
}
__device__ __forceinline__ size_t dense_at(int t, int c, int ntop2) {
  return (((size_t)(t >> 5) * ntop2 + (c >> 1)) * 32 + (t & 31)) * 2 + (c & 1);
}

struct CorrArgs {
  const long long *Lr, *Fr;
  const int *Lc, *Fc;
  const double *Lw, *Fw, *Ld, *Fd;  // 8-byte weight words (ff: float-float pairs)
  const int* pre;
  int ntop, top0;
  double ratio, tol;
  int ff;
};

template <bool FILL>
__device__ int corr_row(const CorrArgs& A, int t, int* __restrict__ ocol, double* __restrict__ ow, bool& ok) {
  long long i = A.Lr[t], j = A.Fr[t];
  const long long ie = A.Lr[t + 1], je = A.Fr[t + 1];
  int n = 0;
  while (i < ie || j < je) {
    const int ca = (i < ie) ? A.Lc[i] : -1, cb = (j < je) ? A.Fc[j] : -1;
    const int pa = (ca >= 0) ? A.pre[ca] : 0x7fffffff, pb = (cb >= 0) ? A.pre[cb] : 0x7fffffff;
    if (pa == pb) {
      ok &= w_close(wval(A.Lw, i, A.ff), wval(A.Fw, j, A.ff), A.ratio, A.tol);
      ++i;
      ++j;
    } else if (pa < pb) {
      if (FILL) { ocol[n] = ca; ow[n] = -A.ratio * wval(A.Lw, i, A.ff); }
      ++n;
      ++i;
    } else {
      if (FILL) { ocol[n] = cb; ow[n] = wval(A.Fw, j, A.ff); }
      ++n;
      ++j;
    }
  }
  if (A.Ld) {
    const int ntop2 = (A.ntop + 1) >> 1;
    for (int c = 0; c < A.ntop; ++c) {
      const double a = wval(A.Ld, dense_at(t, c, ntop2), A.ff), b = wval(A.Fd, dense_at(t, c, ntop2), A.ff);
      const bool za = a == 0.0, zb = b == 0.0;
      if (za != zb) {
        if (FILL) { ocol[n] = A.top0 + c; ow[n] = b - A.ratio * a; }
        ++n;
      } else if (!za) {
        ok &= w_close(a, b, A.ratio, A.tol);
      }
    }
  }
  return n;
}

__global__ void k_corr_count(CorrArgs A, const int* __restrict__ Lt, const int* __restrict__ Ft, int ntarget,
                             int* __restrict__ cnt, int* __restrict__ bad) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntarget) return;
  bool ok = Lt[t] == Ft[t];
  cnt[t] = corr_row<false>(A, t, nullptr, nullptr, ok);
  if (!ok) atomicOr(bad, 1);
}

__global__ void k_corr_fill(CorrArgs A, const int* __restrict__ rows, const long long* __restrict__ crp, int nrows,
                            int* __restrict__ col, double* __restrict__ w) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  bool ok = true;
  corr_row<true>(A, rows[i], col + crp[i], w + crp[i], ok);
}

// sol(node of row) += -1/(4 pi) * sum of the correction row (FP64; warp per row).
__global__ void k_apply_corr(const int* __restrict__ rows, const long long* __restrict__ crp, int nrows,
                             const int* __restrict__ col, const double* __restrict__ w, const double* __restrict__ src,
                             int ncell, const int* __restrict__ tgt_node, double scale, double* __restrict__ o0,
                             double* __restrict__ o1, double* __restrict__ o2) {
  const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (i >= nrows) return;
  double a0 = 0.0, a1 = 0.0, a2 = 0.0;
  for (long long k = crp[i] + lane; k < crp[i + 1]; k += 32) {
    const int c = col[k];
    const double wk = w[k];
    a0 = fma(wk, src[c], a0);
    a1 = fma(wk, src[(size_t)ncell + c], a1);
    a2 = fma(wk, src[2 * (size_t)ncell + c], a2);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a0 += __shfl_xor_sync(0xffffffffu, a0, o);
    a1 += __shfl_xor_sync(0xffffffffu, a1, o);
    a2 += __shfl_xor_sync(0xffffffffu, a2, o);
  }
  if (lane == 0) {
    const int node = tgt_node[rows[i]];
    o0[node] += a0 * scale;
    o1[node] += a1 * scale;
    o2[node] += a2 * scale;
  }
}

// calc_normalderiv_3d: one thread per panel.
__global__ void k_normal_deriv(const double* __restrict__ sol0, int NX, int NY, int NZ, const int* __restrict__ face,
                               const int* __restrict__ pi, const int* __restrict__ pj, const int* __restrict__ pk,
                               int nbound, double invx, double invy, double invz, double* __restrict__ src) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nbound) return;
  const double a1 = 25.0 / 12.0, a2 = -4.0, a3 = 3.0, a4 = -4.0 / 3.0, a5 = 0.25;
  const int f = face[p];
  const int i = pi[p] - 1, j = pj[p] - 1, k = pk[p] - 1;  // 0-based
  const long long sx = 1, sy = NX, sz = (long long)NX * NY;
  long long step, e1, e2;
  double inv;
  if (f < 2) { step = (f == 0) ? sx : -sx; e1 = sy; e2 = sz; inv = invx; }
  else if (f < 4) { step = (f == 2) ? sy : -sy; e1 = sx; e2 = sz; inv = invy; }
  else { step = (f == 4) ? sz : -sz; e1 = sx; e2 = sy; inv = invz; }
  const long long base = i * sx + j * sy + k * sz;
  // corner order of the reference: (0,0), (1,0), (1,1), (0,1) in the face's (fast, slow) axes
  const long long corner[4] = {base, base + e1, base + e1 + e2, base + e2};
  double ps[4];
#pragma unroll
  for (int m = 0; m < 4; ++m) {
    const long long n0 = corner[m];
    const double v0 = sol0[n0], v1 = sol0[n0 + step], v2 = sol0[n0 + 2 * step], v3 = sol0[n0 + 3 * step],
                 v4 = sol0[n0 + 4 * step];
    ps[m] = inv * ((((a1 * v0 + a2 * v1) + a3 * v2) + a4 * v3) + a5 * v4);
  }
  src[p] = 0.25 * (((ps[0] + ps[1]) + ps[2]) + ps[3]);
}

// build_level_nbound_3d sources: area-weighted mean over the istep^2 leaves.
__global__ void k_aggregate(const int* __restrict__ leaf0, const int* __restrict__ rowlen, const int* __restrict__ istep,
                            const double* __restrict__ cds, int first, int ncell, double* __restrict__ s0,
                            double* __restrict__ s1, double* __restrict__ s2) {
  const int c = first + blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= first + ncell) return;
  const int l0 = leaf0[c];
  if (l0 < 0) return;
  const int n1 = rowlen[c], st = istep[c];
  double w0 = 0.0, w1 = 0.0, w2 = 0.0;
  for (int mm = 0; mm < st; ++mm)
    for (int nn = 0; nn < st; ++nn) {
      const int leaf = l0 + mm * n1 + nn;
      const double s = cds[leaf];
      w0 = s0[leaf] * s + w0;
      w1 = s1[leaf] * s + w1;
      w2 = s2[leaf] * s + w2;
    }
  const double sc = cds[c];
  s0[c] = w0 / sc;
  s1[c] = w1 / sc;
  s2[c] = w2 / sc;
}

template <class T>
void upload(DBuf<T>& b, const std::vector<T>& h) {
  b.ensure(h.size());
  if (!h.empty()) VPMG_CUDA(cudaMemcpy(b.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
}

WalkDev walk_dev(const BoundaryOp& B) {
  WalkDev W;
  W.cx = B.cx.p; W.cy = B.cy.p; W.cz = B.cz.p; W.cds = B.cds.p; W.cthr = B.cthr.p;
  W.child = B.child.p; W.flags = B.flags.p;
  W.s0 = B.csrc.p; W.s1 = B.csrc.p + B.ncell_total; W.s2 = B.csrc.p + 2 * (size_t)B.ncell_total;
  W.tgt_node = B.tgt_node.p; W.tx = B.tx.p; W.ty = B.ty.p; W.tz = B.tz.p;
  W.top0 = B.lev_off[B.levmax];
  W.ntop = B.nbound_lev[B.levmax];
  W.levmax = B.levmax;
  W.ntarget = B.ntarget;
  W.lg = std::log((std::sqrt(2.0) - 1.0) / (std::sqrt(2.0) + 1.0));
  W.inv_pi4 = 1.0 / (4.0 * kPI);
  W.pi4 = 4.0 * kPI;
  W.bctype = B.ibctyp;
  W.tree = B.tree ? 1 : 0;
  W.tgt_frame = B.tgt_frame.p;
  W.dense = B.dense ? 1 : 0;
  W.ff = B.arith == VPMG_ARITH_FF48 ? 1 : 0;
  for (int f = 0; f < 6; ++f) W.frame[f] = B.frame[f];
  return W;
}

// Slot of Bounds3d_lev's plane argument: 2/-2 X min/max, 1/-1 Y, 3/-3 Z.
int frame_slot(int iplane) { return 2 * ((iplane > 0 ? iplane : -iplane) - 1) + (iplane < 0 ? 1 : 0); }

// Constants of calc_boundinf_3d_s / calc_boundinf_3d_lev_s for one plane
// (source/pmbound.f90:536-606, 1270-1340).
PanelFrame make_frame(int iplane, const double d[3]) {
  PanelFrame F;
  const double DX = d[0], DY = d[1], DZ = d[2];
  const double si = iplane > 0 ? 1.0 : -1.0;
  for (int m = 0; m < 3; ++m) F.E1[m] = F.E2[m] = F.E3[m] = 0.0;
  double a, b;  // cell sides along E1 and E2
  switch (iplane > 0 ? iplane : -iplane) {
    case 1:
      F.E1[0] = si; F.E2[2] = 1.0; F.E3[1] = -si;
      F.diag = std::sqrt(DX * DX + DZ * DZ); F.area = DX * DZ; a = DX; b = DZ;
      break;
    case 2:
      F.E1[2] = 1.0; F.E2[1] = -si; F.E3[0] = -si;
      F.diag = std::sqrt(DY * DY + DZ * DZ); F.area = DY * DZ; a = DY; b = DZ;
      break;
    default:
      F.E1[0] = 1.0; F.E2[1] = -si; F.E3[2] = -si;
      F.diag = std::sqrt(DX * DX + DY * DY); F.area = DX * DY; a = DX; b = DY;
      break;
  }
  F.S[0] = -0.5 * a; F.S[1] = -0.5 * a; F.S[2] = 0.5 * a; F.S[3] = 0.5 * a;
  F.T[0] = -0.5 * b; F.T[1] = 0.5 * b; F.T[2] = 0.5 * b; F.T[3] = -0.5 * b;
  F.D[0] = b; F.D[1] = a; F.D[2] = b; F.D[3] = a;
  return F;
}

}  // namespace

long long BoundaryOp::bytes() const {
  return (long long)(rowptr.bytes() + col.bytes() + w.bytes() + colptr.bytes() + trow.bytes() + tw.bytes() +
                     cx.bytes() * 5 + child.bytes() + csrc.bytes() + wtop.bytes() + dsum.bytes()) +
         ff.bytes();
}

void boundary_prepare(BoundaryOp& B, const Grid& g, int levmax, long long budget_bytes, cudaStream_t s, int ibctyp,
                      bool tree, int arith) {
  VPMG_CHECK(arith == VPMG_ARITH_FP64 || arith == VPMG_ARITH_FF48, VPMG_ERR_ARG, "unknown arithmetic");
  B.arith = arith;
  VPMG_CHECK(levmax >= 0 && levmax < kMaxLev - 1, VPMG_ERR_ARG, "levmax out of range");
  VPMG_CHECK(ibctyp == 2 || ibctyp == 3, VPMG_ERR_UNSUPPORTED, "ibctyp must be 2 or 3");
  VPMG_CHECK(tree || levmax == 0, VPMG_ERR_ARG, "the untreed sum has one level");
  B.ibctyp = ibctyp;
  B.tree = tree;
  for (int p = 1; p <= 3; ++p) {
    B.frame[frame_slot(p)] = make_frame(p, g.d);
    B.frame[frame_slot(-p)] = make_frame(-p, g.d);
  }
  TreeGeom T;
  try {
    build_tree_geometry(g.xmin, g.d, g.n, levmax, T);
  } catch (const std::exception& e) {
    throw Error{VPMG_ERR_TREE, e.what()};
  }
  B.levmax = levmax;
  B.nbound = T.nbound;
  B.nbound_lev = T.nbound_lev;
  B.lev_off.assign(levmax + 2, 0);
  for (int l = 0; l <= levmax; ++l) B.lev_off[l + 1] = B.lev_off[l] + T.nbound_lev[l];
  B.ncell_total = B.lev_off[levmax + 1];
  const int NC = B.ncell_total;
  std::vector<double> cx(NC), cy(NC), cz(NC), cds(NC), thr(NC);
  std::vector<int> child(4 * (size_t)NC, -1), flags(NC), leaf0(NC), rowlen(NC), istep(NC);
  for (int l = 0; l <= levmax; ++l)
    for (int ic = 0; ic < T.nbound_lev[l]; ++ic) {
      const Cell& c = T.cells[(size_t)l * T.nbound + ic];
      const int f = B.lev_off[l] + ic;
      cx[f] = c.x; cy[f] = c.y; cz[f] = c.z; cds[f] = c.ds; thr[f] = c.thr;
      flags[f] = c.ilev[5];
      VPMG_CHECK(c.ilev[5] != 0, VPMG_ERR_TREE, "Something is wrong with the tree (ilev_t(.,.,6) == 0)");
      leaf0[f] = (l > 0) ? c.leaf0 : -1;
      rowlen[f] = c.rowlen;
      istep[f] = c.istep;
      if (l > 0) {
        const int nch = (c.ilev[5] < 0) ? 2 : 4;
        for (int m = 0; m < nch; ++m) {
          const int ch = c.ilev[m];
          VPMG_CHECK(ch >= 1 && ch <= T.nbound_lev[l - 1], VPMG_ERR_TREE, "tree child index out of range");
          child[4 * (size_t)f + m] = B.lev_off[l - 1] + ch - 1;
        }
      }
    }
  // ancestor of every leaf at each level >= 1 (for the aggregation transpose)
  std::vector<int> anc((size_t)std::max(levmax, 1) * B.nbound, -1);
  for (int l = 1; l <= levmax; ++l)
    for (int ic = 0; ic < T.nbound_lev[l]; ++ic) {
      const Cell& c = T.cells[(size_t)l * T.nbound + ic];
      if (c.leaf0 < 0) continue;
      for (int mm = 0; mm < c.istep; ++mm)
        for (int nn = 0; nn < c.istep; ++nn)
          anc[(size_t)(l - 1) * B.nbound + c.leaf0 + mm * c.rowlen + nn] = B.lev_off[l] + ic;
    }
  upload(B.anc, anc);
  upload(B.cx, cx); upload(B.cy, cy); upload(B.cz, cz); upload(B.cds, cds); upload(B.cthr, thr);
  upload(B.child, child); upload(B.flags, flags); upload(B.agg_leaf0, leaf0); upload(B.agg_rowlen, rowlen);
  upload(B.agg_istep, istep);
  B.csrc.ensure(3 * (size_t)NC);
  std::vector<int> pf(B.nbound), pi(B.nbound), pj(B.nbound), pk(B.nbound);
  for (int p = 0; p < B.nbound; ++p) {
    pf[p] = T.panels[p].face; pi[p] = T.panels[p].i; pj[p] = T.panels[p].j; pk[p] = T.panels[p].k;
  }
  upload(B.pan_face, pf); upload(B.pan_i, pi); upload(B.pan_j, pj); upload(B.pan_k, pk);
  B.ntarget = (int)T.targets.size();
  std::vector<int> tn(B.ntarget), tf(B.ntarget);
  std::vector<double> tx(B.ntarget), ty(B.ntarget), tz(B.ntarget);
  for (int t = 0; t < B.ntarget; ++t) {
    tn[t] = (int)T.targets[t].node; tx[t] = T.targets[t].x; ty[t] = T.targets[t].y; tz[t] = T.targets[t].z;
    tf[t] = frame_slot(T.targets[t].iplane);
  }
  upload(B.tgt_node, tn); upload(B.tx, tx); upload(B.ty, ty); upload(B.tz, tz); upload(B.tgt_frame, tf);
  // ---- record the interaction lists if they fit --------------------------
  B.precomputed = false;
  B.nnz = 0;
  B.rowptr.release(); B.col.release(); B.w.release(); B.wtop.release(); B.dsum.release();
  B.ndense_acc = 0;
  B.ntopd = B.nbound_lev[B.levmax];
  const int nchunk = (B.ntarget + 31) / 32;
  const long long ntop2 = (B.ntopd + 1) / 2;
  const long long dense_bytes =
      (long long)nchunk * ntop2 * 64 * (long long)sizeof(float2) + 3LL * B.ntarget * (long long)sizeof(double);
  // the dense block needs a tree (levmax >= 1), the cells' own columns (not
  // ibctyp 3's start-cell column) and at most half of the budget
  B.dense = B.levmax >= 1 && !(B.ibctyp == 3 && B.tree) && budget_bytes > 0 && dense_bytes <= budget_bytes / 2;
  const WalkDev W = walk_dev(B);
  const int blocks = (B.ntarget + 127) / 128;
  DBuf<int> counts;
  counts.ensure(B.ntarget);
  B.dcount.ensure(1);
  VPMG_CUDA(cudaMemsetAsync(B.dcount.p, 0, sizeof(unsigned long long), s));
  k_walk<kCount><<<blocks, 128, 0, s>>>(W, nullptr, nullptr, nullptr, counts.p, nullptr, nullptr, nullptr, nullptr,
                                        B.dcount.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
  std::vector<int> hc(B.ntarget);
  unsigned long long nd = 0;
  VPMG_CUDA(cudaMemcpyAsync(hc.data(), counts.p, sizeof(int) * B.ntarget, cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaMemcpyAsync(&nd, B.dcount.p, sizeof(nd), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  B.ndense_acc = (long long)nd;
  std::vector<long long> rp(B.ntarget + 1, 0);
  for (int t = 0; t < B.ntarget; ++t) rp[t + 1] = rp[t] + hc[t];
  B.nnz = rp[B.ntarget];
  const long long need = B.nnz * (long long)(sizeof(int) + sizeof(double)) +
                         (long long)sizeof(long long) * (B.ntarget + 1) + (B.dense ? dense_bytes : 0);
  size_t free_b = 0, total_b = 0;
  VPMG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (budget_bytes > 0 && need <= budget_bytes && need < (long long)(0.8 * (double)free_b)) {
    try {
      upload(B.rowptr, rp);
      B.col.ensure((size_t)std::max<long long>(B.nnz, 1));
      B.w.ensure((size_t)std::max<long long>(B.nnz, 1));
      if (B.dense) {
        const size_t nw = (size_t)nchunk * ntop2 * 64;
        B.wtop.ensure(nw);
        VPMG_CUDA(cudaMemsetAsync(B.wtop.p, 0, sizeof(float2) * nw, s));  // opened cells weigh 0
        // segments of the coarsest cells per 32-node chunk: at least three
        // waves of warps (5 resident CTAs of 8 warps per SM), 64+ cells each
        int dev = 0, sms = 0;
        VPMG_CUDA(cudaGetDevice(&dev));
        VPMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        const long long slots = 40LL * sms;
        int seg = 1;
        while (seg < 8 && (long long)nchunk * seg < 3 * slots && B.ntopd / (2 * seg) >= 64) seg *= 2;
        B.dseg = seg;
        B.dsum.ensure(3 * (size_t)B.ntarget * seg);
      }
      k_walk<kFill><<<blocks, 128, 0, s>>>(W, nullptr, nullptr, nullptr, nullptr, B.rowptr.p, B.col.p, B.w.p,
                                           B.dense ? B.wtop.p : nullptr, nullptr);
      VPMG_LAUNCHED();
      VPMG_CUDA(cudaGetLastError());
      VPMG_CUDA(cudaStreamSynchronize(s));
      B.csrc_ff.ensure(4 * (size_t)B.ncell_total);  // here, not in the apply: steps may be captured in graphs
      B.precomputed = true;
    } catch (const Error& e) {
      if (e.status != VPMG_ERR_NOMEM) throw;
      B.rowptr.release(); B.col.release(); B.w.release(); B.wtop.release(); B.dsum.release();
      B.precomputed = false;
    }
  }
  if (!B.precomputed) B.dense = false;  // the walk covers every level
  farfield_prepare(B, g, s);
}

void boundary_panels(BoundaryOp& B, const Grid& g, const double* sol0, int comp, cudaStream_t s) {
  double* dst = B.csrc.p + (size_t)comp * B.ncell_total;  // level-0 part = panels
  k_normal_deriv<<<(B.nbound + 255) / 256, 256, 0, s>>>(sol0, g.n[0], g.n[1], g.n[2], B.pan_face.p, B.pan_i.p,
                                                        B.pan_j.p, B.pan_k.p, B.nbound, 1.0 / g.d[0], 1.0 / g.d[1],
                                                        1.0 / g.d[2], dst);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

// Coarsest cells per dense-block segment (even: cell pairs stay whole) and
// the number of segments that covers them.
static int dense_cseg(const BoundaryOp& B) { return (((B.ntopd + B.dseg - 1) / B.dseg) + 1) & ~1; }
static int dense_nseg(const BoundaryOp& B) { return (B.ntopd + dense_cseg(B) - 1) / dense_cseg(B); }

// Levels 1..levmax aggregate the level-0 panels (source_bound_lev).
static void aggregate_levels(BoundaryOp& B, cudaStream_t s) {
  double* s0 = B.csrc.p;
  double* s1 = B.csrc.p + B.ncell_total;
  double* s2 = B.csrc.p + 2 * (size_t)B.ncell_total;
  for (int l = 1; l <= B.levmax; ++l) {
    const int n = B.nbound_lev[l];
    if (n <= 0) continue;
    k_aggregate<<<(n + 255) / 256, 256, 0, s>>>(B.agg_leaf0.p, B.agg_rowlen.p, B.agg_istep.p, B.cds.p, B.lev_off[l], n,
                                                s0, s1, s2);
    VPMG_LAUNCHED();
  }
}

template <class M>
static void apply_recorded(BoundaryOp& B, double* const sol[3], cudaStream_t s) {
  using H = typename M::H;
  const size_t nc4 = 4 * (size_t)B.ncell_total;
  VPMG_CHECK(B.csrc_ff.n >= nc4, VPMG_ERR_STATE, "boundary operator recorded without its source buffer");
  typename M::V* src = reinterpret_cast<typename M::V*>(B.csrc_ff.p);
  k_split<M><<<(unsigned)std::min<size_t>((nc4 + 255) / 256, 152 * 16), 256, 0, s>>>(B.csrc.p, B.ncell_total, src);
  VPMG_LAUNCHED();
  const H* src2 = reinterpret_cast<const H*>(src);
  if (!M::kFF && B.ff.on) {
    // the coarsest level by FFT over every cell into the partial sums, the
    // finer rows on top, then the opened coarsest cells taken back out
    farfield_apply(B, B.dsum.p, s);
    const long long threads = (long long)B.ntarget * 32;
    k_apply_csr<M><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        B.rowptr.p, B.col.p, reinterpret_cast<const typename M::W*>(B.w.p), src2, B.tgt_node.p, B.ntarget,
        1.0 / (4.0 * kPI), sol[0], sol[1], sol[2], B.dsum.p, 1);
    VPMG_LAUNCHED();
    k_apply_csr<M><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
        B.ff.crow.p, B.ff.ccol.p, reinterpret_cast<const typename M::W*>(B.ff.cw.p), src2, B.tgt_node.p, B.ntarget,
        1.0 / (4.0 * kPI), sol[0], sol[1], sol[2], nullptr, 0);
    VPMG_LAUNCHED();
    return;
  }
  if (B.dense) {
    const long long dthreads = (long long)((B.ntarget + 31) / 32) * 32;
    const int cseg = dense_cseg(B);
    const dim3 grid((unsigned)((dthreads + 255) / 256), (unsigned)dense_nseg(B));
    k_apply_dense<M><<<grid, 256, 0, s>>>(reinterpret_cast<const typename M::W2*>(B.wtop.p), src2,
                                          B.lev_off[B.levmax], B.ntopd, (B.ntopd + 1) / 2, B.ntarget, cseg,
                                          B.dsum.p);
    VPMG_LAUNCHED();
  }
  const long long threads = (long long)B.ntarget * 32;
  k_apply_csr<M><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      B.rowptr.p, B.col.p, reinterpret_cast<const typename M::W*>(B.w.p), src2, B.tgt_node.p, B.ntarget,
      1.0 / (4.0 * kPI), sol[0], sol[1], sol[2], B.dense ? B.dsum.p : nullptr, B.dense ? dense_nseg(B) : 0);
  VPMG_LAUNCHED();
}

void boundary_apply(BoundaryOp& B, const Grid& g, double* const sol[3], cudaStream_t s) {
  (void)g;
  aggregate_levels(B, s);
  if (B.precomputed) {
    if (B.arith == VPMG_ARITH_FF48) apply_recorded<MacFF>(B, sol, s);
    else apply_recorded<Mac64>(B, sol, s);
  } else {
    const WalkDev W = walk_dev(B);
    k_walk<kAccum><<<(B.ntarget + 127) / 128, 128, 0, s>>>(W, sol[0], sol[1], sol[2], nullptr, nullptr, nullptr, nullptr);
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}


bool boundary_group_match(const BoundaryOp& L, const Grid& gl, const BoundaryOp& F, const Grid& gf,
                          double max_frac, double* ratio, GroupCorrection& C, cudaStream_t s) {
  if (!L.precomputed || !F.precomputed || L.ibctyp != 2 || F.ibctyp != 2 || L.tree != F.tree) return false;
  if (L.arith != F.arith) return false;
  // an operator whose coarsest level goes by FFT stays with its problem: the
  // group would apply that level as the dense block, and in FP64 (the only
  // arithmetic of the FFT path) sharing the weights saves memory traffic
  // the step does not wait on, while the dense block costs five times the
  // FFT path's operations
  if (L.ff.on || F.ff.on) return false;
  if (L.ntarget != F.ntarget || L.ncell_total != F.ncell_total || L.levmax != F.levmax || L.dense != F.dense ||
      L.ntopd != F.ntopd || L.lev_off != F.lev_off || L.wtop.n != F.wtop.n)
    return false;
  for (int d = 0; d < 3; ++d)
    if (gl.n[d] != gf.n[d]) return false;
  // weights dS / r scale with the spacing when the cells are similar
  const double r = gf.d[0] / gl.d[0];
  for (int d = 1; d < 3; ++d)
    if (std::fabs(gf.d[d] / gl.d[d] - r) > 1e-14 * r) return false;
  // the tree (children, dummy flags) must be the same; preorder of its cells
  const int nc = L.ncell_total, nt = L.ntarget;
  std::vector<int> lch(4 * (size_t)nc), fch(4 * (size_t)nc), lfl((size_t)nc), ffl((size_t)nc);
  VPMG_CUDA(cudaMemcpyAsync(lch.data(), L.child.p, sizeof(int) * lch.size(), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaMemcpyAsync(fch.data(), F.child.p, sizeof(int) * fch.size(), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaMemcpyAsync(lfl.data(), L.flags.p, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaMemcpyAsync(ffl.data(), F.flags.p, sizeof(int) * nc, cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  if (lch != fch || lfl != ffl) return false;
  std::vector<int> pre((size_t)nc, -1);
  {
    int next = 0;
    std::vector<std::pair<int, int>> st;  // (cell, level)
    const int top0 = L.lev_off[L.levmax];
    for (int c = L.ntopd - 1; c >= 0; --c) st.push_back({top0 + c, L.levmax});
    while (!st.empty()) {
      const auto [c, lev] = st.back();
      st.pop_back();
      if (c < 0 || c >= nc || pre[c] >= 0) continue;
      pre[c] = next++;
      if (lev == 0) continue;
      const int k = (lfl[c] < 0) ? 2 : 4;
      for (int q = k - 1; q >= 0; --q) st.push_back({lch[4 * (size_t)c + q], lev - 1});
    }
    for (int c = 0; c < nc; ++c)
      if (pre[c] < 0) pre[c] = next++;  // not reachable from the top: never in a row
  }
  DBuf<int> dpre, cnt, bad;
  upload(dpre, pre);
  cnt.ensure((size_t)nt);
  bad.ensure(1);
  VPMG_CUDA(cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  auto words = [](const DBuf<float2>& b) { return reinterpret_cast<const double*>(b.p); };
  CorrArgs A{L.rowptr.p, F.rowptr.p, L.col.p, F.col.p, words(L.w), words(F.w), L.dense ? words(L.wtop) : nullptr,
             F.dense ? words(F.wtop) : nullptr, dpre.p, L.ntopd, L.lev_off[L.levmax], r, 1e-12,
             L.arith == VPMG_ARITH_FF48 ? 1 : 0};
  k_corr_count<<<(nt + 127) / 128, 128, 0, s>>>(A, L.tgt_node.p, F.tgt_node.p, nt, cnt.p, bad.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
  std::vector<int> hc((size_t)nt);
  int hb = 1;
  VPMG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(int) * nt, cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaMemcpyAsync(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  if (hb) return false;
  std::vector<int> rows;
  std::vector<long long> crp(1, 0);
  for (int t = 0; t < nt; ++t)
    if (hc[t]) {
      rows.push_back(t);
      crp.push_back(crp.back() + hc[t]);
    }
  const double all = (double)(L.nnz + L.ndense_acc);
  if ((double)crp.back() > max_frac * all) return false;
  C.nrows = (int)rows.size();
  C.nnz = crp.back();
  if (C.nrows) {
    upload(C.rows, rows);
    upload(C.rowptr, crp);
    C.col.ensure((size_t)C.nnz);
    C.w.ensure((size_t)C.nnz);
    k_corr_fill<<<(C.nrows + 127) / 128, 128, 0, s>>>(A, C.rows.p, C.rowptr.p, C.nrows, C.col.p, C.w.p);
    VPMG_LAUNCHED();
    VPMG_CUDA(cudaGetLastError());
    VPMG_CUDA(cudaStreamSynchronize(s));
  }
  *ratio = r;
  return true;
}

void boundary_release_recorded(BoundaryOp& B) {
  B.rowptr.release(); B.col.release(); B.w.release(); B.wtop.release(); B.dsum.release(); B.csrc_ff.release();
  B.colptr.release(); B.trow.release(); B.tw.release(); B.vff.release(); B.dpart.release();
  farfield_release(B);
  B.precomputed = false;
  B.dense = false;
  B.transposed = false;
  B.nnz = 0;
  B.ndense_acc = 0;
}

void boundary_group_correct(const BoundaryOp& F, const GroupCorrection& C, double* const sol[3], cudaStream_t s) {
  if (!C.nrows) return;
  k_apply_corr<<<(unsigned)(((long long)C.nrows * 32 + 255) / 256), 256, 0, s>>>(
      C.rows.p, C.rowptr.p, C.nrows, C.col.p, C.w.p, F.csrc.p, F.ncell_total, F.tgt_node.p, -1.0 / (4.0 * kPI), sol[0],
      sol[1], sol[2]);
  VPMG_LAUNCHED();
}

void boundary_group_sources(BoundaryOp& B, float2* gsrc, int slot, int lanes, cudaStream_t s) {
  aggregate_levels(B, s);
  const size_t nc4 = 4 * (size_t)B.ncell_total;
  const unsigned g = (unsigned)std::min<size_t>((nc4 + 255) / 256, 152 * 16);
  if (B.arith == VPMG_ARITH_FF48)
    k_split_slot<MacFF><<<g, 256, 0, s>>>(B.csrc.p, B.ncell_total, slot, lanes, gsrc);
  else
    k_split_slot<Mac64><<<g, 256, 0, s>>>(B.csrc.p, B.ncell_total, slot, lanes, reinterpret_cast<double*>(gsrc));
  VPMG_LAUNCHED();
}

// Segments of the coarsest cells for k_group_dense: at least three waves of
// CTAs (5 per SM), 64+ cells each; the same split at set-up and per step.
static int group_dense_cseg(const BoundaryOp& L, int nprob) {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int nquad = nprob > 8 ? 4 : (nprob > 4 ? 2 : 1);
  const long long ctas = ((L.ntarget + 31) / 32 + 8 / nquad - 1) / (8 / nquad);
  int seg = 1;
  while (seg < 8 && ctas * seg < 15LL * sms && L.ntopd / (2 * seg) >= 64) seg *= 2;
  return (((L.ntopd + seg - 1) / seg) + 1) & ~1;
}

size_t boundary_group_partial_count(const BoundaryOp& L, int nprob) {
  if (!L.dense) return 0;
  const int cseg = group_dense_cseg(L, nprob);
  const size_t nseg = (size_t)((L.ntopd + cseg - 1) / cseg);
  return nseg * nprob * 3 * (size_t)L.ntarget;
}

template <class M>
static void group_apply_t(const BoundaryOp& L, const float2* gsrc, int nprob, double* part, const GroupOut& G,
                          cudaStream_t s) {
  using H = typename M::H;
  int nseg = 0;
  const H* gs = reinterpret_cast<const H*>(gsrc);
  if (L.dense) {
    VPMG_CHECK(part, VPMG_ERR_STATE, "group apply: no buffer for the dense block's partial sums");
    const int nquad = nprob > 8 ? 4 : (nprob > 4 ? 2 : 1);
    const int cseg = group_dense_cseg(L, nprob);
    nseg = (L.ntopd + cseg - 1) / cseg;
    const int per = 8 / nquad;
    const dim3 grid((unsigned)(((L.ntarget + 31) / 32 + per - 1) / per), (unsigned)nseg);
    const size_t smem = sizeof(H) * 2 * kGroupTile * nprob;
    k_group_dense<M><<<grid, 256, smem, s>>>(reinterpret_cast<const typename M::W2*>(L.wtop.p), gs,
                                             L.lev_off[L.levmax], L.ntopd, (L.ntopd + 1) / 2, L.ntarget, nprob, nquad,
                                             cseg, part);
    VPMG_LAUNCHED();
  }
  const long long threads = (long long)L.ntarget * 32;
  k_apply_group<M><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
      L.rowptr.p, L.col.p, reinterpret_cast<const typename M::W*>(L.w.p), gs, L.tgt_node.p, L.ntarget, nprob, part,
      nseg, G);
  VPMG_LAUNCHED();
}

void boundary_group_apply(const BoundaryOp& L, const float2* gsrc, int nprob, double* part, const GroupOut& G,
                          cudaStream_t s) {
  VPMG_CHECK(L.precomputed && nprob >= 1 && nprob <= kGroupMax, VPMG_ERR_STATE,
             "group apply: operator not recorded or group too large");
  if (L.arith == VPMG_ARITH_FF48) group_apply_t<MacFF>(L, gsrc, nprob, part, G, s);
  else group_apply_t<Mac64>(L, gsrc, nprob, part, G, s);
  VPMG_CUDA(cudaGetLastError());
}

}  // namespace vpmg

// ---------------------------------------------------------- transposes ----
// Adjoints of the boundary-value chain for the whole-step gradient: with
// BC = -(1/4pi) T agg N (sol0), these apply N^T agg^T T^T (-1/4pi) to the
// adjoint of the boundary values of one component.
namespace vpmg {
namespace {

__global__ void __launch_bounds__(256) k_csr_T(const long long* __restrict__ rowptr, const int* __restrict__ col,
                                               const double* __restrict__ wgt, int ff, const int* __restrict__ tgt_node,
                                               int ntarget, double scale, const double* __restrict__ bcbar,
                                               double* __restrict__ cellbar) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntarget) return;
  const double v = scale * bcbar[tgt_node[warp]];
  if (v == 0.0) return;
  for (long long k = rowptr[warp] + lane; k < rowptr[warp + 1]; k += 32)
    atomicAdd(&cellbar[col[k]], wval(wgt, k, ff) * v);
}

// Transposed interaction list: per-cell counts, then a fill through per-cell
// cursors (the order inside a cell's list follows the atomics, fixed once built).
__global__ void k_col_count(const long long* __restrict__ rowptr, const int* __restrict__ col, int ntarget,
                            int* __restrict__ cnt) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntarget) return;
  for (long long k = rowptr[warp] + lane; k < rowptr[warp + 1]; k += 32) atomicAdd(&cnt[col[k]], 1);
}
__global__ void k_col_fill(const long long* __restrict__ rowptr, const int* __restrict__ col,
                           const double* __restrict__ wgt, int ntarget, const long long* __restrict__ colptr,
                           int* __restrict__ cursor, int* __restrict__ trow, double* __restrict__ tw) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ntarget) return;
  for (long long k = rowptr[warp] + lane; k < rowptr[warp + 1]; k += 32) {
    const int c = col[k];
    const long long slot = colptr[c] + atomicAdd(&cursor[c], 1);
    trow[slot] = warp;
    tw[slot] = wgt[k];  // the 8-byte weight word, either arithmetic
  }
}
// The boundary-value adjoint of each target in the policy's arithmetic, once per call.
template <class M>
__global__ void k_split_bc(const double* __restrict__ bcbar, const int* __restrict__ tgt_node, int ntarget,
                           typename M::V* __restrict__ v) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t < ntarget) v[t] = M::vsplit(bcbar[tgt_node[t]]);
}

// cellbar[c] = scale * sum over the cell's targets of w * bcbar(target node);
// warp per cell, products and sums in the policy's arithmetic.
template <class M>
__global__ void __launch_bounds__(256) k_csc_T(const long long* __restrict__ colptr, const int* __restrict__ trow,
                                               const typename M::W* __restrict__ tw,
                                               const typename M::V* __restrict__ v, int ncell, double scale,
                                               double* __restrict__ cellbar) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= ncell) return;
  typename M::Acc f;
  for (long long k = colptr[warp] + lane; k < colptr[warp + 1]; k += 32)
    M::mac(f, __ldg(&tw[k]), __ldg(&v[__ldg(&trow[k])]));
  double a = M::fin(f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) cellbar[warp] = scale * a;
}

// Transpose of the dense block: cellbar[top0 + c] += scale * sum_t w(t, c) bcbar(node t).
// A warp per (cell, group of kDenseTGroup target chunks) forms a partial sum
// (each chunk's 32 weights are one coalesced row), then k_dense_T_sum adds
// a cell's groups in order (deterministic).
constexpr int kDenseTGroup = 64;
template <class M>
__global__ void __launch_bounds__(256) k_dense_T(const typename M::W* __restrict__ wtop,
                                                 const typename M::V* __restrict__ v, int ntop, int ntarget,
                                                 double* __restrict__ part) {
  const long long wid = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nchunk = (ntarget + 31) / 32;
  const int ngroup = (nchunk + kDenseTGroup - 1) / kDenseTGroup;
  if (wid >= (long long)ntop * ngroup) return;
  const int c = (int)(wid % ntop), grp = (int)(wid / ntop);
  const int g1 = min(nchunk, (grp + 1) * kDenseTGroup);
  typename M::Acc f;
  for (int g = grp * kDenseTGroup; g < g1; ++g) {
    const int t = g * 32 + lane;
    if (t >= ntarget) continue;
    const typename M::W w = __ldg(&wtop[(((size_t)g * ((ntop + 1) >> 1) + (c >> 1)) * 32 + lane) * 2 + (c & 1)]);
    M::mac(f, w, __ldg(&v[t]));
  }
  double a = M::fin(f);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  if (lane == 0) part[(size_t)grp * ntop + c] = a;
}

__global__ void k_dense_T_sum(const double* __restrict__ part, int ntop, int ngroup, int top0, double scale,
                              double* __restrict__ cellbar) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ntop) return;
  double a = 0.0;
  for (int grp = 0; grp < ngroup; ++grp) a += part[(size_t)grp * ntop + c];
  cellbar[top0 + c] += scale * a;
}

// leaf adjoint = its own level-0 adjoint + sum over ancestors of ds_leaf / ds_cell * cell adjoint
__global__ void k_agg_T(const int* __restrict__ anc, const double* __restrict__ cds, int nbound, int levmax,
                        const double* __restrict__ cellbar, double* __restrict__ panelbar) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nbound) return;
  double v = cellbar[p];
  const double ds = cds[p];
  for (int l = 1; l <= levmax; ++l) {
    const int a = anc[(size_t)(l - 1) * nbound + p];
    if (a >= 0) v += ds / cds[a] * cellbar[a];
  }
  panelbar[p] = v;
}

__global__ void k_normal_deriv_T(const double* __restrict__ panelbar, int NX, int NY, const int* __restrict__ face,
                                 const int* __restrict__ pi, const int* __restrict__ pj, const int* __restrict__ pk,
                                 int nbound, double invx, double invy, double invz, double* __restrict__ sol0bar) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= nbound) return;
  const double g = 0.25 * panelbar[p];
  if (g == 0.0) return;
  const double a[5] = {25.0 / 12.0, -4.0, 3.0, -4.0 / 3.0, 0.25};
  const int f = face[p];
  const long long sx = 1, sy = NX, sz = (long long)NX * NY;
  long long step, e1, e2;
  double inv;
  if (f < 2) { step = (f == 0) ? sx : -sx; e1 = sy; e2 = sz; inv = invx; }
  else if (f < 4) { step = (f == 2) ? sy : -sy; e1 = sx; e2 = sz; inv = invy; }
  else { step = (f == 4) ? sz : -sz; e1 = sx; e2 = sy; inv = invz; }
  const long long base = (long long)(pi[p] - 1) * sx + (long long)(pj[p] - 1) * sy + (long long)(pk[p] - 1) * sz;
  const long long corner[4] = {base, base + e1, base + e1 + e2, base + e2};
  for (int m = 0; m < 4; ++m)
    for (int k = 0; k < 5; ++k) atomicAdd(&sol0bar[corner[m] + k * step], g * inv * a[k]);
}

}  // namespace

void boundary_transpose_prepare(BoundaryOp& B, cudaStream_t s) {
  if (B.precomputed) {  // at set-up: the transposes may be captured in graphs
    B.vff.ensure((size_t)B.ntarget);
    if (B.dense) B.dpart.ensure((size_t)B.ntopd * (((B.ntarget + 31) / 32 + kDenseTGroup - 1) / kDenseTGroup));
  }
  if (!B.precomputed || B.transposed || B.nnz == 0) return;
  const long long need = B.nnz * (long long)(sizeof(int) + sizeof(float2)) + 8LL * (B.ncell_total + 1);
  size_t free_b = 0, total_b = 0;
  VPMG_CUDA(cudaMemGetInfo(&free_b, &total_b));
  if (need > (long long)(0.5 * (double)free_b)) return;  // keep the atomic scatter
  DBuf<int> cnt;
  cnt.ensure(B.ncell_total);
  VPMG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * B.ncell_total, s));
  const long long threads = (long long)B.ntarget * 32;
  const unsigned blocks = (unsigned)((threads + 255) / 256);
  k_col_count<<<blocks, 256, 0, s>>>(B.rowptr.p, B.col.p, B.ntarget, cnt.p);
  VPMG_LAUNCHED();
  std::vector<int> hc(B.ncell_total);
  VPMG_CUDA(cudaMemcpyAsync(hc.data(), cnt.p, sizeof(int) * B.ncell_total, cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  std::vector<long long> cp(B.ncell_total + 1, 0);
  for (int c = 0; c < B.ncell_total; ++c) cp[c + 1] = cp[c] + hc[c];
  VPMG_CHECK(cp[B.ncell_total] == B.nnz, VPMG_ERR_TREE, "transposed interaction list lost entries");
  try {
    upload(B.colptr, cp);
    B.trow.ensure((size_t)B.nnz);
    B.tw.ensure((size_t)B.nnz);
  } catch (const Error& e) {
    if (e.status != VPMG_ERR_NOMEM) throw;
    B.colptr.release(); B.trow.release(); B.tw.release();
    return;
  }
  VPMG_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int) * B.ncell_total, s));
  k_col_fill<<<blocks, 256, 0, s>>>(B.rowptr.p, B.col.p, reinterpret_cast<const double*>(B.w.p), B.ntarget,
                                    B.colptr.p, cnt.p, B.trow.p, reinterpret_cast<double*>(B.tw.p));
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
  VPMG_CUDA(cudaStreamSynchronize(s));
  B.transposed = true;
}

template <class M>
static void apply_T_recorded(BoundaryOp& B, const double* bcbar, double* cellbar, cudaStream_t s) {
  using V = typename M::V;
  using W = typename M::W;
  const double scale = -1.0 / (4.0 * kPI);
  V* vv = reinterpret_cast<V*>(B.vff.p);
  if (B.transposed || B.dense) {
    VPMG_CHECK(B.vff.n >= (size_t)B.ntarget, VPMG_ERR_STATE, "boundary transpose not prepared");
    k_split_bc<M><<<(B.ntarget + 255) / 256, 256, 0, s>>>(bcbar, B.tgt_node.p, B.ntarget, vv);
    VPMG_LAUNCHED();
  }
  auto dense_T = [&] {
    if (!B.dense) return;
    const int ngroup = ((B.ntarget + 31) / 32 + kDenseTGroup - 1) / kDenseTGroup;
    VPMG_CHECK(B.dpart.n >= (size_t)ngroup * B.ntopd, VPMG_ERR_STATE, "boundary transpose not prepared");
    const long long threads = (long long)B.ntopd * ngroup * 32;
    k_dense_T<M><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(reinterpret_cast<const W*>(B.wtop.p), vv, B.ntopd,
                                                                  B.ntarget, B.dpart.p);
    VPMG_LAUNCHED();
    k_dense_T_sum<<<(B.ntopd + 255) / 256, 256, 0, s>>>(B.dpart.p, B.ntopd, ngroup, B.lev_off[B.levmax], scale,
                                                         cellbar);
    VPMG_LAUNCHED();
  };
  if (B.transposed) {
    const long long threads = (long long)B.ncell_total * 32;
    k_csc_T<M><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(B.colptr.p, B.trow.p,
                                                                 reinterpret_cast<const W*>(B.tw.p), vv,
                                                                 B.ncell_total, scale, cellbar);
    VPMG_LAUNCHED();
    dense_T();
    return;
  }
  VPMG_CUDA(cudaMemsetAsync(cellbar, 0, sizeof(double) * B.ncell_total, s));
  const long long threads = (long long)B.ntarget * 32;
  k_csr_T<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(B.rowptr.p, B.col.p,
                                                            reinterpret_cast<const double*>(B.w.p),
                                                            M::kFF ? 1 : 0, B.tgt_node.p, B.ntarget, scale, bcbar,
                                                            cellbar);
  VPMG_LAUNCHED();
  dense_T();
}

void boundary_apply_T(BoundaryOp& B, const double* bcbar, double* cellbar, cudaStream_t s) {
  if (B.precomputed) {
    if (B.arith == VPMG_ARITH_FF48) apply_T_recorded<MacFF>(B, bcbar, cellbar, s);
    else apply_T_recorded<Mac64>(B, bcbar, cellbar, s);
  } else {
    VPMG_CUDA(cudaMemsetAsync(cellbar, 0, sizeof(double) * B.ncell_total, s));
    const WalkDev W = walk_dev(B);
    k_walk<kTranspose><<<(B.ntarget + 127) / 128, 128, 0, s>>>(W, cellbar, const_cast<double*>(bcbar), nullptr,
                                                               nullptr, nullptr, nullptr, nullptr);
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}

void boundary_agg_T(BoundaryOp& B, const double* cellbar, double* panelbar, cudaStream_t s) {
  k_agg_T<<<(B.nbound + 255) / 256, 256, 0, s>>>(B.anc.p, B.cds.p, B.nbound, B.levmax, cellbar, panelbar);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void boundary_panels_T(BoundaryOp& B, const Grid& g, const double* panelbar, double* sol0bar, cudaStream_t s) {
  k_normal_deriv_T<<<(B.nbound + 255) / 256, 256, 0, s>>>(panelbar, g.n[0], g.n[1], B.pan_face.p, B.pan_i.p, B.pan_j.p,
                                                          B.pan_k.p, B.nbound, 1.0 / g.d[0], 1.0 / g.d[1],
                                                          1.0 / g.d[2], sol0bar);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

}  // namespace vpmg
