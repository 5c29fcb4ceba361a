// particles.cu -- particle <-> mesh kernels.
//
//  * deposition: project_particles_3D + project_vol3d(IDVPM=1)
//    (source/pmproject.f90:43-153) as sort-by-cell plus a per-node gather:
//    run-to-run deterministic, no floating-point atomics;
//  * back_to_particles_3D(itype=1) (source/vpm_time.f90:62-107) fused with
//    the forward Euler update of source/test.f90:104-117;
//  * remesh_particles_3d(1) emission (source/vpm_remesh.f90:137-195) as an
//    ordered stream compaction in (k,j,i) node order.
#include <cmath>

#include "ff.cuh"
#include "particles.h"

namespace vpmg {

namespace {

// M4' and the other projection kernels of source/pmproject.f90:391-431, in
// float-float (ff.cuh), |x| given as a float-float value; the branch tests
// compare the whole value (hi, then lo).
__device__ __forceinline__ bool ff_gt(float2 a, float c) { return a.x > c || (a.x == c && a.y > 0.0f); }
__device__ __forceinline__ bool ff_ge(float2 a, float c) { return a.x > c || (a.x == c && a.y >= 0.0f); }
__device__ __forceinline__ float2 ffc(float c) { return make_float2(c, 0.0f); }
__device__ __forceinline__ float2 proj_fun_ff(int itype, float2 xa) {
  const float2 zero = ffc(0.0f), one = ffc(1.0f);
  if (itype == 4) {
    if (ff_gt(xa, 2.0f)) return zero;
    if (ff_ge(xa, 1.0f)) {
      const float2 a = ff::sub(ffc(2.0f), xa);
      return ff::scale(ff::mul(ff::mul(a, a), ff::sub(one, xa)), 0.5f);
    }
    const float2 x2 = ff::mul(xa, xa);
    return ff::fma(ffc(1.5f), ff::mul(x2, xa), ff::fma(ffc(-2.5f), x2, one));
  }
  if (itype == 3) {
    if (ff_gt(xa, 1.5f)) return zero;
    if (ff_ge(xa, 0.5f)) {
      const float2 a = ff::sub(ffc(1.5f), xa);
      return ff::scale(ff::mul(a, a), 0.5f);
    }
    const float2 a = ff::add(xa, ffc(1.5f)), b = ff::add(xa, ffc(0.5f));
    return ff::sub(ff::scale(ff::mul(a, a), 0.5f), ff::mul(ffc(1.5f), ff::mul(b, b)));
  }
  if (itype == 2) return ff_gt(xa, 1.0f) ? zero : ff::sub(one, xa);
  if (itype == 5 || itype == 6) {
    const float lim = (itype == 5) ? 0.5f : 1.0f;
    if (!ff_gt(xa, lim)) return ff::sub(one, ff::mul(xa, xa));
    if (!ff_gt(xa, lim + 1.0f)) return ff::scale(ff::mul(ff::sub(one, xa), ff::sub(ffc(2.0f), xa)), 0.5f);
    return zero;
  }
  return zero;
}

// The same projection kernels in FP64, written as the reference writes them
// (pmproject.f90:391-431), |x| given.
__device__ __forceinline__ double proj_fun_f64(int itype, double xa) {
  if (itype == 4) {
    if (xa > 2.0) return 0.0;
    if (xa >= 1.0) return 0.5 * ((2.0 - xa) * (2.0 - xa)) * (1.0 - xa);
    return 1.0 - 2.5 * (xa * xa) + 1.5 * (xa * xa * xa);
  }
  if (itype == 3) {
    if (xa > 1.5) return 0.0;
    if (xa >= 0.5) return 0.5 * (-xa + 1.5) * (-xa + 1.5);
    return 0.5 * (xa + 1.5) * (xa + 1.5) - 1.5 * (xa + 0.5) * (xa + 0.5);
  }
  if (itype == 2) return (xa > 1.0) ? 0.0 : 1.0 - xa;
  if (itype == 5 || itype == 6) {
    const double lim = (itype == 5) ? 0.5 : 1.0;
    if (xa <= lim) return 1.0 - xa * xa;
    if (xa <= lim + 1.0) return 0.5 * (1.0 - xa) * (2.0 - xa);
    return 0.0;
  }
  return 0.0;
}

// Cell index exactly as int((x - XMIN)/DX) (IEEE division, truncation).
__device__ __forceinline__ int cell_of(double x, double xmin, double d) { return (int)__ddiv_rn(__dsub_rn(x, xmin), d); }

__global__ void k_keys(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                       const int* __restrict__ np_dev, MeshDev m, int* __restrict__ key, int* __restrict__ counts,
                       int* __restrict__ err) {
  const int np = *np_dev;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
  const int i0 = cell_of(x[p], m.xmin[0], m.d[0]);
  const int j0 = cell_of(y[p], m.xmin[1], m.d[1]);
  const int k0 = cell_of(z[p], m.xmin[2], m.d[2]);
  // stencil nodes (0-based) c - ips .. c + ipf must lie on the mesh
  const bool ok = (x[p] - m.xmin[0] >= 0.0) && (y[p] - m.xmin[1] >= 0.0) && (z[p] - m.xmin[2] >= 0.0) &&
                  i0 - m.ips >= 0 && j0 - m.ips >= 0 && k0 - m.ips >= 0 && i0 + m.ipf < m.n[0] &&
                  j0 + m.ipf < m.n[1] && k0 + m.ipf < m.n[2];
  if (!ok) {
    key[p] = -1;
    atomicExch(err, 1);
    continue;
  }
  const int kk = i0 + m.n[0] * (j0 + m.n[1] * k0);
  key[p] = kk;
  atomicAdd(&counts[kk], 1);
  }
}

__global__ void k_scatter(const int* __restrict__ key, const int* __restrict__ np_dev, const int* __restrict__ starts,
                          int* __restrict__ cursor, int* __restrict__ perm) {
  const int np = *np_dev;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const int kk = key[p];
    if (kk < 0) continue;
    const int slot = starts[kk] + atomicAdd(&cursor[kk], 1);
    perm[slot] = p;
  }
}

// Restores particle-index order inside each cell (determinism).
__global__ void k_cell_order(const int* __restrict__ starts, int ncell, int* __restrict__ perm) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncell) return;
  const int s = starts[c], e = starts[c + 1];
  if (e - s < 2) return;
  for (int a = s + 1; a < e; ++a) {
    const int v = perm[a];
    int b = a - 1;
    while (b >= s && perm[b] > v) {
      perm[b + 1] = perm[b];
      --b;
    }
    perm[b + 1] = v;
  }
}

// Sorted records: per slot 4+4+4 stencil weights, 3 strengths, base cell x.
__global__ void k_records(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                          const double* __restrict__ q0, const double* __restrict__ q1, const double* __restrict__ q2,
                          const int* __restrict__ perm, const int* __restrict__ nsorted_dev, MeshDev m,
                          float2* __restrict__ rec) {
  const int nsorted = *nsorted_dev;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsorted; s += gridDim.x * blockDim.x) {
  const int p = perm[s];
  const double pos[3] = {x[p], y[p], z[p]};
  float2* r = rec + (size_t)s * kRecLen;
  float2 wgt[3][4];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    const int c0 = cell_of(pos[d], m.xmin[d], m.d[d]);
    // t of the first stencil node in FP64, the next ones t - a in float-float,
    // the kernel in float-float (ff.cuh)
    const int node0 = c0 - m.ips;  // 0-based node = (i-1) of the reference
    const float2 t0 = ff::split((pos[d] - m.xmin[d] - (double)node0 * m.d[d]) * m.inv[d]);
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      float2 t = ff::add(t0, make_float2(-(float)a, 0.0f));
      if (t.x < 0.0f) t = ff::neg(t);
      wgt[d][a] = (a <= m.ips + m.ipf) ? proj_fun_ff(m.itype, t) : make_float2(0.0f, 0.0f);
    }
    if (d == 0) r[23] = cell_bits(c0);
  }
#pragma unroll
  for (int a = 0; a < 4; ++a) r[a] = wgt[0][a];
#pragma unroll
  for (int b = 0; b < 4; ++b)
#pragma unroll
    for (int c = 0; c < 4; ++c) r[4 + 4 * b + c] = ff::mul(wgt[1][b], wgt[2][c]);
  r[kRecQ] = ff::split(q0[p]);
  r[kRecQ + 1] = ff::split(q1[p]);
  r[kRecQ + 2] = ff::split(q2[p]);
  }
}

// One thread per node: gathers the particles of the (ips+ipf+1)^3 cells
// whose stencil covers the node, in fixed cell and slot order.  The weight
// products and sums run in float-float on the FP32 pipes (ff.cuh).
__global__ void k_deposit(const int* __restrict__ starts, const float2* __restrict__ rec, MeshDev m, double inv_dv,
                          double* __restrict__ r0, double* __restrict__ r1, double* __restrict__ r2) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= N) return;
  const int i = (int)(id % m.n[0]);
  const int j = (int)((id / m.n[0]) % m.n[1]);
  const int k = (int)(id / ((size_t)m.n[0] * m.n[1]));
  const int w = m.ips + m.ipf;  // stencil width - 1
  // particle base cell c covers nodes c-ips .. c+ipf  =>  c in [node-ipf, node+ips]
  const int xlo = max(i - m.ipf, 0), xhi = min(i + m.ips, m.n[0] - 1);
  float2 a0 = make_float2(0.0f, 0.0f), a1 = a0, a2 = a0;
  for (int ck = max(k - m.ipf, 0); ck <= min(k + m.ips, m.n[2] - 1); ++ck) {
    const int iz = k - ck + m.ips;
    for (int cj = max(j - m.ipf, 0); cj <= min(j + m.ips, m.n[1] - 1); ++cj) {
      const int iy = j - cj + m.ips;
      const size_t row = (size_t)m.n[0] * (cj + (size_t)m.n[1] * ck);
      const int s = starts[row + xlo], e = starts[row + xhi + 1];
      for (int t = s; t < e; ++t) {
        const float2* r = rec + (size_t)t * kRecLen;
        // strengths and cell index as two 16-byte loads (slots 20-21, 22-23)
        const float4 q2c = __ldg(reinterpret_cast<const float4*>(r) + 11);
        const int ix = i - __float_as_int(q2c.z) + m.ips;
        if ((unsigned)ix > (unsigned)w) continue;  // only for a binning that does not match rec
        const float4 q01 = __ldg(reinterpret_cast<const float4*>(r) + 10);
        const float2 f = ff::mul(__ldg(&r[ix]), __ldg(&r[4 + 4 * iy + iz]));
        a0 = ff::fma(f, make_float2(q01.x, q01.y), a0);
        a1 = ff::fma(f, make_float2(q01.z, q01.w), a1);
        a2 = ff::fma(f, make_float2(q2c.x, q2c.y), a2);
      }
    }
  }
  r0[id] = ff::to_double(a0) * inv_dv;
  r1[id] = ff::to_double(a1) * inv_dv;
  r2[id] = ff::to_double(a2) * inv_dv;
}

// FP64 records, slot-major: slot k of sorted particle s at rec[k * cs + s]
// (cs = the record stride, the particle capacity), so that a warp's lanes
// read one slot of consecutive particles with coalesced loads.  Slots: x
// weights (0..3), y-z weight products (4 + 4b + c), strengths (20..22), and
// in slot 23 the base cell's x index (low four bytes) and its linear index
// (high four bytes).  The cell is the binning's (k_keys: the reference's
// int((x - XMIN)/DX) per axis), so no division is repeated here; the
// stencil offsets follow the reference, x_a = (XP - XMIN - (i_a - 1) DX) / DX,
// evaluated with the reciprocal of DX.
__global__ void k_records64(const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                            const double* __restrict__ q0, const double* __restrict__ q1,
                            const double* __restrict__ q2, const int* __restrict__ perm,
                            const int* __restrict__ key, const int* __restrict__ nsorted_dev, MeshDev m,
                            double* __restrict__ rec, size_t cs) {
  const int nsorted = *nsorted_dev;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsorted; s += gridDim.x * blockDim.x) {
    const int p = perm[s];
    const int kk = key[p];
    const int cell[3] = {kk % m.n[0], (kk / m.n[0]) % m.n[1], kk / (m.n[0] * m.n[1])};
    const double pos[3] = {x[p], y[p], z[p]};
    double* r = rec + s;
    double wgt[3][4];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      const int node0 = cell[d] - m.ips;  // 0-based node = (i-1) of the reference
      const double off = pos[d] - m.xmin[d];
      if (m.itype == 4) {
        // M4' at the four distances 1+f, f, 1-f, 2-f from the offset f of
        // the cell's own node (the branches of projection_fun resolved by
        // the stencil's geometry): 16 FP64 operations instead of four
        // offsets and four branchy polynomials
        const double f = (off - (double)(node0 + 1) * m.d[d]) * m.inv[d];
        const double g = 1.0 - f, f2 = f * f, g2 = g * g;
        wgt[d][0] = -0.5 * (f * g2);
        wgt[d][1] = fma(1.5 * f, f2, fma(-2.5, f2, 1.0));
        wgt[d][2] = fma(1.5 * g, g2, fma(-2.5, g2, 1.0));
        wgt[d][3] = -0.5 * (f2 * g);
      } else {
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          const double t = (off - (double)(node0 + a) * m.d[d]) * m.inv[d];
          wgt[d][a] = (a <= m.ips + m.ipf) ? proj_fun_f64(m.itype, fabs(t)) : 0.0;
        }
      }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) r[a * cs] = wgt[0][a];
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int c = 0; c < 4; ++c) r[(4 + 4 * b + c) * cs] = wgt[1][b] * wgt[2][c];
    r[kRecQ * cs] = q0[p];
    r[(kRecQ + 1) * cs] = q1[p];
    r[(kRecQ + 2) * cs] = q2[p];
    r[23 * cs] = __hiloint2double(kk, cell[0]);
  }
}

// FP64 deposition gather, balanced over a warp's lanes.  A warp owns 32
// consecutive x nodes of one (j, k) row.  Node n receives from the
// particles of the (ips+ipf+1)^2 cell rows (cj, ck) covering it, in the
// cell range [n - ipf, n + ips] of each row: its visits, enumerated in
// (row, sorted slot) order.  The warp's visits (node by node) are split
// into 32 equal chunks, one per lane, so every lane does two visits per trip
// (2 DMUL + 6 DFMA) instead of idling while a neighbour with more particles
// finishes.  A lane's running sums are flushed where its chunk leaves a
// node: the first and last node it touches as pieces, nodes it covers
// entirely as totals.  Each node then adds its pieces in lane order: a
// fixed order, so the result is the same bits every run; no atomics.
constexpr int kDepWarps = 8;
__global__ void __launch_bounds__(kDepWarps * 32) k_deposit64(const int* __restrict__ starts,
                                                             const double* __restrict__ rec, size_t cs, MeshDev m,
                                                             double inv_dv, double* __restrict__ r0,
                                                             double* __restrict__ r1, double* __restrict__ r2) {
  __shared__ double pf[kDepWarps][32][3], pl[kDepWarps][32][3], tot[kDepWarps][32][3];
  __shared__ int soff[kDepWarps][32], scnt[kDepWarps][32], snA[kDepWarps][32], snB[kDepWarps][32];
  __shared__ long long srow[kDepWarps][16];  // start of each covering cell row (linear cell index at x = 0)
  __shared__ int swyz[kDepWarps][16];        // the y-z weight slot of that row for this node row
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const int nseg = (m.n[0] + 31) / 32;
  const long long wg = (long long)blockIdx.x * kDepWarps + wl;
  if (wg >= (long long)nseg * m.n[1] * m.n[2]) return;  // whole warps only
  const int seg = (int)(wg % nseg);
  const long long jk = wg / nseg;
  const int j = (int)(jk % m.n[1]), k = (int)(jk / m.n[1]);
  const int i0 = seg * 32;
  const int i = i0 + lane;
  const bool valid = i < m.n[0];
  // the cell rows covering this node row (the same for every lane)
  const int cj0 = max(j - m.ipf, 0), cj1 = min(j + m.ips, m.n[1] - 1);
  const int ck0 = max(k - m.ipf, 0), ck1 = min(k + m.ips, m.n[2] - 1);
  const int ncj = cj1 - cj0 + 1, nrow = ncj * (ck1 - ck0 + 1);  // at most 4 x 4
  if (lane < nrow) {
    const int cj = cj0 + lane % ncj, ck = ck0 + lane / ncj;
    srow[wl][lane] = (long long)m.n[0] * (cj + (long long)m.n[1] * ck);
    swyz[wl][lane] = 4 + 4 * (j - cj + m.ips) + (k - ck + m.ips);
  }
  __syncwarp();
  const double* q0 = rec + kRecQ * cs;
  const double* q1 = rec + (kRecQ + 1) * cs;
  const double* q2 = rec + (kRecQ + 2) * cs;
  // visits of this lane's node, and the warp's scan of them
  int cnt = 0;
  if (valid) {
    const int xl = max(i - m.ipf, 0), xh = min(i + m.ips, m.n[0] - 1);
    for (int r = 0; r < nrow; ++r) {
      const long long rb = srow[wl][r];
      cnt += __ldg(&starts[rb + xh + 1]) - __ldg(&starts[rb + xl]);
    }
  }
  int off = cnt;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const int v = __shfl_up_sync(FULL, off, d);
    if (lane >= d) off += v;
  }
  const int V = __shfl_sync(FULL, off, 31);
  off -= cnt;  // exclusive
  soff[wl][lane] = off;
  scnt[wl][lane] = cnt;
  if (V == 0) {
    if (valid) {
      const size_t id = (size_t)i + (size_t)m.n[0] * (j + (size_t)m.n[1] * k);
      r0[id] = 0.0;
      r1[id] = 0.0;
      r2[id] = 0.0;
    }
    return;
  }
  const int C = (V + 31) / 32;
  const int v0 = min(lane * C, V), v1 = min(v0 + C, V);
  // first node of the chunk: the largest n with off_n <= v0 (it has visits)
  int lo = 0, hi = 31;
  const int vq = min(v0, V - 1);
#pragma unroll
  for (int it = 0; it < 5; ++it) {
    const int mid = (lo + hi + 1) >> 1;
    const int om = __shfl_sync(FULL, off, mid);
    if (om <= vq) lo = mid;
    else hi = mid - 1;
  }
  __syncwarp();
  int nA = -1, n = lo;
  if (v0 < v1) {
    nA = n;
    int ii = i0 + n;
    int xl = max(ii - m.ipf, 0), xh = min(ii + m.ips, m.n[0] - 1);
    // row and slot of visit v0 inside node n
    int local = v0 - soff[wl][n];
    int r = 0, tb = 0, te = 0;
    // the row's cell boundaries: cell xl + k holds slots [b_k, b_{k+1}),
    // b_0 = tb; e1..e4 = b_1..b_4 clamped to the row's end te.  Knowing the
    // slot's cell from them, a visit's loads do not wait on a load of it.
    int e1 = 0, e2 = 0, e3 = 0, e4 = 0;
    auto bounds = [&](long long rb) {
      tb = __ldg(&starts[rb + xl]);
      e1 = __ldg(&starts[rb + min(xl + 1, xh + 1)]);
      e2 = __ldg(&starts[rb + min(xl + 2, xh + 1)]);
      e3 = __ldg(&starts[rb + min(xl + 3, xh + 1)]);
      e4 = __ldg(&starts[rb + min(xl + 4, xh + 1)]);
      te = __ldg(&starts[rb + xh + 1]);
    };
    for (;; ++r) {
      bounds(srow[wl][r]);
      if (local < te - tb) break;
      local -= te - tb;
    }
    int t = tb + local;
    int wyz_slot = swyz[wl][r];
    int kc = 0, nb = e1;  // the slot's cell offset from xl and the next cell's first slot
    while (t >= nb && kc < 3) { ++kc; nb = kc == 1 ? e2 : kc == 2 ? e3 : e4; }
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int v = v0; v < v1;) {
      // two visits of this row per trip, their loads in flight together.
      // Where the row or the chunk has one visit left, the second is the
      // same slot with a zero weight: every lane runs the same FP64
      // instructions (a partly masked one costs the pipe a full issue), and
      // fma(0, q, a) = a keeps the sums those of the visits one by one.
      const int ix = ii - (xl + kc) + m.ips;
      const bool two = v + 1 < v1 && t + 1 < te;
      const int t2 = two ? t + 1 : t;
      int kc2 = kc, nb2 = nb;
      while (t2 >= nb2 && kc2 < 3) { ++kc2; nb2 = kc2 == 1 ? e2 : kc2 == 2 ? e3 : e4; }
      const int ix2 = ii - (xl + kc2) + m.ips;
      const double wa = __ldg(&rec[ix * cs + t]), wb = __ldg(&rec[ix2 * cs + t2]);
      const double ya = __ldg(&rec[wyz_slot * cs + t]), yb = __ldg(&rec[wyz_slot * cs + t2]);
      const double qa0 = __ldg(&q0[t]), qa1 = __ldg(&q1[t]), qa2 = __ldg(&q2[t]);
      const double qb0 = __ldg(&q0[t2]), qb1 = __ldg(&q1[t2]), qb2 = __ldg(&q2[t2]);
      const double fa = wa * ya, fb = two ? wb * yb : 0.0;
      a0 = fma(fb, qb0, fma(fa, qa0, a0));
      a1 = fma(fb, qb1, fma(fa, qa1, a1));
      a2 = fma(fb, qb2, fma(fa, qa2, a2));
      const int step = two ? 2 : 1;
      t += step;
      v += step;
      kc = kc2;
      nb = nb2;
      if (t < te) {
        while (t >= nb && kc < 3) { ++kc; nb = kc == 1 ? e2 : kc == 2 ? e3 : e4; }
        continue;
      }
      if (v == v1) continue;
      // next nonempty row of node n, or the node is complete: flush it
      for (;;) {
        if (++r == nrow) {
          double* dst = (n == nA) ? pf[wl][lane] : tot[wl][n];
          dst[0] = a0; dst[1] = a1; dst[2] = a2;
          a0 = a1 = a2 = 0.0;
          do ++n; while (scnt[wl][n] == 0);
          ii = i0 + n;
          xl = max(ii - m.ipf, 0);
          xh = min(ii + m.ips, m.n[0] - 1);
          r = 0;
        }
        bounds(srow[wl][r]);
        if (te > tb) break;
      }
      t = tb;
      wyz_slot = swyz[wl][r];
      kc = 0;
      nb = e1;
      while (t >= nb && kc < 3) { ++kc; nb = kc == 1 ? e2 : kc == 2 ? e3 : e4; }
    }
    double* dst = (n == nA) ? pf[wl][lane] : pl[wl][lane];  // the chunk's last node
    dst[0] = a0; dst[1] = a1; dst[2] = a2;
  }
  snA[wl][lane] = nA;
  snB[wl][lane] = (v0 < v1) ? n : -1;
  __syncwarp();
  if (!valid) return;
  double b0 = 0.0, b1 = 0.0, b2 = 0.0;
  if (cnt > 0) {
    const int L1 = off / C, L2 = (off + cnt - 1) / C;
    if (L1 == L2 && snA[wl][L1] != lane && snB[wl][L1] != lane) {
      b0 = tot[wl][lane][0]; b1 = tot[wl][lane][1]; b2 = tot[wl][lane][2];  // inside one chunk
    } else {
      for (int L = L1; L <= L2; ++L) {  // pieces in lane order
        const double* src = (snA[wl][L] == lane) ? pf[wl][L] : pl[wl][L];
        b0 += src[0];
        b1 += src[1];
        b2 += src[2];
      }
    }
  }
  const size_t id = (size_t)i + (size_t)m.n[0] * (j + (size_t)m.n[1] * k);
  r0[id] = b0 * inv_dv;
  r1[id] = b1 * inv_dv;
  r2[id] = b2 * inv_dv;
}

// FP64 mesh-to-particle over sorted slots: UP = sum W vel, GP = (sum W def)
// * vol; optionally the forward Euler push.  6 DFMA per particle-node visit.
__global__ void __launch_bounds__(128) k_m2p64(const int* __restrict__ perm, const int* __restrict__ nsorted_dev,
                                               const double* __restrict__ rec, size_t cs, MeshDev m,
                                               const double* __restrict__ v0, const double* __restrict__ v1,
                                               const double* __restrict__ v2, const double* __restrict__ g0,
                                               const double* __restrict__ g1, const double* __restrict__ g2,
                                               double* __restrict__ up, double* __restrict__ gp, int up_add,
                                               double* __restrict__ x, double* __restrict__ y,
                                               double* __restrict__ z, double* __restrict__ q0,
                                               double* __restrict__ q1, double* __restrict__ q2,
                                               const double* __restrict__ vol, int do_euler, double dt, double ux,
                                               double uy, double uz) {
  const int nsorted = *nsorted_dev;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsorted; s += gridDim.x * blockDim.x) {
    const int p = perm[s];
    const double* r = rec + s;  // slot-major records (stride cs)
    double wx[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) wx[a] = r[a * cs];
    const double cw = r[23 * cs];
    const int c0 = __double2loint(cw), kk = __double2hiint(cw);  // the binning's cell
    const int cj = (kk / m.n[0]) % m.n[1], ck = kk / (m.n[0] * m.n[1]);
    const int nw = m.ips + m.ipf + 1;
    double u[3] = {0.0, 0.0, 0.0}, gl[3] = {0.0, 0.0, 0.0};
    for (int c = 0; c < nw; ++c) {
      const int kk = ck - m.ips + c;
      for (int b = 0; b < nw; ++b) {
        const int jj = cj - m.ips + b;
        const double wyz = r[(4 + 4 * b + c) * cs];
        const size_t row = (size_t)m.n[0] * (jj + (size_t)m.n[1] * kk) + (c0 - m.ips);
#pragma unroll
        for (int a = 0; a < 4; ++a) {
          if (a >= nw) break;
          const double f = wx[a] * wyz;
          const size_t id = row + a;
          u[0] = fma(f, __ldg(&v0[id]), u[0]);
          u[1] = fma(f, __ldg(&v1[id]), u[1]);
          u[2] = fma(f, __ldg(&v2[id]), u[2]);
          gl[0] = fma(f, __ldg(&g0[id]), gl[0]);
          gl[1] = fma(f, __ldg(&g1[id]), gl[1]);
          gl[2] = fma(f, __ldg(&g2[id]), gl[2]);
        }
      }
    }
    const double vp = vol[p];
    const double gg0 = gl[0] * vp, gg1 = gl[1] * vp, gg2 = gl[2] * vp;
    if (up) {  // UP = UP + sum W vel (vpm_time.f90:92-94) or UP = sum W vel
      const double b0 = up_add ? up[3 * (size_t)p] : 0.0, b1 = up_add ? up[3 * (size_t)p + 1] : 0.0,
                   b2 = up_add ? up[3 * (size_t)p + 2] : 0.0;
      up[3 * (size_t)p] = b0 + u[0];
      up[3 * (size_t)p + 1] = b1 + u[1];
      up[3 * (size_t)p + 2] = b2 + u[2];
      gp[3 * (size_t)p] = gg0;
      gp[3 * (size_t)p + 1] = gg1;
      gp[3 * (size_t)p + 2] = gg2;
    }
    if (do_euler) {
      x[p] = x[p] + (u[0] + ux) * dt;
      y[p] = y[p] + (u[1] + uy) * dt;
      z[p] = z[p] + (u[2] + uz) * dt;
      q0[p] = q0[p] - gg0 * dt;
      q1[p] = q1[p] - gg1 * dt;
      q2[p] = q2[p] - gg2 * dt;
    }
  }
}

// A field value as a float-float pair: split from FP64, or stored as one.
__device__ __forceinline__ float2 field_ff(const double* __restrict__ f, size_t id) { return ff::split(f[id]); }
__device__ __forceinline__ float2 field_ff(const float2* __restrict__ f, size_t id) { return f[id]; }

// M2P over sorted slots: UP = sum W vel, GP = (sum W def) * vol; optionally
// the forward Euler push.  Weight products and sums in float-float; the
// fields are FP64 arrays or float-float pairs (T).
template <typename T>
__global__ void k_m2p(const int* __restrict__ perm, const int* __restrict__ nsorted_dev, const float2* __restrict__ rec,
                      MeshDev m,
                      const T* __restrict__ v0, const T* __restrict__ v1, const T* __restrict__ v2,
                      const T* __restrict__ g0, const T* __restrict__ g1, const T* __restrict__ g2,
                      double* __restrict__ up, double* __restrict__ gp, int up_add, double* __restrict__ x,
                      double* __restrict__ y, double* __restrict__ z, double* __restrict__ q0, double* __restrict__ q1,
                      double* __restrict__ q2, const double* __restrict__ vol, int do_euler, double dt, double ux,
                      double uy, double uz) {
  const int nsorted = *nsorted_dev;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nsorted; s += gridDim.x * blockDim.x) {
  const int p = perm[s];
  const float2* r = rec + (size_t)s * kRecLen;
  float2 w[4];
#pragma unroll
  for (int a = 0; a < 4; ++a) w[a] = r[a];
  const int c0 = record_cell(r);
  const int cj = cell_of(y[p], m.xmin[1], m.d[1]), ck = cell_of(z[p], m.xmin[2], m.d[2]);
  const int nw = m.ips + m.ipf + 1;
  const float2 zero = make_float2(0.0f, 0.0f);
  float2 u[3] = {zero, zero, zero}, gl[3] = {zero, zero, zero};
  for (int c = 0; c < nw; ++c) {
    const int kk = ck - m.ips + c;
    for (int b = 0; b < nw; ++b) {
      const int jj = cj - m.ips + b;
      const float2 wyz = r[4 + 4 * b + c];
      const size_t row = (size_t)m.n[0] * (jj + (size_t)m.n[1] * kk) + (c0 - m.ips);
#pragma unroll 4
      for (int a = 0; a < nw; ++a) {
        const float2 f = ff::mul(w[a], wyz);
        const size_t id = row + a;
        u[0] = ff::fma(f, field_ff(v0, id), u[0]);
        u[1] = ff::fma(f, field_ff(v1, id), u[1]);
        u[2] = ff::fma(f, field_ff(v2, id), u[2]);
        gl[0] = ff::fma(f, field_ff(g0, id), gl[0]);
        gl[1] = ff::fma(f, field_ff(g1, id), gl[1]);
        gl[2] = ff::fma(f, field_ff(g2, id), gl[2]);
      }
    }
  }
  const double vp = vol[p];
  const double ud[3] = {ff::to_double(u[0]), ff::to_double(u[1]), ff::to_double(u[2])};
  const double gg0 = ff::to_double(gl[0]) * vp, gg1 = ff::to_double(gl[1]) * vp, gg2 = ff::to_double(gl[2]) * vp;
  if (up) {  // UP = UP + sum W vel (vpm_time.f90:92-94) or UP = sum W vel
    const double b0 = up_add ? up[3 * (size_t)p] : 0.0, b1 = up_add ? up[3 * (size_t)p + 1] : 0.0,
                 b2 = up_add ? up[3 * (size_t)p + 2] : 0.0;
    up[3 * (size_t)p] = b0 + ud[0];
    up[3 * (size_t)p + 1] = b1 + ud[1];
    up[3 * (size_t)p + 2] = b2 + ud[2];
    gp[3 * (size_t)p] = gg0;
    gp[3 * (size_t)p + 1] = gg1;
    gp[3 * (size_t)p + 2] = gg2;
  }
  if (do_euler) {
    x[p] = x[p] + (ud[0] + ux) * dt;
    y[p] = y[p] + (ud[1] + uy) * dt;
    z[p] = z[p] + (ud[2] + uz) * dt;
    q0[p] = q0[p] - gg0 * dt;
    q1[p] = q1[p] - gg1 * dt;
    q2[p] = q2[p] - gg2 * dt;
  }
  }
}

// Remesh: flag nodes inside [lo, hi] (0-based, per axis) with |w| >= thr.
// flag = !(sqrt_rn(s) < thr) with s = (a*a + b*b) + c*c rounded as written.
// A correctly rounded square root is monotonic, so sqrt_rn(s) < thr exactly
// when s < tstar, the least double whose root is >= thr (found on the host):
// no square root per node.  Nodes whose three values have biased exponents
// <= emax have s < tstar / 2 and are decided from the exponent bits alone.
__global__ void k_remesh_flags(const double* __restrict__ r0, const double* __restrict__ r1, const double* __restrict__ r2,
                               MeshDev m, int lo0, int lo1, int lo2, int hi0, int hi1, int hi2, double tstar, int emax,
                               int* __restrict__ flag) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= N) return;
  const int i = (int)(id % m.n[0]);
  const int j = (int)((id / m.n[0]) % m.n[1]);
  const int k = (int)(id / ((size_t)m.n[0] * m.n[1]));
  int f = 0;
  if (i >= lo0 && i <= hi0 && j >= lo1 && j <= hi1 && k >= lo2 && k <= hi2) {
    const double a = r0[id], b = r1[id], c = r2[id];
    const int ea = (__double2hiint(a) >> 20) & 0x7FF, eb = (__double2hiint(b) >> 20) & 0x7FF,
              ec = (__double2hiint(c) >> 20) & 0x7FF;
    if (max(ea, max(eb, ec)) > emax) {
      const double s2 = __dadd_rn(__dadd_rn(__dmul_rn(a, a), __dmul_rn(b, b)), __dmul_rn(c, c));
      f = (s2 < tstar) ? 0 : 1;
    }
  }
  flag[id] = f;
}

__global__ void k_remesh_emit(const double* __restrict__ r0, const double* __restrict__ r1, const double* __restrict__ r2,
                              const int* __restrict__ flag, const int* __restrict__ pos, MeshDev m, double dv,
                              int capacity, double* __restrict__ x, double* __restrict__ y, double* __restrict__ z,
                              double* __restrict__ q0, double* __restrict__ q1, double* __restrict__ q2,
                              double* __restrict__ vol) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (id >= N || !flag[id]) return;
  const int s = pos[id];
  if (s >= capacity) return;
  const int i = (int)(id % m.n[0]);
  const int j = (int)((id / m.n[0]) % m.n[1]);
  const int k = (int)(id / ((size_t)m.n[0] * m.n[1]));
  x[s] = m.xmin[0] + m.d[0] * (double)i;
  y[s] = m.xmin[1] + m.d[1] * (double)j;
  z[s] = m.xmin[2] + m.d[2] * (double)k;
  q0[s] = r0[id] * dv;
  q1[s] = r1[id] * dv;
  q2[s] = r2[id] * dv;
  vol[s] = dv;
}

__global__ void k_set_total(int* __restrict__ dst, const int* __restrict__ src) { *dst = *src; }

// New particle count of a remesh, clamped to the capacity (overflow -> error 2).
__global__ void k_set_count(int* __restrict__ np, const int* __restrict__ total, int capacity, int* __restrict__ err) {
  const int t = *total;
  if (t > capacity) {
    *np = capacity;
    atomicExch(err, 2);
  } else {
    *np = t;
  }
}

unsigned stride_grid(int capacity, int threads) {
  return (unsigned)std::max(1, std::min((capacity + threads - 1) / threads, 152 * 32));
}

}  // namespace

void Particles::ensure(int cap) {
  if (cap <= capacity) return;
  x.ensure(cap); y.ensure(cap); z.ensure(cap);
  q0.ensure(cap); q1.ensure(cap); q2.ensure(cap); vol.ensure(cap);
  up.ensure(3 * (size_t)cap); gp.ensure(3 * (size_t)cap);
  key.ensure(cap); perm.ensure(cap);
  rec.ensure((size_t)kRecLen * cap);
  d_np.ensure(1);
  capacity = cap;
}

void Binning::ensure(size_t ncell) {
  if (ncell <= ncells) return;
  starts.ensure(ncell + 1);
  cursor.ensure(ncell);
  sums.ensure(scan_block_sums_needed(ncell) + 1);
  err.ensure(1);
  VPMG_CUDA(cudaMemset(err.p, 0, sizeof(int)));
  ncells = ncell;
}

// Sort by cell + records, all on the stream (no host round trip): the
// particle count is read from P.d_np, the sorted count lands in starts[N].
// Errors (stencil outside the mesh = 1, remesh overflow = 2) accumulate in
// B.err and are reported by check_particle_errors at the next host sync.
void bin_particles(Particles& P, const MeshDev& m, Binning& B, cudaStream_t s) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  B.ensure(N);
  VPMG_CUDA(cudaMemsetAsync(B.cursor.p, 0, sizeof(int) * N, s));
  k_keys<<<stride_grid(P.capacity, 256), 256, 0, s>>>(P.x.p, P.y.p, P.z.p, P.d_np.p, m, P.key.p, B.cursor.p, B.err.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaMemsetAsync(B.sums.p, 0, sizeof(int) * B.sums.n, s));
  exclusive_scan_int(B.cursor.p, B.starts.p, N, B.sums.p, s);
  const int nt = (int)scan_block_sums_needed(N) - 1;
  k_set_total<<<1, 1, 0, s>>>(B.starts.p + N, B.sums.p + nt);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaMemsetAsync(B.cursor.p, 0, sizeof(int) * N, s));
  k_scatter<<<stride_grid(P.capacity, 256), 256, 0, s>>>(P.key.p, P.d_np.p, B.starts.p, B.cursor.p, P.perm.p);
  VPMG_LAUNCHED();
  k_cell_order<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(B.starts.p, (int)N, P.perm.p);
  VPMG_LAUNCHED();
  B.nsorted_dev = B.starts.p + N;
  if (P.arith == VPMG_ARITH_FF48)
    k_records<<<stride_grid(P.capacity, 256), 256, 0, s>>>(P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p, P.perm.p,
                                                           B.nsorted_dev, m, P.rec.p);
  else
    k_records64<<<stride_grid(P.capacity, 256), 256, 0, s>>>(P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p, P.perm.p,
                                                             P.key.p, B.nsorted_dev, m, P.rec64(), P.rec_stride());
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void check_particle_errors(Binning& B, cudaStream_t s) {
  if (!B.err.p) return;
  int e = 0;
  VPMG_CUDA(cudaMemcpyAsync(&e, B.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  if (e) VPMG_CUDA(cudaMemsetAsync(B.err.p, 0, sizeof(int), s));
  VPMG_CHECK(e != 1, VPMG_ERR_OUTSIDE, "a particle's projection stencil leaves the mesh");
  VPMG_CHECK(e != 2, VPMG_ERR_CAPACITY, "remesh produced more particles than the capacity");
}

int read_count(const int* d, cudaStream_t s) {
  int v = 0;
  VPMG_CUDA(cudaMemcpyAsync(&v, d, sizeof(int), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  return v;
}

void deposit(const Particles& P, const MeshDev& m, const Binning& B, double* const rhs[3], cudaStream_t s) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  const double dv = m.d[0] * m.d[1] * m.d[2];
  if (P.arith == VPMG_ARITH_FF48) {
    k_deposit<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(B.starts.p, P.rec.p, m, 1.0 / dv, rhs[0], rhs[1], rhs[2]);
  } else {
    const long long warps = (long long)((m.n[0] + 31) / 32) * m.n[1] * m.n[2];
    k_deposit64<<<(unsigned)((warps + kDepWarps - 1) / kDepWarps), kDepWarps * 32, 0, s>>>(
        B.starts.p, P.rec64(), P.rec_stride(), m, 1.0 / dv, rhs[0], rhs[1], rhs[2]);
  }
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

template <typename T>
static void m2p_launch(Particles& P, const MeshDev& m, const Binning& B, const T* const vel[3], const T* const def[3],
                       int up_mode, bool euler, double dt, const double uinf[3], cudaStream_t s) {
  k_m2p<T><<<stride_grid(P.capacity, 128), 128, 0, s>>>(P.perm.p, B.nsorted_dev, P.rec.p, m, vel[0], vel[1], vel[2],
                                                         def[0], def[1], def[2], up_mode ? P.up.p : nullptr, P.gp.p,
                                                         up_mode == 2 ? 1 : 0, P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p, P.vol.p,
                                                         euler ? 1 : 0, dt, uinf[0], uinf[1], uinf[2]);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void m2p(Particles& P, const MeshDev& m, const Binning& B, const double* const vel[3], const double* const def[3],
         int up_mode, bool euler, double dt, const double uinf[3], cudaStream_t s) {
  if (P.arith == VPMG_ARITH_FF48) {
    m2p_launch(P, m, B, vel, def, up_mode, euler, dt, uinf, s);
    return;
  }
  k_m2p64<<<stride_grid(P.capacity, 128), 128, 0, s>>>(P.perm.p, B.nsorted_dev, P.rec64(), P.rec_stride(), m,
                                                       vel[0], vel[1], vel[2],
                                                       def[0], def[1], def[2], up_mode ? P.up.p : nullptr, P.gp.p,
                                                       up_mode == 2 ? 1 : 0, P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p, P.vol.p,
                                                       euler ? 1 : 0, dt, uinf[0], uinf[1], uinf[2]);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void m2p(Particles& P, const MeshDev& m, const Binning& B, const float2* const vel[3], const float2* const def[3],
         int up_mode, bool euler, double dt, const double uinf[3], cudaStream_t s) {
  VPMG_CHECK(P.arith == VPMG_ARITH_FF48, VPMG_ERR_STATE, "float-float fields with FP64 particle records");
  m2p_launch(P, m, B, vel, def, up_mode, euler, dt, uinf, s);
}

// Ordered compaction of the flagged nodes; the new count goes to P.d_np
// (clamped to the capacity, overflow flagged in B.err), on the stream.
// tstar = least double t with sqrt_rn(t) >= thr (thr > 0): sqrt_rn(s) < thr
// exactly when s < tstar.  emax = largest biased exponent e such that three
// values below 2^(e - 1022) in magnitude give s < tstar / 2.
static void remesh_threshold(double thr, double* tstar, int* emax) {
  double t = thr * thr;
  while (t > 0.0 && std::sqrt(std::nextafter(t, 0.0)) >= thr) t = std::nextafter(t, 0.0);
  while (std::sqrt(t) < thr) t = std::nextafter(t, INFINITY);
  *tstar = t;
  int e = 0;
  while (e < 2046) {
    const double mx = std::ldexp(1.0, e + 1 - 1022);  // bound for exponent e + 1
    if (3.0 * mx * mx >= 0.5 * t) break;
    ++e;
  }
  *emax = e;
}

void remesh_mask(const MeshDev& m, Binning& B, const double* const rhs[3], const int lo[3], const int hi[3],
                 double thr, cudaStream_t s) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  B.ensure(N);
  VPMG_CHECK(thr > 0.0 && std::isfinite(thr), VPMG_ERR_ARG, "remesh threshold must be positive");
  double tstar = 0.0;
  int emax = 0;
  remesh_threshold(thr, &tstar, &emax);
  k_remesh_flags<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(rhs[0], rhs[1], rhs[2], m, lo[0], lo[1], lo[2], hi[0], hi[1],
                                                              hi[2], tstar, emax, B.cursor.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaMemsetAsync(B.sums.p, 0, sizeof(int) * B.sums.n, s));
  exclusive_scan_int(B.cursor.p, B.starts.p, N, B.sums.p, s);
}

namespace {
// Emission of the nodes flagged in B.cursor (slots in B.starts) and the new count.
void emit_flagged(Particles& P, const MeshDev& m, Binning& B, const double* const rhs[3], cudaStream_t s) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  const double dv = m.d[0] * m.d[1] * m.d[2];
  const int nt = (int)scan_block_sums_needed(N) - 1;
  k_remesh_emit<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(rhs[0], rhs[1], rhs[2], B.cursor.p, B.starts.p, m, dv,
                                                             P.capacity, P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p,
                                                             P.vol.p);
  VPMG_LAUNCHED();
  k_set_count<<<1, 1, 0, s>>>(P.d_np.p, B.sums.p + nt, P.capacity, B.err.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}
}  // namespace

void remesh_emit(Particles& P, const MeshDev& m, Binning& B, const double* const rhs[3], const int lo[3],
                 const int hi[3], double thr, cudaStream_t s) {
  remesh_mask(m, B, rhs, lo, hi, thr, s);
  emit_flagged(P, m, B, rhs, s);
}

void remesh_emit_masked(Particles& P, const MeshDev& m, Binning& B, const double* const rhs[3], const int* mask,
                        cudaStream_t s) {
  const size_t N = (size_t)m.n[0] * m.n[1] * m.n[2];
  B.ensure(N);
  VPMG_CUDA(cudaMemcpyAsync(B.cursor.p, mask, sizeof(int) * N, cudaMemcpyDeviceToDevice, s));
  VPMG_CUDA(cudaMemsetAsync(B.sums.p, 0, sizeof(int) * B.sums.n, s));
  exclusive_scan_int(B.cursor.p, B.starts.p, N, B.sums.p, s);
  emit_flagged(P, m, B, rhs, s);
}

}  // namespace vpmg
