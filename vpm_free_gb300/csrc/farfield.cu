// farfield.cu -- the coarsest tree level of the boundary operator by FFT.
//
// In Bounds3d_lev / tree_calc_3d (source/pmbound.f90:980-1249) every
// boundary node visits every cell of the coarsest level and accepts it
// unless r < 10 sqrt(dS); accepted cells add -dS/(4 pi r) times their
// source.  The recorded operator stores these weights as a dense block
// (two thirds of all interactions at 256^3) and applies it with 3 FMA per
// weight.  When the coarsest cells form a uniform lattice on every face
// (each face side a multiple of 2^levmax panels), cell centres and boundary
// nodes are points of one node lattice, and dS/r depends only on their
// index offsets:
//   * between parallel faces (the same face, or the opposite one at the
//     box's distance) the sum over cells is a 2-D convolution on the face
//     lattice;
//   * between perpendicular faces it is a 1-D convolution along their
//     shared axis, and a dense sum over the other two indices (the target's
//     distance to the source plane and the cell's distance to the target
//     plane) in the frequency domain.
// Both are evaluated with FP64 FFTs over every coarsest cell; the cells a
// node opened (the walk's zero slots of the dense block) are subtracted as
// correction rows, so the result is the dense block's sum to rounding.
// The kernels are even in the lattice offsets, so their spectra are real.
// Inverse transforms use IFFT(Y) = conj(FFT(conj(Y))) / P with the 1/P
// folded into the stored kernel spectra.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "arith.cuh"
#include "fft_stages.cuh"
#include "vpmg_internal.h"

namespace vpmg {

namespace {

constexpr int kFFThreads = 128;
constexpr int kFFJobs = 24;
constexpr int kFFSmem = 48 * 1024;  // dynamic shared memory of the line kernel

// in-plane axes of face f (normal f / 2): the panels' fast and slow axes
// (calc_normalderiv_3d: X faces (y, z), Y faces (x, z), Z faces (x, y))
__host__ __device__ __forceinline__ int ax_u(int f) { return (f >> 1) == 0 ? 1 : 0; }
__host__ __device__ __forceinline__ int ax_v(int f) { return (f >> 1) == 2 ? 1 : 2; }

struct AxisDev {
  int P, nst, npair;
  int radix[16];
  const double2* tw;
};

// dS / r for the node-lattice offset (ex, ey, ez) = offset * spacing, with
// every operation rounded explicitly so that all kernels (spectra and
// correction rows) evaluate the same value; 0 at r = 0 (such a cell is
// always opened, and its correction uses the same 0).
__device__ __forceinline__ double ff_kern(double dS, double ex, double ey, double ez) {
  const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez));
  return r2 > 0.0 ? __ddiv_rn(dS, __dsqrt_rn(r2)) : 0.0;
}

// signed offset of circular index e in a transform of length P
__device__ __forceinline__ int circ(int e, int P) { return e <= P / 2 ? e : e - P; }

__device__ double2* ff_fft(double2* a, double2* b, const AxisDev& p, int npair) {
  int Ns = 1;
  for (int s = 0; s < p.nst; ++s) {
    const int r = p.radix[s];
    switch (r) {
      case 2: stage<F64, 2>(a, b, p.P, Ns, p.tw, npair); break;
      case 3: stage<F64, 3>(a, b, p.P, Ns, p.tw, npair); break;
      case 4: stage<F64, 4>(a, b, p.P, Ns, p.tw, npair); break;
      default: stage<F64, 8>(a, b, p.P, Ns, p.tw, npair); break;
    }
    __syncthreads();
    Ns *= r;
    double2* t = a;
    a = b;
    b = t;
  }
  return a;
}

// One batch of line transforms.  Line l = q * nl2 + r (r < nl2) reads from
// sbase + q * sqs + r * sls and writes to dbase + q * dqs + r * dls.
// Element e of the transform: dense (sparse = 0): source index e * ses for
// e < scnt, zero beyond; lattice (sparse = 1): nonzero only at
// e = soff + b * sstep (b < scnt), from source index b * ses.  A real
// source (real = 1) reads doubles: re at the index, im at index + ioff
// (ioff < 0: im = 0).  The first nkeep outputs are written (stride des).
struct FFJob {
  long long sbase, sqs, sls, ses, dbase, dqs, dls, des, ioff;
  int nlines, nl2, nkeep, soff, sstep, scnt, sparse, real, axis;
};
struct FFJobs {
  FFJob j[kFFJobs];
  AxisDev ax[3];
  const double2* src;
  const double* srcr;
  double2* dst;
};

__global__ void __launch_bounds__(kFFThreads) k_ff_lines(const __grid_constant__ FFJobs J) {
  extern __shared__ double2 ffsm[];
  const FFJob& jb = J.j[blockIdx.y];
  const AxisDev& p = J.ax[jb.axis];
  const int P = p.P, npair = p.npair;
  const int l0 = blockIdx.x * npair;
  if (l0 >= jb.nlines) return;  // whole CTA, before any barrier
  const int nl = min(npair, jb.nlines - l0);
  double2* A = ffsm;
  double2* B = ffsm + (size_t)npair * P;
  // consecutive threads: consecutive elements of a line when the source
  // elements are contiguous, else consecutive lines
  const bool along = jb.ses == 1;
  for (int t = threadIdx.x; t < npair * P; t += blockDim.x) {
    const int li = along ? t / P : t % npair, e = along ? t % P : t / npair;
    double2 v = make_double2(0.0, 0.0);
    if (li < nl) {
      int b = -1;
      if (jb.sparse) {
        const int d = e - jb.soff;
        if (d >= 0 && d % jb.sstep == 0 && d / jb.sstep < jb.scnt) b = d / jb.sstep;
      } else if (e < jb.scnt) {
        b = e;
      }
      if (b >= 0) {
        const int l = l0 + li;
        const long long idx = jb.sbase + (long long)(l / jb.nl2) * jb.sqs + (long long)(l % jb.nl2) * jb.sls +
                              (long long)b * jb.ses;
        if (jb.real) v = make_double2(J.srcr[idx], jb.ioff >= 0 ? J.srcr[idx + jb.ioff] : 0.0);
        else v = J.src[idx];
      }
    }
    A[li * P + e] = v;
  }
  __syncthreads();
  const double2* R = ff_fft(A, B, p, npair);
  const bool along_d = jb.des == 1;
  for (int t = threadIdx.x; t < npair * P; t += blockDim.x) {
    const int li = along_d ? t / P : t % npair, e = along_d ? t % P : t / npair;
    if (li < nl && e < jb.nkeep) {
      const int l = l0 + li;
      J.dst[jb.dbase + (long long)(l / jb.nl2) * jb.dqs + (long long)(l % jb.nl2) * jb.dls + (long long)e * jb.des] =
          R[li * P + e];
    }
  }
}

// X[f][phi] = conj(S2[f][phi] Kpar[n][0] + S2[f^1][phi] Kpar[n][1]) over the
// Pv x Pu spectrum of each target face and field.
struct ParDev {
  long long s2[6][2], kp[3][2];
  int Pu[6], Pv[6];
};
__global__ void k_ff_mul_par(const __grid_constant__ ParDev D, const double2* __restrict__ S2,
                             const double* __restrict__ kpar, double2* __restrict__ X) {
  const int f = blockIdx.y / 2, phi = blockIdx.y % 2, n = f >> 1;
  const long long cnt = (long long)D.Pu[f] * D.Pv[f];
  const double2* a = S2 + D.s2[f][phi];
  const double2* b = S2 + D.s2[f ^ 1][phi];
  const double* k0 = kpar + D.kp[n][0];
  const double* k1 = kpar + D.kp[n][1];
  double2* x = X + D.s2[f][phi];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
    const double2 u = a[i], v = b[i];
    const double p0 = k0[i], p1 = k1[i];
    x[i] = make_double2(fma(u.x, p0, v.x * p1), -fma(u.y, p0, v.y * p1));
  }
}

// Perpendicular source faces: for target face F and group g (source
// normal = F's u axis for g = 0, its v axis for g = 1; the shared axis w is
// F's other axis), rows i along the source normal, frequencies w of the
// shared axis, cells c along F's normal:
//   A_comp[i][w] = sum_{G of the group} sum_c Kperp[F,G][i][c][w] Sw[G][comp][c][w]
// written as packed, conjugated full spectra for the inverse transforms:
//   Z01[i] = conj(A_0 + i A_1),  Z2[i / 2] = conj(A_2[2k] + i A_2[2k+1]),
// each with its Hermitian mirror at P - w.
struct PerpDev {
  long long kp[12][2];   // Kperp offsets of the two source faces
  long long sw[12][2];   // Sw offsets (comp 0) of the two source faces
  long long z[12];       // Z offset of the group's lines (Z01 rows, then Z2 rows)
  int Nn[12], Mc[12], P[12];
};
__global__ void __launch_bounds__(128) k_ff_perp_mv(const __grid_constant__ PerpDev D, const double* __restrict__ kperp,
                                                    const double2* __restrict__ Sw, double2* __restrict__ Z) {
  const int gi = blockIdx.y;
  const int Nn = D.Nn[gi], Mc = D.Mc[gi], P = D.P[gi], H = P / 2 + 1;
  const int npr = (Nn + 1) / 2;
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)npr * H) return;
  const int w = (int)(t % H), ip = (int)(t / H);
  const int i0 = 2 * ip, i1 = min(2 * ip + 1, Nn - 1);
  const bool two = 2 * ip + 1 < Nn;
  double a[2][3][2] = {};  // [row][comp][re, im]
  for (int gs = 0; gs < 2; ++gs) {
    const double* k0 = kperp + D.kp[gi][gs] + (long long)i0 * Mc * H + w;
    const double* k1 = kperp + D.kp[gi][gs] + (long long)i1 * Mc * H + w;
    const double2* s = Sw + D.sw[gi][gs] + w;
    const long long cs = (long long)Mc * P;  // comp stride of Sw
    for (int c = 0; c < Mc; ++c) {
      const double q0 = __ldg(&k0[(long long)c * H]), q1 = __ldg(&k1[(long long)c * H]);
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        const double2 v = __ldg(&s[m * cs + (long long)c * P]);
        a[0][m][0] = fma(q0, v.x, a[0][m][0]);
        a[0][m][1] = fma(q0, v.y, a[0][m][1]);
        a[1][m][0] = fma(q1, v.x, a[1][m][0]);
        a[1][m][1] = fma(q1, v.y, a[1][m][1]);
      }
    }
  }
  double2* z01 = Z + D.z[gi];
  double2* z2 = z01 + (long long)Nn * P;
  const bool mirror = w > 0 && 2 * w < P;
  for (int r = 0; r < (two ? 2 : 1); ++r) {
    const int i = r ? i1 : i0;
    const double* A0 = a[r][0];
    const double* A1 = a[r][1];
    // conj(A0 + i A1) and, at P - w, conj(conj(A0) + i conj(A1))
    z01[(long long)i * P + w] = make_double2(A0[0] - A1[1], -(A0[1] + A1[0]));
    if (mirror) z01[(long long)i * P + (P - w)] = make_double2(A0[0] + A1[1], A0[1] - A1[0]);
  }
  {
    const double* C0 = a[0][2];
    double C1r = 0.0, C1i = 0.0;
    if (two) { C1r = a[1][2][0]; C1i = a[1][2][1]; }
    z2[(long long)ip * P + w] = make_double2(C0[0] - C1i, -(C0[1] + C1r));
    if (mirror) z2[(long long)ip * P + (P - w)] = make_double2(C0[0] + C1i, C0[1] - C1r);
  }
}

// Boundary node t: dsum[comp][t] = the parallel part (X of the node's face)
// plus both perpendicular groups (Z), read at the node's lattice position.
struct GatherDev {
  long long x[6][2];     // X offsets per face and field
  long long z[6][2];     // Z offsets per face and group
  int Pu[6], P01[6][2], Nn[6][2];
  int N[3];
};
__global__ void k_ff_gather(const __grid_constant__ GatherDev D, const int* __restrict__ tgt_node, int ntarget,
                            const double2* __restrict__ X, const double2* __restrict__ Z, double* __restrict__ dsum) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntarget) return;
  const int node = tgt_node[t];
  const int idx[3] = {node % D.N[0], (node / D.N[0]) % D.N[1], node / (D.N[0] * D.N[1])};
  int f;
  if (idx[0] == 0) f = 0;
  else if (idx[0] == D.N[0] - 1) f = 1;
  else if (idx[1] == 0) f = 2;
  else if (idx[1] == D.N[1] - 1) f = 3;
  else if (idx[2] == 0) f = 4;
  else f = 5;
  const int u = idx[ax_u(f)], v = idx[ax_v(f)];
  const double2 p01 = X[D.x[f][0] + (long long)v * D.Pu[f] + u];
  const double2 p2 = X[D.x[f][1] + (long long)v * D.Pu[f] + u];
  double c0 = p01.x, c1 = -p01.y, c2 = p2.x;
  // g = 0: rows along u, elements along v; g = 1: rows along v, elements along u
  for (int g = 0; g < 2; ++g) {
    const int i = g ? v : u, j = g ? u : v;
    const int P = D.P01[f][g], Nn = D.Nn[f][g];
    const double2* z01 = Z + D.z[f][g];
    const double2* z2 = z01 + (long long)Nn * P;
    const double2 q = z01[(long long)i * P + j];
    const double2 r = z2[(long long)(i >> 1) * P + j];
    c0 += q.x;
    c1 -= q.y;
    c2 += (i & 1) ? -r.y : r.x;
  }
  dsum[t] = c0;
  dsum[ntarget + t] = c1;
  dsum[2 * (size_t)ntarget + t] = c2;
}

// ---- set-up kernels -------------------------------------------------------

// The parallel-pair kernel on the circular Pv x Pu lattice of faces with
// normal n: dS / r at in-plane offsets (du, dv) and plane distance dn.
__global__ void k_ff_kpar_build(int Pu, int Pv, int axu, int axv, int axn, int dn, double dS, double hx, double hy,
                                double hz, double2* __restrict__ out) {
  const long long cnt = (long long)Pu * Pv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
    const int u = (int)(i % Pu), v = (int)(i / Pu);
    int o[3];
    o[axu] = circ(u, Pu);
    o[axv] = circ(v, Pv);
    o[axn] = dn;
    out[i] = make_double2(ff_kern(dS, __dmul_rn((double)o[0], hx), __dmul_rn((double)o[1], hy),
                                  __dmul_rn((double)o[2], hz)),
                          0.0);
  }
}

// The perpendicular-pair kernel lines [i][c][P]: target row i along the
// source normal ng (offset i - iG from the source plane), cell c along the
// target normal nf (offset iF - centre), circular offset along w.
__global__ void k_ff_kperp_build(int Nn, int Mc, int P, int ng, int nf, int w, int iG, int iF, int istep, double dS,
                                 double hx, double hy, double hz, double2* __restrict__ out) {
  const long long cnt = (long long)Nn * Mc * P;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
    const int e = (int)(i % P);
    const long long lc = i / P;
    const int c = (int)(lc % Mc), r = (int)(lc / Mc);
    int o[3];
    o[ng] = r - iG;
    o[nf] = iF - (c * istep + istep / 2);
    o[w] = circ(e, P);
    out[i] = make_double2(ff_kern(dS, __dmul_rn((double)o[0], hx), __dmul_rn((double)o[1], hy),
                                  __dmul_rn((double)o[2], hz)),
                          0.0);
  }
}

// dst[l][e] = re(src[l][e]) * scale for e < keep (lines of length P).
__global__ void k_ff_real(const double2* __restrict__ src, long long nlines, int P, int keep, double scale,
                          double* __restrict__ dst) {
  const long long cnt = nlines * keep;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cnt; i += (long long)gridDim.x * blockDim.x) {
    const long long l = i / keep;
    const int e = (int)(i % keep);
    dst[i] = src[l * P + e].x * scale;
  }
}

// Correction rows: per boundary node, the coarsest cells whose dense-block
// slot is zero (the walk opened them), weight -dS/r by the lattice formula.
struct CorrDev {
  int cell0[7], ma[6];
  double dS[6], h[3];
  int N[3], istep, ntop, top0;
};
__device__ __forceinline__ void cell_centre(const CorrDev& D, int c, int& f, int o[3]) {
  f = 0;
  while (f < 5 && c >= D.cell0[f + 1]) ++f;
  const int k = c - D.cell0[f];
  const int a = k % D.ma[f], b = k / D.ma[f];
  const int n = f >> 1;
  o[n] = (f & 1) ? D.N[n] - 1 : 0;
  o[ax_u(f)] = a * D.istep + D.istep / 2;
  o[ax_v(f)] = b * D.istep + D.istep / 2;
}
template <bool FILL>
__global__ void k_ff_corr(const __grid_constant__ CorrDev D, const double* __restrict__ wtop,
                          const int* __restrict__ tgt_node, int ntarget, int* __restrict__ counts,
                          const long long* __restrict__ rowptr, int* __restrict__ col, double* __restrict__ wgt) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntarget) return;
  const long long ntop2 = (D.ntop + 1) / 2;
  const double* row = wtop + (size_t)(t >> 5) * ntop2 * 64 + (t & 31) * 2;
  int cnt = 0;
  long long out = FILL ? rowptr[t] : 0;
  const int node = tgt_node[t];
  const int ti[3] = {node % D.N[0], (node / D.N[0]) % D.N[1], node / (D.N[0] * D.N[1])};
  for (int c = 0; c < D.ntop; ++c) {
    if (row[(size_t)(c >> 1) * 64 + (c & 1)] != 0.0) continue;
    if (FILL) {
      int f, o[3];
      cell_centre(D, c, f, o);
      col[out] = D.top0 + c;
      wgt[out] = -ff_kern(D.dS[f], __dmul_rn((double)(ti[0] - o[0]), D.h[0]), __dmul_rn((double)(ti[1] - o[1]), D.h[1]),
                          __dmul_rn((double)(ti[2] - o[2]), D.h[2]));
      ++out;
    } else {
      ++cnt;
    }
  }
  if (!FILL) counts[t] = cnt;
}

// ---- host helpers ---------------------------------------------------------

int smooth_length(int need) {  // least P >= need of the form 2^a 3^b, a >= 1
  int best = 0;
  for (long long p3 = 1; p3 <= 2LL * need + 6; p3 *= 3)
    for (long long p = p3 * 2; p <= 2LL * need + 6; p *= 2)
      if (p >= need && (best == 0 || p < best)) best = (int)p;
  return best;
}

void make_axis(FarFieldAxis& A, int P) {
  A.P = P;
  int m = P, n2 = 0, n3 = 0;
  while (m % 2 == 0) { m /= 2; ++n2; }
  while (m % 3 == 0) { m /= 3; ++n3; }
  VPMG_CHECK(m == 1, VPMG_ERR_UNSUPPORTED, "far-field length not of the form 2^a 3^b");
  A.nst = 0;
  while (n2 >= 3) { A.radix[A.nst++] = 8; n2 -= 3; }
  if (n2 == 2) A.radix[A.nst++] = 4;
  if (n2 == 1) A.radix[A.nst++] = 2;
  while (n3-- > 0) A.radix[A.nst++] = 3;
  VPMG_CHECK(A.nst <= 16, VPMG_ERR_UNSUPPORTED, "too many far-field FFT stages");
  A.npair = std::max(1, std::min(8, kFFSmem / (int)(2 * sizeof(double2) * P)));
  std::vector<double2> h(P);
  for (int t = 0; t < P; ++t) {
    const double a = -2.0 * kPI * (double)t / (double)P;
    h[t] = make_double2(std::cos(a), std::sin(a));
  }
  A.tw.ensure(P);
  VPMG_CUDA(cudaMemcpy(A.tw.p, h.data(), sizeof(double2) * P, cudaMemcpyHostToDevice));
}

AxisDev axis_dev(const FarFieldAxis& A) {
  AxisDev d;
  d.P = A.P;
  d.nst = A.nst;
  d.npair = A.npair;
  for (int i = 0; i < 16; ++i) d.radix[i] = A.radix[i];
  d.tw = A.tw.p;
  return d;
}

// Runs a list of line-transform jobs, at most kFFJobs per launch.
void run_jobs(const FarField& F, const std::vector<FFJob>& jobs, const double2* src, const double* srcr, double2* dst,
              cudaStream_t s) {
  for (size_t j0 = 0; j0 < jobs.size(); j0 += kFFJobs) {
    FFJobs J;
    const int nj = (int)std::min<size_t>(kFFJobs, jobs.size() - j0);
    int gx = 1;
    for (int k = 0; k < nj; ++k) {
      J.j[k] = jobs[j0 + k];
      const int np = F.ax[J.j[k].axis].npair;
      gx = std::max(gx, (J.j[k].nlines + np - 1) / np);
    }
    for (int a = 0; a < 3; ++a) J.ax[a] = axis_dev(F.ax[a]);
    J.src = src;
    J.srcr = srcr;
    J.dst = dst;
    k_ff_lines<<<dim3((unsigned)gx, (unsigned)nj), kFFThreads, kFFSmem, s>>>(J);
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}

FFJob dense_job(int axis, long long sbase, long long sls, long long ses, int scnt, long long dbase, long long dls,
                long long des, int nkeep, int nlines) {
  FFJob j{};
  j.axis = axis;
  j.sbase = sbase; j.sqs = 0; j.sls = sls; j.ses = ses;
  j.dbase = dbase; j.dqs = 0; j.dls = dls; j.des = des;
  j.nlines = nlines; j.nl2 = std::max(nlines, 1); j.nkeep = nkeep;
  j.sparse = 0; j.scnt = scnt; j.soff = 0; j.sstep = 1;
  j.real = 0; j.ioff = -1;
  return j;
}

unsigned grid_for(long long n) { return (unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152 * 32)); }

}  // namespace

long long FarField::bytes() const {
  return (long long)(kpar.bytes() + kperp.bytes() + T.bytes() + S2.bytes() + X.bytes() + Sw.bytes() + Z.bytes() +
                     crow.bytes() + ccol.bytes() + cw.bytes());
}

void farfield_release(BoundaryOp& B) {
  FarField& F = B.ff;
  F.on = false;
  F.kpar.release(); F.kperp.release(); F.T.release(); F.S2.release(); F.X.release(); F.Sw.release(); F.Z.release();
  F.crow.release(); F.ccol.release(); F.cw.release();
  F.ncorr = 0;
}

void farfield_prepare(BoundaryOp& B, const Grid& g, cudaStream_t s) {
  farfield_release(B);
  FarField& F = B.ff;
  const char* env = std::getenv("VPMG_FARFIELD");
  if (env && env[0] == '0') return;
  if (B.arith != VPMG_ARITH_FP64 || B.ibctyp != 2 || !B.tree || B.levmax < 1 || !B.precomputed || !B.dense) return;
  const int istep = 1 << B.levmax;
  for (int a = 0; a < 3; ++a)
    if ((g.n[a] - 1) % istep != 0 || g.n[a] - 1 <= istep) return;  // dummy cells at the coarsest level
  // faces' coarsest lattices, in the tree's face order
  int ma[6], mb[6], cell0[7];
  cell0[0] = 0;
  for (int f = 0; f < 6; ++f) {
    ma[f] = (g.n[ax_u(f)] - 1) / istep;
    mb[f] = (g.n[ax_v(f)] - 1) / istep;
    cell0[f + 1] = cell0[f] + ma[f] * mb[f];
  }
  if (cell0[6] != B.ntopd) return;
  // every coarsest centre on its lattice node and one area per face
  const int top0 = B.lev_off[B.levmax];
  std::vector<double> cx(B.ntopd), cy(B.ntopd), cz(B.ntopd), cds(B.ntopd);
  std::vector<int> fl(B.ntopd);
  VPMG_CUDA(cudaMemcpy(cx.data(), B.cx.p + top0, sizeof(double) * B.ntopd, cudaMemcpyDeviceToHost));
  VPMG_CUDA(cudaMemcpy(cy.data(), B.cy.p + top0, sizeof(double) * B.ntopd, cudaMemcpyDeviceToHost));
  VPMG_CUDA(cudaMemcpy(cz.data(), B.cz.p + top0, sizeof(double) * B.ntopd, cudaMemcpyDeviceToHost));
  VPMG_CUDA(cudaMemcpy(cds.data(), B.cds.p + top0, sizeof(double) * B.ntopd, cudaMemcpyDeviceToHost));
  VPMG_CUDA(cudaMemcpy(fl.data(), B.flags.p + top0, sizeof(int) * B.ntopd, cudaMemcpyDeviceToHost));
  for (int f = 0; f < 6; ++f) {
    const double ds0 = cds[cell0[f]];
    for (int k = 0; k < ma[f] * mb[f]; ++k) {
      const int c = cell0[f] + k;
      if (fl[c] < 0 || std::fabs(cds[c] - ds0) > 1e-13 * ds0) return;
      int o[3];
      const int n = f >> 1;
      o[n] = (f & 1) ? g.n[n] - 1 : 0;
      o[ax_u(f)] = (k % ma[f]) * istep + istep / 2;
      o[ax_v(f)] = (k / ma[f]) * istep + istep / 2;
      const double pc[3] = {cx[c], cy[c], cz[c]};
      for (int a = 0; a < 3; ++a) {
        const double want = g.xmin[a] + (double)o[a] * g.d[a];
        if (std::fabs(pc[a] - want) > 1e-9 * g.d[a]) return;
      }
    }
    F.dS[f] = ds0;
  }
  for (int a = 0; a < 3; ++a) {
    F.N[a] = g.n[a];
    F.h[a] = g.d[a];
    const int P = smooth_length(2 * g.n[a] - 1 - istep);
    if (P > 3 * 512 || P < 8) return;
    make_axis(F.ax[a], P);
  }
  F.istep = istep;
  for (int f = 0; f < 6; ++f) F.cell0[f] = cell0[f];
  // ---- buffers ------------------------------------------------------------
  long long tsz = 0, s2sz = 0, swsz = 0, zsz = 0;
  for (int f = 0; f < 6; ++f) {
    const int Pu = F.ax[ax_u(f)].P, Pv = F.ax[ax_v(f)].P;
    for (int phi = 0; phi < 2; ++phi) {
      F.t_off[f][phi] = tsz;
      tsz += (long long)mb[f] * Pu;
      F.s2_off[f][phi] = s2sz;
      s2sz += (long long)Pu * Pv;
    }
    // Sw[f][wsel]: 3 comps x (cells across w) lines of P_w; wsel 0: w = u
    F.sw_off[f][0] = swsz;
    swsz += 3LL * mb[f] * Pu;
    F.sw_off[f][1] = swsz;
    swsz += 3LL * ma[f] * Pv;
    // Z[f][g]: group g's source normal ng = (g ? v : u) axis of f, w the other
    for (int gg = 0; gg < 2; ++gg) {
      const int ng = gg ? ax_v(f) : ax_u(f), w = gg ? ax_u(f) : ax_v(f);
      const int Nn = g.n[ng], Pw = F.ax[w].P;
      F.z_off[f][gg] = zsz;
      zsz += (long long)(Nn + (Nn + 1) / 2) * Pw;
    }
  }
  F.T.ensure(tsz);
  F.S2.ensure(s2sz);
  F.X.ensure(s2sz);
  F.Sw.ensure(swsz);
  F.Z.ensure(zsz);
  // ---- parallel-pair kernel spectra ---------------------------------------
  long long kpsz = 0;
  for (int n = 0; n < 3; ++n) {
    const int f = 2 * n, Pu = F.ax[ax_u(f)].P, Pv = F.ax[ax_v(f)].P;
    F.kpar_off[n][0] = kpsz;
    kpsz += (long long)Pu * Pv;
    F.kpar_off[n][1] = kpsz;
    kpsz += (long long)Pu * Pv;
  }
  F.kpar.ensure(kpsz);
  for (int n = 0; n < 3; ++n) {
    const int f = 2 * n, au = ax_u(f), av = ax_v(f);
    const int Pu = F.ax[au].P, Pv = F.ax[av].P;
    DBuf<double2> tmp;
    tmp.ensure((size_t)Pu * Pv);
    for (int side = 0; side < 2; ++side) {
      k_ff_kpar_build<<<grid_for((long long)Pu * Pv), 256, 0, s>>>(Pu, Pv, au, av, n, side ? g.n[n] - 1 : 0, F.dS[f],
                                                                    g.d[0], g.d[1], g.d[2], tmp.p);
      VPMG_LAUNCHED();
      std::vector<FFJob> jobs;
      jobs.push_back(dense_job(au, 0, Pu, 1, Pu, 0, Pu, 1, Pu, Pv));  // rows
      run_jobs(F, jobs, tmp.p, nullptr, tmp.p, s);
      jobs.clear();
      jobs.push_back(dense_job(av, 0, 1, Pu, Pv, 0, 1, Pu, Pv, Pu));  // columns
      run_jobs(F, jobs, tmp.p, nullptr, tmp.p, s);
      k_ff_real<<<grid_for((long long)Pu * Pv), 256, 0, s>>>(tmp.p, Pv, Pu, Pu, 1.0 / ((double)Pu * Pv),
                                                              F.kpar.p + F.kpar_off[n][side]);
      VPMG_LAUNCHED();
    }
    VPMG_CUDA(cudaStreamSynchronize(s));
  }
  // ---- perpendicular-pair kernel spectra ----------------------------------
  long long kqsz = 0;
  for (int f = 0; f < 6; ++f)
    for (int gg = 0; gg < 2; ++gg)
      for (int side = 0; side < 2; ++side) {
        const int ng = gg ? ax_v(f) : ax_u(f), w = gg ? ax_u(f) : ax_v(f), nf = f >> 1;
        const int Mc = (g.n[nf] - 1) / istep, Pw = F.ax[w].P;
        F.kperp_off[f * 4 + gg * 2 + side] = kqsz;
        kqsz += (long long)g.n[ng] * Mc * (Pw / 2 + 1);
      }
  F.kperp.ensure(kqsz);
  for (int f = 0; f < 6; ++f)
    for (int gg = 0; gg < 2; ++gg) {
      const int ng = gg ? ax_v(f) : ax_u(f), w = gg ? ax_u(f) : ax_v(f), nf = f >> 1;
      const int Nn = g.n[ng], Mc = (g.n[nf] - 1) / istep, Pw = F.ax[w].P;
      DBuf<double2> tmp;
      tmp.ensure((size_t)Nn * Mc * Pw);
      for (int side = 0; side < 2; ++side) {
        const int G = 2 * ng + side;
        k_ff_kperp_build<<<grid_for((long long)Nn * Mc * Pw), 256, 0, s>>>(
            Nn, Mc, Pw, ng, nf, w, side ? g.n[ng] - 1 : 0, (f & 1) ? g.n[nf] - 1 : 0, istep, F.dS[G], g.d[0], g.d[1],
            g.d[2], tmp.p);
        VPMG_LAUNCHED();
        std::vector<FFJob> jobs;
        jobs.push_back(dense_job(w, 0, Pw, 1, Pw, 0, Pw, 1, Pw, Nn * Mc));
        run_jobs(F, jobs, tmp.p, nullptr, tmp.p, s);
        k_ff_real<<<grid_for((long long)Nn * Mc * (Pw / 2 + 1)), 256, 0, s>>>(
            tmp.p, (long long)Nn * Mc, Pw, Pw / 2 + 1, 1.0 / (double)Pw, F.kperp.p + F.kperp_off[f * 4 + gg * 2 + side]);
        VPMG_LAUNCHED();
      }
      VPMG_CUDA(cudaStreamSynchronize(s));
    }
  // ---- correction rows: the opened coarsest cells --------------------------
  CorrDev D{};
  for (int f = 0; f < 7; ++f) D.cell0[f] = cell0[f];
  for (int f = 0; f < 6; ++f) { D.ma[f] = ma[f]; D.dS[f] = F.dS[f]; }
  for (int a = 0; a < 3; ++a) { D.h[a] = g.d[a]; D.N[a] = g.n[a]; }
  D.istep = istep;
  D.ntop = B.ntopd;
  D.top0 = top0;
  DBuf<int> counts;
  counts.ensure(B.ntarget);
  const double* wt = reinterpret_cast<const double*>(B.wtop.p);
  k_ff_corr<false><<<(B.ntarget + 127) / 128, 128, 0, s>>>(D, wt, B.tgt_node.p, B.ntarget, counts.p, nullptr, nullptr,
                                                           nullptr);
  VPMG_LAUNCHED();
  std::vector<int> hc(B.ntarget);
  VPMG_CUDA(cudaMemcpyAsync(hc.data(), counts.p, sizeof(int) * B.ntarget, cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  std::vector<long long> rp(B.ntarget + 1, 0);
  for (int t = 0; t < B.ntarget; ++t) rp[t + 1] = rp[t] + hc[t];
  F.ncorr = rp[B.ntarget];
  F.crow.ensure(B.ntarget + 1);
  VPMG_CUDA(cudaMemcpy(F.crow.p, rp.data(), sizeof(long long) * (B.ntarget + 1), cudaMemcpyHostToDevice));
  F.ccol.ensure((size_t)std::max<long long>(F.ncorr, 1));
  F.cw.ensure((size_t)std::max<long long>(F.ncorr, 1));
  k_ff_corr<true><<<(B.ntarget + 127) / 128, 128, 0, s>>>(D, wt, B.tgt_node.p, B.ntarget, nullptr, F.crow.p, F.ccol.p,
                                                          F.cw.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
  VPMG_CUDA(cudaStreamSynchronize(s));
  // FP64 flops of one apply: 5 P log2 P per line transform, 4 FMA per
  // spectrum product, 2 FMA per kernel value, component and part
  auto fft = [&](int a) { return 5.0 * F.ax[a].P * std::log2((double)F.ax[a].P); };
  double flop = 0.0;
  for (int f = 0; f < 6; ++f) {
    const int au = ax_u(f), av = ax_v(f);
    flop += 2.0 * (mb[f] * fft(au) + F.ax[au].P * fft(av));                 // source rows and columns
    flop += 2.0 * 8.0 * F.ax[au].P * F.ax[av].P;                            // products
    flop += 2.0 * (F.ax[au].P * fft(av) + g.n[av] * fft(au));              // inverse columns and rows
    flop += 3.0 * (mb[f] * fft(au) + ma[f] * fft(av));                      // perpendicular sources
    for (int gg = 0; gg < 2; ++gg) {
      const int ng = gg ? av : au, w = gg ? au : av, nf = f >> 1;
      const double Nn = g.n[ng], Mc = (g.n[nf] - 1) / istep, H = F.ax[w].P / 2 + 1;
      flop += 2.0 * Nn * Mc * H * 12.0;                                     // two source faces, 3 comps x re/im FMA
      flop += (Nn + (g.n[ng] + 1) / 2) * fft(w);                            // inverse lines
    }
  }
  F.flops = flop;
  F.on = true;
}

void farfield_apply(BoundaryOp& B, double* dsum, cudaStream_t s) {
  FarField& F = B.ff;
  const int istep = F.istep, h2 = istep / 2;
  const int NC = B.ncell_total, top0 = B.lev_off[B.levmax];
  int ma[6], mb[6];
  for (int f = 0; f < 6; ++f) {
    ma[f] = (F.N[ax_u(f)] - 1) / istep;
    mb[f] = (F.N[ax_v(f)] - 1) / istep;
  }
  // 1. rows of the 2-D source transforms: line b of face f holds the
  //    face's cell row b at u = a * istep + istep / 2 (phi 0: s0 + i s1, phi 1: s2)
  std::vector<FFJob> jobs;
  for (int f = 0; f < 6; ++f)
    for (int phi = 0; phi < 2; ++phi) {
      const int au = ax_u(f), Pu = F.ax[au].P;
      FFJob j{};
      j.axis = au;
      j.sbase = (long long)(phi ? 2 : 0) * NC + top0 + F.cell0[f];
      j.sqs = 0; j.sls = ma[f]; j.ses = 1;
      j.real = 1; j.ioff = phi ? -1 : NC;
      j.sparse = 1; j.soff = h2; j.sstep = istep; j.scnt = ma[f];
      j.dbase = F.t_off[f][phi]; j.dqs = 0; j.dls = Pu; j.des = 1;
      j.nlines = mb[f]; j.nl2 = mb[f]; j.nkeep = Pu;
      jobs.push_back(j);
    }
  run_jobs(F, jobs, nullptr, B.csrc.p, F.T.p, s);
  // 2. columns: column w_u of face f has the rows' values at v = b * istep + istep / 2
  jobs.clear();
  for (int f = 0; f < 6; ++f)
    for (int phi = 0; phi < 2; ++phi) {
      const int au = ax_u(f), av = ax_v(f), Pu = F.ax[au].P, Pv = F.ax[av].P;
      FFJob j{};
      j.axis = av;
      j.sbase = F.t_off[f][phi]; j.sqs = 0; j.sls = 1; j.ses = Pu;
      j.real = 0; j.ioff = -1;
      j.sparse = 1; j.soff = h2; j.sstep = istep; j.scnt = mb[f];
      j.dbase = F.s2_off[f][phi]; j.dqs = 0; j.dls = 1; j.des = Pu;
      j.nlines = Pu; j.nl2 = Pu; j.nkeep = Pv;
      jobs.push_back(j);
    }
  run_jobs(F, jobs, F.T.p, nullptr, F.S2.p, s);
  // 3. products with the same-face and opposite-face kernels (conjugated)
  ParDev PD{};
  for (int f = 0; f < 6; ++f) {
    PD.Pu[f] = F.ax[ax_u(f)].P;
    PD.Pv[f] = F.ax[ax_v(f)].P;
    PD.s2[f][0] = F.s2_off[f][0];
    PD.s2[f][1] = F.s2_off[f][1];
  }
  for (int n = 0; n < 3; ++n) { PD.kp[n][0] = F.kpar_off[n][0]; PD.kp[n][1] = F.kpar_off[n][1]; }
  k_ff_mul_par<<<dim3(152 * 2, 12), 256, 0, s>>>(PD, F.S2.p, F.kpar.p, F.X.p);
  VPMG_LAUNCHED();
  // 4. inverse columns (rows v < N_v kept), 5. inverse rows v < N_v (u < N_u kept)
  jobs.clear();
  for (int f = 0; f < 6; ++f)
    for (int phi = 0; phi < 2; ++phi) {
      const int au = ax_u(f), av = ax_v(f), Pu = F.ax[au].P, Pv = F.ax[av].P;
      jobs.push_back(dense_job(av, F.s2_off[f][phi], 1, Pu, Pv, F.s2_off[f][phi], 1, Pu, F.N[av], Pu));
    }
  run_jobs(F, jobs, F.X.p, nullptr, F.X.p, s);
  jobs.clear();
  for (int f = 0; f < 6; ++f)
    for (int phi = 0; phi < 2; ++phi) {
      const int au = ax_u(f), av = ax_v(f), Pu = F.ax[au].P;
      jobs.push_back(dense_job(au, F.s2_off[f][phi], Pu, 1, Pu, F.s2_off[f][phi], Pu, 1, F.N[au], F.N[av]));
    }
  run_jobs(F, jobs, F.X.p, nullptr, F.X.p, s);
  // 6. perpendicular sources: face G's cells along its axis w at
  //    b * istep + istep / 2, one line per (comp, cell across w)
  jobs.clear();
  for (int G = 0; G < 6; ++G)
    for (int ws = 0; ws < 2; ++ws) {
      const int w = ws ? ax_v(G) : ax_u(G), Pw = F.ax[w].P;
      const int nacross = ws ? ma[G] : mb[G], nalong = ws ? mb[G] : ma[G];
      FFJob j{};
      j.axis = w;
      j.sbase = top0 + F.cell0[G]; j.sqs = NC;
      j.sls = ws ? 1 : ma[G];   // next cell across w
      j.ses = ws ? ma[G] : 1;   // next cell along w
      j.real = 1; j.ioff = -1;
      j.sparse = 1; j.soff = h2; j.sstep = istep; j.scnt = nalong;
      j.dbase = F.sw_off[G][ws]; j.dqs = (long long)nacross * Pw; j.dls = Pw; j.des = 1;
      j.nlines = 3 * nacross; j.nl2 = nacross; j.nkeep = Pw / 2 + 1;
      jobs.push_back(j);
    }
  run_jobs(F, jobs, nullptr, B.csrc.p, F.Sw.p, s);
  // 7. the dense sums per frequency, packed for the inverse transforms
  PerpDev QD{};
  long long maxthreads = 0;
  for (int f = 0; f < 6; ++f)
    for (int gg = 0; gg < 2; ++gg) {
      const int gi = f * 2 + gg;
      const int ng = gg ? ax_v(f) : ax_u(f), w = gg ? ax_u(f) : ax_v(f), nf = f >> 1;
      QD.Nn[gi] = F.N[ng];
      QD.Mc[gi] = (F.N[nf] - 1) / istep;
      QD.P[gi] = F.ax[w].P;
      QD.z[gi] = F.z_off[f][gg];
      for (int side = 0; side < 2; ++side) {
        const int G = 2 * ng + side;
        const int ws = (w == ax_u(G)) ? 0 : 1;  // w is G's u or v axis; the other is f's normal
        QD.kp[gi][side] = F.kperp_off[f * 4 + gg * 2 + side];
        QD.sw[gi][side] = F.sw_off[G][ws];
      }
      maxthreads = std::max(maxthreads, (long long)((F.N[ng] + 1) / 2) * (F.ax[w].P / 2 + 1));
    }
  k_ff_perp_mv<<<dim3((unsigned)((maxthreads + 127) / 128), 12), 128, 0, s>>>(QD, F.kperp.p, F.Sw.p, F.Z.p);
  VPMG_LAUNCHED();
  // 8. inverse transforms of the packed lines (N_w outputs kept)
  jobs.clear();
  for (int f = 0; f < 6; ++f)
    for (int gg = 0; gg < 2; ++gg) {
      const int ng = gg ? ax_v(f) : ax_u(f), w = gg ? ax_u(f) : ax_v(f);
      const int Nn = F.N[ng], Pw = F.ax[w].P, nl = Nn + (Nn + 1) / 2;
      jobs.push_back(dense_job(w, F.z_off[f][gg], Pw, 1, Pw, F.z_off[f][gg], Pw, 1, F.N[w], nl));
    }
  run_jobs(F, jobs, F.Z.p, nullptr, F.Z.p, s);
  // 9. every boundary node reads its face's three parts
  GatherDev GD{};
  for (int f = 0; f < 6; ++f) {
    GD.x[f][0] = F.s2_off[f][0];
    GD.x[f][1] = F.s2_off[f][1];
    GD.Pu[f] = F.ax[ax_u(f)].P;
    for (int gg = 0; gg < 2; ++gg) {
      const int ng = gg ? ax_v(f) : ax_u(f), w = gg ? ax_u(f) : ax_v(f);
      GD.z[f][gg] = F.z_off[f][gg];
      GD.P01[f][gg] = F.ax[w].P;
      GD.Nn[f][gg] = F.N[ng];
    }
  }
  for (int a = 0; a < 3; ++a) GD.N[a] = F.N[a];
  k_ff_gather<<<(B.ntarget + 255) / 256, 256, 0, s>>>(GD, B.tgt_node.p, B.ntarget, F.X.p, F.Z.p, dsum);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

}  // namespace vpmg
