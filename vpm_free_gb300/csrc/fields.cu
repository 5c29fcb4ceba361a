// fields.cu -- mesh-to-mesh kernels of the step.
//
//  * rhsscat_3d / solget_3d for one block (source/vpm_mpi.f90:199-328):
//    box copies between the global mesh and the padded block;
//  * YAPS sampling, coarse Laplacian and face interpolation
//    (source/yaps3d.f90:104-138, 1914-2016) driven by host-built maps;
//  * calc_velocity_serial_3d(1) (source/vpm_gcalc.f90:1-136): central-
//    difference curl and the conservative stretching term.
#include "fields.h"
#include "ff.cuh"

namespace vpmg {

namespace {

// One node per thread; blockIdx.y is the plane k, and the threads of a
// plane run over its e0 x e1 nodes without gaps (one 32-bit division per
// node, no partly filled CTA per row).
__global__ void k_box_copy(const double* __restrict__ src, int sx, int sy, int so0, int so1, int so2,
                           double* __restrict__ dst, int dx, int dy, int do0, int do1, int do2, int e0, int e1) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= e0 * e1) return;
  const int j = t / e0, i = t - j * e0, k = blockIdx.y;
  dst[(size_t)(do0 + i) + (size_t)dx * ((do1 + j) + (size_t)dy * (do2 + k))] =
      src[(size_t)(so0 + i) + (size_t)sx * ((so1 + j) + (size_t)sy * (so2 + k))];
}

__global__ void k_sample(const double* __restrict__ a0, const double* __restrict__ a1, const double* __restrict__ a2,
                         const long long* __restrict__ src, const long long* __restrict__ dst, int n,
                         double* __restrict__ c0, double* __restrict__ c1, double* __restrict__ c2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  c0[dst[t]] = a0[src[t]];
  c1[dst[t]] = a1[src[t]];
  c2[dst[t]] = a2[src[t]];
}

__global__ void k_coarse_lap(const double* __restrict__ s, double* __restrict__ r, int CX, int CY, int lo0, int lo1,
                             int lo2, int e0, int e1, int e2, double ih0, double ih1, double ih2) {
  const size_t n = (size_t)e0 * e1 * e2;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = lo0 + (int)(t % e0);
  const int j = lo1 + (int)((t / e0) % e1);
  const int k = lo2 + (int)(t / ((size_t)e0 * e1));
  const size_t sy = CX, sz = (size_t)CX * CY;
  const size_t id = (size_t)i + sy * j + sz * k;
  const double c = s[id];
  r[id] = ((s[id + 1] - 2.0 * c) + s[id - 1]) * ih0 + ((s[id + sy] - 2.0 * c) + s[id - sy]) * ih1 +
          ((s[id + sz] - 2.0 * c) + s[id - sz]) * ih2;
}

__global__ void k_face_interp(const long long* __restrict__ node, const long long* __restrict__ cbase,
                              const double* __restrict__ w, const int* __restrict__ flagged, int n,
                              const double* __restrict__ csol, const double* __restrict__ samp, int CX, int CY,
                              double* __restrict__ sol) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double* wt = w + 9 * (size_t)t;
  const size_t b = cbase[t];
  const size_t sy = CX, sz = (size_t)CX * CY;
  const bool fl = flagged[t] != 0;
  double v = sol[node[t]];
  for (int kc = 0; kc < 3; ++kc)
    for (int jc = 0; jc < 3; ++jc)
      for (int ic = 0; ic < 3; ++ic) {
        const double f = (wt[ic] * wt[3 + jc]) * wt[6 + kc];
        const size_t cid = b + ic + sy * jc + sz * kc;
        const double sm = samp[cid];
        const double add = fl ? sm : 0.0;
        v = v + f * ((csol[cid] - sm) + add);
      }
  sol[node[t]] = v;
}

// u = curl psi on nodes 1..N-2 (0-based); other nodes keep zero.
// With f0 (nullable), the velocity is also written as float-float pairs
// f0/f1/f2 for the mesh-to-particle gather.
__global__ void k_velocity(const double* __restrict__ p0, const double* __restrict__ p1, const double* __restrict__ p2,
                           int NX, int NY, int NZ, double i2x, double i2y, double i2z, double* __restrict__ u0,
                           double* __restrict__ u1, double* __restrict__ u2, float2* __restrict__ f0,
                           float2* __restrict__ f1, float2* __restrict__ f2) {
  // grid: (x blocks, y, z) over the interior, no index divisions
  const int i = 1 + blockIdx.x * blockDim.x + threadIdx.x, j = 1 + blockIdx.y, k = 1 + blockIdx.z;
  if (i > NX - 2) return;
  const size_t sy = NX, sz = (size_t)NX * NY;
  const size_t id = i + sy * j + sz * k;
  // central differences; each component's two scalings by 1/(2h) fused
  // into one multiply and one FMA (12 FP64 operations per node)
  const double ex1 = p1[id + 1] - p1[id - 1], ex2 = p2[id + 1] - p2[id - 1];
  const double ey0 = p0[id + sy] - p0[id - sy], ey2 = p2[id + sy] - p2[id - sy];
  const double ez0 = p0[id + sz] - p0[id - sz], ez1 = p1[id + sz] - p1[id - sz];
  const double v0 = fma(ey2, i2y, -(ez1 * i2z)), v1 = fma(ez0, i2z, -(ex2 * i2x)), v2 = fma(ex1, i2x, -(ey0 * i2y));
  u0[id] = v0;
  u1[id] = v1;
  u2[id] = v2;
  if (f0) {
    f0[id] = ff::split(v0);
    f1[id] = ff::split(v1);
    f2[id] = ff::split(v2);
  }
}

// Stretching  SOL(m) = -sum_j d(RHS_j u_m)/dx_j  on nodes 2..N-3 (0-based).
__global__ void k_deformation(const double* __restrict__ r0, const double* __restrict__ r1, const double* __restrict__ r2,
                              const double* __restrict__ u0, const double* __restrict__ u1,
                              const double* __restrict__ u2, int NX, int NY, int NZ, double i2x, double i2y, double i2z,
                              double* __restrict__ g0, double* __restrict__ g1, double* __restrict__ g2,
                              float2* __restrict__ f0, float2* __restrict__ f1, float2* __restrict__ f2) {
  // grid: (x blocks, y, z) over nodes 2..N-3, no index divisions
  const int i = 2 + blockIdx.x * blockDim.x + threadIdx.x, j = 2 + blockIdx.y, k = 2 + blockIdx.z;
  if (i > NX - 3) return;
  const size_t sy = NX, sz = (size_t)NX * NY;
  const size_t id = i + sy * j + sz * k;
  const double rxp = r0[id + 1], rxm = r0[id - 1], ryp = r1[id + sy], rym = r1[id - sy], rzp = r2[id + sz],
               rzm = r2[id - sz];
  const double* U[3] = {u0, u1, u2};
  double* G[3] = {g0, g1, g2};
  float2* F[3] = {f0, f1, f2};
  if (rxp == 0.0 && rxm == 0.0 && ryp == 0.0 && rym == 0.0 && rzp == 0.0 && rzm == 0.0) {
    // no vorticity around the node (most of the mesh): the stretching is zero
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      G[m][id] = 0.0;
      if (f0) F[m][id] = make_float2(0.0f, 0.0f);
    }
    return;
  }
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    // -sum_j (R_j u_m (+) - R_j u_m (-)) / (2 h_j): each difference one
    // multiply and one FMA, the three scalings and sums two FMAs and a multiply
    const double* u = U[m];
    const double a = fma(rxm, u[id - 1], -(rxp * u[id + 1]));
    const double b = fma(rym, u[id - sy], -(ryp * u[id + sy]));
    const double c = fma(rzm, u[id - sz], -(rzp * u[id + sz]));
    const double v = fma(a, i2x, fma(b, i2y, c * i2z));
    G[m][id] = v;
    if (f0) F[m][id] = ff::split(v);
  }
}

// The stretching stencil in float-float arithmetic, writing both the FP64
// field and its float-float pairs: the products and differences run on the
// FP32 pipes, the only FP64 operation is the join of each output.  It reads
// the velocity's float-float pairs.  (The velocity's curl stays FP64: it has
// few operations per node and runs at the memory rate.)
__global__ void k_deformation_ff(const double* __restrict__ r0, const double* __restrict__ r1,
                                 const double* __restrict__ r2, const float2* __restrict__ u0,
                                 const float2* __restrict__ u1, const float2* __restrict__ u2, int NX, int NY, int NZ,
                                 double i2x, double i2y, double i2z, double* __restrict__ g0, double* __restrict__ g1,
                                 double* __restrict__ g2, float2* __restrict__ f0, float2* __restrict__ f1,
                                 float2* __restrict__ f2) {
  const int ex = NX - 4, ey = NY - 4, ez = NZ - 4;
  const size_t n = (size_t)ex * ey * ez;
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = 2 + (int)(t % ex), j = 2 + (int)((t / ex) % ey), k = 2 + (int)(t / ((size_t)ex * ey));
  const size_t sy = NX, sz = (size_t)NX * NY;
  const size_t id = i + sy * j + sz * k;
  const float2 IX = ff::split(i2x), IY = ff::split(i2y), IZ = ff::split(i2z);
  const float2 rxp = ff::split(r0[id + 1]), rxm = ff::split(r0[id - 1]), ryp = ff::split(r1[id + sy]),
               rym = ff::split(r1[id - sy]), rzp = ff::split(r2[id + sz]), rzm = ff::split(r2[id - sz]);
  const float2* U[3] = {u0, u1, u2};
  double* G[3] = {g0, g1, g2};
  float2* F[3] = {f0, f1, f2};
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const float2* u = U[m];
    const float2 a = ff::neg(ff::mul(ff::sub(ff::mul(rxp, u[id + 1]), ff::mul(rxm, u[id - 1])), IX));
    const float2 b = ff::neg(ff::mul(ff::sub(ff::mul(ryp, u[id + sy]), ff::mul(rym, u[id - sy])), IY));
    const float2 c = ff::neg(ff::mul(ff::sub(ff::mul(rzp, u[id + sz]), ff::mul(rzm, u[id - sz])), IZ));
    const float2 v = ff::add(ff::add(a, b), c);
    G[m][id] = ff::to_double(v);
    F[m][id] = v;
  }
}

// diffuse_vort_3d (source/vpm_gcalc.f90:138-210), neqpm = 3 (VIS = NI):
// SOL(m) = -NI Lap_h RHS(m) on the nodes strictly inside [lo, hi] (0-based);
// SOL is zero elsewhere (cleared by the caller).
__global__ void k_diffuse(const double* __restrict__ r0, const double* __restrict__ r1, const double* __restrict__ r2,
                          int NX, int NY, int lo0, int lo1, int lo2, int e0, int e1, int e2, double idx2, double idy2,
                          double idz2, double ni, double* __restrict__ s0, double* __restrict__ s1,
                          double* __restrict__ s2) {
  const size_t n = (size_t)e0 * e1 * e2;
  const size_t sy = NX, sz = (size_t)NX * NY;
  const double* R[3] = {r0, r1, r2};
  double* S[3] = {s0, s1, s2};
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int i = lo0 + (int)(t % e0), j = lo1 + (int)((t / e0) % e1), k = lo2 + (int)(t / ((size_t)e0 * e1));
    const size_t id = (size_t)i + sy * j + sz * k;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
      const double* r = R[m];
      const double c = r[id];
      const double dxx = ((r[id + 1] - 2.0 * c) + r[id - 1]) * idx2;
      const double dyy = ((r[id + sy] - 2.0 * c) + r[id - sy]) * idy2;
      const double dzz = ((r[id + sz] - 2.0 * c) + r[id - sz]) * idz2;
      S[m][id] = -ni * ((dxx + dyy) + dzz);
    }
  }
}

template <class T>
void upload(DBuf<T>& b, const std::vector<T>& h) {
  b.ensure(h.size());
  if (!h.empty()) VPMG_CUDA(cudaMemcpy(b.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
}

unsigned grid_for(size_t n, int threads) { return (unsigned)std::max<size_t>(1, (n + threads - 1) / threads); }

}  // namespace

void box_copy(const double* src, const int sdims[3], const int so[3], double* dst, const int ddims[3], const int dof[3],
              const int ext[3], cudaStream_t s) {
  const size_t n = (size_t)ext[0] * ext[1] * ext[2];
  if (!n) return;
  VPMG_CHECK(ext[2] <= 65535 && (size_t)ext[0] * ext[1] <= (size_t)INT32_MAX, VPMG_ERR_UNSUPPORTED,
             "box copy extent above the grid limit");
  const dim3 grid((unsigned)(((size_t)ext[0] * ext[1] + 255) / 256), (unsigned)ext[2]);
  k_box_copy<<<grid, 256, 0, s>>>(src, sdims[0], sdims[1], so[0], so[1], so[2], dst, ddims[0], ddims[1], dof[0], dof[1],
                                  dof[2], ext[0], ext[1]);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void YapsDev::prepare(const YapsGeom& Y) {
  std::vector<long long> fnode(Y.faces.size()), fcb(Y.faces.size());
  std::vector<double> fw(9 * Y.faces.size());
  std::vector<int> ffl(Y.faces.size());
  for (size_t t = 0; t < Y.faces.size(); ++t) {
    fnode[t] = Y.faces[t].node;
    fcb[t] = Y.faces[t].cbase;
    for (int m = 0; m < 9; ++m) fw[9 * t + m] = Y.faces[t].w[m];
    ffl[t] = Y.faces[t].flagged;
  }
  upload(samp_src, Y.samp_src);
  upload(samp_dst, Y.samp_dst);
  upload(face_node, fnode);
  upload(face_cbase, fcb);
  upload(face_w, fw);
  upload(face_flag, ffl);
  nsamp = (int)Y.samp_src.size();
  nface = (int)Y.faces.size();
  for (int d = 0; d < 6; ++d) map[d] = Y.map[d];
}

void yaps_sample(const YapsDev& Y, const double* const sbl[3], double* const samp[3], cudaStream_t s) {
  k_sample<<<grid_for(Y.nsamp, 256), 256, 0, s>>>(sbl[0], sbl[1], sbl[2], Y.samp_src.p, Y.samp_dst.p, Y.nsamp, samp[0],
                                                  samp[1], samp[2]);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void yaps_coarse_rhs(const YapsDev& Y, const int cdims[3], const double dc[3], const double* const samp[3],
                     double* const crhs[3], cudaStream_t s) {
  const int lo[3] = {Y.map[0], Y.map[1], Y.map[2]};  // 1-based map(1:3)+1  ->  0-based map(1:3)
  const int e[3] = {Y.map[3] - Y.map[0] - 1, Y.map[4] - Y.map[1] - 1, Y.map[5] - Y.map[2] - 1};
  if (e[0] <= 0 || e[1] <= 0 || e[2] <= 0) return;
  const size_t n = (size_t)e[0] * e[1] * e[2];
  for (int c = 0; c < 3; ++c) {
    k_coarse_lap<<<grid_for(n, 256), 256, 0, s>>>(samp[c], crhs[c], cdims[0], cdims[1], lo[0], lo[1], lo[2], e[0], e[1],
                                                  e[2], 1.0 / (dc[0] * dc[0]), 1.0 / (dc[1] * dc[1]),
                                                  1.0 / (dc[2] * dc[2]));
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}

void yaps_face_interp(const YapsDev& Y, const int cdims[3], const double* const csol[3], const double* const samp[3],
                      double* const sbl[3], cudaStream_t s) {
  for (int c = 0; c < 3; ++c) {
    k_face_interp<<<grid_for(Y.nface, 128), 128, 0, s>>>(Y.face_node.p, Y.face_cbase.p, Y.face_w.p, Y.face_flag.p,
                                                         Y.nface, csol[c], samp[c], cdims[0], cdims[1], sbl[c]);
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}

void viscous_diffusion(const int dims[3], const int nn_bl[6], const double h[3], double ni, const double* const rhs[3],
                       double* const sol[3], cudaStream_t s) {
  // interior of the block range: 1-based NXs_bl+1 .. NXf_bl-1 -> 0-based nn_bl[d] .. nn_bl[d+3]-2
  const int lo[3] = {nn_bl[0], nn_bl[1], nn_bl[2]};
  const int e[3] = {nn_bl[3] - nn_bl[0] - 1, nn_bl[4] - nn_bl[1] - 1, nn_bl[5] - nn_bl[2] - 1};
  for (int c = 0; c < 3; ++c) fill_zero(sol[c], (size_t)dims[0] * dims[1] * dims[2], s);
  if (e[0] <= 0 || e[1] <= 0 || e[2] <= 0) return;
  const size_t n = (size_t)e[0] * e[1] * e[2];
  k_diffuse<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 32), 256, 0, s>>>(
      rhs[0], rhs[1], rhs[2], dims[0], dims[1], lo[0], lo[1], lo[2], e[0], e[1], e[2], 1.0 / (h[0] * h[0]),
      1.0 / (h[1] * h[1]), 1.0 / (h[2] * h[2]), ni, sol[0], sol[1], sol[2]);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

// Nodes where the FP64 stretching stencil has work: an interior node
// (2..N-3) with a non-zero RHS among its six neighbours (instrumentation).
__global__ void k_count_vortical(const double* __restrict__ r0, const double* __restrict__ r1,
                                 const double* __restrict__ r2, int NX, int NY, int NZ,
                                 unsigned long long* __restrict__ count) {
  const int ex = NX - 4, ey = NY - 4, ez = NZ - 4;
  const size_t n = (size_t)ex * ey * ez;
  const size_t sy = NX, sz = (size_t)NX * NY;
  unsigned long long c = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int i = 2 + (int)(t % ex), j = 2 + (int)((t / ex) % ey), k = 2 + (int)(t / ((size_t)ex * ey));
    const size_t id = i + sy * j + sz * k;
    if (r0[id + 1] != 0.0 || r0[id - 1] != 0.0 || r1[id + sy] != 0.0 || r1[id - sy] != 0.0 || r2[id + sz] != 0.0 ||
        r2[id - sz] != 0.0)
      ++c;
  }
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(count, c);
}

long long count_vortical_nodes(const int dims[3], const double* const rhs[3], cudaStream_t s) {
  if (dims[0] <= 4 || dims[1] <= 4 || dims[2] <= 4) return 0;
  DBuf<unsigned long long> d;
  d.ensure(1);
  VPMG_CUDA(cudaMemsetAsync(d.p, 0, sizeof(unsigned long long), s));
  k_count_vortical<<<152 * 8, 256, 0, s>>>(rhs[0], rhs[1], rhs[2], dims[0], dims[1], dims[2], d.p);
  VPMG_LAUNCHED();
  unsigned long long c = 0;
  VPMG_CUDA(cudaMemcpyAsync(&c, d.p, sizeof(c), cudaMemcpyDeviceToHost, s));
  VPMG_CUDA(cudaStreamSynchronize(s));
  return (long long)c;
}

void velocity_and_stretching(const int dims[3], const double h[3], const double* const psi[3], const double* const rhs[3],
                             double* const vel[3], double* const def[3], cudaStream_t s, int parts,
                             float2* const vel_ff[3], float2* const def_ff[3]) {
  const int NX = dims[0], NY = dims[1], NZ = dims[2];
  const double i2x = 1.0 / (2 * h[0]), i2y = 1.0 / (2 * h[1]), i2z = 1.0 / (2 * h[2]);
  if ((parts & 1) && NX > 2 && NY > 2 && NZ > 2) {
    const dim3 g((unsigned)((NX - 2 + 127) / 128), (unsigned)(NY - 2), (unsigned)(NZ - 2));
    k_velocity<<<g, 128, 0, s>>>(psi[0], psi[1], psi[2], NX, NY, NZ, i2x, i2y, i2z, vel[0], vel[1], vel[2],
                                                vel_ff ? vel_ff[0] : nullptr, vel_ff ? vel_ff[1] : nullptr,
                                                vel_ff ? vel_ff[2] : nullptr);
    VPMG_LAUNCHED();
  }
  if ((parts & 2) && NX > 4 && NY > 4 && NZ > 4) {
    const size_t n = (size_t)(NX - 4) * (NY - 4) * (NZ - 4);
    if (vel_ff && def_ff)  // the velocity's float-float pairs are current whenever vel_ff is passed
      k_deformation_ff<<<grid_for(n, 256), 256, 0, s>>>(rhs[0], rhs[1], rhs[2], vel_ff[0], vel_ff[1], vel_ff[2], NX, NY,
                                                        NZ, i2x, i2y, i2z, def[0], def[1], def[2], def_ff[0],
                                                        def_ff[1], def_ff[2]);
    else
      k_deformation<<<dim3((unsigned)((NX - 4 + 127) / 128), (unsigned)(NY - 4), (unsigned)(NZ - 4)), 128, 0, s>>>(
          rhs[0], rhs[1], rhs[2], vel[0], vel[1], vel[2], NX, NY, NZ, i2x, i2y, i2z, def[0], def[1], def[2],
          def_ff ? def_ff[0] : nullptr, def_ff ? def_ff[1] : nullptr, def_ff ? def_ff[2] : nullptr);
    VPMG_LAUNCHED();
  }
  VPMG_CUDA(cudaGetLastError());
}

}  // namespace vpmg
