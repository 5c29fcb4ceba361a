// adjoint.cu -- reverse mode of the whole particle-mesh step.
//
// One step of the forward map (source/vpm.f90 WhatToDo = 2, the Euler push
// of source/test.f90:104-117, remesh_particles_3d(1)) is
//   R   = D(X) Q / DV                      deposition (pmproject.f90:43-153)
//   psi = L R                              rhsscat, yaps3d, solget (linear)
//   u   = C psi,  g = S(R, u)              vpm_gcalc.f90:1-136
//   UP  = I(X) u, GP = V I(X) g            vpm_time.f90:62-107
//   X'  = X + dt UP,  Q' = Q - dt GP
//   Q'' = mask . D_r(X') Q'                remesh (vpm_remesh.f90:50-195)
// and the loss is a function of the velocity field of the final particles.
// Every linear piece is transposed exactly (L is not symmetric: one-sided
// normal derivatives, the quadtree far field, the coarse coupling of
// YAPS), positions enter through the M4' weights and their derivative, the
// remesh threshold is a fixed mask, and remeshed particles sit on mesh
// nodes, so their positions carry no gradient.  Particle states are
// checkpointed on the forward pass; the backward pass recomputes one step
// from its checkpoint and then runs that step's transpose.  No kernel of
// the backward pass needs a host round trip (particle counts stay on the
// device).
#include <algorithm>
#include <cmath>
#include <vector>

#include "ff.cuh"
#include "handle.h"

struct AdjointState {
  int cap = 0;
  vpmg::DBuf<double> ckpt;  // (K+1) checkpoints x 7 particle arrays x capacity
  vpmg::DBuf<int> ckpt_np;  // (K+1)
  vpmg::DBuf<double> xq1;   // X', Q' after the Euler push: 6 x cap
  vpmg::DBuf<double> pbar;  // xbar qbar upbar gpbar qnew xb1 qb1: 21 x cap
  vpmg::DBuf<double> rbar, psibar, ubar, gbar, nodeA;  // 3 x N each
  vpmg::DBuf<double> blA, blB, blC, blD;               // block arrays (NB)
  vpmg::DBuf<double> cA, cB, cC;                       // coarse arrays (NC)
  vpmg::DBuf<double> cellbar, panelbar;
  vpmg::DBuf<double> sampbar, crhsbar, csolbar;  // NC each
  vpmg::DBuf<double> rhsbarbl;                   // NB
  vpmg::DBuf<double> probes, uprobe;             // 3 x nprobe each (component-major)
  vpmg::DBuf<double> lossv;                      // block partial sums
  vpmg::DBuf<double> out;                        // AoS gradients for the host copy
  vpmg::DBuf<int> masks;                         // remesh node masks of the last recorded run: K x N
  vpmg::DBuf<int> kidx;                          // checkpoint index read by the copies (device side)
  int nprobe = 0;
  int masks_steps = -1;                          // steps recorded in masks (-1: none)
  // one backward step captured as a CUDA graph, replayed once per step
  cudaGraphExec_t bwd = nullptr;
  double bwd_dt = 0.0;
  const void* bwd_key[3] = {nullptr, nullptr, nullptr};
  long long bwd_launches = 0;
  ~AdjointState() {
    if (bwd) cudaGraphExecDestroy(bwd);
  }
};

namespace vpmg {
namespace {

// ---------------------------------------------------------------- M4' ----
__device__ __forceinline__ double m4(double t) {
  const double a = fabs(t);
  if (a > 2.0) return 0.0;
  if (a >= 1.0) return 0.5 * ((2.0 - a) * (2.0 - a)) * (1.0 - a);
  return 1.0 - 2.5 * (a * a) + 1.5 * (a * a * a);
}
__device__ __forceinline__ double dm4(double t) {  // d m4 / dt
  const double a = fabs(t), sg = t < 0.0 ? -1.0 : 1.0;
  if (a > 2.0) return 0.0;
  if (a >= 1.0) return sg * (-0.5 * (2.0 - a) * (4.0 - 3.0 * a));
  return -5.0 * t + 4.5 * t * a;
}
__device__ __forceinline__ int cell_of(double x, double xmin, double d) { return (int)__ddiv_rn(__dsub_rn(x, xmin), d); }

// The 4 x 4 x 4 M4' stencil of a point: base cell, weights and their
// derivatives with respect to the point's coordinates.  False when the
// stencil leaves the mesh (the binning reports that case as an error).
struct Stencil {
  int c0[3];
  double w[3][4], dw[3][4];
};
__device__ __forceinline__ bool stencil(const MeshDev& m, double px, double py, double pz, Stencil& S) {
  const double p[3] = {px, py, pz};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    if (!(p[d] - m.xmin[d] >= 0.0)) return false;
    S.c0[d] = cell_of(p[d], m.xmin[d], m.d[d]);
    if (S.c0[d] - 1 < 0 || S.c0[d] + 2 >= m.n[d]) return false;
    const double inv = 1.0 / m.d[d];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int node = S.c0[d] - 1 + a;
      const double t = (p[d] - m.xmin[d] - (double)node * m.d[d]) * inv;
      S.w[d][a] = m4(t);
      S.dw[d][a] = dm4(t) * inv;
    }
  }
  return true;
}
__device__ __forceinline__ size_t node_id(const MeshDev& m, const Stencil& S, int a, int b, int c) {
  return (size_t)(S.c0[0] - 1 + a) + (size_t)m.n[0] * ((size_t)(S.c0[1] - 1 + b) + (size_t)m.n[1] * (S.c0[2] - 1 + c));
}

struct Vec3 {
  const double* c[3];
};

// Per particle p (count on the device):
//   qbar_p += sA sum_n W(X_p, n) A(n)
//   xbar_p += sum_n grad W(X_p, n) [ sA a_p . A(n) + sB bw_p b_p . B(n) ]
// A, B: three node fields back to back (N apart); a, b: three particle
// arrays; qbar, xbar: three particle arrays cap apart.
__global__ void k_particle_adj(MeshDev m, const int* __restrict__ np_dev, const double* __restrict__ x,
                               const double* __restrict__ y, const double* __restrict__ z,
                               const double* __restrict__ A, const double* __restrict__ B, size_t N, Vec3 a, Vec3 b,
                               const double* __restrict__ bw, double sA, double sB, double* __restrict__ qbar,
                               double* __restrict__ xbar, int cap) {
  const int np = *np_dev;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    Stencil S;
    if (!stencil(m, x[p], y[p], z[p], S)) continue;
    const double av[3] = {sA * a.c[0][p], sA * a.c[1][p], sA * a.c[2][p]};
    double bv[3] = {0.0, 0.0, 0.0};
    if (B) {
      const double f = sB * (bw ? bw[p] : 1.0);
      bv[0] = f * b.c[0][p];
      bv[1] = f * b.c[1][p];
      bv[2] = f * b.c[2][p];
    }
    double q[3] = {0, 0, 0}, g[3] = {0, 0, 0};
    for (int c = 0; c < 4; ++c)
      for (int bb = 0; bb < 4; ++bb) {
        const double wyz = S.w[1][bb] * S.w[2][c], dyz = S.dw[1][bb] * S.w[2][c], ydz = S.w[1][bb] * S.dw[2][c];
#pragma unroll
        for (int aa = 0; aa < 4; ++aa) {
          const size_t id = node_id(m, S, aa, bb, c);
          const double A0 = A[id], A1 = A[N + id], A2 = A[2 * N + id];
          double s = av[0] * A0 + av[1] * A1 + av[2] * A2;
          if (B) s += bv[0] * B[id] + bv[1] * B[N + id] + bv[2] * B[2 * N + id];
          const double wx = S.w[0][aa];
          if (qbar) {
            const double f = wx * wyz * sA;
            q[0] += f * A0;
            q[1] += f * A1;
            q[2] += f * A2;
          }
          g[0] += S.dw[0][aa] * wyz * s;
          g[1] += wx * dyz * s;
          g[2] += wx * ydz * s;
        }
      }
    if (qbar)
      for (int d = 0; d < 3; ++d) qbar[(size_t)d * cap + p] += q[d];
    for (int d = 0; d < 3; ++d) xbar[(size_t)d * cap + p] += g[d];
  }
}

// Strength slots of the sorted records <- scale * w_p * v_p (w = QP(4) or 1):
// FP64 records (ff == 0) are slot-major with stride cs, float-float records
// (ff != 0) particle-major.
__global__ void k_records_set_q(float2* __restrict__ rec, int ff, size_t cs, const int* __restrict__ perm,
                                const int* __restrict__ nsorted, const double* __restrict__ v, int cap, double scale,
                                const double* __restrict__ w) {
  const int n = *nsorted;
  double* rd = reinterpret_cast<double*>(rec);
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < n; s += gridDim.x * blockDim.x) {
    const int p = perm[s];
    const double f = scale * (w ? w[p] : 1.0);
    const double q[3] = {f * v[p], f * v[cap + p], f * v[2 * (size_t)cap + p]};
    for (int c = 0; c < 3; ++c) {
      if (ff) rec[(size_t)s * kRecLen + kRecQ + c] = ff::split(q[c]);
      else rd[(kRecQ + c) * cs + s] = q[c];
    }
  }
}

__device__ __forceinline__ void unflatten(size_t id, int NX, int NY, int& i, int& j, int& k) {
  i = (int)(id % NX);
  j = (int)((id / NX) % NY);
  k = (int)(id / ((size_t)NX * NY));
}

// Transposed stretching.  Forward, on nodes 2..N-3:
//   g_m(n) = -sum_j (a_jm(n + e_j) - a_jm(n - e_j)) / (2 h_j),  a_jm = R_j u_m,
// so abar_jm(k) = (gbar_m(k + e_j) - gbar_m(k - e_j)) / (2 h_j) with gbar
// restricted to the region; Rbar_j += abar_jm u_m and ubar_m += abar_jm R_j.
__global__ void k_stretch_T(const double* __restrict__ gbar, const double* __restrict__ R, const double* __restrict__ u,
                            int NX, int NY, int NZ, double i2x, double i2y, double i2z, double* __restrict__ rbar,
                            double* __restrict__ ubar) {
  const size_t N = (size_t)NX * NY * NZ;
  const size_t st[3] = {1, (size_t)NX, (size_t)NX * NY};
  const int ext[3] = {NX, NY, NZ};
  const double i2[3] = {i2x, i2y, i2z};
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < N; id += (size_t)gridDim.x * blockDim.x) {
    int pos[3];
    unflatten(id, NX, NY, pos[0], pos[1], pos[2]);
    auto inreg = [&](int d, int off) {
      for (int e = 0; e < 3; ++e) {
        const int q = pos[e] + (e == d ? off : 0);
        if (q < 2 || q > ext[e] - 3) return false;
      }
      return true;
    };
    double rb[3] = {0, 0, 0}, ub[3] = {0, 0, 0};
    for (int jd = 0; jd < 3; ++jd) {
      const bool lo = inreg(jd, -1), hi = inreg(jd, +1);
      if (!lo && !hi) continue;
      for (int mm = 0; mm < 3; ++mm) {
        const double gl = lo ? gbar[(size_t)mm * N + id - st[jd]] : 0.0;
        const double gh = hi ? gbar[(size_t)mm * N + id + st[jd]] : 0.0;
        const double G = (gh - gl) * i2[jd];
        rb[jd] += G * u[(size_t)mm * N + id];
        ub[mm] += G * R[(size_t)jd * N + id];
      }
    }
    for (int c = 0; c < 3; ++c) {
      rbar[(size_t)c * N + id] += rb[c];
      ubar[(size_t)c * N + id] += ub[c];
    }
  }
}

// Transposed curl.  Forward on nodes 1..N-2 with D_d f(n) = (f(n+e_d) - f(n-e_d)) / (2 h_d):
//   u0 = Dy psi2 - Dz psi1,  u1 = Dz psi0 - Dx psi2,  u2 = Dx psi1 - Dy psi0.
__global__ void k_curl_T(const double* __restrict__ ubar, int NX, int NY, int NZ, double i2x, double i2y, double i2z,
                         double* __restrict__ psibar) {
  const size_t N = (size_t)NX * NY * NZ;
  const size_t st[3] = {1, (size_t)NX, (size_t)NX * NY};
  const int ext[3] = {NX, NY, NZ};
  const double i2[3] = {i2x, i2y, i2z};
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < N; id += (size_t)gridDim.x * blockDim.x) {
    int pos[3];
    unflatten(id, NX, NY, pos[0], pos[1], pos[2]);
    // (D_d^T f)(n) = (f(n - e_d) - f(n + e_d)) / (2 h_d), f restricted to nodes 1..N-2
    auto DT = [&](int cu, int d) {
      double r = 0.0;
      for (int sgn = -1; sgn <= 1; sgn += 2) {
        bool ok = true;
        for (int e = 0; e < 3; ++e) {
          const int q = pos[e] + (e == d ? sgn : 0);
          if (q < 1 || q > ext[e] - 2) ok = false;
        }
        if (ok) {
          const double v = ubar[(size_t)cu * N + (sgn < 0 ? id - st[d] : id + st[d])];
          r += sgn < 0 ? v : -v;
        }
      }
      return r * i2[d];
    };
    psibar[id] = DT(1, 2) - DT(2, 1);
    psibar[N + id] = DT(2, 0) - DT(0, 2);
    psibar[2 * N + id] = DT(0, 1) - DT(1, 0);
  }
}

// Boundary-value adjoint of a Dirichlet solve on box [lo, hi] whose face
// values pass through to the output: on face-interior nodes
// bbar = ubar - fbar(interior neighbour) / h^2, on box edges bbar = ubar.
__global__ void k_face_bc_T(const double* __restrict__ ubar, const double* __restrict__ fbar, int NX, int NY, int lo0,
                            int lo1, int lo2, int hi0, int hi1, int hi2, double ihx2, double ihy2, double ihz2,
                            double* __restrict__ bbar) {
  const int ex = hi0 - lo0 + 1, ey = hi1 - lo1 + 1, ez = hi2 - lo2 + 1;
  const long long total = (long long)ex * ey * ez;
  const size_t sy = NX, sz = (size_t)NX * NY;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const int i = lo0 + (int)(t % ex), j = lo1 + (int)((t / ex) % ey), k = lo2 + (int)(t / ((long long)ex * ey));
    const bool bx = (i == lo0 || i == hi0), by = (j == lo1 || j == hi1), bz = (k == lo2 || k == hi2);
    if (!bx && !by && !bz) continue;
    const size_t id = (size_t)i + sy * j + sz * k;
    double v = ubar[id];
    if ((int)bx + (int)by + (int)bz == 1) {
      if (bx) v -= fbar[i == lo0 ? id + 1 : id - 1] * ihx2;
      if (by) v -= fbar[j == lo1 ? id + sy : id - sy] * ihy2;
      if (bz) v -= fbar[k == lo2 ? id + sz : id - sz] * ihz2;
    }
    bbar[id] = v;
  }
}

__global__ void k_zero(double* __restrict__ p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = 0.0;
}
__global__ void k_axpy(double* __restrict__ y, const double* __restrict__ x, double a, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] += a * x[i];
}
// dst(box at dof) += src(box at so), box extent e.
__global__ void k_box_add(const double* __restrict__ src, int sx, int sy, int so0, int so1, int so2,
                          double* __restrict__ dst, int dx, int dy, int do0, int do1, int do2, int e0, int e1, int e2) {
  const size_t n = (size_t)e0 * e1 * e2;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(t % e0), j = (int)((t / e0) % e1), k = (int)(t / ((size_t)e0 * e1));
    dst[(size_t)(do0 + i) + (size_t)dx * ((do1 + j) + (size_t)dy * (do2 + k))] +=
        src[(size_t)(so0 + i) + (size_t)sx * ((so1 + j) + (size_t)sy * (so2 + k))];
  }
}

// Transposed face interpolation: sol(node) += sum f (csol - samp + flag samp).
__global__ void k_face_interp_T(const long long* __restrict__ node, const long long* __restrict__ cbase,
                                const double* __restrict__ w, const int* __restrict__ flagged, int n, int CX, int CY,
                                const double* __restrict__ fbar, double* __restrict__ csolbar,
                                double* __restrict__ sampbar) {
  const size_t sy = CX, sz = (size_t)CX * CY;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const double F = fbar[node[t]];
    if (F == 0.0) continue;
    const double* wt = w + 9 * (size_t)t;
    const size_t b = cbase[t];
    const bool fl = flagged[t] != 0;  // then d/dsamp = -1 + 1 = 0
    for (int kc = 0; kc < 3; ++kc)
      for (int jc = 0; jc < 3; ++jc)
        for (int ic = 0; ic < 3; ++ic) {
          const double f = (wt[ic] * wt[3 + jc]) * wt[6 + kc];
          const size_t cid = b + ic + sy * jc + sz * kc;
          atomicAdd(&csolbar[cid], f * F);
          if (!fl) atomicAdd(&sampbar[cid], -f * F);
        }
  }
}

// Transposed coarse Laplacian (restricted to the map interior): sampbar += Lap(crhsbar masked).
__global__ void k_coarse_lap_T(const double* __restrict__ cr, double* __restrict__ sb, int CX, int CY, int CZ, int lo0,
                               int lo1, int lo2, int e0, int e1, int e2, double ih0, double ih1, double ih2) {
  const size_t N = (size_t)CX * CY * CZ;
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < N; id += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    unflatten(id, CX, CY, i, j, k);
    auto v = [&](int a, int b, int c) {
      const bool in = a >= lo0 && a < lo0 + e0 && b >= lo1 && b < lo1 + e1 && c >= lo2 && c < lo2 + e2;
      return in ? cr[(size_t)a + (size_t)CX * (b + (size_t)CY * c)] : 0.0;
    };
    const double c0 = v(i, j, k);
    sb[id] += (v(i + 1, j, k) + v(i - 1, j, k) - 2.0 * c0) * ih0 + (v(i, j + 1, k) + v(i, j - 1, k) - 2.0 * c0) * ih1 +
              (v(i, j, k + 1) + v(i, j, k - 1) - 2.0 * c0) * ih2;
  }
}

__global__ void k_sample_T(const long long* __restrict__ src, const long long* __restrict__ dst, int n,
                           const double* __restrict__ sampbar, double* __restrict__ ubl) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    atomicAdd(&ubl[src[t]], sampbar[dst[t]]);
}

// X' = X + dt UP, Q' = Q - dt GP (the push of back_to_particles with uinf = 0).
__global__ void k_after_euler(const int* __restrict__ np_dev, const double* x, const double* y, const double* z,
                              const double* q0, const double* q1, const double* q2, const double* __restrict__ up,
                              const double* __restrict__ gp, double dt, double* __restrict__ xq1, int cap) {
  const int np = *np_dev;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    xq1[p] = x[p] + up[3 * (size_t)p] * dt;
    xq1[cap + p] = y[p] + up[3 * (size_t)p + 1] * dt;
    xq1[2 * (size_t)cap + p] = z[p] + up[3 * (size_t)p + 2] * dt;
    xq1[3 * (size_t)cap + p] = q0[p] - gp[3 * (size_t)p] * dt;
    xq1[4 * (size_t)cap + p] = q1[p] - gp[3 * (size_t)p + 1] * dt;
    xq1[5 * (size_t)cap + p] = q2[p] - gp[3 * (size_t)p + 2] * dt;
  }
}
__global__ void k_load_pushed(const int* __restrict__ np_dev, const double* __restrict__ xq1, int cap, double* x,
                              double* y, double* z, double* q0, double* q1, double* q2) {
  const int np = *np_dev;
  double* dst[6] = {x, y, z, q0, q1, q2};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
    for (int a = 0; a < 6; ++a) dst[a][p] = xq1[(size_t)a * cap + p];
}

// Node field of the emitted particles' strength adjoints (zero off the mask).
__global__ void k_mask_field(const int* __restrict__ flag, const int* __restrict__ pos, size_t N,
                             const double* __restrict__ qnew, int cap, double* __restrict__ A) {
  for (size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x; id < N; id += (size_t)gridDim.x * blockDim.x) {
    const int s = pos[id];
    const bool f = flag[id] != 0 && s < cap;
    for (int c = 0; c < 3; ++c) A[(size_t)c * N + id] = f ? qnew[(size_t)c * cap + s] : 0.0;
  }
}

// Euler transpose: xbar = xbar', qbar = qbar', upbar = dt xbar', gpbar = -dt qbar'.
__global__ void k_euler_T(const int* __restrict__ np_dev, int cap, double dt, const double* __restrict__ xb1,
                          const double* __restrict__ qb1, double* __restrict__ xbar, double* __restrict__ qbar,
                          double* __restrict__ upbar, double* __restrict__ gpbar) {
  const int np = *np_dev;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) {
      const size_t i = (size_t)d * cap + p;
      xbar[i] = xb1[i];
      qbar[i] = qb1[i];
      upbar[i] = dt * xb1[i];
      gpbar[i] = -dt * qb1[i];
    }
}

// Probe velocities u(probe) = sum_n W(probe, n) u(n) (probes component-major).
__global__ void k_probe_u(MeshDev m, int np, const double* __restrict__ pr, const double* __restrict__ u, size_t N,
                          double* __restrict__ up) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    Stencil S;
    double a[3] = {0, 0, 0};
    if (stencil(m, pr[p], pr[np + p], pr[2 * (size_t)np + p], S))
      for (int c = 0; c < 4; ++c)
        for (int b = 0; b < 4; ++b)
          for (int aa = 0; aa < 4; ++aa) {
            const size_t id = node_id(m, S, aa, b, c);
            const double f = S.w[0][aa] * S.w[1][b] * S.w[2][c];
            for (int d = 0; d < 3; ++d) a[d] += f * u[d * N + id];
          }
    for (int d = 0; d < 3; ++d) up[(size_t)d * np + p] = a[d];
  }
}
// ubar(n) += 2 W(probe, n) u(probe)
__global__ void k_probe_scatter_T(MeshDev m, int np, const double* __restrict__ pr, const double* __restrict__ up,
                                  size_t N, double* __restrict__ ubar) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    Stencil S;
    if (!stencil(m, pr[p], pr[np + p], pr[2 * (size_t)np + p], S)) continue;
    for (int c = 0; c < 4; ++c)
      for (int b = 0; b < 4; ++b)
        for (int aa = 0; aa < 4; ++aa) {
          const size_t id = node_id(m, S, aa, b, c);
          const double f = 2.0 * S.w[0][aa] * S.w[1][b] * S.w[2][c];
          for (int d = 0; d < 3; ++d) atomicAdd(&ubar[d * N + id], f * up[(size_t)d * np + p]);
        }
  }
}
// Sum of squares, per block (fixed reduction shape: deterministic).
constexpr int kSumBlocks = 512;
__global__ void k_sumsq(const double* __restrict__ v, size_t n, double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    s += v[i] * v[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Checkpoint copies of the particle arrays (dir 0: particles -> checkpoint
// *kidx, 1: back); the index is read on the device so that one captured
// backward step serves every step.
__global__ void k_copy_particles(int dir, const int* __restrict__ kidx, const int* __restrict__ np_live,
                                 const int* __restrict__ ckpt_np, int cap, double* x, double* y, double* z, double* q0,
                                 double* q1, double* q2, double* vol, double* __restrict__ ckpt) {
  const int k = *kidx;
  const int n = dir == 0 ? *np_live : ckpt_np[k];
  double* ck = ckpt + (size_t)k * 7 * cap;
  double* arr[7] = {x, y, z, q0, q1, q2, vol};
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    for (int a = 0; a < 7; ++a) {
      if (dir == 0) ck[(size_t)a * cap + p] = arr[a][p];
      else arr[a][p] = ck[(size_t)a * cap + p];
    }
}
// The count moves after the copy, whose blocks all read it.
__global__ void k_copy_count(int dir, const int* __restrict__ kidx, int* __restrict__ np_live, int* __restrict__ ckpt_np) {
  const int k = *kidx;
  if (dir == 0) ckpt_np[k] = *np_live;
  else *np_live = ckpt_np[k];
}
__global__ void k_set_index(int* __restrict__ kidx, int v) { *kidx = v; }
__global__ void k_step_back(int* __restrict__ kidx) { *kidx -= 1; }

// Three component arrays (cap apart) -> AoS (3, n).
__global__ void k_to_aos(const int* __restrict__ np_dev, const double* __restrict__ v, int cap, double* __restrict__ o) {
  const int n = *np_dev;
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) o[3 * (size_t)p + d] = v[(size_t)d * cap + p];
}

// AoS (3, n) -> three component arrays (cap apart).
__global__ void k_from_aos(int n, const double* __restrict__ o, int cap, double* __restrict__ v) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    for (int d = 0; d < 3; ++d) v[(size_t)d * cap + p] = o[3 * (size_t)p + d];
}

unsigned grid(size_t n, int t = 256) { return (unsigned)std::max<size_t>(1, std::min<size_t>((n + t - 1) / t, 152 * 16)); }

// ----------------------------------------------------------- L^T ---------
// Transposed Dirichlet solve with the box faces of the output as boundary
// values (dirichlet_solve with zero_bc = false).  ubar: adjoint of the
// output, zero outside the box.  rhsbar += A^-1 ubar (interior; the 7-point
// Laplacian is symmetric), bbar <- adjoint of the boundary values (box faces,
// zero elsewhere).  fbar: scratch of the array's size.
void dirichlet_T(vpmg_handle* h, DirichletPlan& dp, const double* ubar, double* rhsbar, double* bbar, double* fbar,
                 size_t n) {
  cudaStream_t st = h->stream;
  k_zero<<<grid(n), 256, 0, st>>>(fbar, n);
  VPMG_LAUNCHED();
  dirichlet_solve(dp, ubar, fbar, true, h->work.p, st);
  k_axpy<<<grid(n), 256, 0, st>>>(rhsbar, fbar, 1.0, n);
  k_zero<<<grid(n), 256, 0, st>>>(bbar, n);
  k_face_bc_T<<<grid((size_t)(dp.m[0] + 2) * (dp.m[1] + 2) * (dp.m[2] + 2)), 256, 0, st>>>(
      ubar, fbar, dp.dims[0], dp.dims[1], dp.box[0], dp.box[1], dp.box[2], dp.box[3], dp.box[4], dp.box[5],
      1.0 / (dp.h[0] * dp.h[0]), 1.0 / (dp.h[1] * dp.h[1]), 1.0 / (dp.h[2] * dp.h[2]), bbar);
  count_launch(3);
  VPMG_CUDA(cudaGetLastError());
}

// Transposed infinite-domain solve of one component (pmesh, iynbc = 1):
// sol = D2(rhs, bc),  bc = -(1/4pi) T agg N D0(rhs).  rhsbar += ...
void infinite_domain_T(vpmg_handle* h, DirichletPlan& dp, BoundaryOp& bo, const Grid& g, const double* solbar,
                       double* rhsbar, double* A, double* B, double* C) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const size_t n = g.count();
  dirichlet_T(h, dp, solbar, rhsbar, A, B, n);  // A = boundary-value adjoint
  boundary_apply_T(bo, A, S.cellbar.p, st);
  boundary_agg_T(bo, S.cellbar.p, S.panelbar.p, st);
  k_zero<<<grid(n), 256, 0, st>>>(C, n);
  VPMG_LAUNCHED();
  boundary_panels_T(bo, g, S.panelbar.p, C, st);   // C = adjoint of the zero-BC solution
  dirichlet_solve(dp, C, B, true, h->work.p, st);  // D0^T (interior of B; B spans the whole box)
  k_axpy<<<grid(n), 256, 0, st>>>(rhsbar, B, 1.0, n);
  VPMG_LAUNCHED();
}

// rbar (3 global components) += L^T psibar.
void poisson_T(vpmg_handle* h, const double* psibar, double* rbar) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  const size_t N = h->gglob.count(), NB = h->gbl.count(), NC = h->gco.count();
  const int go[3] = {s.nn_bl[0] - 1, s.nn_bl[1] - 1, s.nn_bl[2] - 1};
  const YapsDev& Y = h->yaps;
  const int lo[3] = {Y.map[0], Y.map[1], Y.map[2]};
  const int e[3] = {Y.map[3] - Y.map[0] - 1, Y.map[4] - Y.map[1] - 1, Y.map[5] - Y.map[2] - 1};
  for (int c = 0; c < 3; ++c) {
    double* ubl = S.blA.p;  // adjoint of the block solution
    double* rbl = S.rhsbarbl.p;
    fill_zero(ubl, NB, st);
    fill_zero(rbl, NB, st);
    // solget^T
    box_copy(psibar + (size_t)c * N, s.nn, go, ubl, s.nnbl, h->inner_lo, h->inner_ext, st);
    // final solve on the inner box: rhs part -> rbl, face values -> blB
    dirichlet_T(h, h->dp_inner, ubl, rbl, S.blB.p, S.blC.p, NB);
    // face interpolation: the faces kept their values and received the coarse correction
    fill_zero(S.csolbar.p, NC, st);
    fill_zero(S.sampbar.p, NC, st);
    k_face_interp_T<<<grid(Y.nface, 128), 128, 0, st>>>(Y.face_node.p, Y.face_cbase.p, Y.face_w.p, Y.face_flag.p,
                                                         Y.nface, s.nn_coarse[0], s.nn_coarse[1], S.blB.p,
                                                         S.csolbar.p, S.sampbar.p);
    VPMG_LAUNCHED();
    VPMG_CUDA(cudaMemcpyAsync(ubl, S.blB.p, sizeof(double) * NB, cudaMemcpyDeviceToDevice, st));
    // coarse infinite-domain solve, then the coarse Laplacian of the samples
    fill_zero(S.crhsbar.p, NC, st);
    infinite_domain_T(h, h->dp_c, h->bo_c, h->gco, S.csolbar.p, S.crhsbar.p, S.cA.p, S.cB.p, S.cC.p);
    if (e[0] > 0 && e[1] > 0 && e[2] > 0) {
      k_coarse_lap_T<<<grid(NC), 256, 0, st>>>(S.crhsbar.p, S.sampbar.p, s.nn_coarse[0], s.nn_coarse[1],
                                               s.nn_coarse[2], lo[0], lo[1], lo[2], e[0], e[1], e[2],
                                               1.0 / (s.dpm_coarse[0] * s.dpm_coarse[0]),
                                               1.0 / (s.dpm_coarse[1] * s.dpm_coarse[1]),
                                               1.0 / (s.dpm_coarse[2] * s.dpm_coarse[2]));
      VPMG_LAUNCHED();
    }
    // sampling of the fine block solution
    k_sample_T<<<grid(Y.nsamp), 256, 0, st>>>(Y.samp_src.p, Y.samp_dst.p, Y.nsamp, S.sampbar.p, ubl);
    VPMG_LAUNCHED();
    // fine infinite-domain solve on the padded block
    infinite_domain_T(h, h->dp_bl, h->bo_bl, h->gbl, ubl, rbl, S.blB.p, S.blC.p, S.blD.p);
    // rhsscat^T: the block RHS holds the global RHS on the inner box
    k_box_add<<<grid((size_t)h->inner_ext[0] * h->inner_ext[1] * h->inner_ext[2]), 256, 0, st>>>(
        rbl, s.nnbl[0], s.nnbl[1], h->inner_lo[0], h->inner_lo[1], h->inner_lo[2], rbar + (size_t)c * N, s.nn[0],
        s.nn[1], go[0], go[1], go[2], h->inner_ext[0], h->inner_ext[1], h->inner_ext[2]);
    VPMG_LAUNCHED();
    VPMG_CUDA(cudaGetLastError());
  }
}

// ------------------------------------------------------------ steps ------
void set_index(vpmg_handle* h, int k) {
  k_set_index<<<1, 1, 0, h->stream>>>(h->adj->kidx.p, k);
  VPMG_LAUNCHED();
}
// Copy between the particles and checkpoint *kidx (set_index).
void copy_ckpt(vpmg_handle* h, int dir) {
  AdjointState& S = *h->adj;
  Particles& P = h->parts;
  k_copy_particles<<<grid(S.cap), 256, 0, h->stream>>>(dir, S.kidx.p, P.d_np.p, S.ckpt_np.p, S.cap, P.x.p, P.y.p, P.z.p,
                                                      P.q0.p, P.q1.p, P.q2.p, P.vol.p, S.ckpt.p);
  k_copy_count<<<1, 1, 0, h->stream>>>(dir, S.kidx.p, P.d_np.p, S.ckpt_np.p);
  count_launch(2);
}

void ensure_state(vpmg_handle* h, int K, int nprobe) {
  VPMG_CHECK(h->nblk == 1, VPMG_ERR_UNSUPPORTED, "the reverse mode runs one YAPS block (NBI = NBJ = NBK = 1)");
  if (!h->adj) h->adj = new AdjointState();
  AdjointState& S = *h->adj;
  const size_t N = h->gglob.count(), NB = h->gbl.count(), NC = h->gco.count();
  S.cap = h->parts.capacity;
  S.ckpt.ensure((size_t)(K + 1) * 7 * S.cap);
  S.ckpt_np.ensure(K + 1);
  S.xq1.ensure(6 * (size_t)S.cap);
  S.pbar.ensure(21 * (size_t)S.cap);
  for (DBuf<double>* b : {&S.rbar, &S.psibar, &S.ubar, &S.gbar, &S.nodeA}) b->ensure(3 * N);
  for (DBuf<double>* b : {&S.blA, &S.blB, &S.blC, &S.blD, &S.rhsbarbl}) b->ensure(NB);
  for (DBuf<double>* b : {&S.cA, &S.cB, &S.cC, &S.sampbar, &S.crhsbar, &S.csolbar}) b->ensure(NC);
  S.cellbar.ensure(std::max(h->bo_bl.ncell_total, h->bo_c.ncell_total));
  S.panelbar.ensure(std::max(h->bo_bl.nbound, h->bo_c.nbound));
  S.probes.ensure(3 * (size_t)std::max(nprobe, 1));
  S.uprobe.ensure(3 * (size_t)std::max(nprobe, 1));
  S.lossv.ensure(2 * kSumBlocks);
  S.out.ensure(3 * (size_t)S.cap);
  S.kidx.ensure(1);
  S.nprobe = nprobe;
  boundary_transpose_prepare(h->bo_bl, h->stream);
  boundary_transpose_prepare(h->bo_c, h->stream);
}

// Probe stencils must stay on the mesh (checked on the host, as the kernels do).
void check_probes(const vpmg_handle* h, const double* pr, int n) {
  const Grid& g = h->gglob;
  for (int p = 0; p < n; ++p)
    for (int d = 0; d < 3; ++d) {
      const double x = pr[3 * (size_t)p + d];
      VPMG_CHECK(std::isfinite(x) && x - g.xmin[d] >= 0.0, VPMG_ERR_ARG, "a probe lies outside the mesh");
      const int c = (int)((x - g.xmin[d]) / g.d[d]);
      VPMG_CHECK(c - 1 >= 0 && c + 2 < g.n[d], VPMG_ERR_ARG, "a probe's M4' stencil leaves the mesh");
    }
}

// Bin the current particles on the global mesh and solve their fields.
void forward_fields(vpmg_handle* h) {
  bin_particles(h->parts, hx::mesh_dev(h->gglob, h->cfg.interf_iproj), h->bins, h->stream);
  hx::field_step(h);
}

// loss = sum_probes |u(probe)|^2 + ke * 0.5 DV sum_nodes |u|^2 of the current velocity field.
double field_loss(vpmg_handle* h, double ke) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const size_t N = h->gglob.count();
  const MeshDev mg = hx::mesh_dev(h->gglob, 4);
  const double dv = h->gglob.d[0] * h->gglob.d[1] * h->gglob.d[2];
  if (S.nprobe > 0) {
    k_probe_u<<<grid(S.nprobe, 128), 128, 0, st>>>(mg, S.nprobe, S.probes.p, h->vel.p, N, S.uprobe.p);
    VPMG_LAUNCHED();
  }
  k_sumsq<<<kSumBlocks, 256, 0, st>>>(S.uprobe.p, 3 * (size_t)S.nprobe, S.lossv.p);
  k_sumsq<<<kSumBlocks, 256, 0, st>>>(h->vel.p, 3 * N, S.lossv.p + kSumBlocks);
  count_launch(2);
  std::vector<double> part(2 * kSumBlocks);
  VPMG_CUDA(cudaMemcpyAsync(part.data(), S.lossv.p, sizeof(double) * part.size(), cudaMemcpyDeviceToHost, st));
  VPMG_CUDA(cudaStreamSynchronize(st));
  double a = 0, b = 0;
  for (int i = 0; i < kSumBlocks; ++i) {
    a += part[i];
    b += part[kSumBlocks + i];
  }
  return a + ke * 0.5 * dv * b;
}

// ubar <- d loss / d u of the current field (after field_loss).
void seed_loss(vpmg_handle* h, double ke) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const size_t N = h->gglob.count();
  const double dv = h->gglob.d[0] * h->gglob.d[1] * h->gglob.d[2];
  fill_zero(S.ubar.p, 3 * N, st);
  k_axpy<<<grid(3 * N), 256, 0, st>>>(S.ubar.p, h->vel.p, ke * dv, 3 * N);
  VPMG_LAUNCHED();
  if (S.nprobe > 0) {
    k_probe_scatter_T<<<grid(S.nprobe, 128), 128, 0, st>>>(hx::mesh_dev(h->gglob, 4), S.nprobe, S.probes.p,
                                                            S.uprobe.p, N, S.ubar.p);
    VPMG_LAUNCHED();
  }
}

// Field chain transposed, from ubar (and gbar when with_stretch) to the
// current particles: xbar, qbar += ...  Needs h->rhs and h->vel of the
// current particles.  Consumes ubar.
void fields_T(vpmg_handle* h, bool with_stretch, double* xbar, double* qbar) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  const size_t N = h->gglob.count();
  const double i2x = 1.0 / (2 * s.dpm[0]), i2y = 1.0 / (2 * s.dpm[1]), i2z = 1.0 / (2 * s.dpm[2]);
  fill_zero(S.rbar.p, 3 * N, st);
  if (with_stretch) {
    k_stretch_T<<<grid(N), 256, 0, st>>>(S.gbar.p, h->rhs.p, h->vel.p, s.nn[0], s.nn[1], s.nn[2], i2x, i2y, i2z,
                                         S.rbar.p, S.ubar.p);
    VPMG_LAUNCHED();
  }
  k_curl_T<<<grid(N), 256, 0, st>>>(S.ubar.p, s.nn[0], s.nn[1], s.nn[2], i2x, i2y, i2z, S.psibar.p);
  VPMG_LAUNCHED();
  poisson_T(h, S.psibar.p, S.rbar.p);
  // deposition^T:  qbar += W rbar / DV,  xbar += grad W (Q . rbar) / DV
  const MeshDev mg = hx::mesh_dev(h->gglob, 4);
  const double dv = mg.d[0] * mg.d[1] * mg.d[2];
  Particles& P = h->parts;
  const Vec3 q{{P.q0.p, P.q1.p, P.q2.p}}, none{{nullptr, nullptr, nullptr}};
  k_particle_adj<<<grid(S.cap, 128), 128, 0, st>>>(mg, P.d_np.p, P.x.p, P.y.p, P.z.p, S.rbar.p, nullptr, N, q, none,
                                                    nullptr, 1.0 / dv, 0.0, qbar, xbar, S.cap);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

// Vector-Jacobian product of the field step (vpm WhatToDo = 2) on the
// handle's particles, which must be binned on the global mesh with their
// fields solved (h->rhs, h->vel, h->def):
//   UP = I(X) u,  GP = vol I(X) g,  u = C L D(X) Q / DV,  g = S(D(X) Q / DV, u)
// xb, qb += (d(UP, GP) / d(X, Q))^T (upb, gpb); all particle arrays 3 x cap.
void fields_vjp(vpmg_handle* h, const double* upb, const double* gpb, double* xb, double* qb) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const int cap = S.cap;
  const size_t N = h->gglob.count();
  Particles& P = h->parts;
  const MeshDev mg = hx::mesh_dev(h->gglob, 4);
  const double dvg = mg.d[0] * mg.d[1] * mg.d[2];
  fill_zero(S.ubar.p, 3 * N, st);
  fill_zero(S.gbar.p, 3 * N, st);
  double* U[3] = {S.ubar.p, S.ubar.p + N, S.ubar.p + 2 * N};
  double* G[3] = {S.gbar.p, S.gbar.p + N, S.gbar.p + 2 * N};
  // M2P^T: ubar = sum_p W upbar_p,  gbar = sum_p W vol_p gpbar_p  (the deposit divides by DV)
  const int rff = P.arith == VPMG_ARITH_FF48 ? 1 : 0;
  k_records_set_q<<<grid(cap), 256, 0, st>>>(P.rec.p, rff, P.rec_stride(), P.perm.p, h->bins.nsorted_dev, upb, cap,
                                             dvg, nullptr);
  VPMG_LAUNCHED();
  deposit(P, mg, h->bins, U, st);
  k_records_set_q<<<grid(cap), 256, 0, st>>>(P.rec.p, rff, P.rec_stride(), P.perm.p, h->bins.nsorted_dev, gpb, cap,
                                             dvg, P.vol.p);
  VPMG_LAUNCHED();
  deposit(P, mg, h->bins, G, st);
  // positions through the M2P weights
  const Vec3 a{{upb, upb + cap, upb + 2 * (size_t)cap}}, b{{gpb, gpb + cap, gpb + 2 * (size_t)cap}};
  k_particle_adj<<<grid(cap, 128), 128, 0, st>>>(mg, P.d_np.p, P.x.p, P.y.p, P.z.p, h->vel.p, h->def.p, N, a, b,
                                                  P.vol.p, 1.0, 1.0, nullptr, xb, cap);
  VPMG_LAUNCHED();
  // stretching, curl, Poisson, deposition
  fields_T(h, true, xb, qb);
}

// Vector-Jacobian product of remesh_particles_3d(1) on the handle's
// particles (any positions): Q''(slot(n)) = DV_r R_r(n) on the flagged
// nodes, R_r = D_r(X) Q / DV_r.  qnew: adjoint of the emitted strengths
// (3 x cap, slot order); xb, qb <- d/d(X, Q).  Leaves the emission mask in
// the binning (cursor = flag, starts = slot).
void remesh_vjp(vpmg_handle* h, const double* qnew, double* xb, double* qb) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const int cap = S.cap;
  const size_t N = h->gglob.count();
  Particles& P = h->parts;
  const Grid gr = hx::remesh_grid(h);
  const MeshDev mr = hx::mesh_dev(gr, 4);
  bin_particles(P, mr, h->bins, st);
  double* RR[3] = {S.nodeA.p, S.nodeA.p + N, S.nodeA.p + 2 * N};
  deposit(P, mr, h->bins, RR, st);
  const vpmg_sizes& s = h->sz;
  const int hh = h->cfg.interf_iproj / 2;
  const int lo[3] = {s.nn_bl[0] - 1 + hh, s.nn_bl[1] - 1 + hh, s.nn_bl[2] - 1 + hh};
  const int hi[3] = {s.nn_bl[3] - 1 - hh, s.nn_bl[4] - 1 - hh, s.nn_bl[5] - 1 - hh};
  remesh_mask(mr, h->bins, RR, lo, hi, (double)1e-09f, st);
  // A(n) = qnew[slot(n)] on the mask; qbar = W A, xbar = grad W (Q . A)
  k_mask_field<<<grid(N), 256, 0, st>>>(h->bins.cursor.p, h->bins.starts.p, N, qnew, cap, S.nodeA.p);
  VPMG_LAUNCHED();
  fill_zero(xb, 3 * (size_t)cap, st);
  fill_zero(qb, 3 * (size_t)cap, st);
  const Vec3 q{{P.q0.p, P.q1.p, P.q2.p}}, none{{nullptr, nullptr, nullptr}};
  k_particle_adj<<<grid(cap, 128), 128, 0, st>>>(mr, P.d_np.p, P.x.p, P.y.p, P.z.p, S.nodeA.p, nullptr, N, q, none,
                                                  nullptr, 1.0, 0.0, qb, xb, cap);
  VPMG_LAUNCHED();
}

// Adjoint of step k = *kidx (particles X_k, Q_k from checkpoint k): on
// entry qnew = d loss / d Q_{k+1}; on exit qnew = d loss / d Q_k,
// xb = d loss / d X_k, and *kidx = k - 1.  Stream work only (capturable).
void backward_step(vpmg_handle* h, double dt) {
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  const int cap = S.cap;
  const size_t N = h->gglob.count();
  Particles& P = h->parts;
  double* xb = S.pbar.p;
  double* qb = S.pbar.p + 3 * (size_t)cap;
  double* upb = S.pbar.p + 6 * (size_t)cap;
  double* gpb = S.pbar.p + 9 * (size_t)cap;
  double* qnew = S.pbar.p + 12 * (size_t)cap;
  double* xb1 = S.pbar.p + 15 * (size_t)cap;
  double* qb1 = S.pbar.p + 18 * (size_t)cap;
  const MeshDev mg = hx::mesh_dev(h->gglob, 4);
  // 1. recompute: fields at X_k, UP and GP, the pushed state X', Q'
  copy_ckpt(h, 1);
  forward_fields(h);
  {
    const double u0[3] = {0.0, 0.0, 0.0};
    hx::m2p_fields(h, kUpSet, false, dt, u0);
  }
  k_after_euler<<<grid(cap), 256, 0, st>>>(P.d_np.p, P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p, P.up.p, P.gp.p, dt,
                                          S.xq1.p, cap);
  k_load_pushed<<<grid(cap), 256, 0, st>>>(P.d_np.p, S.xq1.p, cap, P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p);
  count_launch(2);
  // 2. remesh^T at X', Q' (the step's own mask)
  remesh_vjp(h, qnew, xb1, qb1);
  // 3. Euler^T
  k_euler_T<<<grid(cap), 256, 0, st>>>(P.d_np.p, cap, dt, xb1, qb1, xb, qb, upb, gpb);
  VPMG_LAUNCHED();
  // 4. back at X_k (the fields are still those of X_k): the field step's VJP
  copy_ckpt(h, 1);
  bin_particles(P, mg, h->bins, st);
  VPMG_CUDA(cudaMemcpyAsync(qnew, qb, sizeof(double) * 3 * cap, cudaMemcpyDeviceToDevice, st));
  fields_vjp(h, upb, gpb, xb, qnew);
  k_step_back<<<1, 1, 0, st>>>(S.kidx.p);
  VPMG_LAUNCHED();
}

// The backward step as a CUDA graph (re-captured when dt or a buffer moves).
void ensure_backward_graph(vpmg_handle* h, double dt) {
  AdjointState& S = *h->adj;
  const void* key[3] = {S.ckpt.p, S.pbar.p, h->parts.x.p};
  if (S.bwd && S.bwd_dt == dt && key[0] == S.bwd_key[0] && key[1] == S.bwd_key[1] && key[2] == S.bwd_key[2]) return;
  if (S.bwd) {
    cudaGraphExecDestroy(S.bwd);
    S.bwd = nullptr;
  }
  const long long l0 = h->launches;
  cudaGraph_t g = nullptr;
  VPMG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  try {
    backward_step(h, dt);
  } catch (...) {
    cudaStreamEndCapture(h->stream, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    h->launches = l0;
    throw;
  }
  VPMG_CUDA(cudaStreamEndCapture(h->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&S.bwd, g, 0);
  cudaGraphDestroy(g);
  VPMG_CUDA(e);
  S.bwd_launches = h->launches - l0;
  h->launches = l0;
  S.bwd_dt = dt;
  for (int i = 0; i < 3; ++i) S.bwd_key[i] = key[i];
}

// One step with the remesh's |w| cut replaced by a recorded node mask.
void step_masked(vpmg_handle* h, double dt, const int* mask) {
  cudaStream_t st = h->stream;
  const size_t N = h->gglob.count();
  Particles& P = h->parts;
  forward_fields(h);
  const double u0[3] = {0.0, 0.0, 0.0};
  hx::m2p_fields(h, kUpSet, true, dt, u0);
  const Grid gr = hx::remesh_grid(h);
  const MeshDev mr = hx::mesh_dev(gr, 4);
  bin_particles(P, mr, h->bins, st);
  double* R[3] = {h->rhs.p, h->rhs.p + N, h->rhs.p + 2 * N};
  deposit(P, mr, h->bins, R, st);
  remesh_emit_masked(P, mr, h->bins, R, mask, st);
}

// mask_mode 0: the reference's |w| cut; 1: the cut, recording each step's
// mask; 2: the masks recorded by the last mode-1 run (the fixed-mask map).
void forward_pass(vpmg_handle* h, int nsteps, double dt, int mask_mode) {
  AdjointState& S = *h->adj;
  const size_t N = h->gglob.count();
  for (int k = 0; k < nsteps; ++k) {
    set_index(h, k);
    copy_ckpt(h, 0);
    if (mask_mode == 2) {
      step_masked(h, dt, S.masks.p + (size_t)k * N);
    } else {
      hx::step_on_stream(h, dt);
      if (mask_mode == 1)  // the step's flags stay in the binning's cursor
        VPMG_CUDA(cudaMemcpyAsync(S.masks.p + (size_t)k * N, h->bins.cursor.p, sizeof(int) * N,
                                  cudaMemcpyDeviceToDevice, h->stream));
    }
  }
  set_index(h, nsteps);
  copy_ckpt(h, 0);
  forward_fields(h);
}

struct Timer {
  cudaEvent_t e[3] = {nullptr, nullptr, nullptr};
  Timer() {
    for (auto& x : e) VPMG_CUDA(cudaEventCreate(&x));
  }
  ~Timer() {
    for (auto& x : e)
      if (x) cudaEventDestroy(x);
  }
};

// Shared by the loss-only and the gradient entry points.
double adjoint_common(vpmg_handle* h, int nsteps, double dt, const double* probes, int nprobe, double ke,
                      bool backward, int mask_mode, double* xbar, double* qbar, double* ms_fwd, double* ms_bwd) {
  VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
  VPMG_CHECK(mask_mode >= 0 && mask_mode <= 2, VPMG_ERR_ARG, "mask_mode must be 0, 1 or 2");
  VPMG_CHECK(mask_mode != 2 || (h->adj && h->adj->masks_steps >= nsteps), VPMG_ERR_STATE,
             "no recorded remesh masks for that many steps (run vpmg_adjoint_run first)");
  VPMG_CHECK(h->cfg.interf_iproj == 4, VPMG_ERR_UNSUPPORTED, "the adjoint is written for the M4' kernel");
  VPMG_CHECK(nsteps >= 0 && nprobe >= 0 && (nprobe == 0 || probes), VPMG_ERR_ARG, "bad sizes");
  VPMG_CHECK(!h->keep_intermediates, VPMG_ERR_STATE, "the adjoint runs with profiling level < 2");
  check_probes(h, probes, nprobe);
  hx::sync_np(h);
  const int np0 = h->np;
  ensure_state(h, nsteps, nprobe);
  AdjointState& S = *h->adj;
  cudaStream_t st = h->stream;
  if (mask_mode == 1) {
    S.masks.ensure(std::max<size_t>((size_t)nsteps * h->gglob.count(), 1));
    S.masks_steps = -1;
  }
  if (nprobe > 0) {  // AoS (3, nprobe) -> component-major
    std::vector<double> pc(3 * (size_t)nprobe);
    for (int p = 0; p < nprobe; ++p)
      for (int d = 0; d < 3; ++d) pc[(size_t)d * nprobe + p] = probes[3 * (size_t)p + d];
    VPMG_CUDA(cudaMemcpyAsync(S.probes.p, pc.data(), sizeof(double) * pc.size(), cudaMemcpyHostToDevice, st));
    VPMG_CUDA(cudaStreamSynchronize(st));
  }
  const bool prof = h->profile;
  h->profile = false;
  Timer T;
  double L = 0.0;
  try {
    VPMG_CUDA(cudaEventRecord(T.e[0], st));
    forward_pass(h, nsteps, dt, mask_mode);
    L = field_loss(h, ke);
    if (mask_mode == 1) S.masks_steps = nsteps;
    VPMG_CUDA(cudaEventRecord(T.e[1], st));
    if (backward) {
      const int cap = S.cap;
      seed_loss(h, ke);
      fill_zero(S.pbar.p, 3 * (size_t)cap, st);                 // xbar
      fill_zero(S.pbar.p + 12 * (size_t)cap, 3 * (size_t)cap, st);  // qnew
      fields_T(h, false, S.pbar.p, S.pbar.p + 12 * (size_t)cap);
      if (nsteps > 0) {
        const bool graphs = !h->no_graphs;
        if (graphs) ensure_backward_graph(h, dt);
        set_index(h, nsteps - 1);
        for (int k = nsteps - 1; k >= 0; --k) {
          if (graphs) {
            VPMG_CUDA(cudaGraphLaunch(S.bwd, st));
            h->launches += S.bwd_launches;
          } else {
            backward_step(h, dt);
          }
        }
      }
    }
    VPMG_CUDA(cudaEventRecord(T.e[2], st));
    VPMG_CUDA(cudaEventSynchronize(T.e[2]));
    // leave the handle holding the initial particles
    set_index(h, 0);
    copy_ckpt(h, 1);
    hx::sync_np(h);
  } catch (...) {
    h->profile = prof;
    throw;
  }
  h->profile = prof;
  float tf = 0.f, tb = 0.f;
  VPMG_CUDA(cudaEventElapsedTime(&tf, T.e[0], T.e[1]));
  VPMG_CUDA(cudaEventElapsedTime(&tb, T.e[1], T.e[2]));
  if (ms_fwd) *ms_fwd = tf;
  if (ms_bwd) *ms_bwd = tb;
  if (backward && np0 > 0) {
    const int cap = S.cap;
    for (int w = 0; w < 2; ++w) {
      double* dst = w == 0 ? xbar : qbar;
      if (!dst) continue;
      const double* src = w == 0 ? S.pbar.p : S.pbar.p + 12 * (size_t)cap;
      k_to_aos<<<grid(cap), 256, 0, st>>>(h->parts.d_np.p, src, cap, S.out.p);
      VPMG_LAUNCHED();
      VPMG_CUDA(cudaMemcpyAsync(dst, S.out.p, sizeof(double) * 3 * (size_t)np0, cudaMemcpyDeviceToHost, st));
      VPMG_CUDA(cudaStreamSynchronize(st));
    }
  }
  return L;
}

// Host (3, n) AoS -> 3 x cap device components (through S.out).
void upload_vec3(vpmg_handle* h, const double* src, int n, double* dst) {
  AdjointState& S = *h->adj;
  fill_zero(dst, 3 * (size_t)S.cap, h->stream);
  if (n <= 0) return;
  VPMG_CUDA(cudaMemcpyAsync(S.out.p, src, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, h->stream));
  k_from_aos<<<grid(n), 256, 0, h->stream>>>(n, S.out.p, S.cap, dst);
  VPMG_LAUNCHED();
}
void download_vec3(vpmg_handle* h, const double* src, int n, double* dst) {
  AdjointState& S = *h->adj;
  if (!dst || n <= 0) return;
  k_to_aos<<<grid(n), 256, 0, h->stream>>>(h->parts.d_np.p, src, S.cap, S.out.p);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaMemcpyAsync(dst, S.out.p, sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
  VPMG_CUDA(cudaStreamSynchronize(h->stream));
}

}  // namespace

namespace hx {
void destroy_adjoint(vpmg_handle* h) {
  delete h->adj;
  h->adj = nullptr;
}
}  // namespace hx

}  // namespace vpmg

using namespace vpmg;

// ==================================================================== C ===
extern "C" {

int vpmg_apply_poisson(vpmg_handle* h, const double* r, double* psi) {
  return hx::guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
    VPMG_CHECK(r && psi, VPMG_ERR_ARG, "null array");
    const size_t N = h->gglob.count();
    VPMG_CUDA(cudaMemcpyAsync(h->rhs.p, r, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, h->stream));
    hx::poisson_part(h);
    VPMG_CUDA(cudaMemcpyAsync(psi, h->sol.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int vpmg_adjoint_poisson(vpmg_handle* h, const double* psibar, double* rbar) {
  return hx::guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
    VPMG_CHECK(psibar && rbar, VPMG_ERR_ARG, "null array");
    ensure_state(h, 0, 0);
    AdjointState& S = *h->adj;
    const size_t N = h->gglob.count();
    VPMG_CUDA(cudaMemcpyAsync(S.psibar.p, psibar, sizeof(double) * 3 * N, cudaMemcpyHostToDevice, h->stream));
    fill_zero(S.rbar.p, 3 * N, h->stream);
    poisson_T(h, S.psibar.p, S.rbar.p);
    VPMG_CUDA(cudaMemcpyAsync(rbar, S.rbar.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int vpmg_vjp_fields(vpmg_handle* h, const double* xp, const double* qp, int nvr, const double* upbar,
                    const double* gpbar, double* xbar, double* qbar) {
  return hx::guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
    VPMG_CHECK(h->cfg.interf_iproj == 4, VPMG_ERR_UNSUPPORTED, "the adjoint is written for the M4' kernel");
    VPMG_CHECK(xp && qp && upbar && gpbar && nvr >= 0, VPMG_ERR_ARG, "null array");
    ensure_state(h, 0, 0);
    AdjointState& S = *h->adj;
    const int cap = S.cap;
    hx::upload_particles(h, xp, qp, nvr);
    forward_fields(h);
    double* xb = S.pbar.p;
    double* qb = S.pbar.p + 3 * (size_t)cap;
    double* upb = S.pbar.p + 6 * (size_t)cap;
    double* gpb = S.pbar.p + 9 * (size_t)cap;
    upload_vec3(h, upbar, nvr, upb);
    upload_vec3(h, gpbar, nvr, gpb);
    fill_zero(xb, 3 * (size_t)cap, h->stream);
    fill_zero(qb, 3 * (size_t)cap, h->stream);
    fields_vjp(h, upb, gpb, xb, qb);
    hx::sync_np(h);
    download_vec3(h, xb, nvr, xbar);
    download_vec3(h, qb, nvr, qbar);
  });
}

int vpmg_vjp_remesh(vpmg_handle* h, const double* xp, const double* qp, int nvr, const double* qbar_new, int nnew,
                    double* xbar, double* qbar) {
  return hx::guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
    VPMG_CHECK(h->cfg.interf_iproj == 4, VPMG_ERR_UNSUPPORTED, "the adjoint is written for the M4' kernel");
    VPMG_CHECK(xp && qp && qbar_new && nvr >= 0 && nnew >= 0, VPMG_ERR_ARG, "null array");
    ensure_state(h, 0, 0);
    AdjointState& S = *h->adj;
    const int cap = S.cap;
    VPMG_CHECK(nnew <= cap, VPMG_ERR_CAPACITY, "more emitted particles than mesh nodes");
    hx::upload_particles(h, xp, qp, nvr);
    double* qnew = S.pbar.p + 12 * (size_t)cap;
    double* xb = S.pbar.p + 15 * (size_t)cap;
    double* qb = S.pbar.p + 18 * (size_t)cap;
    upload_vec3(h, qbar_new, nnew, qnew);
    remesh_vjp(h, qnew, xb, qb);
    hx::sync_np(h);
    // the emission count of this remesh must be the caller's
    const size_t N = h->gglob.count();
    const int nf = read_count(h->bins.starts.p + N - 1, h->stream), last = read_count(h->bins.cursor.p + N - 1, h->stream);
    VPMG_CHECK(nf + last == nnew, VPMG_ERR_ARG, "qbar_new must hold one row per particle the remesh emits");
    download_vec3(h, xb, nvr, xbar);
    download_vec3(h, qb, nvr, qbar);
  });
}

int vpmg_adjoint_loss(vpmg_handle* h, int nsteps, double dt, const double* probes, int nprobe, double ke_weight,
                      int mask_mode, double* loss) {
  return hx::guarded(h, [&] {
    const double L =
        adjoint_common(h, nsteps, dt, probes, nprobe, ke_weight, false, mask_mode, nullptr, nullptr, nullptr, nullptr);
    if (loss) *loss = L;
  });
}

int vpmg_adjoint_run(vpmg_handle* h, int nsteps, double dt, const double* probes, int nprobe, double ke_weight,
                     double* loss, double* xbar, double* qbar, double* ms_forward, double* ms_backward) {
  return hx::guarded(h, [&] {
    const double L =
        adjoint_common(h, nsteps, dt, probes, nprobe, ke_weight, true, 1, xbar, qbar, ms_forward, ms_backward);
    if (loss) *loss = L;
  });
}

}  // extern "C"
