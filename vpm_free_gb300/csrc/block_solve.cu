// block_solve.cu -- the padded YAPS block's infinite-domain solve, evaluated
// only where the reference's step reads it.
//
// yaps3d (source/yaps3d.f90:52-53 -> pmlib.f90:115-154) solves the padded
// block twice per component with the same right-hand side:
//   1. zero boundary values (solve_eq_0_3d, pmsolve.f90:367-432), of which
//      calc_normalderiv_3d (pinfdomain.f90:294-547) reads only the 4
//      interior layers next to each face;
//   2. the quadtree boundary values (solve_eq_3d, pmsolve.f90:284-365), of
//      which the step reads only the every-nc-th samples
//      (yaps3d.f90:104-138) and the six faces of the inner block box
//      (interp_stencil targets, yaps3d.f90:340-395; final-solve boundary).
// Both share the forward transform ghat = DST_y DST_x RHS: the boundary
// values of solve 2 enter in transform space as rank-structured face terms
// added inside the Thomas sweep.  The inverse transforms are evaluated only
// on the needed layers: dot products with the selected sine rows along one
// axis, then a full inverse DST along the other.  The values produced are
// those of the full discrete solves (same linear algebra, different
// rounding).
#include <algorithm>
#include <cmath>
#include <cstring>

#include "arith.cuh"
#include "block_solve.h"

namespace vpmg {

namespace {

constexpr int kLines = 16;  // lines per CTA of the x dot-product kernel

__device__ __forceinline__ double shfl_xor(double v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }
__device__ __forceinline__ float2 shfl_xor(float2 v, int m) {
  return make_float2(__shfl_xor_sync(0xffffffffu, v.x, m), __shfl_xor_sync(0xffffffffu, v.y, m));
}

// The dot products below run in the policy's arithmetic (arith.cuh): the
// sine rows are stored in it (doubles, or float-float pairs), W enters it
// as it is staged, and each result is joined back into a double.

// out[i + nsel*(q + m1*kk)] = sum_p S[i][p] * W[p + m0*(q + m1*k)],  k = klist ? klist[kk] : kk
// Persistent CTAs walk tiles of up to kLines lines; the sine rows are
// staged once per CTA.  In FP64 (dbl) the next tile is staged with
// asynchronous copies (cp.async, 8 bytes each) while the current one is
// reduced, so the loads' latency hides behind the FMAs.  Float-float
// staging converts each value as it lands, which cannot run ahead: one
// buffer, and the smaller footprint keeps more CTAs on an SM instead.
__device__ __forceinline__ void cp_async8(void* smem, const void* gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

template <class A>
__device__ __forceinline__ void stage_x_tile(typename A::R* tile, const double* __restrict__ W, int m0, int m1,
                                             int nlines, const int* __restrict__ klist, int l0, int lines) {
  for (int t = threadIdx.x; t < lines * m0; t += blockDim.x) {
    const int li = t / m0, p = t - li * m0;
    const int l = l0 + li;
    if (l < nlines) {
      const int q = l % m1, kk = l / m1;
      const int k = klist ? klist[kk] : kk;
      const double* src = W + (size_t)p + (size_t)m0 * (q + (size_t)m1 * k);
      if constexpr (A::kFF) tile[t] = A::from(*src);
      else cp_async8(&tile[t], src);
    } else {
      tile[t] = A::zero();
    }
  }
  if constexpr (!A::kFF) cp_async_commit();
}

template <class A>
__global__ void __launch_bounds__(128) k_partial_x(const double* __restrict__ W, int m0, int m1, int nk,
                                                   const int* __restrict__ klist, const typename A::R* __restrict__ S,
                                                   int nsel, double* __restrict__ out, int lines, int dbl) {
  using R = typename A::R;
  extern __shared__ double smx[];
  R* Ss = reinterpret_cast<R*>(smx);               // nsel x m0
  R* const buf0 = Ss + (size_t)nsel * m0;           // one or two (dbl) tiles of `lines` x m0 (lines <= kLines)
  R* const buf1 = buf0 + (size_t)lines * m0;
  const int nlines = m1 * nk;
  const int ntiles = (nlines + lines - 1) / lines;
  for (int t = threadIdx.x; t < nsel * m0; t += blockDim.x) Ss[t] = S[t];
  int cur = 0;
  if (dbl && (int)blockIdx.x < ntiles)
    stage_x_tile<A>(buf0, W, m0, m1, nlines, klist, blockIdx.x * lines, lines);
  // R adjacent threads share one dot product (R = 128 / outputs, a power of
  // two up to 8, when the CTA has fewer outputs than threads), each summing
  // every R-th term; their partials meet in a fixed shuffle tree.
  const int nout = lines * nsel;
  int Rs = 1;
  while (Rs < 8 && nout * Rs * 2 <= (int)blockDim.x) Rs *= 2;
  const int r = threadIdx.x % Rs;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int next = tile + gridDim.x;
    if (dbl) {
      if (next < ntiles) {
        stage_x_tile<A>(cur ? buf0 : buf1, W, m0, m1, nlines, klist, next * lines, lines);
        if constexpr (!A::kFF) cp_async_wait<1>();  // the current tile's copies are done
      } else {
        if constexpr (!A::kFF) cp_async_wait<0>();
      }
    } else {
      stage_x_tile<A>(buf0, W, m0, m1, nlines, klist, tile * lines, lines);
      if constexpr (!A::kFF) cp_async_wait<0>();
    }
    __syncthreads();
    const R* tl = cur ? buf1 : buf0;
    const int l0 = tile * lines;
    for (int o0 = 0; o0 < nout; o0 += blockDim.x / Rs) {
      const int o = o0 + threadIdx.x / Rs;
      const int li = o % lines, i = o / lines;
      const int l = l0 + li;
      const bool ok = o < nout && l < nlines;
      R a0 = A::zero(), a1 = a0, a2 = a0, a3 = a0;
      if (ok) {
        const R* a = tl + (size_t)li * m0;
        const R* b = Ss + (size_t)i * m0;
        int p = r;
        for (; p + 3 * Rs < m0; p += 4 * Rs) {
          a0 = A::fma(a[p], b[p], a0);
          a1 = A::fma(a[p + Rs], b[p + Rs], a1);
          a2 = A::fma(a[p + 2 * Rs], b[p + 2 * Rs], a2);
          a3 = A::fma(a[p + 3 * Rs], b[p + 3 * Rs], a3);
        }
        for (; p < m0; p += Rs) a0 = A::fma(a[p], b[p], a0);
      }
      R v = A::add(A::add(a0, a1), A::add(a2, a3));
      for (int m = 1; m < Rs; m <<= 1) {
        const R w = shfl_xor(v, m);
        v = (r & m) ? A::add(w, v) : A::add(v, w);
      }
      if (ok && r == 0) {
        const int q = l % m1, kk = l / m1;
        out[i + (size_t)nsel * (q + (size_t)m1 * kk)] = A::to(v);
      }
    }
    __syncthreads();  // the buffer is refilled next (one buffer) or two tiles on (dbl)
    if (dbl) cur ^= 1;
  }
}

// out[p + m0*(j + nsel*kk)] = sum_q S[j][q] * W[p + m0*(q + m1*k)]
// A CTA stages the m1 x 32 column tile (p0..p0+31, all q) of plane k in
// shared memory with coalesced row loads -- W is read from HBM once -- and
// its threads then form the nsel x 32 dot products from the tile.
constexpr int kColTile = 32;
// A second row set (S2, nsel2 -> out2, same layout) is served from the
// same staged tile when given, so two face sets cost one pass over W.
template <class A>
__device__ __forceinline__ void stage_y_tile(typename A::R* tile, const double* __restrict__ W, int m0, int m1,
                                             const int* __restrict__ klist, int p0, int kk) {
  const int k = klist ? klist[kk] : kk;
  const double* plane = W + (size_t)m0 * m1 * k;
  const int lane = threadIdx.x % kColTile, row = threadIdx.x / kColTile, rows = blockDim.x / kColTile;
  const int p = p0 + lane;
  for (int q = row; q < m1; q += rows) {
    if (p < m0) {
      if constexpr (A::kFF) tile[q * kColTile + lane] = A::from(plane[(size_t)m0 * q + p]);
      else cp_async8(&tile[q * kColTile + lane], plane + (size_t)m0 * q + p);
    } else {
      tile[q * kColTile + lane] = A::zero();
    }
  }
  if constexpr (!A::kFF) cp_async_commit();
}

// Persistent CTAs walk (column tile, plane) pairs; with dbl (FP64, when two
// tiles fit) the next pair's tile is staged asynchronously while the
// current one is reduced.
template <class A>
__global__ void __launch_bounds__(256) k_partial_y(const double* __restrict__ W, int m0, int m1, int nk,
                                                   const int* __restrict__ klist, const typename A::R* __restrict__ S,
                                                   int nsel, double* __restrict__ out,
                                                   const typename A::R* __restrict__ S2, int nsel2,
                                                   double* __restrict__ out2, int dbl) {
  using R = typename A::R;
  extern __shared__ double smy[];
  R* const buf0 = reinterpret_cast<R*>(smy);              // [q][lane], m1 x kColTile
  R* const buf1 = buf0 + (size_t)m1 * kColTile;             // the second tile (dbl)
  R* const partial = (dbl ? buf1 : buf0) + (size_t)m1 * kColTile;  // partial sums [row][lane]
  const int nbx = (m0 + kColTile - 1) / kColTile;
  const int ntiles = nbx * nk;
  const int lane = threadIdx.x % kColTile, row = threadIdx.x / kColTile, rows = blockDim.x / kColTile;
  // R rows share one output row set when there are fewer outputs than rows
  // (R a power of two), each summing every R-th q; the partials are added
  // in row order through shared memory.
  const int nout = nsel + nsel2;
  int Rs = 1;
  while (Rs < rows && nout * Rs * 2 <= rows) Rs *= 2;
  const int r = row % Rs;
  int cur = 0;
  if (dbl && (int)blockIdx.x < ntiles)
    stage_y_tile<A>(buf0, W, m0, m1, klist, ((int)blockIdx.x % nbx) * kColTile, (int)blockIdx.x / nbx);
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int p0 = (tile % nbx) * kColTile, kk = tile / nbx;
    const int next = tile + gridDim.x;
    if (dbl) {
      if (next < ntiles) {
        stage_y_tile<A>(cur ? buf0 : buf1, W, m0, m1, klist, (next % nbx) * kColTile, next / nbx);
        if constexpr (!A::kFF) cp_async_wait<1>();
      } else {
        if constexpr (!A::kFF) cp_async_wait<0>();
      }
    } else {
      stage_y_tile<A>(buf0, W, m0, m1, klist, p0, kk);
      if constexpr (!A::kFF) cp_async_wait<0>();
    }
    __syncthreads();
    const R* tl = cur ? buf1 : buf0;
    const int p = p0 + lane;
    for (int j0 = 0; j0 < nout; j0 += rows / Rs) {
      const int jj = j0 + row / Rs;
      R a0 = A::zero(), a1 = a0, a2 = a0, a3 = a0;
      if (jj < nout && p < m0) {
        const bool second = jj >= nsel;
        const int j = second ? jj - nsel : jj;
        const R* Sj = (second ? S2 : S) + (size_t)j * m1;
        int q = r;
        for (; q + 3 * Rs < m1; q += 4 * Rs) {
          a0 = A::fma(__ldg(&Sj[q]), tl[q * kColTile + lane], a0);
          a1 = A::fma(__ldg(&Sj[q + Rs]), tl[(q + Rs) * kColTile + lane], a1);
          a2 = A::fma(__ldg(&Sj[q + 2 * Rs]), tl[(q + 2 * Rs) * kColTile + lane], a2);
          a3 = A::fma(__ldg(&Sj[q + 3 * Rs]), tl[(q + 3 * Rs) * kColTile + lane], a3);
        }
        for (; q < m1; q += Rs) a0 = A::fma(__ldg(&Sj[q]), tl[q * kColTile + lane], a0);
      }
      R v = A::add(A::add(a0, a1), A::add(a2, a3));
      if (Rs > 1) {
        partial[row * kColTile + lane] = v;
        __syncthreads();
        if (r == 0)
          for (int m = 1; m < Rs; ++m) v = A::add(v, partial[(row + m) * kColTile + lane]);
        __syncthreads();
      }
      if (r == 0 && jj < nout && p < m0) {
        const bool second = jj >= nsel;
        const int j = second ? jj - nsel : jj;
        if (second) out2[(size_t)p + (size_t)m0 * (j + (size_t)nsel2 * kk)] = A::to(v);
        else out[(size_t)p + (size_t)m0 * (j + (size_t)nsel * kk)] = A::to(v);
      }
    }
    __syncthreads();  // the tile's buffer is refilled next
    if (dbl) cur ^= 1;
  }
}

// dst node (ia[a], ib[b], ic[c]) <- src[a + na*(b + nb*c)]; a null list means identity + off.
__global__ void k_scatter3(const double* __restrict__ src, int na, int nb, int nc, const int* __restrict__ ia,
                           const int* __restrict__ ib, const int* __restrict__ ic, int off, double* __restrict__ dst,
                           int dx, int dy) {
  const size_t n = (size_t)na * nb * nc;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
    const int a = (int)(t % na), b = (int)((t / na) % nb), c = (int)(t / ((size_t)na * nb));
    const int i = ia ? ia[a] : a + off, j = ib ? ib[b] : b + off, k = ic ? ic[c] : c + off;
    dst[(size_t)i + (size_t)dx * (j + (size_t)dy * k)] = src[t];
  }
}

// The first and last interior layers' sines along an axis of m nodes are
// sin(pi (p+1)/(m+1)) and sin(pi m (p+1)/(m+1)) = (-1)^p sin(pi (p+1)/(m+1)),
// so a pair of opposite faces enters mode p of the sweep as its sum (p
// even) or its difference (p odd) times the first layer's sine.  The face
// extractions below store the x and y pairs that way (the transforms along
// the faces' own axes are linear): one FMA per axis and node in the sweep.
//
// Interior values of the six faces of the block: x pair (sum, difference)
// [k][j], y pair [k][i], z faces [j][i].
__global__ void k_extract_faces(const double* __restrict__ s, int NX, int NY, int NZ, double* __restrict__ fxs,
                                double* __restrict__ fxd, double* __restrict__ fys, double* __restrict__ fyd,
                                double* __restrict__ fz0, double* __restrict__ fzN) {
  const int m0 = NX - 2, m1 = NY - 2, m2 = NZ - 2;
  const size_t sy = NX, sz = (size_t)NX * NY;
  const long nx = (long)m1 * m2, ny = (long)m0 * m2, nz = (long)m0 * m1;
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nx + ny + nz; t += (long)gridDim.x * blockDim.x) {
    if (t < nx) {
      const int j = (int)(t % m1) + 1, k = (int)(t / m1) + 1;
      const double a = s[sy * j + sz * k], b = s[(NX - 1) + sy * j + sz * k];
      fxs[t] = a + b;
      fxd[t] = a - b;
    } else if (t < nx + ny) {
      const long u = t - nx;
      const int i = (int)(u % m0) + 1, k = (int)(u / m0) + 1;
      const double a = s[i + sz * k], b = s[i + sy * (NY - 1) + sz * k];
      fys[u] = a + b;
      fyd[u] = a - b;
    } else {
      const long u = t - nx - ny;
      const int i = (int)(u % m0) + 1, j = (int)(u / m0) + 1;
      fz0[u] = s[i + sy * j];
      fzN[u] = s[i + sy * j + sz * (NZ - 1)];
    }
  }
}

// The six faces of the box whose node (0,0,0) sits at (o0,o1,o2) of an
// NX x NY x * array, interior m0 x m1 x m2: x pair (sum, difference) [k][j],
// y pair [k][i], z faces [j][i].
__global__ void k_extract_box_faces(const double* __restrict__ s, int NX, int NY, int o0, int o1, int o2, int m0,
                                    int m1, int m2, double* __restrict__ fxs, double* __restrict__ fxd,
                                    double* __restrict__ fys, double* __restrict__ fyd, double* __restrict__ fz0,
                                    double* __restrict__ fzN) {
  const size_t sy = NX, sz = (size_t)NX * NY;
  const long nx = (long)m1 * m2, ny = (long)m0 * m2, nz = (long)m0 * m1;
  auto at = [&](int a, int b, int c) { return s[(size_t)(o0 + a) + sy * (o1 + b) + sz * (o2 + c)]; };
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < nx + ny + nz; t += (long)gridDim.x * blockDim.x) {
    if (t < nx) {
      const int j = (int)(t % m1) + 1, k = (int)(t / m1) + 1;
      const double a = at(0, j, k), b = at(m0 + 1, j, k);
      fxs[t] = a + b;
      fxd[t] = a - b;
    } else if (t < nx + ny) {
      const long u = t - nx;
      const int i = (int)(u % m0) + 1, k = (int)(u / m0) + 1;
      const double a = at(i, 0, k), b = at(i, m1 + 1, k);
      fys[u] = a + b;
      fyd[u] = a - b;
    } else {
      const long u = t - nx - ny;
      const int i = (int)(u % m0) + 1, j = (int)(u / m0) + 1;
      fz0[u] = at(i, j, 0);
      fzN[u] = at(i, j, m2 + 1);
    }
  }
}

struct FaceTerms {
  const double *fxs, *fxd, *fys, *fyd, *fz0, *fzN;  // transforms: [k][q], [k][p], [q][p]
  const double *ex1, *ey1;                          // sin(pi (p+1)/(m+1)) along x and y
  double cx, cy, cz;                                // -scale / h^2
};

// Thomas sweep of -u[k-1] + d u[k] - u[k+1] = r[k] with the reciprocal pivot
// table; r = ghat (+ the transformed Dirichlet face terms when bc).  The
// recurrence stays in FP64: each line is a dependent chain and the lines
// are too few to hide the longer chain of float-float operations.
__global__ void k_thomas_faces(const double* __restrict__ g, double* __restrict__ out, const double* __restrict__ rinvt,
                               int m0, int m1, int m2, int bc, FaceTerms F) {
  const int pq = blockIdx.x * blockDim.x + threadIdx.x;
  if (pq >= m0 * m1) return;
  const int p = pq % m0, q = pq / m0;
  const size_t plane = (size_t)m0 * m1;
  auto rinv = [&](size_t id) { return rinvt[id]; };
  double ax = 0.0, ay = 0.0;
  const double *fx = nullptr, *fy = nullptr;
  if (bc) {
    ax = F.cx * F.ex1[p];
    ay = F.cy * F.ey1[q];
    fx = (p & 1) ? F.fxd : F.fxs;  // the x pair's sum (p even) or difference
    fy = (q & 1) ? F.fyd : F.fys;
  }
  auto rhs = [&](int k) -> double {
    double r = g[pq + plane * k];
    if (bc) {
      r = fma(ay, fy[(size_t)k * m0 + p], fma(ax, fx[(size_t)k * m1 + q], r));
      if (k == 0) r += F.cz * F.fz0[pq];
      if (k == m2 - 1) r += F.cz * F.fzN[pq];
    }
    return r;
  };
  // loads twelve planes ahead of the dependent chain (one thread per line
  // leaves few warps per SM: the loads in flight set the speed); same
  // arithmetic order
  constexpr int U = 12;
  double y = rhs(0);
  out[pq] = y;
  double ri = rinv(pq);
  int k = 1;
  for (; k + U - 1 < m2; k += U) {
    const size_t id = pq + plane * k;
    double qv[U], rv[U];
#pragma unroll
    for (int u = 0; u < U; ++u) qv[u] = rhs(k + u);
#pragma unroll
    for (int u = 0; u < U; ++u) rv[u] = rinv(id + plane * u);
#pragma unroll
    for (int u = 0; u < U; ++u) {
      y = fma(y, u ? rv[u - 1] : ri, qv[u]);
      out[id + plane * u] = y;
    }
    ri = rv[U - 1];
  }
  for (; k < m2; ++k) {
    const size_t id = pq + plane * k;
    y = fma(y, ri, rhs(k));
    out[id] = y;
    ri = rinv(id);
  }
  double u = y * ri;
  out[pq + plane * (m2 - 1)] = u;
  k = m2 - 2;
  for (; k - (U - 1) >= 0; k -= U) {
    const size_t id = pq + plane * k;
    double ov[U], rv[U];
#pragma unroll
    for (int v = 0; v < U; ++v) ov[v] = out[id - plane * v];
#pragma unroll
    for (int v = 0; v < U; ++v) rv[v] = rinv(id - plane * v);
#pragma unroll
    for (int v = 0; v < U; ++v) {
      u = (ov[v] + u) * rv[v];
      out[id - plane * v] = u;
    }
  }
  for (; k >= 0; --k) {
    const size_t id = pq + plane * k;
    u = (out[id] + u) * rinv(id);
    out[id] = u;
  }
}

// sin(pi (i+1)(p+1)/N) of the selected rows, one 8-byte word each: the
// double (FP64) or its float-float pair (hi, lo) in the word's bytes.
std::vector<double> sine_rows(const std::vector<int>& sel, int m, int arith) {
  std::vector<double> S(sel.size() * (size_t)m);
  const double N = m + 1;
  for (size_t i = 0; i < sel.size(); ++i)
    for (int p = 0; p < m; ++p) {
      const double v = std::sin(kPI * (double)(sel[i] + 1) * (double)(p + 1) / N);
      if (arith == VPMG_ARITH_FF48) {
        const float hi = (float)v;
        const float2 f = make_float2(hi, (float)(v - (double)hi));
        std::memcpy(&S[i * m + p], &f, sizeof(double));
      } else {
        S[i * m + p] = v;
      }
    }
  return S;
}

template <class T>
void up(DBuf<T>& b, const std::vector<T>& h) {
  b.ensure(std::max<size_t>(h.size(), 1));
  if (!h.empty()) VPMG_CUDA(cudaMemcpy(b.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
}

std::vector<int> plus1(const std::vector<int>& v) {
  std::vector<int> r(v);
  for (int& x : r) x += 1;
  return r;
}

// Dynamic shared memory granted to k_partial_x and k_partial_y so far, per
// device: the limit is an attribute of each kernel on each device, and one
// process may hold handles on several devices.  Raised at set-up only
// (outside any stream capture), never lowered.
constexpr int kMaxDev = 64;
size_t g_partial_smem[kMaxDev] = {0};
size_t g_partial_y_smem[kMaxDev] = {0};
size_t& granted(size_t* table) {
  int dev = 0;
  VPMG_CUDA(cudaGetDevice(&dev));
  VPMG_CHECK(dev >= 0 && dev < kMaxDev, VPMG_ERR_UNSUPPORTED, "device index beyond the per-device tables");
  return table[dev];
}

// k_partial_x's shared memory: the sine rows and one or two (dbl) tiles,
// 8 bytes per value in both arithmetics.
size_t partial_x_smem(int m0, int nsel, int lines, bool dbl) {
  return sizeof(double) * ((dbl ? 2 : 1) * (size_t)lines * m0 + (size_t)nsel * m0);
}
// Tile height of k_partial_x: the most lines (up to kLines) whose staged
// tiles and the sine rows fit in a CTA's shared memory.
int partial_x_lines(int m0, int nsel, bool dbl) {
  int lines = kLines;
  while (lines > 1 && partial_x_smem(m0, nsel, lines, dbl) > 227 * 1024) lines /= 2;
  return lines;
}

void partial_x_reserve(int m0, int nsel) {
  const size_t sm = partial_x_smem(m0, nsel, partial_x_lines(m0, nsel, true), true);
  VPMG_CHECK(sm <= 227 * 1024, VPMG_ERR_UNSUPPORTED, "partial transform tile too large");
  // the whole per-CTA maximum: every call's tile height keeps it within
  const size_t cap = 227 * 1024;
  size_t& have = granted(g_partial_smem);
  if (cap > have) {
    VPMG_CUDA(cudaFuncSetAttribute(k_partial_x<F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
    VPMG_CUDA(cudaFuncSetAttribute(k_partial_x<FF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)cap));
    have = cap;
  }
}

void partial_x(int arith, const double* W, int m0, int m1, int nk, const int* klist, const double* S, int nsel,
               double* out, cudaStream_t s) {
  const int nlines = m1 * nk;
  const bool dbl = arith != VPMG_ARITH_FF48;
  const int lines = partial_x_lines(m0, nsel, dbl);
  const size_t sm = partial_x_smem(m0, nsel, lines, dbl);
  VPMG_CHECK(sm <= granted(g_partial_smem), VPMG_ERR_STATE, "k_partial_x shared memory not reserved");
  // persistent CTAs: as many as fit on the SMs at this shared-memory size
  const unsigned ntiles = (nlines + lines - 1) / lines;
  const unsigned per_sm = (unsigned)std::max<size_t>(1, std::min<size_t>(8, (227 * 1024) / (sm + 1024)));
  const unsigned g = std::min(ntiles, 152u * per_sm);
  if (arith == VPMG_ARITH_FF48)
    k_partial_x<FF><<<g, 128, sm, s>>>(W, m0, m1, nk, klist, reinterpret_cast<const float2*>(S), nsel, out, lines, 0);
  else
    k_partial_x<F64><<<g, 128, sm, s>>>(W, m0, m1, nk, klist, S, nsel, out, lines, 1);
  VPMG_LAUNCHED();
}

// k_partial_y's shared memory: one or two column tiles and the partial sums
// of 8 rows; two tiles (double buffering) when they fit.
size_t partial_y_smem(int m1, bool dbl) { return sizeof(double) * ((dbl ? 2 : 1) * (size_t)m1 + 8) * kColTile; }
bool partial_y_dbl(int m1) { return partial_y_smem(m1, true) <= 227 * 1024; }

void partial_y_reserve(int m1) {
  const size_t sm = partial_y_smem(m1, partial_y_dbl(m1));
  VPMG_CHECK(sm <= 227 * 1024, VPMG_ERR_UNSUPPORTED, "partial transform tile too large");
  size_t& have = granted(g_partial_y_smem);
  if (sm > have) {
    VPMG_CUDA(cudaFuncSetAttribute(k_partial_y<F64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    VPMG_CUDA(cudaFuncSetAttribute(k_partial_y<FF>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    have = sm;
  }
}

void partial_y(int arith, const double* W, int m0, int m1, int nk, const int* klist, const double* S, int nsel,
               double* out, cudaStream_t s, const double* S2 = nullptr, int nsel2 = 0, double* out2 = nullptr) {
  const int dbl = (arith != VPMG_ARITH_FF48 && partial_y_dbl(m1)) ? 1 : 0;
  const size_t sm = partial_y_smem(m1, dbl);  // tiles + partial sums of 8 rows
  VPMG_CHECK(sm <= granted(g_partial_y_smem), VPMG_ERR_STATE, "k_partial_y shared memory not reserved");
  // persistent CTAs: as many as fit on the SMs at this shared-memory size
  const unsigned ntiles = (unsigned)(((m0 + kColTile - 1) / kColTile) * nk);
  const unsigned per_sm = (unsigned)std::max<size_t>(1, std::min<size_t>(8, (227 * 1024) / (sm + 1024)));
  const unsigned g = std::min(ntiles, 152u * per_sm);
  if (arith == VPMG_ARITH_FF48)
    k_partial_y<FF><<<g, 256, sm, s>>>(W, m0, m1, nk, klist, reinterpret_cast<const float2*>(S), nsel, out,
                                      reinterpret_cast<const float2*>(S2), nsel2, out2, dbl);
  else
    k_partial_y<F64><<<g, 256, sm, s>>>(W, m0, m1, nk, klist, S, nsel, out, S2, nsel2, out2, dbl);
  VPMG_LAUNCHED();
}

void scatter3(const double* src, int na, int nb, int nc, const int* ia, const int* ib, const int* ic, int off,
              double* dst, const int dims[3], cudaStream_t s) {
  const size_t n = (size_t)na * nb * nc;
  k_scatter3<<<(unsigned)std::min<size_t>((n + 255) / 256, 152 * 16), 256, 0, s>>>(src, na, nb, nc, ia, ib, ic, off,
                                                                                   dst, dims[0], dims[1]);
  VPMG_LAUNCHED();
}

}  // namespace

void BlockSolve::prepare(const DirichletPlan& P, const int nnbl_bl[6], int ncoarse) {
  arith = P.arith;
  for (int d = 0; d < 3; ++d) { dims[d] = P.dims[d]; m[d] = P.m[d]; }
  VPMG_CHECK(m[0] >= 8 && m[1] >= 8 && m[2] >= 8, VPMG_ERR_UNSUPPORTED, "block too small for the partial solve");
  const size_t nint = (size_t)m[0] * m[1] * m[2];
  ghat.ensure(3 * nint);
  W.ensure(nint);
  // normal-derivative layers: interior indices 0..3 and m-4..m-1
  std::vector<int> fx = {0, 1, 2, 3, m[0] - 4, m[0] - 3, m[0] - 2, m[0] - 1};
  std::vector<int> fylo = {0, 1, 2, 3}, fyhi = {m[1] - 4, m[1] - 3, m[1] - 2, m[1] - 1};
  up(S_fx, sine_rows(fx, m[0], arith));
  up(S_fy_lo, sine_rows(fylo, m[1], arith));
  up(S_fy_hi, sine_rows(fyhi, m[1], arith));
  up(l_fx, plus1(fx));
  // inner-box faces: 1-based node nnbl_bl -> interior index nnbl_bl - 2
  for (int d = 0; d < 3; ++d) {
    inner_lo[d] = nnbl_bl[d] - 2;
    inner_hi[d] = nnbl_bl[d + 3] - 2;
    VPMG_CHECK(inner_lo[d] >= 0 && inner_hi[d] < m[d] && inner_lo[d] < inner_hi[d], VPMG_ERR_ARG,
               "inner block box outside the padded block");
  }
  std::vector<int> ix = {inner_lo[0], inner_hi[0]};
  up(S_ix, sine_rows(ix, m[0], arith));
  up(S_iy_lo, sine_rows({inner_lo[1]}, m[1], arith));
  up(S_iy_hi, sine_rows({inner_hi[1]}, m[1], arith));
  up(l_ix, plus1(ix));
  // samples: 0-based nodes nc*t inside the block interior -> interior index nc*t - 1
  auto samples = [&](int d) {
    std::vector<int> v;
    for (int t = 1; ncoarse * t <= dims[d] - 2; ++t) v.push_back(ncoarse * t - 1);
    return v;
  };
  std::vector<int> sx = samples(0), sy = samples(1), sz = samples(2);
  nsx = (int)sx.size(); nsy = (int)sy.size(); nsz = (int)sz.size();
  up(S_sx, sine_rows(sx, m[0], arith));
  up(S_sy, sine_rows(sy, m[1], arith));
  up(l_sx, plus1(sx));
  up(l_sy, plus1(sy));
  up(l_sz, sz);  // plane list (interior index) for the y dots
  std::vector<int> idz(sz);
  up(l_idz, plus1(idz));  // node list for the scatter
  // first layer sines for the face terms
  auto edge = [&](int mm) {
    std::vector<double> e(mm);
    const double N = mm + 1;
    for (int p = 0; p < mm; ++p) e[p] = std::sin(kPI * (double)(p + 1) / N);
    return e;
  };
  up(e_x1, edge(m[0]));
  up(e_y1, edge(m[1]));
  partial_x_reserve(m[0], std::max(8, nsx));
  partial_y_reserve(m[1]);
  X8.ensure((size_t)8 * m[1] * m[2]);
  Y4.ensure((size_t)m[0] * 8 * m[2]);  // low and high face rows
  X2.ensure((size_t)2 * m[1] * m[2]);
  Y1.ensure((size_t)m[0] * 2 * m[2]);
  Ys.ensure((size_t)m[0] * nsy * nsz);
  XS.ensure((size_t)nsx * nsy * nsz);
  fxs.ensure((size_t)m[1] * m[2]); fxd.ensure((size_t)m[1] * m[2]);
  fys.ensure((size_t)m[0] * m[2]); fyd.ensure((size_t)m[0] * m[2]);
  fz0.ensure((size_t)m[0] * m[1]); fzN.ensure((size_t)m[0] * m[1]);
  ready = true;
}

void block_solve_zero_bc(BlockSolve& B, DirichletPlan& P, const double* rhs_c, int c, double* sol0, cudaStream_t s) {
  const int m0 = B.m[0], m1 = B.m[1], m2 = B.m[2];
  const size_t nint = (size_t)m0 * m1 * m2, plane = (size_t)m0 * m1;
  double* g = B.ghat.p + (size_t)c * nint;
  dst_forward_xy(P, rhs_c, nullptr, true, g, s);
  FaceTerms F{};
  k_thomas_faces<<<(int)((plane + 127) / 128), 128, 0, s>>>(g, B.W.p, P.rinvd.p, m0, m1, m2, 0, F);
  VPMG_LAUNCHED();
  // x faces: 8 layers by dot products along x; y faces: 4 + 4 rows by dot products along y
  partial_x(B.arith, B.W.p, m0, m1, m2, nullptr, B.S_fx.p, 8, B.X8.p, s);
  double* Y4b = B.Y4.p + (size_t)m0 * 4 * m2;
  partial_y(B.arith, B.W.p, m0, m1, m2, nullptr, B.S_fy_lo.p, 4, B.Y4.p, s, B.S_fy_hi.p, 4, Y4b);
  // one launch of inverse y transforms: the x-face layers and the first and
  // last 4 planes (z faces, in place on W after the dots) ...
  double* top = B.W.p + plane * (m2 - 4);
  const DstYLines ys[3] = {{&P.fy, B.X8.p, 8, m1, m2}, {&P.fy, B.W.p, m0, m1, 4}, {&P.fy, top, m0, m1, 4}};
  dst_lines_y_jobs(ys, 3, s);
  scatter3(B.X8.p, 8, m1, m2, B.l_fx.p, nullptr, nullptr, 1, sol0, B.dims, s);
  // ... then inverse x transforms into sol0: the y-face rows, then the z
  // planes.  Jobs of one launch write disjoint nodes; where the rows and the
  // planes meet (box edges) the planes' launch writes last, every run.
  const DstXInvLines xr[2] = {
      {&P.fx, B.Y4.p, sol0, {B.dims[0], B.dims[1], B.dims[2]}, {1, 1, 1}, {m0, 4, m2}},
      {&P.fx, Y4b, sol0, {B.dims[0], B.dims[1], B.dims[2]}, {1, 1 + m1 - 4, 1}, {m0, 4, m2}}};
  dst_x_inv_jobs(xr, 2, s);
  const DstXInvLines xz[2] = {
      {&P.fx, B.W.p, sol0, {B.dims[0], B.dims[1], B.dims[2]}, {1, 1, 1}, {m0, m1, 4}},
      {&P.fx, top, sol0, {B.dims[0], B.dims[1], B.dims[2]}, {1, 1, 1 + m2 - 4}, {m0, m1, 4}}};
  dst_x_inv_jobs(xz, 2, s);
  VPMG_CUDA(cudaGetLastError());
}

void block_solve_bc(BlockSolve& B, DirichletPlan& P, int c, double* sol_c, cudaStream_t s) {
  const int m0 = B.m[0], m1 = B.m[1], m2 = B.m[2];
  const size_t nint = (size_t)m0 * m1 * m2, plane = (size_t)m0 * m1;
  // boundary values of the faces, transformed along the face's axes
  k_extract_faces<<<256, 256, 0, s>>>(sol_c, B.dims[0], B.dims[1], B.dims[2], B.fxs.p, B.fxd.p, B.fys.p, B.fyd.p,
                                      B.fz0.p, B.fzN.p);
  VPMG_LAUNCHED();
  // transformed along the face's axes: rows over j -> q (x faces), over i ->
  // p (y faces, and the z faces' rows), in one launch; then the z faces'
  // columns over j
  const DstYLines rows[6] = {{&P.fy, B.fxs.p, 1, m1, m2}, {&P.fy, B.fxd.p, 1, m1, m2},
                             {&P.fx, B.fys.p, 1, m0, m2}, {&P.fx, B.fyd.p, 1, m0, m2},
                             {&P.fx, B.fz0.p, 1, m0, m1}, {&P.fx, B.fzN.p, 1, m0, m1}};
  dst_lines_y_jobs(rows, 6, s);
  const DstYLines cols[2] = {{&P.fy, B.fz0.p, m0, m1, 1}, {&P.fy, B.fzN.p, m0, m1, 1}};
  dst_lines_y_jobs(cols, 2, s);
  const double scale = dirichlet_scale(P);
  FaceTerms F;
  F.fxs = B.fxs.p; F.fxd = B.fxd.p; F.fys = B.fys.p; F.fyd = B.fyd.p; F.fz0 = B.fz0.p; F.fzN = B.fzN.p;
  F.ex1 = B.e_x1.p; F.ey1 = B.e_y1.p;
  F.cx = -scale / (P.h[0] * P.h[0]);
  F.cy = -scale / (P.h[1] * P.h[1]);
  F.cz = -scale / (P.h[2] * P.h[2]);
  const double* g = B.ghat.p + (size_t)c * nint;
  k_thomas_faces<<<(int)((plane + 127) / 128), 128, 0, s>>>(g, B.W.p, P.rinvd.p, m0, m1, m2, 1, F);
  VPMG_LAUNCHED();
  // dot products: the inner-box x faces along x, its y faces along y, and
  // the interior samples along y then x
  partial_x(B.arith, B.W.p, m0, m1, m2, nullptr, B.S_ix.p, 2, B.X2.p, s);
  double* Y1b = B.Y1.p + (size_t)m0 * m2;
  partial_y(B.arith, B.W.p, m0, m1, m2, nullptr, B.S_iy_lo.p, 1, B.Y1.p, s, B.S_iy_hi.p, 1, Y1b);
  partial_y(B.arith, B.W.p, m0, m1, B.nsz, B.l_sz.p, B.S_sy.p, B.nsy, B.Ys.p, s);
  partial_x(B.arith, B.Ys.p, m0, B.nsy, B.nsz, nullptr, B.S_sx.p, B.nsx, B.XS.p, s);
  scatter3(B.XS.p, B.nsx, B.nsy, B.nsz, B.l_sx.p, B.l_sy.p, B.l_idz.p, 0, sol_c, B.dims, s);
  // one launch of inverse y transforms: the x-face layers and the inner-box
  // z planes (in place on W, after the dots) ...
  double* pl0 = B.W.p + plane * B.inner_lo[2];
  double* pl1 = B.W.p + plane * B.inner_hi[2];
  const DstYLines ys[3] = {{&P.fy, B.X2.p, 2, m1, m2}, {&P.fy, pl0, m0, m1, 1}, {&P.fy, pl1, m0, m1, 1}};
  dst_lines_y_jobs(ys, 3, s);
  scatter3(B.X2.p, 2, m1, m2, B.l_ix.p, nullptr, nullptr, 1, sol_c, B.dims, s);
  // ... then inverse x transforms into sol_c: the y-face rows, then the z
  // planes (jobs of one launch write disjoint nodes; at the box edges the
  // planes' launch writes last, every run)
  const int dm[3] = {B.dims[0], B.dims[1], B.dims[2]};
  const DstXInvLines xr[2] = {
      {&P.fx, B.Y1.p, sol_c, {dm[0], dm[1], dm[2]}, {1, B.inner_lo[1] + 1, 1}, {m0, 1, m2}},
      {&P.fx, Y1b, sol_c, {dm[0], dm[1], dm[2]}, {1, B.inner_hi[1] + 1, 1}, {m0, 1, m2}}};
  dst_x_inv_jobs(xr, 2, s);
  const DstXInvLines xz[2] = {
      {&P.fx, pl0, sol_c, {dm[0], dm[1], dm[2]}, {1, 1, B.inner_lo[2] + 1}, {m0, m1, 1}},
      {&P.fx, pl1, sol_c, {dm[0], dm[1], dm[2]}, {1, 1, B.inner_hi[2] + 1}, {m0, m1, 1}}};
  dst_x_inv_jobs(xz, 2, s);
  VPMG_CUDA(cudaGetLastError());
}

void FaceSolve::prepare(const DirichletPlan& P) {
  const int m0 = P.m[0], m1 = P.m[1], m2 = P.m[2];
  f.ensure(2 * ((size_t)m1 * m2 + (size_t)m0 * m2 + (size_t)m0 * m1));
  std::vector<double> e((size_t)m0 + (size_t)m1);
  for (int p = 0; p < m0; ++p) e[p] = std::sin(kPI * (double)(p + 1) / (double)(m0 + 1));
  for (int q = 0; q < m1; ++q) e[m0 + q] = std::sin(kPI * (double)(q + 1) / (double)(m1 + 1));
  this->e.ensure(e.size());
  VPMG_CUDA(cudaMemcpy(this->e.p, e.data(), sizeof(double) * e.size(), cudaMemcpyHostToDevice));
  ready = true;
}

void dirichlet_solve_faces(DirichletPlan& P, FaceSolve& FS, const double* rhs, double* sol, double* work,
                           double* out, cudaStream_t s) {
  VPMG_CHECK(FS.ready, VPMG_ERR_STATE, "face solve not prepared");
  const int m0 = P.m[0], m1 = P.m[1], m2 = P.m[2];
  const size_t plane = (size_t)m0 * m1;
  // forward transforms of the RHS alone (zero tiles skip their FFTs)
  dst_forward_xy(P, rhs, nullptr, true, work, s);
  // the faces' values, transformed along their own axes
  double* fxs = FS.f.p;
  double* fxd = fxs + (size_t)m1 * m2;
  double* fys = fxd + (size_t)m1 * m2;
  double* fyd = fys + (size_t)m0 * m2;
  double* fz0 = fyd + (size_t)m0 * m2;
  double* fzN = fz0 + (size_t)m0 * m1;
  k_extract_box_faces<<<256, 256, 0, s>>>(sol, P.dims[0], P.dims[1], P.box[0], P.box[1], P.box[2], m0, m1, m2, fxs,
                                          fxd, fys, fyd, fz0, fzN);
  VPMG_LAUNCHED();
  const DstYLines rows[6] = {{&P.fy, fxs, 1, m1, m2}, {&P.fy, fxd, 1, m1, m2}, {&P.fx, fys, 1, m0, m2},
                             {&P.fx, fyd, 1, m0, m2}, {&P.fx, fz0, 1, m0, m1}, {&P.fx, fzN, 1, m0, m1}};
  dst_lines_y_jobs(rows, 6, s);
  const DstYLines cols[2] = {{&P.fy, fz0, m0, m1, 1}, {&P.fy, fzN, m0, m1, 1}};
  dst_lines_y_jobs(cols, 2, s);
  // the sweep with the face terms, then the full inverse transforms
  const double scale = dirichlet_scale(P);
  FaceTerms F;
  F.fxs = fxs; F.fxd = fxd; F.fys = fys; F.fyd = fyd; F.fz0 = fz0; F.fzN = fzN;
  F.ex1 = FS.e.p; F.ey1 = FS.e.p + m0;
  F.cx = -scale / (P.h[0] * P.h[0]);
  F.cy = -scale / (P.h[1] * P.h[1]);
  F.cz = -scale / (P.h[2] * P.h[2]);
  k_thomas_faces<<<(int)((plane + 127) / 128), 128, 0, s>>>(work, out, P.rinvd.p, m0, m1, m2, 1, F);
  VPMG_LAUNCHED();
  dst_lines_y(P.fy, out, m0, m1, m2, s);
  const int o[3] = {P.box[0] + 1, P.box[1] + 1, P.box[2] + 1};
  dst_x_inv_to_box(P.fx, out, sol, P.dims, o, P.m, s);
  VPMG_CUDA(cudaGetLastError());
}

}  // namespace vpmg
