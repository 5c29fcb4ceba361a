// vpm_oracle.cpp -- CPU restatement of vpm_free's particle-mesh step.
//
// TEST INFRASTRUCTURE ONLY (the checker of the CUDA library).  See
// vpm_oracle.h for the parity status.  Build with -ffp-contract=off: the
// tree opening test and the cell-index arithmetic are compared bit for bit
// with the CUDA library, which evaluates the same expressions with
// explicitly rounded operations.
#include "vpm_oracle.h"

#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstring>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

typedef std::complex<double> cd;

const double PI = 4.0 * std::atan(1.0);
const double PI4 = 4.0 * PI;

inline size_t lin(int nx, int ny, int i, int j, int k) {  // 1-based (i,j,k)
  return (size_t)(i - 1) + (size_t)nx * ((size_t)(j - 1) + (size_t)ny * (size_t)(k - 1));
}

// Fortran NINT: round half away from zero.
inline int fnint(double x) { return (int)std::lround(x); }

// ---------------------------------------------------------------- FFT ----
// Recursive mixed-radix decimation-in-time DFT (exp(-2 pi i jk/n)), used
// for the DST-I of the Dirichlet solver.  Twiddles come from one table of
// the full length.
struct FFTPlan {
  int n = 0;
  std::vector<int> fac;
  std::vector<cd> tw;
  explicit FFTPlan(int n_ = 1) : n(n_) {
    int m = n;
    for (int p = 2; m > 1;) {
      if (m % p == 0) { fac.push_back(p); m /= p; } else { ++p; }
    }
    tw.resize(n);
    for (int t = 0; t < n; ++t) tw[t] = std::polar(1.0, -2.0 * PI * (double)t / (double)n);
  }
};

void fft_rec(const cd* in, cd* out, int n, int s, const FFTPlan& P, int twstride, int fi, cd* tmp) {
  if (n == 1) { out[0] = in[0]; return; }
  const int p = P.fac[fi];
  const int m = n / p;
  for (int r = 0; r < p; ++r) fft_rec(in + (size_t)r * s, out + (size_t)r * m, m, s * p, P, twstride * p, fi + 1, tmp);
  for (int k = 0; k < m; ++k) {
    for (int r = 0; r < p; ++r) tmp[r] = out[(size_t)r * m + k];
    for (int q = 0; q < p; ++q) {
      cd acc = 0.0;
      const long kk = k + (long)q * m;
      for (int r = 0; r < p; ++r) acc += tmp[r] * P.tw[(size_t)(((long)r * kk) % n) * twstride];
      out[(size_t)q * m + k] = acc;
    }
  }
}

// Unnormalised DST-I of two real sequences of length n = N-1 at once:
// X_k = sum_{j=1}^{n} x_j sin(pi j k / N).  Packs a + i b, odd-extends to
// 2N, one complex DFT; Re W_k = 2 B_k, Im W_k = -2 A_k.
struct DST2 {
  int n, N;
  FFTPlan plan;
  explicit DST2(int n_) : n(n_), N(n_ + 1), plan(2 * (n_ + 1)) {}
  void run(double* a, double* b, std::vector<cd>& z, std::vector<cd>& w, std::vector<cd>& tmp) const {
    const int M = 2 * N;
    z.assign(M, cd(0.0, 0.0));
    w.resize(M);
    tmp.resize(M);
    for (int j = 1; j <= n; ++j) {
      cd v(a[j - 1], b ? b[j - 1] : 0.0);
      z[j] = v;
      z[M - j] = -v;
    }
    fft_rec(z.data(), w.data(), M, 1, plan, 1, 0, tmp.data());
    for (int k = 1; k <= n; ++k) {
      a[k - 1] = -0.5 * w[k].imag();
      if (b) b[k - 1] = 0.5 * w[k].real();
    }
  }
};

// ------------------------------------------------------ projection fun ----
double projection_fun(int itype, double x) {  // source/pmproject.f90:391-431
  double xabs = std::fabs(x), f = 0.0;
  if (itype == 2) {
    f = (xabs > 1.0) ? 0.0 : 1.0 - xabs;
  } else if (itype == 3) {
    if (xabs > 1.5) f = 0.0;
    if (xabs >= 0.5 && xabs <= 1.5) f = 0.5 * (-xabs + 1.5) * (-xabs + 1.5);
    if (xabs >= 0.0 && xabs < 0.5) f = 0.5 * (xabs + 1.5) * (xabs + 1.5) - 1.5 * (xabs + 0.5) * (xabs + 0.5);
  } else if (itype == 4) {
    if (xabs > 2.0) f = 0.0;
    if (xabs >= 1.0 && xabs <= 2.0) f = 0.5 * ((2.0 - xabs) * (2.0 - xabs)) * (1.0 - xabs);
    if (xabs < 1.0) f = 1.0 - 2.5 * (xabs * xabs) + 1.5 * (xabs * xabs * xabs);
  } else if (itype == 5) {
    if (xabs <= 0.5) f = 1.0 - xabs * xabs;
    if (xabs > 0.5 && xabs <= 1.5) f = 0.5 * (1.0 - xabs) * (2.0 - xabs);
    if (xabs > 1.5) f = 0.0;
  } else if (itype == 6) {
    if (xabs <= 1.0) f = 1.0 - xabs * xabs;
    if (xabs > 1.0 && xabs <= 2.0) f = 0.5 * (1.0 - xabs) * (2.0 - xabs);
    if (xabs > 2.0) f = 0.0;
  }
  return f;
}

// ------------------------------------------------------------- solver ----
int nthr(int t) {
#ifdef _OPENMP
  return t > 0 ? t : omp_get_max_threads();
#else
  (void)t;
  return 1;
#endif
}

// Dirichlet 7-point solve; semantics of MKL d_Helmholtz_3D('DDDDDD', q=0)
// as called from source/pmsolve.f90:284-432: f = -RHS on the box, boundary
// values bd_* taken from SOL (or zero), solution written to the interior.
void dirichlet(int nx, int ny, int nz, const int box[6], const double d[3], const double* rhs,
               double* sol, bool zero_bc, int nthreads) {
  const int is = box[0], js = box[1], ks = box[2], ie = box[3], je = box[4], ke = box[5];
  const int n1 = ie - is - 1, n2 = je - js - 1, n3 = ke - ks - 1;  // interior counts
  if (n1 < 1 || n2 < 1 || n3 < 1) return;
  const double hx2 = d[0] * d[0], hy2 = d[1] * d[1], hz2 = d[2] * d[2];
  auto S = [&](int i, int j, int k) -> double& { return sol[lin(nx, ny, i, j, k)]; };
  auto R = [&](int i, int j, int k) -> double { return rhs[lin(nx, ny, i, j, k)]; };
  // g(a,b,c) on interior, a fastest (a = 1..n1)
  std::vector<double> g((size_t)n1 * n2 * n3);
  auto G = [&](int a, int b, int c) -> double& { return g[(size_t)(a - 1) + (size_t)n1 * ((b - 1) + (size_t)n2 * (c - 1))]; };
  const int T = nthr(nthreads);
#pragma omp parallel for num_threads(T) schedule(static)
  for (int c = 1; c <= n3; ++c)
    for (int b = 1; b <= n2; ++b)
      for (int a = 1; a <= n1; ++a) {
        const int i = is + a, j = js + b, k = ks + c;
        double v = R(i, j, k);
        if (!zero_bc) {
          if (a == 1) v -= S(is, j, k) / hx2;
          if (a == n1) v -= S(ie, j, k) / hx2;
          if (b == 1) v -= S(i, js, k) / hy2;
          if (b == n2) v -= S(i, je, k) / hy2;
          if (c == 1) v -= S(i, j, ks) / hz2;
          if (c == n3) v -= S(i, j, ke) / hz2;
        }
        G(a, b, c) = v;
      }
  DST2 dx(n1), dy(n2);
  // forward DST along x (pairs of lines)
  const long nlx = (long)n2 * n3;
#pragma omp parallel num_threads(T)
  {
    std::vector<cd> z, w, tmp;
#pragma omp for schedule(static)
    for (long l = 0; l < nlx; l += 2) {
      double* a = &g[(size_t)l * n1];
      double* b = (l + 1 < nlx) ? &g[(size_t)(l + 1) * n1] : nullptr;
      dx.run(a, b, z, w, tmp);
    }
  }
  // forward DST along y: lines (a, c) gathered
#pragma omp parallel num_threads(T)
  {
    std::vector<cd> z, w, tmp;
    std::vector<double> la(n2), lb(n2);
#pragma omp for schedule(static)
    for (long l = 0; l < (long)n1 * n3; l += 2) {
      const int a0 = (int)(l % n1) + 1, c0 = (int)(l / n1) + 1;
      const bool two = (l + 1 < (long)n1 * n3);
      const int a1 = (int)((l + 1) % n1) + 1, c1 = (int)((l + 1) / n1) + 1;
      for (int b = 1; b <= n2; ++b) { la[b - 1] = G(a0, b, c0); if (two) lb[b - 1] = G(a1, b, c1); }
      dy.run(la.data(), two ? lb.data() : nullptr, z, w, tmp);
      for (int b = 1; b <= n2; ++b) { G(a0, b, c0) = la[b - 1]; if (two) G(a1, b, c1) = lb[b - 1]; }
    }
  }
  // tridiagonal along z for each (p,q)
  const double N1 = n1 + 1, N2 = n2 + 1;
  const double scale = 4.0 / (N1 * N2);
#pragma omp parallel num_threads(T)
  {
    std::vector<double> m(n3), y(n3);
#pragma omp for schedule(static)
    for (long l = 0; l < (long)n1 * n2; ++l) {
      const int p = (int)(l % n1) + 1, q = (int)(l / n1) + 1;
      const double sp = std::sin(PI * p / (2.0 * N1)), sq = std::sin(PI * q / (2.0 * N2));
      const double mup = 4.0 * sp * sp, muq = 4.0 * sq * sq;
      const double dd = 2.0 + hz2 * (mup / hx2 + muq / hy2);
      // -u_{k-1} + dd u_k - u_{k+1} = -hz2 * ghat_k * scale
      for (int c = 1; c <= n3; ++c) {
        const double r = -hz2 * G(p, q, c) * scale;
        if (c == 1) { m[0] = dd; y[0] = r; }
        else { m[c - 1] = dd - 1.0 / m[c - 2]; y[c - 1] = r + y[c - 2] / m[c - 2]; }
      }
      double u = y[n3 - 1] / m[n3 - 1];
      G(p, q, n3) = u;
      for (int c = n3 - 1; c >= 1; --c) { u = (y[c - 1] + u) / m[c - 1]; G(p, q, c) = u; }
    }
  }
  // inverse DST along y then x (unnormalised; scale folded above)
#pragma omp parallel num_threads(T)
  {
    std::vector<cd> z, w, tmp;
    std::vector<double> la(n2), lb(n2);
#pragma omp for schedule(static)
    for (long l = 0; l < (long)n1 * n3; l += 2) {
      const int a0 = (int)(l % n1) + 1, c0 = (int)(l / n1) + 1;
      const bool two = (l + 1 < (long)n1 * n3);
      const int a1 = (int)((l + 1) % n1) + 1, c1 = (int)((l + 1) / n1) + 1;
      for (int b = 1; b <= n2; ++b) { la[b - 1] = G(a0, b, c0); if (two) lb[b - 1] = G(a1, b, c1); }
      dy.run(la.data(), two ? lb.data() : nullptr, z, w, tmp);
      for (int b = 1; b <= n2; ++b) { G(a0, b, c0) = la[b - 1]; if (two) G(a1, b, c1) = lb[b - 1]; }
    }
  }
#pragma omp parallel num_threads(T)
  {
    std::vector<cd> z, w, tmp;
#pragma omp for schedule(static)
    for (long l = 0; l < nlx; l += 2) {
      double* a = &g[(size_t)l * n1];
      double* b = (l + 1 < nlx) ? &g[(size_t)(l + 1) * n1] : nullptr;
      dx.run(a, b, z, w, tmp);
    }
  }
#pragma omp parallel for num_threads(T) schedule(static)
  for (int c = 1; c <= n3; ++c)
    for (int b = 1; b <= n2; ++b)
      for (int a = 1; a <= n1; ++a) S(is + a, js + b, ks + c) = G(a, b, c);
  if (zero_bc) {  // boundary of the box is zero (solve_eq_0_3d writes bd = 0)
    for (int k = ks; k <= ke; ++k)
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i)
          if (i == is || i == ie || j == js || j == je || k == ks || k == ke) S(i, j, k) = 0.0;
  }
}

// ------------------------------------------------- infinite domain BCs ----
struct Panels {  // calc_normalderiv_3d output (source/pinfdomain.f90:294-547)
  int nbound = 0;
  std::vector<double> src[3];
  std::vector<double> xc, yc, zc, ds;  // 0.25*(c1+c2+c3+c4) panel centres, areas
  int n1f[6], n2f[6];                  // per face: fast and slow cell counts
};

struct Tree {  // build_level_nbound_3d output (source/pinfdomain.f90:875-1530)
  int levmax = 0, nbound = 0;
  std::vector<int> nbound_lev;  // cumulative count per level (all faces)
  std::vector<double> xs, ys, zs, dsl, s[3];  // [lev*nbound + (icount-1)]
  std::vector<int> ilev;                      // [((lev*nbound)+(icount-1))*6 + m]
  int& IL(int c, int lev, int m) { return ilev[((size_t)lev * nbound + (c - 1)) * 6 + (m - 1)]; }
  int IL(int c, int lev, int m) const { return ilev[((size_t)lev * nbound + (c - 1)) * 6 + (m - 1)]; }
  size_t at(int c, int lev) const { return (size_t)lev * nbound + (c - 1); }
};

inline double coord(double xmin, int i, double d) { return xmin + (double)(i - 1) * d; }
inline double mean4(double a, double b, double c, double e) { return 0.25 * (((a + b) + c) + e); }

void normal_deriv(int NX, int NY, int NZ, const double xb[6], const double D[3], double* const s0[3], Panels& P) {
  const double a1 = 25.0 / 12.0, a2 = -4.0, a3 = 3.0, a4 = -4.0 / 3.0, a5 = 0.25;
  const double XMIN = xb[0], YMIN = xb[1], ZMIN = xb[2], DX = D[0], DY = D[1], DZ = D[2];
  auto S = [&](int c, int i, int j, int k) { return s0[c][lin(NX, NY, i, j, k)]; };
  const int NXs = 1, NXf = NX, NYs = 1, NYf = NY, NZs = 1, NZf = NZ;
  P.nbound = 0;
  size_t tot = 2 * (size_t)(NY - 1) * (NZ - 1) + 2 * (size_t)(NX - 1) * (NZ - 1) + 2 * (size_t)(NX - 1) * (NY - 1);
  for (int c = 0; c < 3; ++c) P.src[c].assign(tot, 0.0);
  P.xc.assign(tot, 0.0); P.yc.assign(tot, 0.0); P.zc.assign(tot, 0.0); P.ds.assign(tot, 0.0);
  auto d5 = [&](double inv, double v0, double v1, double v2, double v3, double v4) {
    return inv * ((((a1 * v0 + a2 * v1) + a3 * v2) + a4 * v3) + a5 * v4);
  };
  auto put = [&](double x1, double x2, double x3, double x4, double y1, double y2, double y3, double y4,
                 double z1, double z2, double z3, double z4, double dsv) {
    int n = P.nbound;
    P.xc[n] = mean4(x1, x2, x3, x4); P.yc[n] = mean4(y1, y2, y3, y4); P.zc[n] = mean4(z1, z2, z3, z4);
    P.ds[n] = dsv;
    P.nbound++;
  };
  // XMIN / XMAX: k outer, j inner
  for (int face = 0; face < 2; ++face) {
    const int i = face == 0 ? NXs : NXf, sg = face == 0 ? 1 : -1;
    const double inv = 1.0 / DX;
    for (int k = NZs; k <= NZf - 1; ++k)
      for (int j = NYs; j <= NYf - 1; ++j) {
        const int n = P.nbound, j1 = j + 1, k1 = k + 1;
        for (int c = 0; c < 3; ++c) {
          double p1 = d5(inv, S(c, i, j, k), S(c, i + sg, j, k), S(c, i + 2 * sg, j, k), S(c, i + 3 * sg, j, k), S(c, i + 4 * sg, j, k));
          double p2 = d5(inv, S(c, i, j1, k), S(c, i + sg, j1, k), S(c, i + 2 * sg, j1, k), S(c, i + 3 * sg, j1, k), S(c, i + 4 * sg, j1, k));
          double p3 = d5(inv, S(c, i, j1, k1), S(c, i + sg, j1, k1), S(c, i + 2 * sg, j1, k1), S(c, i + 3 * sg, j1, k1), S(c, i + 4 * sg, j1, k1));
          double p4 = d5(inv, S(c, i, j, k1), S(c, i + sg, j, k1), S(c, i + 2 * sg, j, k1), S(c, i + 3 * sg, j, k1), S(c, i + 4 * sg, j, k1));
          P.src[c][n] = 0.25 * (((p1 + p2) + p3) + p4);
        }
        const double x = coord(XMIN, i, DX), y0 = coord(YMIN, j, DY), y1 = coord(YMIN, j + 1, DY);
        const double z0 = coord(ZMIN, k, DZ), z1 = coord(ZMIN, k + 1, DZ);
        if (face == 0) put(x, x, x, x, y0, y0, y1, y1, z0, z1, z1, z0, DY * DZ);
        else put(x, x, x, x, y1, y1, y0, y0, z0, z1, z1, z0, DY * DZ);
      }
    P.n1f[face] = NY - 1; P.n2f[face] = NZ - 1;
  }
  // YMIN / YMAX: k outer, i inner
  for (int face = 0; face < 2; ++face) {
    const int j = face == 0 ? NYs : NYf, sg = face == 0 ? 1 : -1;
    const double inv = 1.0 / DY;
    for (int k = NZs; k <= NZf - 1; ++k)
      for (int i = NXs; i <= NXf - 1; ++i) {
        const int n = P.nbound, i1 = i + 1, k1 = k + 1;
        for (int c = 0; c < 3; ++c) {
          double p1 = d5(inv, S(c, i, j, k), S(c, i, j + sg, k), S(c, i, j + 2 * sg, k), S(c, i, j + 3 * sg, k), S(c, i, j + 4 * sg, k));
          double p2 = d5(inv, S(c, i1, j, k), S(c, i1, j + sg, k), S(c, i1, j + 2 * sg, k), S(c, i1, j + 3 * sg, k), S(c, i1, j + 4 * sg, k));
          double p3 = d5(inv, S(c, i1, j, k1), S(c, i1, j + sg, k1), S(c, i1, j + 2 * sg, k1), S(c, i1, j + 3 * sg, k1), S(c, i1, j + 4 * sg, k1));
          double p4 = d5(inv, S(c, i, j, k1), S(c, i, j + sg, k1), S(c, i, j + 2 * sg, k1), S(c, i, j + 3 * sg, k1), S(c, i, j + 4 * sg, k1));
          P.src[c][n] = 0.25 * (((p1 + p2) + p3) + p4);
        }
        const double y = coord(YMIN, j, DY), x0 = coord(XMIN, i, DX), x1 = coord(XMIN, i + 1, DX);
        const double z0 = coord(ZMIN, k, DZ), z1 = coord(ZMIN, k + 1, DZ);
        if (face == 0) put(x0, x0, x1, x1, y, y, y, y, z0, z1, z1, z0, DX * DZ);
        else put(x1, x1, x0, x0, y, y, y, y, z0, z1, z1, z0, DX * DZ);
      }
    P.n1f[2 + face] = NX - 1; P.n2f[2 + face] = NZ - 1;
  }
  // ZMIN / ZMAX: j outer, i inner
  for (int face = 0; face < 2; ++face) {
    const int k = face == 0 ? NZs : NZf, sg = face == 0 ? 1 : -1;
    const double inv = 1.0 / DZ;
    for (int j = NYs; j <= NYf - 1; ++j)
      for (int i = NXs; i <= NXf - 1; ++i) {
        const int n = P.nbound, i1 = i + 1, j1 = j + 1;
        for (int c = 0; c < 3; ++c) {
          double p1 = d5(inv, S(c, i, j, k), S(c, i, j, k + sg), S(c, i, j, k + 2 * sg), S(c, i, j, k + 3 * sg), S(c, i, j, k + 4 * sg));
          double p2 = d5(inv, S(c, i1, j, k), S(c, i1, j, k + sg), S(c, i1, j, k + 2 * sg), S(c, i1, j, k + 3 * sg), S(c, i1, j, k + 4 * sg));
          double p3 = d5(inv, S(c, i1, j1, k), S(c, i1, j1, k + sg), S(c, i1, j1, k + 2 * sg), S(c, i1, j1, k + 3 * sg), S(c, i1, j1, k + 4 * sg));
          double p4 = d5(inv, S(c, i, j1, k), S(c, i, j1, k + sg), S(c, i, j1, k + 2 * sg), S(c, i, j1, k + 3 * sg), S(c, i, j1, k + 4 * sg));
          P.src[c][n] = 0.25 * (((p1 + p2) + p3) + p4);
        }
        const double z = coord(ZMIN, k, DZ), x0 = coord(XMIN, i, DX), x1 = coord(XMIN, i + 1, DX);
        const double y0 = coord(YMIN, j, DY), y1 = coord(YMIN, j + 1, DY);
        if (face == 0) put(x0, x0, x1, x1, y0, y1, y1, y0, z, z, z, z, DX * DY);
        else put(x1, x1, x0, x0, y0, y1, y1, y0, z, z, z, z, DX * DY);
      }
    P.n1f[4 + face] = NX - 1; P.n2f[4 + face] = NY - 1;
  }
}

// Per-face quadtree, literal restatement of build_level_nbound_3d.
bool build_tree(const Panels& P, int levmax, Tree& T) {
  T.levmax = levmax;
  T.nbound = P.nbound;
  const size_t NL = (size_t)(levmax + 1) * P.nbound;
  T.xs.assign(NL, 0.0); T.ys.assign(NL, 0.0); T.zs.assign(NL, 0.0); T.dsl.assign(NL, 0.0);
  for (int c = 0; c < 3; ++c) T.s[c].assign(NL, 0.0);
  T.ilev.assign(NL * 6, 0);
  std::vector<int> nbl(levmax + 1, 0), ncount(levmax + 1, 0);
  for (int face = 0; face < 6; ++face) {
    const int n1 = P.n1f[face], n2 = P.n2f[face];
    std::vector<int> nnf(levmax + 1);
    for (int lev = 0; lev <= levmax; ++lev) {
      const int istep = 1 << lev;
      nnf[lev] = n1 / istep + ((n1 % istep) ? 1 : 0);
    }
    const int lf = nbl[0];
    for (int lev = 0; lev <= levmax; ++lev) {
      const int istep = 1 << lev;
      int icount = nbl[lev];
      for (int so = 0; so <= n2 - istep; so += istep) {
        for (int fo = 0; fo <= n1 - istep; fo += istep) {
          double xc = 0, yc = 0, zc = 0, sc = 0, sw[3] = {0, 0, 0};
          for (int mm = 1; mm <= istep; ++mm)
            for (int nn = 1; nn <= istep; ++nn) {
              const int leaf = lf + so * n1 + fo + (mm - 1) * n1 + nn;  // 1-based
              const double x = P.xc[leaf - 1], y = P.yc[leaf - 1], z = P.zc[leaf - 1], s = P.ds[leaf - 1];
              xc = x + xc; yc = y + yc; zc = z + zc; sc = s + sc;
              for (int c = 0; c < 3; ++c) sw[c] = P.src[c][leaf - 1] * s + sw[c];
            }
          icount++;
          const size_t a = T.at(icount, lev);
          const double q = (double)(float)(istep * istep);
          T.xs[a] = xc / q; T.ys[a] = yc / q; T.zs[a] = zc / q; T.dsl[a] = sc;
          for (int c = 0; c < 3; ++c) T.s[c][a] = sw[c] / sc;
          const int npre = nnf[lev];
          if (lev > 0) {
            const int nn = nnf[lev - 1];
            int nj;
            if (fo == 0 && icount - 1 == nbl[lev]) nj = nbl[lev - 1] + 1;
            else if (fo == 0 && icount - 1 > nbl[lev]) {
              nj = T.IL(icount - 1, lev, 3) + 1;
              if (T.IL(icount - 1, lev, 6) < 0) nj = T.IL(icount - 1, lev, 2) + 1;
            } else nj = T.IL(icount - 1, lev, 2) + 1;
            T.IL(icount, lev, 1) = nj; T.IL(icount, lev, 2) = nj + 1;
            T.IL(icount, lev, 3) = nj + nn + 1; T.IL(icount, lev, 4) = nj + nn; T.IL(icount, lev, 5) = 4;
          }
          T.IL(icount, lev, 6) = npre;
        }
        if ((n1 % istep) != 0 || n1 <= istep) {
          if (lev == 0) return false;
          icount++;
          const int nn = nnf[lev - 1];
          const int nj = T.IL(icount - 1, lev, 2) + 1;
          T.IL(icount, lev, 1) = nj; T.IL(icount, lev, 2) = nj + nn; T.IL(icount, lev, 5) = 2; T.IL(icount, lev, 6) = -1;
        }
      }
      if ((n2 % istep) != 0 || n2 <= istep) {
        if (lev == 0) return false;
        for (int fo = 0; fo <= n1 - istep; fo += istep) {
          if (fo == n1 - istep && (n1 % istep) != 0) continue;
          icount++;
          int nj;
          if (fo == 0 && T.IL(icount - 1, lev, 6) > 0) nj = T.IL(icount - 1, lev, 3) + 1;
          else nj = T.IL(icount - 1, lev, 2) + 1;
          T.IL(icount, lev, 1) = nj; T.IL(icount, lev, 2) = nj + 1; T.IL(icount, lev, 5) = 2; T.IL(icount, lev, 6) = -2;
        }
      }
      ncount[lev] = icount;
    }
    nbl = ncount;
  }
  T.nbound_lev = nbl;
  return nbl[0] == P.nbound;
}

// Recursive walk, literal restatement of tree_calc_3d (source/pmbound.f90:1135-1249).
void tree_calc(const Tree& T, int nv, int nlev, double X, double Y, double Z, double src[3], long& nint) {
  int list[4] = {0, 0, 0, 0};
  int ls = 1, lfin;
  bool all = false;
  if (nlev == T.levmax) { all = true; lfin = T.nbound_lev[nlev]; }
  else if (T.IL(nv, nlev + 1, 6) < 0) { list[0] = T.IL(nv, nlev + 1, 1); list[1] = T.IL(nv, nlev + 1, 2); lfin = 2; }
  else { for (int m = 0; m < 4; ++m) list[m] = T.IL(nv, nlev + 1, m + 1); lfin = 4; }
  const double lg = std::log((std::sqrt(2.0) - 1) / (std::sqrt(2.0) + 1));
  for (int nlf = ls; nlf <= lfin; ++nlf) {
    const int nleaf = all ? nlf : list[nlf - 1];
    const size_t a = T.at(nleaf, nlev);
    const double XR = T.xs[a] - X, YR = T.ys[a] - Y, ZR = T.zs[a] - Z;
    const double r = std::sqrt(XR * XR + YR * YR + ZR * ZR);
    const double DS = T.dsl[a];
    if ((r < 10.0 * std::sqrt(DS) && nlev > 0) || T.IL(nleaf, nlev, 6) < 0) {
      tree_calc(T, nleaf, nlev - 1, X, Y, Z, src, nint);
    } else {
      ++nint;
      if (r > 1e-05) {
        for (int c = 0; c < 3; ++c) src[c] = src[c] - T.s[c][a] * DS / r;
      } else {
        for (int c = 0; c < 3; ++c) src[c] = src[c] + T.s[c][a] * 2.0 * std::sqrt(DS) * lg;
      }
    }
  }
}

// ---- ibctyp = 3: constant-source panels ---------------------------------
// Target-plane constants of calc_boundinf_3d_s / calc_boundinf_3d_lev_s
// (source/pmbound.f90:536-606, 1270-1340).  iplane: +-1 Y plane, +-2 X plane,
// +-3 Z plane; the sign is negative on the max faces (Bounds3d_lev,
// pmbound.f90:1004-1054).
struct Frame {
  double E1[3], E2[3], E3[3], S[4], T[4], D[4], diag, area;
};

Frame make_frame(int iplane, const double Dpm[3]) {
  Frame F;
  const double DX = Dpm[0], DY = Dpm[1], DZ = Dpm[2];
  const double si = iplane > 0 ? 1.0 : -1.0;
  for (int m = 0; m < 3; ++m) F.E1[m] = F.E2[m] = F.E3[m] = 0.0;
  double a = 0, b = 0;  // in-plane spacings along E1 and E2
  switch (iplane > 0 ? iplane : -iplane) {
    case 1:  // Y = const
      F.E1[0] = 1.0 * si; F.E2[2] = 1.0; F.E3[1] = -1.0 * si;
      F.diag = std::sqrt(DX * DX + DZ * DZ); F.area = DX * DZ; a = DX; b = DZ;
      break;
    case 2:  // X = const
      F.E1[2] = 1.0; F.E2[1] = -1.0 * si; F.E3[0] = -1.0 * si;
      F.diag = std::sqrt(DY * DY + DZ * DZ); F.area = DY * DZ; a = DY; b = DZ;
      break;
    default:  // Z = const
      F.E1[0] = 1.0; F.E2[1] = -1.0 * si; F.E3[2] = -1.0 * si;
      F.diag = std::sqrt(DX * DX + DY * DY); F.area = DX * DY; a = DX; b = DY;
      break;
  }
  F.S[0] = -0.5 * a; F.S[1] = -0.5 * a; F.S[2] = 0.5 * a; F.S[3] = 0.5 * a;
  F.T[0] = -0.5 * b; F.T[1] = 0.5 * b; F.T[2] = 0.5 * b; F.T[3] = -0.5 * b;
  F.D[0] = b; F.D[1] = a; F.D[2] = b; F.D[3] = a;
  return F;
}

// FSOUR_A4 (source/pmbound.f90:1540-1620) with NSIDE = 0, ISING = 0,
// EPSS = 1e-14: potential at XO of a flat quadrilateral of unit constant
// source centred at RG, corners (S, T) in the frame (E1, E2, E3).
double fsour_a4(const double XO[3], const double RG[3], const Frame& F, double AREA) {
  const double COSB[4] = {0.0, 1.0, 0.0, -1.0}, SINB[4] = {1.0, 0.0, -1.0, 0.0};
  const double TINY = 1e-10, EPSS = 1e-14;
  const double d0 = XO[0] - RG[0], d1 = XO[1] - RG[1], d2 = XO[2] - RG[2];
  const double X = (d0 * F.E1[0] + d1 * F.E1[1]) + d2 * F.E1[2];
  const double Y = (d0 * F.E2[0] + d1 * F.E2[1]) + d2 * F.E2[2];
  double Z = (d0 * F.E3[0] + d1 * F.E3[1]) + d2 * F.E3[2];
  const double RO = std::sqrt((X * X + Y * Y) + Z * Z);
  const double RATIO = RO / F.diag;
  if (RATIO > 10) {
    const double AREA1 = AREA / PI4;
    return -AREA1 / RO;
  }
  double FIL = 0.0;
  const double ZP = (Z < 0.0) ? -1.0 : 1.0;
  double AZ = std::max(EPSS, std::fabs(Z));
  Z = AZ * ZP;
  const double ZK = Z * Z;
  double R[4], E[4], H[4];
  for (int k = 0; k < 4; ++k) {
    const double XK = (X - F.S[k]) * (X - F.S[k]);
    const double YK = (Y - F.T[k]) * (Y - F.T[k]);
    H[k] = (X - F.S[k]) * (Y - F.T[k]);
    R[k] = std::sqrt((XK + YK) + ZK);
    E[k] = ZK + XK;
  }
  for (int k = 0; k < 4; ++k) {
    const int k1 = k, k2 = (k == 3) ? 0 : k + 1;
    const double A2 = (R[k1] + R[k2]) + F.D[k];
    const double A1 = (R[k1] + R[k2]) - F.D[k];
    if (std::fabs(A1 * A2) < TINY) continue;
    const double AK = std::log(A1 / A2);
    const double TOO = -(X - F.S[k1]) * SINB[k] + (Y - F.T[k1]) * COSB[k];
    FIL = FIL - TOO * AK;
  }
  AZ = std::max(TINY, AZ);
  Z = AZ * ZP;
  double UL3 = 0.0;
  for (int k = 0; k < 4; ++k) {
    if (std::fabs(COSB[k]) < TINY) continue;
    const int k1 = k, k2 = (k == 3) ? 0 : k + 1;
    UL3 = UL3 + std::atan((SINB[k] * E[k1] - COSB[k] * H[k1]) / ((Z * COSB[k]) * R[k1])) -
          std::atan((SINB[k] * E[k2] - COSB[k] * H[k2]) / ((Z * COSB[k]) * R[k2]));
  }
  return (FIL + Z * UL3) / PI4;
}

// Recursive walk, literal restatement of tree_calc_3d_s (source/pmbound.f90:1379-1501).
// Kept as written: the opening test divides (r / sqrt(dS) < 10); only
// ilev_t(.,.,6) == -1 dummies are always opened (a -2 dummy has dS = 0, so
// it is never opened and its children are not visited); at the coarsest
// level an unopened cell contributes FSOUR_A4(cell) times the source of
// the cell the walk started from (nv = 1), not of the visited cell.
void tree_calc_s(const Tree& T, int nv, int nlev, const double XO[3], const Frame& F, double src[3], long& nint) {
  int list[4] = {0, 0, 0, 0};
  int lfin;
  bool all = false;
  if (nlev == T.levmax) { all = true; lfin = T.nbound_lev[nlev]; }
  else if (T.IL(nv, nlev + 1, 6) < 0) { list[0] = T.IL(nv, nlev + 1, 1); list[1] = T.IL(nv, nlev + 1, 2); lfin = 2; }
  else { for (int m = 0; m < 4; ++m) list[m] = T.IL(nv, nlev + 1, m + 1); lfin = 4; }
  for (int nlf = 1; nlf <= lfin; ++nlf) {
    const int nleaf = all ? nlf : list[nlf - 1];
    const size_t a = T.at(nleaf, nlev);
    const double RG[3] = {T.xs[a], T.ys[a], T.zs[a]};
    const double r = std::sqrt(((XO[0] - RG[0]) * (XO[0] - RG[0]) + (XO[1] - RG[1]) * (XO[1] - RG[1])) +
                               (XO[2] - RG[2]) * (XO[2] - RG[2]));
    const double DS = T.dsl[a];
    const double RATIO = r / std::sqrt(DS);
    if ((RATIO < 10 && nlev > 0) || T.IL(nleaf, nlev, 6) == -1) {
      tree_calc_s(T, nleaf, nlev - 1, XO, F, src, nint);
    } else {
      ++nint;
      if (nlev != T.levmax) {
        for (int c = 0; c < 3; ++c) src[c] = src[c] - T.s[c][a] * DS / (PI4 * r);
      } else {
        const double FIS = fsour_a4(XO, RG, F, DS);
        const size_t av = T.at(nv, nlev);
        for (int c = 0; c < 3; ++c) src[c] = src[c] + T.s[c][av] * FIS;
      }
    }
  }
}

// Bounds3d_lev (source/pmbound.f90:980-1133) on the whole grid 1..N; and
// the untreed Bounds3d (source/pmbound.f90:80-157) when direct.  ibctyp 2:
// calc_boundinf_3d_lev / calc_boundinf_3d; ibctyp 3: calc_boundinf_3d_lev_s
// / calc_boundinf_3d_s (source/pmbound.f90:1255-1353, 520-648).
long bounds(int NX, int NY, int NZ, const double xb[6], const double D[3], const Tree* T, const Panels* P,
            double* const sol[3], int nthreads, int ibctyp) {
  const double XMIN = xb[0], YMIN = xb[1], ZMIN = xb[2], DX = D[0], DY = D[1], DZ = D[2];
  struct Tg { int i, j, k, iplane; };
  std::vector<Tg> tg;
  for (int k = 1; k <= NZ; ++k) for (int j = 1; j <= NY; ++j) tg.push_back({1, j, k, 2});
  for (int k = 1; k <= NZ; ++k) for (int j = 1; j <= NY; ++j) tg.push_back({NX, j, k, -2});
  for (int k = 1; k <= NZ; ++k) for (int i = 2; i <= NX - 1; ++i) tg.push_back({i, 1, k, 1});
  for (int k = 1; k <= NZ; ++k) for (int i = 2; i <= NX - 1; ++i) tg.push_back({i, NY, k, -1});
  for (int j = 2; j <= NY - 1; ++j) for (int i = 2; i <= NX - 1; ++i) tg.push_back({i, j, 1, 3});
  for (int j = 2; j <= NY - 1; ++j) for (int i = 2; i <= NX - 1; ++i) tg.push_back({i, j, NZ, -3});
  Frame frames[7];
  for (int p = -3; p <= 3; ++p)
    if (p != 0) frames[p + 3] = make_frame(p, D);
  long total = 0;
  const int Tn = nthr(nthreads);
  const double lg = std::log((std::sqrt(2.0) - 1) / (std::sqrt(2.0) + 1));
#pragma omp parallel for num_threads(Tn) schedule(dynamic, 64) reduction(+ : total)
  for (long t = 0; t < (long)tg.size(); ++t) {
    const int i = tg[t].i, j = tg[t].j, k = tg[t].k;
    const double X = coord(XMIN, i, DX), Y = coord(YMIN, j, DY), Z = coord(ZMIN, k, DZ);
    const size_t node = lin(NX, NY, i, j, k);
    const Frame& F = frames[tg[t].iplane + 3];
    const double XO[3] = {X, Y, Z};
    double src[3] = {0, 0, 0};
    long ni = 0;
    if (ibctyp == 3 && T) {
      tree_calc_s(*T, 1, T->levmax, XO, F, src, ni);
      for (int c = 0; c < 3; ++c) sol[c][node] += src[c];
    } else if (ibctyp == 3) {
      double acc[3] = {sol[0][node], sol[1][node], sol[2][node]};
      for (int nv = 0; nv < P->nbound; ++nv) {
        const double RG[3] = {P->xc[nv], P->yc[nv], P->zc[nv]};
        const double FIS = fsour_a4(XO, RG, F, F.area);  // AREA of the target plane, as written
        ++ni;
        for (int c = 0; c < 3; ++c) acc[c] = acc[c] + FIS * P->src[c][nv];
      }
      for (int c = 0; c < 3; ++c) sol[c][node] = acc[c];
    } else if (T) {
      tree_calc(*T, 1, T->levmax, X, Y, Z, src, ni);
      for (int c = 0; c < 3; ++c) sol[c][node] += src[c] / PI4;
    } else {
      // direct sum; target-plane-dependent self term (h1 + h2) as in the reference
      const int plane = (i == 1 || i == NX) ? 2 : ((j == 1 || j == NY) ? 1 : 3);
      const double hsum = plane == 2 ? (DY + DZ) : (plane == 1 ? (DX + DZ) : (DX + DY));
      double acc[3] = {sol[0][node], sol[1][node], sol[2][node]};
      for (int nv = 0; nv < P->nbound; ++nv) {
        const double XR = P->xc[nv] - X, YR = P->yc[nv] - Y, ZR = P->zc[nv] - Z;
        const double r = std::sqrt(XR * XR + YR * YR + ZR * ZR);
        const double DS = P->ds[nv];
        ++ni;
        for (int c = 0; c < 3; ++c) {
          if (r > 1e-05) acc[c] = acc[c] - P->src[c][nv] * DS / (PI4 * r);
          else acc[c] = acc[c] + P->src[c][nv] * hsum * lg / PI4;
        }
      }
      for (int c = 0; c < 3; ++c) sol[c][node] = acc[c];
    }
    total += ni;
  }
  return total;
}

// pmesh (source/pmlib.f90:69-192), 3-D, ibctyp 2 or 3.
long g_last_interactions = 0;
int pmesh(double* const sol[3], double* const rhs[3], const double xb[6], const double D[3], const int NN[3],
          const int NN_bl[6], int iynbc, int itree, int levmax, int nthreads, int ibctyp = 2) {
  const int NX = NN[0], NY = NN[1], NZ = NN[2];
  if (iynbc == 1) {
    // infdomain_3d (source/pinfdomain.f90:86-158)
    std::vector<double> s0v[3];
    double* s0[3];
    for (int c = 0; c < 3; ++c) { s0v[c].assign((size_t)NX * NY * NZ, 0.0); s0[c] = s0v[c].data(); }
    const int full[6] = {1, 1, 1, NX, NY, NZ};
    for (int c = 0; c < 3; ++c) dirichlet(NX, NY, NZ, full, D, rhs[c], s0[c], true, nthreads);
    Panels P;
    normal_deriv(NX, NY, NZ, xb, D, s0, P);
    if (itree == 1) {
      Tree T;
      if (!build_tree(P, levmax, T)) return -3;
      g_last_interactions = bounds(NX, NY, NZ, xb, D, &T, nullptr, sol, nthreads, ibctyp);
    } else {
      g_last_interactions = bounds(NX, NY, NZ, xb, D, nullptr, &P, sol, nthreads, ibctyp);
    }
    for (int c = 0; c < 3; ++c) dirichlet(NX, NY, NZ, full, D, rhs[c], sol[c], false, nthreads);
  } else {
    for (int c = 0; c < 3; ++c) dirichlet(NX, NY, NZ, NN_bl, D, rhs[c], sol[c], false, nthreads);
  }
  return 0;
}

struct Scratch {
  int nn[3] = {0, 0, 0}, nnbl[3] = {0, 0, 0}, nnc[3] = {0, 0, 0};
  std::vector<double> rhs[3], sol[3], vel[3], def[3], bl_sol1[3], bl_final[3], c_rhs[3], c_sol[3];
};
Scratch g_scr;

}  // namespace

// ============================================================ C API =====
extern "C" {

double vpmo_projection_fun(int itype, double x) { return projection_fun(itype, x); }

void vpmo_definepm(int itype, double Xbound[6], double Dpm[3], int ndum, const int nsize[3], int NN[3],
                   int NN_bl[6]) {
  // source/pmlib.f90:216-432 with ND = 3 (itype 1 and 3 are the live paths)
  int ndum_new[3] = {ndum, ndum, ndum};
  if (itype == 1) {
    for (int d = 0; d < 3; ++d) {
      Xbound[d] = Xbound[d] - ((double)ndum_new[d] * Dpm[d]);
      Xbound[d + 3] = Xbound[d + 3] + ((double)ndum_new[d] * Dpm[d]);
    }
    for (int d = 0; d < 3; ++d) NN[d] = fnint(std::fabs(Xbound[d + 3] - Xbound[d]) / Dpm[d]) + 1;
    for (int d = 0; d < 3; ++d) { NN_bl[d] = ndum_new[d] + 1; NN_bl[d + 3] = NN[d] - ndum_new[d]; }
    return;
  }
  if (itype == 3) {
    for (int d = 0; d < 3; ++d) {
      Xbound[d] = Xbound[d] - ((double)ndum_new[d] * Dpm[d]);
      Xbound[d + 3] = Xbound[d + 3] + ((double)ndum_new[d] * Dpm[d]);
    }
    for (int d = 0; d < 3; ++d) NN[d] = fnint(std::fabs(Xbound[d + 3] - Xbound[d]) / Dpm[d]) + 1;
    for (int d = 0; d < 3; ++d) ndum_new[d] = nsize[d] - ((NN[d] - 1) % nsize[d]);
    for (int d = 0; d < 3; ++d) {
      if (ndum_new[d] % 2 == 0) {
        ndum_new[d] = ndum_new[d] / 2;
        Xbound[d] = Xbound[d] - ((double)ndum_new[d] * Dpm[d]);
        Xbound[d + 3] = Xbound[d + 3] + ((double)ndum_new[d] * Dpm[d]);
        NN[d] = fnint(std::fabs(Xbound[d + 3] - Xbound[d]) / Dpm[d]) + 1;
      } else {
        const int nn1 = ndum_new[d] % 2, nn2 = ndum_new[d] / 2;
        Xbound[d] = Xbound[d] - ((double)(nn1 + nn2) * Dpm[d]);
        Xbound[d + 3] = Xbound[d + 3] + ((double)nn2 * Dpm[d]);
        NN[d] = fnint(std::fabs(Xbound[d + 3] - Xbound[d]) / Dpm[d]) + 1;
      }
      NN_bl[d] = ndum + 1;
      NN_bl[d + 3] = NN[d] - ndum;
    }
    return;
  }
  // itype 2 / 4 are not on the 3-D single-block path
  for (int d = 0; d < 3; ++d) { NN[d] = 0; NN_bl[d] = NN_bl[d + 3] = 0; }
}

int vpmo_define_sizes(const vpmo_config* cfg, const double* xp, int nvr, int ntime, vpmo_sizes* s) {
  // source/vpm.f90:477-660; the sizes are block 1's, which all blocks share
  if (cfg->nbi < 1 || cfg->nbj < 1 || cfg->nbk < 1) return -2;
  const bool recompute = (ntime == 0 && cfg->idefine == 1) || cfg->idefine == 0 || !s->defined;
  if (recompute) {
    double Xb[6], Dpm[3] = {cfg->dpm[0], cfg->dpm[1], cfg->dpm[2]};
    int NN[3], NN_bl[6];
    if (cfg->use_box) {
      for (int d = 0; d < 6; ++d) Xb[d] = cfg->box[d];
      for (int d = 0; d < 3; ++d) {
        NN[d] = fnint(std::fabs(Xb[d + 3] - Xb[d]) / Dpm[d]) + 1;
        NN_bl[d] = 1; NN_bl[d + 3] = NN[d];
        if ((NN[d] - 1) % cfg->ncoarse != 0) return -4;
      }
    } else {
      if (nvr <= 0) return -1;
      double mn[3] = {xp[0], xp[1], xp[2]}, mx[3] = {xp[0], xp[1], xp[2]};
      for (int p = 1; p < nvr; ++p)
        for (int d = 0; d < 3; ++d) { mn[d] = std::min(mn[d], xp[3 * (size_t)p + d]); mx[d] = std::max(mx[d], xp[3 * (size_t)p + d]); }
      for (int d = 0; d < 3; ++d) {
        Xb[d] = mn[d] - (double)cfg->interf_iproj * cfg->dpm[d];
        Xb[d + 3] = mx[d] + (double)cfg->interf_iproj * cfg->dpm[d];
      }
      const int nsiz[3] = {cfg->nbi * cfg->ncoarse, cfg->nbj * cfg->ncoarse, cfg->nbk * cfg->ncoarse};
      vpmo_definepm(3, Xb, Dpm, 0, nsiz, NN, NN_bl);
    }
    for (int d = 0; d < 6; ++d) s->xbound[d] = Xb[d];
    for (int d = 0; d < 3; ++d) { s->dpm[d] = Dpm[d]; s->nn[d] = NN[d]; }
    for (int d = 0; d < 6; ++d) s->nn_bl[d] = NN_bl[d];
  }
  // block grid (vpm.f90:556-596), nb = 1
  const double* Xb = s->xbound;
  const double* Dpm = s->dpm;
  int NXB = fnint((Xb[3] - Xb[0]) / Dpm[0]), NYB = fnint((Xb[4] - Xb[1]) / Dpm[1]), NZB = fnint((Xb[5] - Xb[2]) / Dpm[2]);
  int NXbl = NXB / cfg->nbi, NYbl = NYB / cfg->nbj, NZbl = NZB / cfg->nbk;
  double Xt[6];
  Xt[0] = Xb[0] + (double)(0 * NXbl) * Dpm[0]; Xt[3] = Xb[0] + (double)(1 * NXbl) * Dpm[0];
  Xt[1] = Xb[1] + (double)(0 * NYbl) * Dpm[1]; Xt[4] = Xb[1] + (double)(1 * NYbl) * Dpm[1];
  Xt[2] = Xb[2] + (double)(0 * NZbl) * Dpm[2]; Xt[5] = Xb[2] + (double)(1 * NZbl) * Dpm[2];
  double Dt[3] = {Dpm[0], Dpm[1], Dpm[2]};
  const int nsb[3] = {cfg->ncoarse, cfg->ncoarse, cfg->ncoarse};
  vpmo_definepm(1, Xt, Dt, cfg->ncoarse, nsb, s->nnbl, s->nnbl_bl);
  for (int d = 0; d < 6; ++d) s->xbound_bl[d] = Xt[d];
  // coarse grid (vpm.f90:602-612)
  for (int d = 0; d < 6; ++d) s->xbound_coarse[d] = Xb[d];
  for (int d = 0; d < 3; ++d) s->dpm_coarse[d] = (double)cfg->ncoarse * Dpm[d];
  const int ns2 = 1 << cfg->ilevmax;
  const int nsc[3] = {ns2, ns2, ns2};
  vpmo_definepm(1, s->xbound_coarse, s->dpm_coarse, 4, nsc, s->nn_coarse, s->nn_bl_coarse);
  // level clamp (vpm.f90:627-652)
  int ilev = cfg->ilevmax;
  for (int lev = 0; lev <= ilev; ++lev) {
    const int istep = 1 << lev;
    if ((s->nnbl_bl[3] - s->nnbl_bl[0]) / istep == 0 || (s->nnbl_bl[4] - s->nnbl_bl[1]) / istep == 0 ||
        (s->nnbl_bl[5] - s->nnbl_bl[2]) / istep == 0) { ilev = lev - 1; break; }
  }
  s->ilevmax = ilev;
  s->dvpm = Dpm[0] * Dpm[1] * Dpm[2];
  s->defined = 1;
  return 0;
}

int vpmo_project_particles(const vpmo_sizes* s, int itype, const double* xp, const double* qp, int nvr,
                           double* rhs0, double* rhs1, double* rhs2, int nthreads) {
  // project_particles_3D (pmproject.f90:43-98) then project_vol3d IDVPM=1 (:136-148).
  // Row 4 (volume) is overwritten by DVpm in project_vol3d, so it is not deposited.
  const int NX = s->nn[0], NY = s->nn[1], NZ = s->nn[2];
  const double XMIN = s->xbound[0], YMIN = s->xbound[1], ZMIN = s->xbound[2];
  const double DX = s->dpm[0], DY = s->dpm[1], DZ = s->dpm[2];
  double* R[3] = {rhs0, rhs1, rhs2};
  const size_t N = (size_t)NX * NY * NZ;
  for (int c = 0; c < 3; ++c) std::fill(R[c], R[c] + N, 0.0);
  const int ips = (itype == 2) ? 0 : 1, ipf = (itype == 2) ? 1 : 2;
  int err = 0;
  for (int nv = 0; nv < nvr; ++nv) {
    const double px = xp[3 * (size_t)nv], py = xp[3 * (size_t)nv + 1], pz = xp[3 * (size_t)nv + 2];
    const int inode = (int)((px - XMIN) / DX) + 1, jnode = (int)((py - YMIN) / DY) + 1, knode = (int)((pz - ZMIN) / DZ) + 1;
    for (int k = knode - ips; k <= knode + ipf; ++k)
      for (int j = jnode - ips; j <= jnode + ipf; ++j)
        for (int i = inode - ips; i <= inode + ipf; ++i) {
          const double x = (px - XMIN - (double)(i - 1) * DX) / DX;
          const double fx = projection_fun(itype, x);
          const double y = (py - YMIN - (double)(j - 1) * DY) / DY;
          const double fy = projection_fun(itype, y);
          const double z = (pz - ZMIN - (double)(k - 1) * DZ) / DZ;
          const double fz = projection_fun(itype, z);
          const double f = fx * fy * fz;
          if (i < 1 || i > NX || j < 1 || j > NY || k < 1 || k > NZ) { err = -1; continue; }
          const size_t id = lin(NX, NY, i, j, k);
          for (int c = 0; c < 3; ++c) R[c][id] = R[c][id] + f * qp[4 * (size_t)nv + c];
        }
  }
  const double DV = DX * DY * DZ;
  (void)nthreads;
  for (int c = 0; c < 3; ++c)
    for (size_t n = 0; n < N; ++n) R[c][n] = R[c][n] / DV;
  return err;
}

void vpmo_dirichlet(int nx, int ny, int nz, const int box[6], const double d[3], const double* rhs, double* sol,
                    int zero_bc, int nthreads) {
  dirichlet(nx, ny, nz, box, d, rhs, sol, zero_bc != 0, nthreads);
}

int vpmo_pmesh(double* const sol[3], double* const rhs[3], const double xbound[6], const double dpm[3],
               const int nn[3], const int nn_bl[6], int iynbc, int itree, int levmax, int nthreads) {
  return pmesh(sol, rhs, xbound, dpm, nn, nn_bl, iynbc, itree, levmax, nthreads);
}

int vpmo_pmesh_bc(double* const sol[3], double* const rhs[3], const double xbound[6], const double dpm[3],
                  const int nn[3], const int nn_bl[6], int iynbc, int itree, int levmax, int nthreads, int ibctyp) {
  if (ibctyp != 2 && ibctyp != 3) return -6;
  return pmesh(sol, rhs, xbound, dpm, nn, nn_bl, iynbc, itree, levmax, nthreads, ibctyp);
}

long vpmo_boundary_values_bc(double* const sol0[3], double* const bnd[3], const double xb[6], const double D[3],
                             const int nn[3], int levmax, int direct, int nthreads, int ibctyp) {
  if (ibctyp != 2 && ibctyp != 3) return -6;
  Panels P;
  normal_deriv(nn[0], nn[1], nn[2], xb, D, sol0, P);
  if (direct) return bounds(nn[0], nn[1], nn[2], xb, D, nullptr, &P, bnd, nthreads, ibctyp);
  Tree T;
  if (!build_tree(P, levmax, T)) return -3;
  return bounds(nn[0], nn[1], nn[2], xb, D, &T, nullptr, bnd, nthreads, ibctyp);
}

long vpmo_boundary_values(double* const sol0[3], double* const bnd[3], const double xb[6], const double D[3],
                          const int nn[3], int levmax, int direct, int nthreads) {
  return vpmo_boundary_values_bc(sol0, bnd, xb, D, nn, levmax, direct, nthreads, 2);
}

double vpmo_fsour_a4(const double xo[3], const double rg[3], int iplane, const double dpm[3], double area) {
  return fsour_a4(xo, rg, make_frame(iplane, dpm), area);
}

// yaps3d (source/yaps3d.f90:1-453) for NBI x NBJ x NBK blocks, the blocks
// run one after the other as the ranks would; with rhsscat_3d and
// solget_3d (source/vpm_mpi.f90:199-328).  Writes the global SOL into W.sol.
static double g_yaps_seam = 0.0;
static int yaps_multi(const vpmo_config* cfg, const vpmo_sizes* s, Scratch& W, int nthreads) {
  const int NBI = cfg->nbi, NBJ = cfg->nbj, NBK = cfg->nbk, B = NBI * NBJ * NBK;
  const int NX = s->nn[0], NY = s->nn[1];
  const int BX = s->nnbl[0], BY = s->nnbl[1], BZ = s->nnbl[2];
  const size_t NB = (size_t)BX * BY * BZ;
  const int CX = s->nn_coarse[0], CY = s->nn_coarse[1], CZ = s->nn_coarse[2];
  const size_t NC = (size_t)CX * CY * CZ;
  const int* nbb = s->nnbl_bl;
  const int NXs = nbb[0], NYs = nbb[1], NZs = nbb[2], NXf = nbb[3], NYf = nbb[4], NZf = nbb[5];
  const int nc = cfg->ncoarse;
  const double* Xb = s->xbound;
  const double* D = s->dpm;
  // block boxes (vpm.f90:561-596): all blocks have the sizes of block 1
  const int NXbl = fnint((Xb[3] - Xb[0]) / D[0]) / NBI, NYbl = fnint((Xb[4] - Xb[1]) / D[1]) / NBJ,
            NZbl = fnint((Xb[5] - Xb[2]) / D[2]) / NBK;
  std::vector<double> xbl(6 * (size_t)B);
  for (int k = 1; k <= NBK; ++k)
    for (int j = 1; j <= NBJ; ++j)
      for (int i = 1; i <= NBI; ++i) {
        const int nb = (k - 1) * NBJ * NBI + (j - 1) * NBI + i;
        double Xt[6] = {Xb[0] + (double)((i - 1) * NXbl) * D[0], Xb[1] + (double)((j - 1) * NYbl) * D[1],
                        Xb[2] + (double)((k - 1) * NZbl) * D[2], Xb[0] + (double)(i * NXbl) * D[0],
                        Xb[1] + (double)(j * NYbl) * D[1], Xb[2] + (double)(k * NZbl) * D[2]};
        double Dt[3] = {D[0], D[1], D[2]};
        const int nsb[3] = {nc, nc, nc};
        int nnt[3], nnbt[6];
        vpmo_definepm(1, Xt, Dt, nc, nsb, nnt, nnbt);
        for (int d = 0; d < 3; ++d)
          if (nnt[d] != s->nnbl[d]) return -7;
        for (int d = 0; d < 6; ++d) xbl[6 * (size_t)(nb - 1) + d] = Xt[d];
      }
  auto coords = [&](int nb, int& bi, int& bj, int& bk) {  // 1-based block position of block nb (1-based)
    bi = (nb - 1) % NBI + 1; bj = ((nb - 1) / NBI) % NBJ + 1; bk = (nb - 1) / (NBI * NBJ) + 1;
  };
  std::vector<std::vector<double>> rbl((size_t)B * 3), sbl((size_t)B * 3);
  for (int b = 0; b < B; ++b) {
    int bi, bj, bk;
    coords(b + 1, bi, bj, bk);
    // rhsscat_3d
    const int ixs = (bi - 1) * (NXf - NXs) + s->nn_bl[0], jxs = (bj - 1) * (NYf - NYs) + s->nn_bl[1],
              kxs = (bk - 1) * (NZf - NZs) + s->nn_bl[2];
    for (int c = 0; c < 3; ++c) {
      std::vector<double>& R = rbl[3 * b + c];
      R.assign(NB, 0.0);
      sbl[3 * b + c].assign(NB, 0.0);
      for (int k = NZs; k <= NZf; ++k)
        for (int j = NYs; j <= NYf; ++j)
          for (int i = NXs; i <= NXf; ++i)
            R[lin(BX, BY, i, j, k)] = W.rhs[c][lin(NX, NY, ixs + i - NXs, jxs + j - NYs, kxs + k - NZs)];
      for (int k = 1; k <= BZ; ++k)
        for (int j = 1; j <= BY; ++j)
          for (int i = 1; i <= BX; ++i)
            if ((bi > 1 && i == NXs) || (bj > 1 && j == NYs) || (bk > 1 && k == NZs)) R[lin(BX, BY, i, j, k)] = 0.0;
    }
    // pmesh(iynbc = 1) on the padded block
    double* sp[3] = {sbl[3 * b].data(), sbl[3 * b + 1].data(), sbl[3 * b + 2].data()};
    double* rp[3] = {rbl[3 * b].data(), rbl[3 * b + 1].data(), rbl[3 * b + 2].data()};
    const int e = pmesh(sp, rp, &xbl[6 * (size_t)b], s->dpm, s->nnbl, s->nnbl_bl, 1, cfg->iyntree, s->ilevmax,
                        nthreads, cfg->ibctyp);
    if (e) return e;
  }
  // sampling and map_nodes of every block (yaps3d.f90:104-138)
  std::vector<std::vector<double>> samp((size_t)B * 3);
  std::vector<std::vector<char>> mapn(B);
  std::vector<int> cmap(6 * (size_t)B, -1);
  for (int b = 0; b < B; ++b) {
    for (int c = 0; c < 3; ++c) samp[3 * b + c].assign(NC, 0.0);
    mapn[b].assign(NC, 0);
    const double* xb = &xbl[6 * (size_t)b];
    int* mp = &cmap[6 * (size_t)b];
    for (int k = 1; k <= BZ; k += nc)
      for (int j = 1; j <= BY; j += nc)
        for (int i = 1; i <= BX; i += nc) {
          const double X0 = xb[0] + (double)(i - 1) * s->dpm[0];
          const double X1 = xb[1] + (double)(j - 1) * s->dpm[1];
          const double X2 = xb[2] + (double)(k - 1) * s->dpm[2];
          const int in = fnint((X0 - s->xbound_coarse[0]) / s->dpm_coarse[0]) + 1;
          const int jn = fnint((X1 - s->xbound_coarse[1]) / s->dpm_coarse[1]) + 1;
          const int kn = fnint((X2 - s->xbound_coarse[2]) / s->dpm_coarse[2]) + 1;
          if (i == 1) mp[0] = in;
          if (i == BX) mp[3] = in;
          if (j == 1) mp[1] = jn;
          if (j == BY) mp[4] = jn;
          if (k == 1) mp[2] = kn;
          if (k == BZ) mp[5] = kn;
          if (in < 1 || in > CX || jn < 1 || jn > CY || kn < 1 || kn > CZ) return -5;
          for (int c = 0; c < 3; ++c) samp[3 * b + c][lin(CX, CY, in, jn, kn)] = sbl[3 * b + c][lin(BX, BY, i, j, k)];
          mapn[b][lin(CX, CY, in, jn, kn)] = 1;
        }
  }
  // coarse RHS: sum over blocks of calc_laplacian_coarse_3d inside each map (yaps3d.f90:254-261, 1990-2016)
  const double dc2[3] = {s->dpm_coarse[0] * s->dpm_coarse[0], s->dpm_coarse[1] * s->dpm_coarse[1],
                         s->dpm_coarse[2] * s->dpm_coarse[2]};
  for (int c = 0; c < 3; ++c) W.c_rhs[c].assign(NC, 0.0);
  for (int b = 0; b < B; ++b) {
    const int* mp = &cmap[6 * (size_t)b];
    for (int c = 0; c < 3; ++c) {
      const std::vector<double>& S = samp[3 * b + c];
      auto Sm = [&](int i, int j, int k) { return S[lin(CX, CY, i, j, k)]; };
      std::vector<double> tmp(NC, 0.0);
      for (int k = mp[2] + 1; k <= mp[5] - 1; ++k)
        for (int j = mp[1] + 1; j <= mp[4] - 1; ++j)
          for (int i = mp[0] + 1; i <= mp[3] - 1; ++i)
            tmp[lin(CX, CY, i, j, k)] = ((Sm(i + 1, j, k) - 2.0 * Sm(i, j, k)) + Sm(i - 1, j, k)) / dc2[0] +
                                        ((Sm(i, j + 1, k) - 2.0 * Sm(i, j, k)) + Sm(i, j - 1, k)) / dc2[1] +
                                        ((Sm(i, j, k + 1) - 2.0 * Sm(i, j, k)) + Sm(i, j, k - 1)) / dc2[2];
      for (size_t n = 0; n < NC; ++n) W.c_rhs[c][n] = W.c_rhs[c][n] + tmp[n];
    }
  }
  // coarse infinite-domain solve (yaps3d.f90:286-299)
  {
    for (int c = 0; c < 3; ++c) W.c_sol[c].assign(NC, 0.0);
    double* cs[3] = {W.c_sol[0].data(), W.c_sol[1].data(), W.c_sol[2].data()};
    double* cr[3] = {W.c_rhs[0].data(), W.c_rhs[1].data(), W.c_rhs[2].data()};
    const int itree = cfg->iyntree == 1 ? 1 : 0;
    const int lmax = itree ? s->ilevmax - 1 : 1;
    const int e = pmesh(cs, cr, s->xbound_coarse, s->dpm_coarse, s->nn_coarse, s->nn_bl_coarse, 1, itree, lmax,
                        nthreads, cfg->ibctyp);
    if (e) return e;
  }
  // mapnodes_bl (yaps3d.f90:457-1912): every block sends each of its 26
  // neighbours the values of its first solution at the neighbour's inner-face
  // nodes that lie in its padded block, faces facing it only.  Restated from
  // the 26 transfers as one rule: along an axis with offset o = +1 (receiver
  // above the sender) the receiver range is [s, s+nc], o = -1 gives [f-nc, f],
  // o = 0 the inner range [s, f]; the sender index is the receiver's plus
  // o * (f - s); a face is sent when the offset along its normal is 0 or
  // points from the sender to it.  BBound(node, 1:3, sender) per receiver.
  const int isx = BX, isy = BY, isz = BZ;
  const int iface12 = isy * isz, iface34 = isx * isz, iface56 = isx * isy;
  const int ibound = 2 * (iface12 + iface34 + iface56);
  std::vector<double> bbound((size_t)B * B * ibound * 3, 0.0);  // [recv][sender][node][c]
  auto BBv = [&](int r, int snd, int node, int c) -> double& {
    return bbound[(((size_t)r * B + snd) * ibound + (node - 1)) * 3 + c];
  };
  const int lo[3] = {NXs, NYs, NZs}, hi[3] = {NXf, NYf, NZf};
  for (int sb = 1; sb <= B; ++sb) {
    int si, sj, sk;
    coords(sb, si, sj, sk);
    for (int oz = -1; oz <= 1; ++oz)
      for (int oy = -1; oy <= 1; ++oy)
        for (int ox = -1; ox <= 1; ++ox) {
          if (!ox && !oy && !oz) continue;
          const int ri = si + ox, rj = sj + oy, rk = sk + oz;
          if (ri < 1 || ri > NBI || rj < 1 || rj > NBJ || rk < 1 || rk > NBK) continue;
          const int rb = (rk - 1) * NBJ * NBI + (rj - 1) * NBI + ri;
          const int o[3] = {ox, oy, oz};
          auto range = [&](int d, int& a, int& z) {
            if (o[d] > 0) { a = lo[d]; z = lo[d] + nc; }
            else if (o[d] < 0) { a = hi[d] - nc; z = hi[d]; }
            else { a = lo[d]; z = hi[d]; }
          };
          for (int face = 0; face < 6; ++face) {
            const int ax = face / 2, side = face % 2;  // side 0: min face, 1: max face
            if (side == 0 && o[ax] < 0) continue;
            if (side == 1 && o[ax] > 0) continue;
            const int plane = side == 0 ? lo[ax] : hi[ax];
            const int u = ax == 0 ? 1 : 0, v = ax == 2 ? 1 : 2;  // in-plane axes, u fastest
            int ua, uz, va, vz;
            range(u, ua, uz);
            range(v, va, vz);
            const int nodstart = ax == 0 ? side * iface12 : (ax == 1 ? 2 * iface12 + side * iface34
                                                                     : 2 * iface12 + 2 * iface34 + side * iface56);
            const int ustride = ax == 0 ? isy : isx;
            for (int vv = va; vv <= vz; ++vv)
              for (int uu = ua; uu <= uz; ++uu) {
                int rcv[3];
                rcv[ax] = plane; rcv[u] = uu; rcv[v] = vv;
                int snd[3];
                for (int d = 0; d < 3; ++d) snd[d] = rcv[d] + o[d] * (hi[d] - lo[d]);
                const int node = nodstart + (vv - 1) * ustride + uu;
                for (int c = 0; c < 3; ++c)
                  BBv(rb - 1, sb - 1, node, c) = BBv(rb - 1, sb - 1, node, c) +
                                                 sbl[3 * (sb - 1) + c][lin(BX, BY, snd[0], snd[1], snd[2])];
              }
          }
        }
  }
  // interp_stencil on every block's inner faces (yaps3d.f90:340-395, 1914-1983)
  for (int nb = 1; nb <= B; ++nb) {
    int bi, bj, bk;
    coords(nb, bi, bj, bk);
    const double* xb = &xbl[6 * (size_t)(nb - 1)];
    std::vector<double>* S = &sbl[3 * (size_t)(nb - 1)];
    std::vector<int> nnb(B);
    auto interp = [&](int i, int j, int k, int node) {
      const double X0 = xb[0] + (double)(i - 1) * s->dpm[0];
      const double X1 = xb[1] + (double)(j - 1) * s->dpm[1];
      const double X2 = xb[2] + (double)(k - 1) * s->dpm[2];
      const int in = fnint((X0 - s->xbound_coarse[0]) / s->dpm_coarse[0]) + 1;
      const int jn = fnint((X1 - s->xbound_coarse[1]) / s->dpm_coarse[1]) + 1;
      const int kn = fnint((X2 - s->xbound_coarse[2]) / s->dpm_coarse[2]) + 1;
      for (int b = 0; b < B; ++b)
        nnb[b] = !(mapn[b][lin(CX, CY, in - 1, jn - 1, kn - 1)] == 1 && mapn[b][lin(CX, CY, in + 1, jn + 1, kn + 1)] == 1);
      for (int kc = kn - 1; kc <= kn + 1; ++kc)
        for (int jc = jn - 1; jc <= jn + 1; ++jc)
          for (int ic = in - 1; ic <= in + 1; ++ic) {
            const size_t cid = lin(CX, CY, ic, jc, kc);
            double add[3] = {0, 0, 0}, add_sample[3] = {0, 0, 0};
            for (int b = 0; b < B; ++b)
              for (int c = 0; c < 3; ++c) {
                add_sample[c] = samp[3 * b + c][cid] + add_sample[c];
                if (nnb[b] == 1) add[c] = samp[3 * b + c][cid] + add[c];
              }
            const double xc = (X0 - s->xbound_coarse[0] - (double)(ic - 1) * s->dpm_coarse[0]) / s->dpm_coarse[0];
            const double fx = projection_fun(3, xc);
            const double yc = (X1 - s->xbound_coarse[1] - (double)(jc - 1) * s->dpm_coarse[1]) / s->dpm_coarse[1];
            const double fy = projection_fun(3, yc);
            const double zc = (X2 - s->xbound_coarse[2] - (double)(kc - 1) * s->dpm_coarse[2]) / s->dpm_coarse[2];
            const double fz = projection_fun(3, zc);
            const double f = fx * fy * fz;
            for (int c = 0; c < 3; ++c) {
              double& v = S[c][lin(BX, BY, i, j, k)];
              v = v + f * ((W.c_sol[c][cid] - add_sample[c]) + add[c]);
            }
          }
      for (int kb = bk - 1; kb <= bk + 1; ++kb)
        for (int jb = bj - 1; jb <= bj + 1; ++jb)
          for (int ib = bi - 1; ib <= bi + 1; ++ib) {
            if (ib < 1 || ib > NBI || jb < 1 || jb > NBJ || kb < 1 || kb > NBK) continue;
            const int nbc = (kb - 1) * NBI * NBJ + (jb - 1) * NBI + ib;
            if (nnb[nbc - 1] == 1 || nbc == nb) continue;
            for (int c = 0; c < 3; ++c) {
              double& v = S[c][lin(BX, BY, i, j, k)];
              v = v + BBv(nb - 1, nbc - 1, node, c);
            }
          }
    };
    // BBound is read from the first solutions: interp_stencil of every block
    // runs after mapnodes_bl has copied them, so updating S here is safe.
    for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) interp(NXs, j, k, (k - 1) * isy + j);
    for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) interp(NXf, j, k, iface12 + (k - 1) * isy + j);
    for (int k = NZs; k <= NZf; ++k)
      for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, NYs, k, 2 * iface12 + (k - 1) * isx + i);
    for (int k = NZs; k <= NZf; ++k)
      for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, NYf, k, 2 * iface12 + iface34 + (k - 1) * isx + i);
    for (int j = NYs + 1; j <= NYf - 1; ++j)
      for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, j, NZs, 2 * iface12 + 2 * iface34 + (j - 1) * isx + i);
    for (int j = NYs + 1; j <= NYf - 1; ++j)
      for (int i = NXs + 1; i <= NXf - 1; ++i)
        interp(i, j, NZf, 2 * iface12 + 2 * iface34 + iface56 + (j - 1) * isx + i);
  }
  // seam check: nodes shared by the inner faces of several blocks must get
  // the same boundary value from every block (same terms, other order)
  {
    std::vector<double> first(3 * (size_t)W.rhs[0].size(), 0.0);
    std::vector<char> seen(W.rhs[0].size(), 0);
    double worst = 0.0, scale = 0.0;
    for (int b = 0; b < B; ++b) {
      int bi, bj, bk;
      coords(b + 1, bi, bj, bk);
      const int ixs = (bi - 1) * (NXf - NXs) + s->nn_bl[0], jxs = (bj - 1) * (NYf - NYs) + s->nn_bl[1],
                kxs = (bk - 1) * (NZf - NZs) + s->nn_bl[2];
      for (int k = NZs; k <= NZf; ++k)
        for (int j = NYs; j <= NYf; ++j)
          for (int i = NXs; i <= NXf; ++i) {
            if (i != NXs && i != NXf && j != NYs && j != NYf && k != NZs && k != NZf) continue;
            const size_t g = lin(NX, NY, ixs + i - NXs, jxs + j - NYs, kxs + k - NZs);
            for (int c = 0; c < 3; ++c) {
              const double v = sbl[3 * b + c][lin(BX, BY, i, j, k)];
              scale = std::max(scale, std::fabs(v));
              if (seen[g]) worst = std::max(worst, std::fabs(v - first[3 * g + c]));
              else first[3 * g + c] = v;
            }
            seen[g] = 1;
          }
    }
    g_yaps_seam = scale > 0 ? worst / scale : 0.0;
  }
  // final Dirichlet solve on each inner box (yaps3d.f90:415-421), then solget_3d in block order
  for (int b = 0; b < B; ++b) {
    double* sp[3] = {sbl[3 * b].data(), sbl[3 * b + 1].data(), sbl[3 * b + 2].data()};
    double* rp[3] = {rbl[3 * b].data(), rbl[3 * b + 1].data(), rbl[3 * b + 2].data()};
    const int e = pmesh(sp, rp, &xbl[6 * (size_t)b], s->dpm, s->nnbl, s->nnbl_bl, 0, 0, 0, nthreads);
    if (e) return e;
  }
  for (int b = 0; b < B; ++b) {
    int bi, bj, bk;
    coords(b + 1, bi, bj, bk);
    const int ixs = (bi - 1) * (NXf - NXs) + s->nn_bl[0], jxs = (bj - 1) * (NYf - NYs) + s->nn_bl[1],
              kxs = (bk - 1) * (NZf - NZs) + s->nn_bl[2];
    for (int c = 0; c < 3; ++c)
      for (int k = NZs; k <= NZf; ++k)
        for (int j = NYs; j <= NYf; ++j)
          for (int i = NXs; i <= NXf; ++i)
            W.sol[c][lin(NX, NY, ixs + i - NXs, jxs + j - NYs, kxs + k - NZs)] = sbl[3 * b + c][lin(BX, BY, i, j, k)];
  }
  if (B >= 1) {  // block 1's fields for vpmo_get_field
    for (int c = 0; c < 3; ++c) W.bl_final[c] = sbl[c];
  }
  return 0;
}

double vpmo_yaps_seam(void) { return g_yaps_seam; }

int vpmo_step_fields(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, double* up,
                     double* gp, int nvr, int nthreads) {
  Scratch& W = g_scr;
  const int NX = s->nn[0], NY = s->nn[1], NZ = s->nn[2];
  const size_t N = (size_t)NX * NY * NZ;
  const int BX = s->nnbl[0], BY = s->nnbl[1], BZ = s->nnbl[2];
  const size_t NB = (size_t)BX * BY * BZ;
  const int CX = s->nn_coarse[0], CY = s->nn_coarse[1], CZ = s->nn_coarse[2];
  const size_t NC = (size_t)CX * CY * CZ;
  for (int d = 0; d < 3; ++d) { W.nn[d] = s->nn[d]; W.nnbl[d] = s->nnbl[d]; W.nnc[d] = s->nn_coarse[d]; }
  for (int c = 0; c < 3; ++c) {
    W.rhs[c].assign(N, 0.0); W.sol[c].assign(N, 0.0); W.vel[c].assign(N, 0.0); W.def[c].assign(N, 0.0);
    W.bl_sol1[c].assign(NB, 0.0); W.bl_final[c].assign(NB, 0.0); W.c_rhs[c].assign(NC, 0.0); W.c_sol[c].assign(NC, 0.0);
  }
  // 1. deposition + volume division (vpm.f90:408-444)
  int e = vpmo_project_particles(s, cfg->interf_iproj, xp, qp, nvr, W.rhs[0].data(), W.rhs[1].data(), W.rhs[2].data(), nthreads);
  if (e) return e;
  if (cfg->nbi * cfg->nbj * cfg->nbk > 1) {
    e = yaps_multi(cfg, s, W, nthreads);
    if (e) return e;
  } else {
  // 2. rhsscat_3d (vpm_mpi.f90:199-238), one block
  std::vector<double> rbl[3], sbl[3];
  for (int c = 0; c < 3; ++c) { rbl[c].assign(NB, 0.0); sbl[c].assign(NB, 0.0); }
  const int* nbb = s->nnbl_bl;
  for (int c = 0; c < 3; ++c)
    for (int k = nbb[2]; k <= nbb[5]; ++k)
      for (int j = nbb[1]; j <= nbb[4]; ++j)
        for (int i = nbb[0]; i <= nbb[3]; ++i)
          rbl[c][lin(BX, BY, i, j, k)] = W.rhs[c][lin(NX, NY, i - nbb[0] + s->nn_bl[0], j - nbb[1] + s->nn_bl[1], k - nbb[2] + s->nn_bl[2])];
  // 3. yaps3d (yaps3d.f90:1-453), one block
  double* sp[3] = {sbl[0].data(), sbl[1].data(), sbl[2].data()};
  double* rp[3] = {rbl[0].data(), rbl[1].data(), rbl[2].data()};
  e = pmesh(sp, rp, s->xbound_bl, s->dpm, s->nnbl, s->nnbl_bl, 1, cfg->iyntree, s->ilevmax, nthreads, cfg->ibctyp);
  if (e) return e;
  for (int c = 0; c < 3; ++c) W.bl_sol1[c] = sbl[c];
  // 3b. sampling every nc-th node (yaps3d.f90:104-138)
  const int nc = cfg->ncoarse;
  std::vector<double> samp[3];
  for (int c = 0; c < 3; ++c) samp[c].assign(NC, 0.0);
  std::vector<char> mapn(NC, 0);
  int map[6] = {-1, -1, -1, -1, -1, -1};
  for (int k = 1; k <= BZ; k += nc)
    for (int j = 1; j <= BY; j += nc)
      for (int i = 1; i <= BX; i += nc) {
        const double X0 = s->xbound_bl[0] + (double)(i - 1) * s->dpm[0];
        const double X1 = s->xbound_bl[1] + (double)(j - 1) * s->dpm[1];
        const double X2 = s->xbound_bl[2] + (double)(k - 1) * s->dpm[2];
        const int in = fnint((X0 - s->xbound_coarse[0]) / s->dpm_coarse[0]) + 1;
        const int jn = fnint((X1 - s->xbound_coarse[1]) / s->dpm_coarse[1]) + 1;
        const int kn = fnint((X2 - s->xbound_coarse[2]) / s->dpm_coarse[2]) + 1;
        if (i == 1) map[0] = in;
        if (i == BX) map[3] = in;
        if (j == 1) map[1] = jn;
        if (j == BY) map[4] = jn;
        if (k == 1) map[2] = kn;
        if (k == BZ) map[5] = kn;
        if (in < 1 || in > CX || jn < 1 || jn > CY || kn < 1 || kn > CZ) return -5;
        for (int c = 0; c < 3; ++c) samp[c][lin(CX, CY, in, jn, kn)] = sbl[c][lin(BX, BY, i, j, k)];
        mapn[lin(CX, CY, in, jn, kn)] = 1;
      }
  // 3c. coarse RHS = 7-point Laplacian of the samples (yaps3d.f90:1990-2016)
  const double dc2[3] = {s->dpm_coarse[0] * s->dpm_coarse[0], s->dpm_coarse[1] * s->dpm_coarse[1], s->dpm_coarse[2] * s->dpm_coarse[2]};
  for (int c = 0; c < 3; ++c) {
    auto Sm = [&](int i, int j, int k) { return samp[c][lin(CX, CY, i, j, k)]; };
    for (int k = map[2] + 1; k <= map[5] - 1; ++k)
      for (int j = map[1] + 1; j <= map[4] - 1; ++j)
        for (int i = map[0] + 1; i <= map[3] - 1; ++i)
          W.c_rhs[c][lin(CX, CY, i, j, k)] =
              ((Sm(i + 1, j, k) - 2.0 * Sm(i, j, k)) + Sm(i - 1, j, k)) / dc2[0] +
              ((Sm(i, j + 1, k) - 2.0 * Sm(i, j, k)) + Sm(i, j - 1, k)) / dc2[1] +
              ((Sm(i, j, k + 1) - 2.0 * Sm(i, j, k)) + Sm(i, j, k - 1)) / dc2[2];
  }
  // 3d. coarse infinite-domain solve (yaps3d.f90:286-299)
  {
    double* cs[3] = {W.c_sol[0].data(), W.c_sol[1].data(), W.c_sol[2].data()};
    double* cr[3] = {W.c_rhs[0].data(), W.c_rhs[1].data(), W.c_rhs[2].data()};
    const int itree = cfg->iyntree == 1 ? 1 : 0;
    const int lmax = itree ? s->ilevmax - 1 : 1;
    e = pmesh(cs, cr, s->xbound_coarse, s->dpm_coarse, s->nn_coarse, s->nn_bl_coarse, 1, itree, lmax, nthreads, cfg->ibctyp);
    if (e) return e;
  }
  // 3e. interp_stencil on the inner-box faces (yaps3d.f90:340-395, 1914-1983), one block:
  // SOL_bl += sum TSC * (SOL_coarse - sample); nnb = 0 since the 3x3x3 stencil stays inside the map.
  {
    const int NXs = nbb[0], NXf = nbb[3], NYs = nbb[1], NYf = nbb[4], NZs = nbb[2], NZf = nbb[5];
    auto interp = [&](int i, int j, int k) {
      const double X0 = s->xbound_bl[0] + (double)(i - 1) * s->dpm[0];
      const double X1 = s->xbound_bl[1] + (double)(j - 1) * s->dpm[1];
      const double X2 = s->xbound_bl[2] + (double)(k - 1) * s->dpm[2];
      const int in = fnint((X0 - s->xbound_coarse[0]) / s->dpm_coarse[0]) + 1;
      const int jn = fnint((X1 - s->xbound_coarse[1]) / s->dpm_coarse[1]) + 1;
      const int kn = fnint((X2 - s->xbound_coarse[2]) / s->dpm_coarse[2]) + 1;
      const bool flagged = !(mapn[lin(CX, CY, in - 1, jn - 1, kn - 1)] == 1 && mapn[lin(CX, CY, in + 1, jn + 1, kn + 1)] == 1);
      for (int kc = kn - 1; kc <= kn + 1; ++kc)
        for (int jc = jn - 1; jc <= jn + 1; ++jc)
          for (int ic = in - 1; ic <= in + 1; ++ic) {
            const double xc = (X0 - s->xbound_coarse[0] - (double)(ic - 1) * s->dpm_coarse[0]) / s->dpm_coarse[0];
            const double fx = projection_fun(3, xc);
            const double yc = (X1 - s->xbound_coarse[1] - (double)(jc - 1) * s->dpm_coarse[1]) / s->dpm_coarse[1];
            const double fy = projection_fun(3, yc);
            const double zc = (X2 - s->xbound_coarse[2] - (double)(kc - 1) * s->dpm_coarse[2]) / s->dpm_coarse[2];
            const double fz = projection_fun(3, zc);
            const double f = fx * fy * fz;
            const size_t cid = lin(CX, CY, ic, jc, kc);
            for (int c = 0; c < 3; ++c) {
              const double add_sample = 0.0 + samp[c][cid];
              const double add = flagged ? (0.0 + samp[c][cid]) : 0.0;
              double& v = sbl[c][lin(BX, BY, i, j, k)];
              v = v + f * ((W.c_sol[c][cid] - add_sample) + add);
            }
          }
    };
    for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) interp(NXs, j, k);
    for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) interp(NXf, j, k);
    for (int k = NZs; k <= NZf; ++k) for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, NYs, k);
    for (int k = NZs; k <= NZf; ++k) for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, NYf, k);
    for (int j = NYs + 1; j <= NYf - 1; ++j) for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, j, NZs);
    for (int j = NYs + 1; j <= NYf - 1; ++j) for (int i = NXs + 1; i <= NXf - 1; ++i) interp(i, j, NZf);
  }
  // 3f. final Dirichlet solve on the inner box (yaps3d.f90:415-421)
  e = pmesh(sp, rp, s->xbound_bl, s->dpm, s->nnbl, s->nnbl_bl, 0, 0, 0, nthreads);
  if (e) return e;
  for (int c = 0; c < 3; ++c) W.bl_final[c] = sbl[c];
  // 4. solget_3d (vpm_mpi.f90:240-328), one block
  for (int c = 0; c < 3; ++c)
    for (int k = nbb[2]; k <= nbb[5]; ++k)
      for (int j = nbb[1]; j <= nbb[4]; ++j)
        for (int i = nbb[0]; i <= nbb[3]; ++i)
          W.sol[c][lin(NX, NY, i - nbb[0] + s->nn_bl[0], j - nbb[1] + s->nn_bl[1], k - nbb[2] + s->nn_bl[2])] = sbl[c][lin(BX, BY, i, j, k)];
  }
  // 5. calc_velocity_serial_3d(1) (vpm_gcalc.f90:1-136)
  {
    const double DX2 = 2 * s->dpm[0], DY2 = 2 * s->dpm[1], DZ2 = 2 * s->dpm[2];
    const int* nb = s->nn_bl;
    auto SO = [&](int c, int i, int j, int k) { return W.sol[c][lin(NX, NY, i, j, k)]; };
    for (int k = nb[2] + 1; k <= nb[5] - 1; ++k)
      for (int j = nb[1] + 1; j <= nb[4] - 1; ++j)
        for (int i = nb[0] + 1; i <= nb[3] - 1; ++i) {
          double dx[3], dy[3], dz[3];
          for (int c = 0; c < 3; ++c) {
            dx[c] = (SO(c, i + 1, j, k) - SO(c, i - 1, j, k)) / DX2;
            dy[c] = (SO(c, i, j + 1, k) - SO(c, i, j - 1, k)) / DY2;
            dz[c] = (SO(c, i, j, k + 1) - SO(c, i, j, k - 1)) / DZ2;
          }
          const size_t id = lin(NX, NY, i, j, k);
          W.vel[0][id] = W.vel[0][id] + dy[2] - dz[1];
          W.vel[1][id] = W.vel[1][id] - (dx[2] - dz[0]);
          W.vel[2][id] = W.vel[2][id] + dx[1] - dy[0];
        }
    auto V = [&](int c, int i, int j, int k) { return W.vel[c][lin(NX, NY, i, j, k)]; };
    auto RH = [&](int c, int i, int j, int k) { return W.rhs[c][lin(NX, NY, i, j, k)]; };
    for (int k = nb[2] + 2; k <= nb[5] - 2; ++k)
      for (int j = nb[1] + 2; j <= nb[4] - 2; ++j)
        for (int i = nb[0] + 2; i <= nb[3] - 2; ++i) {
          const size_t id = lin(NX, NY, i, j, k);
          for (int m = 0; m < 3; ++m) {
            const double wdudx = -(RH(0, i + 1, j, k) * V(m, i + 1, j, k) - RH(0, i - 1, j, k) * V(m, i - 1, j, k)) / DX2;
            const double wdvdy = -(RH(1, i, j + 1, k) * V(m, i, j + 1, k) - RH(1, i, j - 1, k) * V(m, i, j - 1, k)) / DY2;
            const double wdwdz = -(RH(2, i, j, k + 1) * V(m, i, j, k + 1) - RH(2, i, j, k - 1) * V(m, i, j, k - 1)) / DZ2;
            W.def[m][id] = wdudx + wdvdy + wdwdz;
          }
        }
  }
  // 6. back_to_particles_3D(itype=1) (vpm_time.f90:62-107)
  {
    const int itype = cfg->interf_iproj;
    const int ips = (itype == 2) ? 0 : 1, ipf = (itype == 2) ? 1 : 2;
    const double XMIN = s->xbound[0], YMIN = s->xbound[1], ZMIN = s->xbound[2];
    const double DX = s->dpm[0], DY = s->dpm[1], DZ = s->dpm[2];
    for (int nv = 0; nv < nvr; ++nv) {
      const double px = xp[3 * (size_t)nv], py = xp[3 * (size_t)nv + 1], pz = xp[3 * (size_t)nv + 2];
      const int inode = (int)((px - XMIN) / DX) + 1, jnode = (int)((py - YMIN) / DY) + 1, knode = (int)((pz - ZMIN) / DZ) + 1;
      double u[3] = {0, 0, 0}, gl[3] = {0, 0, 0};
      for (int k = knode - ips; k <= knode + ipf; ++k)
        for (int j = jnode - ips; j <= jnode + ipf; ++j)
          for (int i = inode - ips; i <= inode + ipf; ++i) {
            const double x = (px - XMIN - (double)(i - 1) * DX) / DX;
            const double fx = projection_fun(itype, x);
            const double y = (py - YMIN - (double)(j - 1) * DY) / DY;
            const double fy = projection_fun(itype, y);
            const double z = (pz - ZMIN - (double)(k - 1) * DZ) / DZ;
            const double fz = projection_fun(itype, z);
            const double f = fx * fy * fz;
            if (i < 1 || i > NX || j < 1 || j > NY || k < 1 || k > NZ) return -1;
            const size_t id = lin(NX, NY, i, j, k);
            for (int c = 0; c < 3; ++c) { u[c] = u[c] + f * W.vel[c][id]; gl[c] = gl[c] + f * W.def[c][id]; }
          }
      for (int c = 0; c < 3; ++c) { up[3 * (size_t)nv + c] = u[c]; gp[3 * (size_t)nv + c] = gl[c] * qp[4 * (size_t)nv + 3]; }
    }
  }
  return 0;
}

int vpmo_whattodo4(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, double* up,
                   double* gp, int nvr, int nthreads) {
  // vpm(WhatToDo = 4) (vpm.f90:316-343) after an earlier solve: deposition
  // of these particles (vpm.f90:408-444), calc_velocity_serial_3d(-1)
  // (vpm_gcalc.f90:1-136: SOL = 0, then the stretching from the new RHS and
  // the velocity kept from the last solve), back_to_particles_3D(itype = 1)
  // (vpm_time.f90:62-107: UP = UP + sum W vel, GP = vol sum W SOL).
  Scratch& W = g_scr;
  const int NX = s->nn[0], NY = s->nn[1], NZ = s->nn[2];
  const size_t N = (size_t)NX * NY * NZ;
  for (int c = 0; c < 3; ++c)
    if (W.vel[c].size() != N) return -2;  // no resident velocity of this mesh
  int e = vpmo_project_particles(s, cfg->interf_iproj, xp, qp, nvr, W.rhs[0].data(), W.rhs[1].data(),
                                 W.rhs[2].data(), nthreads);
  if (e) return e;
  const double DX2 = 2 * s->dpm[0], DY2 = 2 * s->dpm[1], DZ2 = 2 * s->dpm[2];
  const int* nb = s->nn_bl;
  for (int c = 0; c < 3; ++c) W.def[c].assign(N, 0.0);
  auto V = [&](int c, int i, int j, int k) { return W.vel[c][lin(NX, NY, i, j, k)]; };
  auto RH = [&](int c, int i, int j, int k) { return W.rhs[c][lin(NX, NY, i, j, k)]; };
  for (int k = nb[2] + 2; k <= nb[5] - 2; ++k)
    for (int j = nb[1] + 2; j <= nb[4] - 2; ++j)
      for (int i = nb[0] + 2; i <= nb[3] - 2; ++i) {
        const size_t id = lin(NX, NY, i, j, k);
        for (int m = 0; m < 3; ++m) {
          const double wdudx = -(RH(0, i + 1, j, k) * V(m, i + 1, j, k) - RH(0, i - 1, j, k) * V(m, i - 1, j, k)) / DX2;
          const double wdvdy = -(RH(1, i, j + 1, k) * V(m, i, j + 1, k) - RH(1, i, j - 1, k) * V(m, i, j - 1, k)) / DY2;
          const double wdwdz = -(RH(2, i, j, k + 1) * V(m, i, j, k + 1) - RH(2, i, j, k - 1) * V(m, i, j, k - 1)) / DZ2;
          W.def[m][id] = wdudx + wdvdy + wdwdz;
        }
      }
  const int itype = cfg->interf_iproj;
  const int ips = (itype == 2) ? 0 : 1, ipf = (itype == 2) ? 1 : 2;
  const double XMIN = s->xbound[0], YMIN = s->xbound[1], ZMIN = s->xbound[2];
  const double DX = s->dpm[0], DY = s->dpm[1], DZ = s->dpm[2];
  for (int nv = 0; nv < nvr; ++nv) {
    const double px = xp[3 * (size_t)nv], py = xp[3 * (size_t)nv + 1], pz = xp[3 * (size_t)nv + 2];
    const int inode = (int)((px - XMIN) / DX) + 1, jnode = (int)((py - YMIN) / DY) + 1, knode = (int)((pz - ZMIN) / DZ) + 1;
    double* u = up + 3 * (size_t)nv;
    double gl[3] = {0, 0, 0};
    for (int k = knode - ips; k <= knode + ipf; ++k)
      for (int j = jnode - ips; j <= jnode + ipf; ++j)
        for (int i = inode - ips; i <= inode + ipf; ++i) {
          const double fx = projection_fun(itype, (px - XMIN - (double)(i - 1) * DX) / DX);
          const double fy = projection_fun(itype, (py - YMIN - (double)(j - 1) * DY) / DY);
          const double fz = projection_fun(itype, (pz - ZMIN - (double)(k - 1) * DZ) / DZ);
          const double f = fx * fy * fz;
          if (i < 1 || i > NX || j < 1 || j > NY || k < 1 || k > NZ) return -1;
          const size_t id = lin(NX, NY, i, j, k);
          for (int c = 0; c < 3; ++c) { u[c] = u[c] + f * W.vel[c][id]; gl[c] = gl[c] + f * W.def[c][id]; }
        }
    for (int c = 0; c < 3; ++c) gp[3 * (size_t)nv + c] = gl[c] * qp[4 * (size_t)nv + 3];
  }
  return 0;
}

int vpmo_diffuse(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, double ni, double* gp,
                 int nvr, int nthreads) {
  // vpm(WhatToDo = 5) (vpm.f90:345-372): deposition, diffuse_vort_3d
  // (vpm_gcalc.f90:138-210, neqpm = 3: VIS = NI), back_to_particles_3D(itype = 2)
  // (vpm_time.f90:109-151).
  Scratch& W = g_scr;
  const int NX = s->nn[0], NY = s->nn[1], NZ = s->nn[2];
  const size_t N = (size_t)NX * NY * NZ;
  for (int d = 0; d < 3; ++d) { W.nn[d] = s->nn[d]; W.nnbl[d] = s->nnbl[d]; W.nnc[d] = s->nn_coarse[d]; }
  for (int c = 0; c < 3; ++c) { W.rhs[c].assign(N, 0.0); W.sol[c].assign(N, 0.0); W.vel[c].assign(N, 0.0); W.def[c].assign(N, 0.0); }
  int e = vpmo_project_particles(s, cfg->interf_iproj, xp, qp, nvr, W.rhs[0].data(), W.rhs[1].data(), W.rhs[2].data(), nthreads);
  if (e) return e;
  const double DXpm2 = s->dpm[0] * s->dpm[0], DYpm2 = s->dpm[1] * s->dpm[1], DZpm2 = s->dpm[2] * s->dpm[2];
  const int* nb = s->nn_bl;
  const double VIS = ni;
  for (int k = nb[2] + 1; k <= nb[5] - 1; ++k)
    for (int j = nb[1] + 1; j <= nb[4] - 1; ++j)
      for (int i = nb[0] + 1; i <= nb[3] - 1; ++i)
        for (int c = 0; c < 3; ++c) {
          const std::vector<double>& R = W.rhs[c];
          const double dwxdx = (R[lin(NX, NY, i + 1, j, k)] - 2 * R[lin(NX, NY, i, j, k)] + R[lin(NX, NY, i - 1, j, k)]) / DXpm2;
          const double dwydy = (R[lin(NX, NY, i, j + 1, k)] - 2 * R[lin(NX, NY, i, j, k)] + R[lin(NX, NY, i, j - 1, k)]) / DYpm2;
          const double dwzdz = (R[lin(NX, NY, i, j, k + 1)] - 2 * R[lin(NX, NY, i, j, k)] + R[lin(NX, NY, i, j, k - 1)]) / DZpm2;
          W.sol[c][lin(NX, NY, i, j, k)] = -VIS * (dwxdx + dwydy + dwzdz);  // because RHS = -w
        }
  const int itype = cfg->interf_iproj;
  const int ips = (itype == 2) ? 0 : 1, ipf = (itype == 2) ? 1 : 2;
  const double XMIN = s->xbound[0], YMIN = s->xbound[1], ZMIN = s->xbound[2];
  const double DX = s->dpm[0], DY = s->dpm[1], DZ = s->dpm[2];
  for (int nv = 0; nv < nvr; ++nv) {
    const double px = xp[3 * (size_t)nv], py = xp[3 * (size_t)nv + 1], pz = xp[3 * (size_t)nv + 2];
    const int inode = (int)((px - XMIN) / DX) + 1, jnode = (int)((py - YMIN) / DY) + 1, knode = (int)((pz - ZMIN) / DZ) + 1;
    double g[3] = {0, 0, 0};
    for (int k = knode - ips; k <= knode + ipf; ++k)
      for (int j = jnode - ips; j <= jnode + ipf; ++j)
        for (int i = inode - ips; i <= inode + ipf; ++i) {
          const double fx = projection_fun(itype, (px - XMIN - (double)(i - 1) * DX) / DX);
          const double fy = projection_fun(itype, (py - YMIN - (double)(j - 1) * DY) / DY);
          const double fz = projection_fun(itype, (pz - ZMIN - (double)(k - 1) * DZ) / DZ);
          const double f = fx * fy * fz;
          if (i < 1 || i > NX || j < 1 || j > NY || k < 1 || k > NZ) return -1;
          const size_t id = lin(NX, NY, i, j, k);
          for (int c = 0; c < 3; ++c) g[c] = g[c] + f * W.sol[c][id];
        }
    for (int c = 0; c < 3; ++c) gp[3 * (size_t)nv + c] = g[c] * qp[4 * (size_t)nv + 3];
  }
  return 0;
}

long vpmo_get_field(int which, double* out, long capacity) {
  Scratch& W = g_scr;
  std::vector<double>* f = nullptr;
  switch (which) {
    case VPMO_F_RHS: f = W.rhs; break;
    case VPMO_F_SOL: f = W.sol; break;
    case VPMO_F_VEL: f = W.vel; break;
    case VPMO_F_DEF: f = W.def; break;
    case VPMO_F_BL_SOL1: f = W.bl_sol1; break;
    case VPMO_F_COARSE_RHS: f = W.c_rhs; break;
    case VPMO_F_COARSE_SOL: f = W.c_sol; break;
    case VPMO_F_BL_FINAL: f = W.bl_final; break;
    default: return -1;
  }
  const long n = (long)f[0].size();
  if (out) {
    if (capacity < 3 * n) return -1;
    for (int c = 0; c < 3; ++c) std::memcpy(out + c * n, f[c].data(), sizeof(double) * n);
  }
  return n;
}

void vpmo_euler(double* xp, double* qp, const double* up, const double* gp, int nvr, double dt, const double uinf[3]) {
  // source/test.f90:104-117 (FACDEF = 1)
  for (int j = 0; j < nvr; ++j)
    for (int c = 0; c < 3; ++c) {
      xp[3 * (size_t)j + c] = xp[3 * (size_t)j + c] + (up[3 * (size_t)j + c] + uinf[c]) * dt;
      qp[4 * (size_t)j + c] = qp[4 * (size_t)j + c] - 1.0 * gp[3 * (size_t)j + c] * dt;
    }
}

long vpmo_remesh(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, int nvr,
                 double* xp_out, double* qp_out, long capacity, int nthreads) {
  return vpmo_remesh_masked(cfg, s, xp, qp, nvr, xp_out, qp_out, capacity, nthreads, nullptr, 0);
}

long vpmo_remesh_masked(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, int nvr,
                        double* xp_out, double* qp_out, long capacity, int nthreads, int* mask, int mode) {
  // remesh_particles_3d(1), ncell_rem = 1, mrem = 1 (vpm_remesh.f90:5-225)
  vpmo_sizes r = *s;
  const int NX = s->nn[0], NY = s->nn[1], NZ = s->nn[2];
  for (int d = 0; d < 3; ++d) r.dpm[d] = (s->xbound[d + 3] - s->xbound[d]) / (double)(s->nn[d] - 1);
  const double DV = r.dpm[0] * r.dpm[1] * r.dpm[2];
  const size_t N = (size_t)NX * NY * NZ;
  std::vector<double> R0(N), R1(N), R2(N);
  int e = vpmo_project_particles(&r, cfg->interf_iproj, xp, qp, nvr, R0.data(), R1.data(), R2.data(), nthreads);
  if (e) return e;
  // vpmo_project_particles already divided by the recomputed DVpm (project_vol3d)
  const int h = cfg->interf_iproj / 2;
  const int* nb = s->nn_bl;
  const double thr = (double)1e-09f;  // default-REAL literal of vpm_remesh.f90:184
  long npar = 0;
  if (mask && mode == 1) std::fill(mask, mask + N, 0);
  for (int k = nb[2] + h; k <= nb[5] - h; ++k)
    for (int j = nb[1] + h; j <= nb[4] - h; ++j)
      for (int i = nb[0] + h; i <= nb[3] - h; ++i) {
        const size_t id = lin(NX, NY, i, j, k);
        const double wmag = std::sqrt(R0[id] * R0[id] + R1[id] * R1[id] + R2[id] * R2[id]);
        const bool emit = (mask && mode == 2) ? mask[id] != 0 : !(wmag < thr);
        if (mask && mode == 1) mask[id] = emit ? 1 : 0;
        if (!emit) continue;
        if (npar < capacity) {
          xp_out[3 * npar + 0] = s->xbound[0] + r.dpm[0] * (double)(i - 1);
          xp_out[3 * npar + 1] = s->xbound[1] + r.dpm[1] * (double)(j - 1);
          xp_out[3 * npar + 2] = s->xbound[2] + r.dpm[2] * (double)(k - 1);
          qp_out[4 * npar + 0] = R0[id] * DV;
          qp_out[4 * npar + 1] = R1[id] * DV;
          qp_out[4 * npar + 2] = R2[id] * DV;
          qp_out[4 * npar + 3] = DV;
        }
        ++npar;
      }
  return npar;
}

}  // extern "C"
