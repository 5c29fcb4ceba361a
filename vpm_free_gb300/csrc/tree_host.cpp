// tree_host.cpp -- host construction of the boundary quadtree of one grid.
//
// The tree topology and every coordinate it compares depend only on the
// mesh, which is frozen after the first step (idefine = 1), so they are
// built once on the host and uploaded; only the source strengths are
// aggregated on the device each step.
//
// Follows source/pinfdomain.f90:294-547 (panel corners, areas, face order)
// and :875-1530 (per-face levels, ilev_t child table, dummy cells), and the
// target order of source/pmbound.f90:980-1133.  Compiled with
// -ffp-contract=off: panel centres, level centres and the opening radii
// 10*sqrt(dS) must round exactly as written so that the device's opening
// decisions reproduce the reference's.
#include <cmath>
#include <stdexcept>

#include "tree_host.h"

namespace vpmg {

namespace {
inline double node_coord(double xmin, int i1, double d) { return xmin + (double)(i1 - 1) * d; }  // 1-based node
inline double mean4(double a, double b, double c, double e) { return 0.25 * (((a + b) + c) + e); }
}  // namespace

void build_tree_geometry(const double xmin[3], const double d[3], const int n[3], int levmax, TreeGeom& T) {
  const int NX = n[0], NY = n[1], NZ = n[2];
  const double XMIN = xmin[0], YMIN = xmin[1], ZMIN = xmin[2], DX = d[0], DY = d[1], DZ = d[2];
  T.levmax = levmax;
  T.panels.clear();
  // ---- panels, in calc_normalderiv_3d order -------------------------------
  auto add = [&](int face, int i, int j, int k, double x1, double x2, double x3, double x4, double y1, double y2,
                 double y3, double y4, double z1, double z2, double z3, double z4, double ds) {
    Panel p;
    p.face = face; p.i = i; p.j = j; p.k = k;
    p.xc = mean4(x1, x2, x3, x4); p.yc = mean4(y1, y2, y3, y4); p.zc = mean4(z1, z2, z3, z4);
    p.ds = ds;
    T.panels.push_back(p);
  };
  for (int face = 0; face < 2; ++face) {  // XMIN, XMAX: k outer, j inner
    const int i = face == 0 ? 1 : NX;
    for (int k = 1; k <= NZ - 1; ++k)
      for (int j = 1; j <= NY - 1; ++j) {
        const double x = node_coord(XMIN, i, DX), y0 = node_coord(YMIN, j, DY), y1 = node_coord(YMIN, j + 1, DY);
        const double z0 = node_coord(ZMIN, k, DZ), z1 = node_coord(ZMIN, k + 1, DZ);
        if (face == 0) add(face, i, j, k, x, x, x, x, y0, y0, y1, y1, z0, z1, z1, z0, DY * DZ);
        else add(face, i, j, k, x, x, x, x, y1, y1, y0, y0, z0, z1, z1, z0, DY * DZ);
      }
    T.n1f[face] = NY - 1; T.n2f[face] = NZ - 1;
  }
  for (int face = 2; face < 4; ++face) {  // YMIN, YMAX: k outer, i inner
    const int j = face == 2 ? 1 : NY;
    for (int k = 1; k <= NZ - 1; ++k)
      for (int i = 1; i <= NX - 1; ++i) {
        const double y = node_coord(YMIN, j, DY), x0 = node_coord(XMIN, i, DX), x1 = node_coord(XMIN, i + 1, DX);
        const double z0 = node_coord(ZMIN, k, DZ), z1 = node_coord(ZMIN, k + 1, DZ);
        if (face == 2) add(face, i, j, k, x0, x0, x1, x1, y, y, y, y, z0, z1, z1, z0, DX * DZ);
        else add(face, i, j, k, x1, x1, x0, x0, y, y, y, y, z0, z1, z1, z0, DX * DZ);
      }
    T.n1f[face] = NX - 1; T.n2f[face] = NZ - 1;
  }
  for (int face = 4; face < 6; ++face) {  // ZMIN, ZMAX: j outer, i inner
    const int k = face == 4 ? 1 : NZ;
    for (int j = 1; j <= NY - 1; ++j)
      for (int i = 1; i <= NX - 1; ++i) {
        const double z = node_coord(ZMIN, k, DZ), x0 = node_coord(XMIN, i, DX), x1 = node_coord(XMIN, i + 1, DX);
        const double y0 = node_coord(YMIN, j, DY), y1 = node_coord(YMIN, j + 1, DY);
        if (face == 4) add(face, i, j, k, x0, x0, x1, x1, y0, y1, y1, y0, z, z, z, z, DX * DY);
        else add(face, i, j, k, x1, x1, x0, x0, y0, y1, y1, y0, z, z, z, z, DX * DY);
      }
    T.n1f[face] = NX - 1; T.n2f[face] = NY - 1;
  }
  const int nbound = (int)T.panels.size();
  T.nbound = nbound;
  // ---- levels, build_level_nbound_3d order --------------------------------
  const size_t NL = (size_t)(levmax + 1) * nbound;
  T.cells.assign(NL, Cell());
  std::vector<int> nbl(levmax + 1, 0), ncount(levmax + 1, 0);
  auto C = [&](int icount, int lev) -> Cell& { return T.cells[(size_t)lev * nbound + (icount - 1)]; };
  for (int face = 0; face < 6; ++face) {
    const int n1 = T.n1f[face], n2 = T.n2f[face];
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
          double xc = 0, yc = 0, zc = 0, sc = 0;
          for (int mm = 1; mm <= istep; ++mm)
            for (int nn = 1; nn <= istep; ++nn) {
              const Panel& P = T.panels[lf + so * n1 + fo + (mm - 1) * n1 + nn - 1];
              xc = P.xc + xc; yc = P.yc + yc; zc = P.zc + zc; sc = P.ds + sc;
            }
          icount++;
          Cell& c = C(icount, lev);
          const double q = (double)(float)(istep * istep);
          c.x = xc / q; c.y = yc / q; c.z = zc / q; c.ds = sc;
          c.leaf0 = lf + so * n1 + fo;  // 0-based first leaf (mm = nn = 1)
          c.rowlen = n1;
          c.istep = istep;
          const int npre = nnf[lev];
          if (lev > 0) {
            const int nn = nnf[lev - 1];
            int nj;
            if (fo == 0 && icount - 1 == nbl[lev]) nj = nbl[lev - 1] + 1;
            else if (fo == 0 && icount - 1 > nbl[lev]) {
              nj = C(icount - 1, lev).ilev[2] + 1;
              if (C(icount - 1, lev).ilev[5] < 0) nj = C(icount - 1, lev).ilev[1] + 1;
            } else nj = C(icount - 1, lev).ilev[1] + 1;
            c.ilev[0] = nj; c.ilev[1] = nj + 1; c.ilev[2] = nj + nn + 1; c.ilev[3] = nj + nn; c.ilev[4] = 4;
          }
          c.ilev[5] = npre;
        }
        if ((n1 % istep) != 0 || n1 <= istep) {
          if (lev == 0) throw std::runtime_error("tree: level 0 cannot hold dummy cells");
          icount++;
          Cell& c = C(icount, lev);
          const int nn = nnf[lev - 1];
          const int nj = C(icount - 1, lev).ilev[1] + 1;
          c.ilev[0] = nj; c.ilev[1] = nj + nn; c.ilev[4] = 2; c.ilev[5] = -1;
          c.leaf0 = -1;
        }
      }
      if ((n2 % istep) != 0 || n2 <= istep) {
        if (lev == 0) throw std::runtime_error("tree: level 0 cannot hold dummy cells");
        for (int fo = 0; fo <= n1 - istep; fo += istep) {
          if (fo == n1 - istep && (n1 % istep) != 0) continue;
          icount++;
          Cell& c = C(icount, lev);
          int nj;
          if (fo == 0 && C(icount - 1, lev).ilev[5] > 0) nj = C(icount - 1, lev).ilev[2] + 1;
          else nj = C(icount - 1, lev).ilev[1] + 1;
          c.ilev[0] = nj; c.ilev[1] = nj + 1; c.ilev[4] = 2; c.ilev[5] = -2;
          c.leaf0 = -1;
        }
      }
      ncount[lev] = icount;
    }
    nbl = ncount;
  }
  if (nbl[0] != nbound) throw std::runtime_error("tree: nbound_lev(0) /= nbound");
  T.nbound_lev = nbl;
  for (int lev = 0; lev <= levmax; ++lev)
    for (int ic = 1; ic <= nbl[lev]; ++ic) {
      Cell& c = C(ic, lev);
      c.thr = 10.0 * std::sqrt(c.ds);
    }
  // ---- targets, Bounds3d_lev order ---------------------------------------
  T.targets.clear();
  auto tgt = [&](int i, int j, int k, int iplane) {
    Target t;
    t.node = (long long)(i - 1) + (long long)NX * ((j - 1) + (long long)NY * (k - 1));
    t.x = node_coord(XMIN, i, DX); t.y = node_coord(YMIN, j, DY); t.z = node_coord(ZMIN, k, DZ);
    t.iplane = iplane;
    T.targets.push_back(t);
  };
  for (int k = 1; k <= NZ; ++k) for (int j = 1; j <= NY; ++j) tgt(1, j, k, 2);
  for (int k = 1; k <= NZ; ++k) for (int j = 1; j <= NY; ++j) tgt(NX, j, k, -2);
  for (int k = 1; k <= NZ; ++k) for (int i = 2; i <= NX - 1; ++i) tgt(i, 1, k, 1);
  for (int k = 1; k <= NZ; ++k) for (int i = 2; i <= NX - 1; ++i) tgt(i, NY, k, -1);
  for (int j = 2; j <= NY - 1; ++j) for (int i = 2; i <= NX - 1; ++i) tgt(i, j, 1, 3);
  for (int j = 2; j <= NY - 1; ++j) for (int i = 2; i <= NX - 1; ++i) tgt(i, j, NZ, -3);
}

}  // namespace vpmg
