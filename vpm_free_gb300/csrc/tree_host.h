// tree_host.h -- host-side boundary quadtree description (see tree_host.cpp).
#pragma once
#include <vector>

namespace vpmg {

struct Panel {      // one boundary cell of calc_normalderiv_3d
  int face;         // 0..5 = XMIN XMAX YMIN YMAX ZMIN ZMAX
  int i, j, k;      // 1-based lower-corner node
  double xc, yc, zc, ds;
};

struct Cell {       // one entry of the level arrays xs_lev.. / ilev_t
  double x = 0, y = 0, z = 0, ds = 0, thr = 0;
  int ilev[6] = {0, 0, 0, 0, 0, 0};  // ilev_t(.,lev,1:6), children 1-based within lev-1
  int leaf0 = -1, rowlen = 0, istep = 0;
};

struct Target {
  long long node;   // linear 0-based node index in the grid array
  double x, y, z;
  int iplane;       // plane argument of Bounds3d_lev: 2/-2 X min/max, 1/-1 Y, 3/-3 Z
};

struct TreeGeom {
  int levmax = 0, nbound = 0;
  int n1f[6], n2f[6];
  std::vector<Panel> panels;
  std::vector<Cell> cells;          // [lev * nbound + (icount-1)]
  std::vector<int> nbound_lev;      // cumulative per level
  std::vector<Target> targets;
};

void build_tree_geometry(const double xmin[3], const double d[3], const int n[3], int levmax, TreeGeom& T);

}  // namespace vpmg
