// yaps_host.cpp -- host geometry of the one-block YAPS coupling.
//
// source/yaps3d.f90:104-138 samples the fine block every nc-th node onto
// the coarse grid (coarse node = nint((X - Xc)/Dc) + 1), :1990-2016 takes
// the coarse Laplacian inside the sampled map, and :1914-1983
// (interp_stencil) adds sum TSC(xi) * (SOL_coarse - sample) on the six faces
// of the inner block box.  All index maps and TSC weights depend only on
// the frozen mesh, so they are computed here once; compiled with
// -ffp-contract=off so nint ties and weights round as the reference's
// expressions do.
#include <cmath>
#include <stdexcept>

#include "yaps_host.h"

namespace vpmg {

namespace {
inline int fnint(double x) { return (int)std::lround(x); }
double tsc(double x) {  // projection_fun itype 3 (source/pmproject.f90:407-411)
  const double xa = std::fabs(x);
  double f = 0.0;
  if (xa > 1.5) f = 0.0;
  if (xa >= 0.5 && xa <= 1.5) f = 0.5 * (-xa + 1.5) * (-xa + 1.5);
  if (xa >= 0.0 && xa < 0.5) f = 0.5 * (xa + 1.5) * (xa + 1.5) - 1.5 * (xa + 0.5) * (xa + 0.5);
  return f;
}
}  // namespace

void build_yaps_geometry(const double xb_bl[6], const double dfine[3], const int nbl[3], const int nnbl_bl[6],
                         const double xb_c[6], const double dc[3], const int nc3[3], int nc, YapsGeom& Y) {
  const int BX = nbl[0], BY = nbl[1], BZ = nbl[2];
  const int CX = nc3[0], CY = nc3[1], CZ = nc3[2];
  Y.samp_src.clear();
  Y.samp_dst.clear();
  std::vector<char> mapn((size_t)CX * CY * CZ, 0);
  int map[6] = {-1, -1, -1, -1, -1, -1};
  auto cidx = [&](int i, int j, int k) { return (long long)(i - 1) + (long long)CX * ((j - 1) + (long long)CY * (k - 1)); };
  for (int k = 1; k <= BZ; k += nc)
    for (int j = 1; j <= BY; j += nc)
      for (int i = 1; i <= BX; i += nc) {
        const double X0 = xb_bl[0] + (double)(i - 1) * dfine[0];
        const double X1 = xb_bl[1] + (double)(j - 1) * dfine[1];
        const double X2 = xb_bl[2] + (double)(k - 1) * dfine[2];
        const int in = fnint((X0 - xb_c[0]) / dc[0]) + 1;
        const int jn = fnint((X1 - xb_c[1]) / dc[1]) + 1;
        const int kn = fnint((X2 - xb_c[2]) / dc[2]) + 1;
        if (i == 1) map[0] = in;
        if (i == BX) map[3] = in;
        if (j == 1) map[1] = jn;
        if (j == BY) map[4] = jn;
        if (k == 1) map[2] = kn;
        if (k == BZ) map[5] = kn;
        if (in < 1 || in > CX || jn < 1 || jn > CY || kn < 1 || kn > CZ)
          throw std::runtime_error("yaps: block sample outside the coarse grid");
        Y.samp_src.push_back((long long)(i - 1) + (long long)BX * ((j - 1) + (long long)BY * (k - 1)));
        Y.samp_dst.push_back(cidx(in, jn, kn));
        mapn[cidx(in, jn, kn)] = 1;
      }
  for (int d = 0; d < 6; ++d) Y.map[d] = map[d];
  // interp_stencil on the inner-box faces, in the reference's face order
  const int NXs = nnbl_bl[0], NXf = nnbl_bl[3], NYs = nnbl_bl[1], NYf = nnbl_bl[4], NZs = nnbl_bl[2], NZf = nnbl_bl[5];
  Y.faces.clear();
  auto add = [&](int i, int j, int k) {
    FaceNode fn;
    fn.node = (long long)(i - 1) + (long long)BX * ((j - 1) + (long long)BY * (k - 1));
    const double X[3] = {xb_bl[0] + (double)(i - 1) * dfine[0], xb_bl[1] + (double)(j - 1) * dfine[1],
                         xb_bl[2] + (double)(k - 1) * dfine[2]};
    int cn[3];
    for (int d = 0; d < 3; ++d) cn[d] = fnint((X[d] - xb_c[d]) / dc[d]) + 1;
    if (cn[0] < 2 || cn[0] > CX - 1 || cn[1] < 2 || cn[1] > CY - 1 || cn[2] < 2 || cn[2] > CZ - 1)
      throw std::runtime_error("yaps: interpolation stencil outside the coarse grid");
    fn.cbase = cidx(cn[0] - 1, cn[1] - 1, cn[2] - 1);
    for (int d = 0; d < 3; ++d)
      for (int m = 0; m < 3; ++m) {
        const int c1 = cn[d] - 1 + m;  // 1-based coarse index along d
        const double xc = (X[d] - xb_c[d] - (double)(c1 - 1) * dc[d]) / dc[d];
        fn.w[3 * d + m] = tsc(xc);
      }
    fn.flagged = !(mapn[cidx(cn[0] - 1, cn[1] - 1, cn[2] - 1)] == 1 && mapn[cidx(cn[0] + 1, cn[1] + 1, cn[2] + 1)] == 1);
    Y.faces.push_back(fn);
  };
  for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) add(NXs, j, k);
  for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) add(NXf, j, k);
  for (int k = NZs; k <= NZf; ++k) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, NYs, k);
  for (int k = NZs; k <= NZf; ++k) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, NYf, k);
  for (int j = NYs + 1; j <= NYf - 1; ++j) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, j, NZs);
  for (int j = NYs + 1; j <= NYf - 1; ++j) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, j, NZf);
}

}  // namespace vpmg
