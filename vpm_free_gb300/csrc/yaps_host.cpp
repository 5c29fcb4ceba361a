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

// Several blocks.  Block boxes as define_sizes builds them (vpm.f90:561-596:
// origin Xbound + (i-1)*NXbl*Dpm, then definepm itype 1 pads by ncoarse).
// mapnodes_bl sends each neighbour the sender's first solution at the
// receiver's inner-face nodes that lie in the sender's padded block (the
// 26 transfers of yaps3d.f90:500-1870 all follow that rule), and
// interp_stencil adds it where the sender's map covers the node's 3x3x3
// coarse stencil (nnb = 0).  Here that exchange is a gather: for each face
// node, the sender blocks and the sender's node at the same position.
void build_yaps_multi(const int nblocks[3], const double xbound[6], const double dfine[3], int ncoarse,
                      const int nbl[3], const int nnbl_bl[6], const double xb_c[6], const double dc[3],
                      const int nc3[3], YapsMultiGeom& Y) {
  const int NBI = nblocks[0], NBJ = nblocks[1], NBK = nblocks[2], B = NBI * NBJ * NBK;
  const int BX = nbl[0], BY = nbl[1], BZ = nbl[2];
  const int CX = nc3[0], CY = nc3[1], CZ = nc3[2];
  const size_t NC = (size_t)CX * CY * CZ;
  const int nc = ncoarse;
  const int lo[3] = {nnbl_bl[0], nnbl_bl[1], nnbl_bl[2]}, hi[3] = {nnbl_bl[3], nnbl_bl[4], nnbl_bl[5]};
  Y = YapsMultiGeom();
  Y.nblk = B;
  const int nbc[3] = {fnint((xbound[3] - xbound[0]) / dfine[0]) / NBI, fnint((xbound[4] - xbound[1]) / dfine[1]) / NBJ,
                      fnint((xbound[5] - xbound[2]) / dfine[2]) / NBK};
  Y.xbl.assign(6 * (size_t)B, 0.0);
  for (int k = 1; k <= NBK; ++k)
    for (int j = 1; j <= NBJ; ++j)
      for (int i = 1; i <= NBI; ++i) {
        const int b = (k - 1) * NBJ * NBI + (j - 1) * NBI + (i - 1);
        const int ijk[3] = {i, j, k};
        for (int d = 0; d < 3; ++d) {
          double a = xbound[d] + (double)((ijk[d] - 1) * nbc[d]) * dfine[d];
          double z = xbound[d] + (double)(ijk[d] * nbc[d]) * dfine[d];
          a = a - ((double)nc * dfine[d]);
          z = z + ((double)nc * dfine[d]);
          if (fnint(std::fabs(z - a) / dfine[d]) + 1 != nbl[d]) throw std::runtime_error("yaps: blocks differ in size");
          Y.xbl[6 * (size_t)b + d] = a;
          Y.xbl[6 * (size_t)b + d + 3] = z;
        }
      }
  auto cidx = [&](int i, int j, int k) { return (long long)(i - 1) + (long long)CX * ((j - 1) + (long long)CY * (k - 1)); };
  // samples and map_nodes of every block
  std::vector<std::vector<char>> mapn(B, std::vector<char>(NC, 0));
  Y.maps.assign(6 * (size_t)B, -1);
  for (int k = 1; k <= BZ; k += nc)
    for (int j = 1; j <= BY; j += nc)
      for (int i = 1; i <= BX; i += nc) Y.samp_src.push_back((long long)(i - 1) + (long long)BX * ((j - 1) + (long long)BY * (k - 1)));
  Y.nsamp = (int)Y.samp_src.size();
  Y.samp_dst.assign((size_t)B * Y.nsamp, 0);
  for (int b = 0; b < B; ++b) {
    const double* xb = &Y.xbl[6 * (size_t)b];
    int* mp = &Y.maps[6 * (size_t)b];
    int m = 0;
    for (int k = 1; k <= BZ; k += nc)
      for (int j = 1; j <= BY; j += nc)
        for (int i = 1; i <= BX; i += nc) {
          const double X0 = xb[0] + (double)(i - 1) * dfine[0];
          const double X1 = xb[1] + (double)(j - 1) * dfine[1];
          const double X2 = xb[2] + (double)(k - 1) * dfine[2];
          const int in = fnint((X0 - xb_c[0]) / dc[0]) + 1;
          const int jn = fnint((X1 - xb_c[1]) / dc[1]) + 1;
          const int kn = fnint((X2 - xb_c[2]) / dc[2]) + 1;
          if (i == 1) mp[0] = in;
          if (i == BX) mp[3] = in;
          if (j == 1) mp[1] = jn;
          if (j == BY) mp[4] = jn;
          if (k == 1) mp[2] = kn;
          if (k == BZ) mp[5] = kn;
          if (in < 1 || in > CX || jn < 1 || jn > CY || kn < 1 || kn > CZ)
            throw std::runtime_error("yaps: block sample outside the coarse grid");
          Y.samp_dst[(size_t)b * Y.nsamp + m++] = cidx(in, jn, kn);
          mapn[b][cidx(in, jn, kn)] = 1;
        }
  }
  // inner-face nodes of every block, interp_stencil order
  std::vector<int> nnb(B);
  for (int b = 0; b < B; ++b) {
    const int bi = b % NBI + 1, bj = (b / NBI) % NBJ + 1, bk = b / (NBI * NBJ) + 1;
    const double* xb = &Y.xbl[6 * (size_t)b];
    auto add = [&](int i, int j, int k) {
      MultiFace fn;
      fn.block = b;
      fn.node = (long long)(i - 1) + (long long)BX * ((j - 1) + (long long)BY * (k - 1));
      const double X[3] = {xb[0] + (double)(i - 1) * dfine[0], xb[1] + (double)(j - 1) * dfine[1],
                           xb[2] + (double)(k - 1) * dfine[2]};
      int cn[3];
      for (int d = 0; d < 3; ++d) cn[d] = fnint((X[d] - xb_c[d]) / dc[d]) + 1;
      if (cn[0] < 2 || cn[0] > CX - 1 || cn[1] < 2 || cn[1] > CY - 1 || cn[2] < 2 || cn[2] > CZ - 1)
        throw std::runtime_error("yaps: interpolation stencil outside the coarse grid");
      fn.cbase = cidx(cn[0] - 1, cn[1] - 1, cn[2] - 1);
      for (int d = 0; d < 3; ++d)
        for (int m = 0; m < 3; ++m) {
          const int c1 = cn[d] - 1 + m;
          const double xc = (X[d] - xb_c[d] - (double)(c1 - 1) * dc[d]) / dc[d];
          fn.w[3 * d + m] = tsc(xc);
        }
      fn.flag0 = (int)Y.flag_blocks.size();
      for (int q = 0; q < B; ++q) {
        nnb[q] = !(mapn[q][cidx(cn[0] - 1, cn[1] - 1, cn[2] - 1)] == 1 && mapn[q][cidx(cn[0] + 1, cn[1] + 1, cn[2] + 1)] == 1);
        if (!nnb[q]) continue;
        bool meets = false;  // samples of q are zero off its map: other blocks add exact zeros
        for (int kc = cn[2] - 1; kc <= cn[2] + 1 && !meets; ++kc)
          for (int jc = cn[1] - 1; jc <= cn[1] + 1 && !meets; ++jc)
            for (int ic = cn[0] - 1; ic <= cn[0] + 1 && !meets; ++ic) meets = mapn[q][cidx(ic, jc, kc)] == 1;
        if (meets) Y.flag_blocks.push_back(q);
      }
      fn.nflag = (int)Y.flag_blocks.size() - fn.flag0;
      fn.bb0 = (int)Y.bb_block.size();
      for (int kb = bk - 1; kb <= bk + 1; ++kb)
        for (int jb = bj - 1; jb <= bj + 1; ++jb)
          for (int ib = bi - 1; ib <= bi + 1; ++ib) {
            if (ib < 1 || ib > NBI || jb < 1 || jb > NBJ || kb < 1 || kb > NBK) continue;
            const int q = (kb - 1) * NBI * NBJ + (jb - 1) * NBI + (ib - 1);
            if (nnb[q] == 1 || q == b) continue;
            const int o[3] = {bi - ib, bj - jb, bk - kb};  // receiver minus sender
            const int rc[3] = {i, j, k};
            int sn[3];
            for (int d = 0; d < 3; ++d) {
              sn[d] = rc[d] + o[d] * (hi[d] - lo[d]);
              if (sn[d] < 1 || sn[d] > nbl[d]) throw std::runtime_error("yaps: neighbour node outside its block");
            }
            Y.bb_block.push_back(q);
            Y.bb_node.push_back((long long)(sn[0] - 1) + (long long)BX * ((sn[1] - 1) + (long long)BY * (sn[2] - 1)));
          }
      fn.nbb = (int)Y.bb_block.size() - fn.bb0;
      Y.faces.push_back(fn);
    };
    const int NXs = lo[0], NYs = lo[1], NZs = lo[2], NXf = hi[0], NYf = hi[1], NZf = hi[2];
    for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) add(NXs, j, k);
    for (int k = NZs; k <= NZf; ++k) for (int j = NYs; j <= NYf; ++j) add(NXf, j, k);
    for (int k = NZs; k <= NZf; ++k) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, NYs, k);
    for (int k = NZs; k <= NZf; ++k) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, NYf, k);
    for (int j = NYs + 1; j <= NYf - 1; ++j) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, j, NZs);
    for (int j = NYs + 1; j <= NYf - 1; ++j) for (int i = NXs + 1; i <= NXf - 1; ++i) add(i, j, NZf);
  }
}

}  // namespace vpmg
