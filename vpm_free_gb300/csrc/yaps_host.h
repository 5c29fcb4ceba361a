// yaps_host.h -- host geometry of the one-block YAPS coupling (yaps_host.cpp).
#pragma once
#include <vector>

namespace vpmg {

struct FaceNode {
  long long node;   // linear block node (0-based)
  long long cbase;  // coarse node (ic-1, jc-1, kc-1), linear 0-based
  double w[9];      // TSC weights: x (3), y (3), z (3)
  int flagged;      // nnb(nb) of interp_stencil
};

struct YapsGeom {
  std::vector<long long> samp_src, samp_dst;  // block node -> coarse node
  int map[6];                                 // NN_coarse_map (1-based)
  std::vector<FaceNode> faces;
};

void build_yaps_geometry(const double xb_bl[6], const double dfine[3], const int nbl[3], const int nnbl_bl[6],
                         const double xb_c[6], const double dc[3], const int nc3[3], int nc, YapsGeom& Y);

}  // namespace vpmg
