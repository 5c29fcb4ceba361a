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

// ---- NBI x NBJ x NBK blocks on one GPU ----------------------------------
struct MultiFace {   // one inner-face node of one block, in interp_stencil order
  int block;         // 0-based block id nb - 1
  long long node;    // linear node of that block (0-based)
  long long cbase;   // coarse node (ic-1, jc-1, kc-1), linear 0-based
  double w[9];       // TSC weights x (3), y (3), z (3)
  int flag0, nflag;  // blocks with nnb = 1 whose map meets the stencil, in block order
  int bb0, nbb;      // neighbour blocks with nnb = 0 (BBound terms), in interp_stencil order
};

struct YapsMultiGeom {
  int nblk = 0, nsamp = 0;
  std::vector<double> xbl;                    // [b*6 + d] padded block boxes
  std::vector<long long> samp_src;            // block node of each sample (same for every block)
  std::vector<long long> samp_dst;            // [b*nsamp + m] coarse node
  std::vector<int> maps;                      // [b*6 + d] NN_coarse_map (1-based)
  std::vector<MultiFace> faces;
  std::vector<int> flag_blocks;
  std::vector<int> bb_block;                  // sender block
  std::vector<long long> bb_node;             // sender's linear node at the receiver's face node
};

// Block boxes of vpm.f90:561-596 and the maps of yaps3d (:104-138,
// :1914-1983, with mapnodes_bl's transfers :457-1912 as gathers).
void build_yaps_multi(const int nblocks[3], const double xbound[6], const double dfine[3], int ncoarse,
                      const int nbl[3], const int nnbl_bl[6], const double xb_c[6], const double dc[3],
                      const int nc3[3], YapsMultiGeom& Y);

}  // namespace vpmg
