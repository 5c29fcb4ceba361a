// yaps_multi.h -- YAPS with several blocks on one GPU (yaps_multi.cu).
#pragma once
#include "vpmg_internal.h"
#include "yaps_host.h"

namespace vpmg {

struct YapsMultiDev {
  int nblk = 0, nsamp = 0, nface = 0;
  DBuf<int> face_block, flag_off, flag_blk, bb_off, bb_blk, maps;
  DBuf<long long> face_node, face_cbase, bb_node, samp_src, samp_dst;
  DBuf<double> face_w, face_val;
  void prepare(const YapsMultiGeom& Y);
};

// rhsscat_3d for every block: rhs (3 x N global) -> rhs_bl [block][3][NB].
void yaps_multi_rhsscat(const YapsMultiDev& Y, const double* rhs, const int nn[3], const int nn_bl[6],
                        const int nbl[3], const int nnbl_bl[6], const int nblocks[3], double* rhs_bl, cudaStream_t s);
// samples [block][3][NC], their sum over blocks [3][NC] and the coarse RHS [3][NC].
void yaps_multi_coarse(YapsMultiDev& Y, const double* sol_bl, size_t NB, const int cdims[3], const double dc[3],
                       double* samp, double* sampsum, double* crhs, cudaStream_t s);
// interp_stencil on every block's inner faces, neighbours' first solutions included.
void yaps_multi_faces(YapsMultiDev& Y, const int cdims[3], const double* csol, const double* sampsum,
                      const double* samp, double* sol_bl, size_t NB, cudaStream_t s);
// solget_3d: block inner boxes -> global sol (3 x N), later blocks win on shared planes.
void yaps_multi_solget(const double* sol_bl, const int nbl[3], const int nnbl_bl[6], const int nblocks[3],
                       const int nn[3], const int nn_bl[6], double* sol, cudaStream_t s);

}  // namespace vpmg
