// fields.h -- mesh-to-mesh kernels (fields.cu).
#pragma once
#include "vpmg_internal.h"
#include "yaps_host.h"

namespace vpmg {

struct YapsDev {
  DBuf<long long> samp_src, samp_dst, face_node, face_cbase;
  DBuf<double> face_w;
  DBuf<int> face_flag;
  int nsamp = 0, nface = 0;
  int map[6] = {0, 0, 0, 0, 0, 0};
  void prepare(const YapsGeom& Y);
};

void box_copy(const double* src, const int sdims[3], const int so[3], double* dst, const int ddims[3], const int dof[3],
              const int ext[3], cudaStream_t s);
void yaps_sample(const YapsDev& Y, const double* const sbl[3], double* const samp[3], cudaStream_t s);
void yaps_coarse_rhs(const YapsDev& Y, const int cdims[3], const double dc[3], const double* const samp[3],
                     double* const crhs[3], cudaStream_t s);
void yaps_face_interp(const YapsDev& Y, const int cdims[3], const double* const csol[3], const double* const samp[3],
                      double* const sbl[3], cudaStream_t s);
// diffuse_vort_3d: sol = -ni Lap_h rhs inside the block range nn_bl (1-based), zero elsewhere.
void viscous_diffusion(const int dims[3], const int nn_bl[6], const double h[3], double ni, const double* const rhs[3],
                       double* const sol[3], cudaStream_t s);
// calc_velocity_serial_3d: parts bit 0 = velocity (curl psi), bit 1 = stretching
// (from rhs and the velocity in vel); idcalc 1 = both, 0 = velocity, -1 = stretching.
// vel_ff / def_ff (nullable): the same values also as float-float pairs.
void velocity_and_stretching(const int dims[3], const double h[3], const double* const psi[3], const double* const rhs[3],
                             double* const vel[3], double* const def[3], cudaStream_t s, int parts = 3,
                             float2* const vel_ff[3] = nullptr, float2* const def_ff[3] = nullptr);
// Interior nodes (2..N-3) with a non-zero RHS among the stretching stencil's
// six neighbours: where the FP64 stretching kernel computes (instrumentation).
long long count_vortical_nodes(const int dims[3], const double* const rhs[3], cudaStream_t s);

}  // namespace vpmg
