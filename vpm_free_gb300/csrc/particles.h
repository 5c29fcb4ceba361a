// particles.h -- device particle storage and the particle/mesh kernels.
#pragma once
#include <algorithm>

#include "vpmg_internal.h"

namespace vpmg {

// A sorted particle record: 24 slots of 8 bytes, 192 bytes -- the 4 x
// stencil weights (0..3), the 16 products of the y and z weights
// wy[b] wz[c] at 4 + 4b + c, the strengths (20..22) and the base cell's x
// index in the first four bytes of slot 23.  FP64 arithmetic: each slot a
// double, slot-major (slot k of sorted particle s at k * capacity + s; the
// high four bytes of slot 23 hold the linear cell index).  Float-float
// arithmetic: each slot a float-float pair, particle-major (24 slots per
// particle back to back).
constexpr int kRecLen = 24;
constexpr int kRecQ = 20;  // first strength slot

// Mesh parameters as the kernels see them (0-based nodes).
struct MeshDev {
  double xmin[3], d[3];
  double inv[3];        // 1 / d, computed once on the host (same IEEE quotient)
  int n[3];
  int itype, ips, ipf;  // projection function and stencil extents
};
// Cell index of a sorted record (slot 15), stored as the integer's bits.
__device__ __forceinline__ float2 cell_bits(int c) { return make_float2(__int_as_float(c), 0.0f); }
__device__ __forceinline__ int record_cell(const float2* r) { return __float_as_int(r[23].x); }

struct Particles {
  int capacity = 0;
  DBuf<double> x, y, z, q0, q1, q2, vol;  // SoA, QP(1:3) and QP(4)
  DBuf<double> up, gp;                    // (3, cap) AoS like UP/GP
  DBuf<int> key, perm;
  DBuf<float2> rec;                       // kRecLen slots per sorted particle (8 bytes each)
  DBuf<int> d_np;                         // particle count, on the device
  int arith = VPMG_ARITH_FP64;            // arithmetic of the records, deposition and gather
  double* rec64() const { return reinterpret_cast<double*>(rec.p); }
  size_t rec_stride() const { return (size_t)capacity; }  // FP64 records: doubles between slots
  void ensure(int cap);
};

struct Binning {
  size_t ncells = 0;
  DBuf<int> starts, cursor, sums, err;
  const int* nsorted_dev = nullptr;       // starts[N] after bin_particles
  void ensure(size_t ncell);
};

// All of these only enqueue work on the stream (no host round trip).
void bin_particles(Particles& P, const MeshDev& m, Binning& B, cudaStream_t s);
void deposit(const Particles& P, const MeshDev& m, const Binning& B, double* const rhs[3], cudaStream_t s);
// up_mode: 0 UP not written, 1 UP = sum W vel, 2 UP += sum W vel (the
// reference's accumulation into the caller's UP, vpm_time.f90:92-94);
// GP = vol * sum W def whenever UP is written.
enum { kUpNone = 0, kUpSet = 1, kUpAdd = 2 };
void m2p(Particles& P, const MeshDev& m, const Binning& B, const double* const vel[3], const double* const def[3],
         int up_mode, bool euler, double dt, const double uinf[3], cudaStream_t s);
// the same with the fields as float-float pairs (no split per node visit)
void m2p(Particles& P, const MeshDev& m, const Binning& B, const float2* const vel[3], const float2* const def[3],
         int up_mode, bool euler, double dt, const double uinf[3], cudaStream_t s);
void remesh_emit(Particles& P, const MeshDev& m, Binning& B, const double* const rhs[3], const int lo[3],
                 const int hi[3], double thr, cudaStream_t s);
// The emission mask alone: B.cursor = node flag, B.starts = emit slot (exclusive scan).
void remesh_mask(const MeshDev& m, Binning& B, const double* const rhs[3], const int lo[3], const int hi[3],
                 double thr, cudaStream_t s);
// Emission of exactly the nodes flagged in mask (N ints, 0/1): the remesh
// with a frozen |w| cut.
void remesh_emit_masked(Particles& P, const MeshDev& m, Binning& B, const double* const rhs[3], const int* mask,
                        cudaStream_t s);
// Host sync points.
void check_particle_errors(Binning& B, cudaStream_t s);
int read_count(const int* d, cudaStream_t s);

}  // namespace vpmg
