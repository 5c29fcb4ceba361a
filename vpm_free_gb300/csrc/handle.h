// handle.h -- the C-ABI handle (the reference's vpm_lib module state) and
// the step helpers shared by api.cu and adjoint.cu.
#pragma once
#include <string>

#include "block_solve.h"
#include "fields.h"
#include "particles.h"
#include "vpmg_internal.h"
#include "yaps_multi.h"

#include <memory>
#include <vector>

struct AdjointState;  // adjoint.cu

struct vpmg_handle {
  vpmg_config cfg{};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  long long launches = 0;
  vpmg_sizes sz{};
  bool sized = false, prepared = false;
  long long op_budget = 100LL << 30;
  int arith = VPMG_ARITH_FP64;  // arithmetic of the heavy kernels (vpmg_set_arithmetic)
  // grids
  vpmg::Grid gglob{}, gbl{}, gco{};
  int inner_lo[3] = {0, 0, 0}, inner_ext[3] = {0, 0, 0};  // block inner box (0-based) and extent
  // fields (3 components back to back)
  vpmg::DBuf<double> rhs, sol, vel, def;
  vpmg::DBuf<double> rhs_bl, sol_bl, sol0, work, bl_sol1_copy;
  vpmg::DBuf<double> samp, crhs, csol, csol0;
  vpmg::DirichletPlan dp_bl, dp_inner, dp_c;
  vpmg::BlockSolve bsolve;         // partially evaluated block solves
  vpmg::FaceSolve fsolve;          // the inner box's solve with its faces in DST space
  bool full_block_solves = false;  // evaluate the block solves everywhere (parity / debugging)
  vpmg::BoundaryOp bo_bl, bo_c;
  vpmg::YapsDev yaps;
  // NBI x NBJ x NBK blocks (nblk > 1): rhs_bl / sol_bl hold [block][3][NB],
  // samp [block][3][NC]; one boundary operator per block
  int nblk = 1, nb3[3] = {1, 1, 1};
  std::vector<std::unique_ptr<vpmg::BoundaryOp>> bo_blk;
  std::vector<vpmg::Grid> g_blk;
  vpmg::YapsMultiDev ym;
  vpmg::DBuf<double> sampsum;
  bool keep_intermediates = false;
  // particles
  vpmg::Particles parts;
  vpmg::Binning bins;
  int np = 0;
  vpmg::DBuf<float2> vel_ff, def_ff;  // velocity and stretching as float-float pairs (float-float arithmetic)
  vpmg::DBuf<double> stage;          // AoS staging for host copies
  vpmg::DBuf<double> bench_scratch;  // replay outputs of vpmg_bench_kernel
  // timing
  bool profile = false;
  bool no_graphs = false;
  cudaEvent_t ev[10] = {};
  // graph of one device-resident step, and the per-step particle-count log
  struct {
    cudaGraphExec_t exec = nullptr;
    double dt = 0, u[3] = {0, 0, 0};
    int remesh = -1;
    long long launches = 0;
  } graph;
  vpmg::DBuf<int> hist, hist_counter;
  double phase_ms[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  AdjointState* adj = nullptr;
  // writers called by vpm(WhatToDo = 2): bit 0 solution windows, bit 1 hist lines
  std::string out_dir;
  int out_flags = 0;
};

namespace vpmg {
namespace hx {

struct LaunchScope {  // routes VPMG_LAUNCHED() to the handle's counter
  long long* prev;
  explicit LaunchScope(vpmg_handle* h) : prev(g_launch_counter) { g_launch_counter = &h->launches; }
  ~LaunchScope() { g_launch_counter = prev; }
};

template <class F>
int guarded(vpmg_handle* h, F&& f) {
  if (!h) return VPMG_ERR_ARG;
  try {
    LaunchScope ls(h);
    VPMG_CUDA(cudaSetDevice(h->device));
    f();
    return VPMG_OK;
  } catch (const Error& e) {
    h->err = e.msg;
    return e.status;
  } catch (const std::exception& e) {
    h->err = e.what();
    return VPMG_ERR_ARG;
  }
}

inline double* comp(DBuf<double>& b, size_t n, int c) { return b.p + (size_t)c * n; }

MeshDev mesh_dev(const Grid& g, int itype);
Grid remesh_grid(const vpmg_handle* h);       // global mesh with the remesh's recomputed spacing
void field_step(vpmg_handle* h);              // deposit ... stretching on binned particles
void poisson_part(vpmg_handle* h);            // h->rhs -> h->sol (rhsscat, yaps3d, solget)
// back_to_particles_3D(1) (+ Euler) from the resident fields in the handle's arithmetic
void m2p_fields(vpmg_handle* h, int up_mode, bool euler, double dt, const double uinf[3]);
void remesh(vpmg_handle* h);                  // remesh_particles_3d(1), on the stream
void step_on_stream(vpmg_handle* h, double dt);  // one full step (uinf = 0, remesh), graph replay when enabled
void sync_np(vpmg_handle* h);
void upload_particles(vpmg_handle* h, const double* xp, const double* qp, int n);
void download_particles(vpmg_handle* h, double* xp, double* qp, int n);
void destroy_adjoint(vpmg_handle* h);

}  // namespace hx
}  // namespace vpmg
