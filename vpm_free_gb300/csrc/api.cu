// api.cu -- the C-ABI (include/vpmg.h): handle, sizing, step orchestration.
//
// One handle = one CUDA stream + the device state that the reference keeps
// in module variables (vpm_vars / vpm_size / pmgrid / parvar,
// source/vpm.f90:1-32, source/main_pm.f90:2-45).  Fields stay resident in
// HBM between calls; the Fortran-facing vpm() copies particles in and out.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <sstream>
#include <string>

#include "handle.h"
#include "io_files.h"

using namespace vpmg;

using vpmg::hx::guarded;
using vpmg::hx::LaunchScope;
using vpmg::hx::comp;

namespace {

inline int fnint(double x) { return (int)std::lround(x); }

// definepm (source/pmlib.f90:216-432), itype 1 and 3, ND = 3.
void definepm(int itype, double Xb[6], const double D[3], int ndum, const int nsize[3], int NN[3], int NN_bl[6]) {
  for (int d = 0; d < 3; ++d) {
    Xb[d] = Xb[d] - ((double)ndum * D[d]);
    Xb[d + 3] = Xb[d + 3] + ((double)ndum * D[d]);
    NN[d] = fnint(std::fabs(Xb[d + 3] - Xb[d]) / D[d]) + 1;
  }
  if (itype == 1) {
    for (int d = 0; d < 3; ++d) { NN_bl[d] = ndum + 1; NN_bl[d + 3] = NN[d] - ndum; }
    return;
  }
  // itype 3: pad symmetrically so that NN-1 divides by nsize (odd remainder on the min side)
  for (int d = 0; d < 3; ++d) {
    const int nd = nsize[d] - ((NN[d] - 1) % nsize[d]);
    if (nd % 2 == 0) {
      Xb[d] = Xb[d] - ((double)(nd / 2) * D[d]);
      Xb[d + 3] = Xb[d + 3] + ((double)(nd / 2) * D[d]);
    } else {
      Xb[d] = Xb[d] - ((double)(nd % 2 + nd / 2) * D[d]);
      Xb[d + 3] = Xb[d + 3] + ((double)(nd / 2) * D[d]);
    }
    NN[d] = fnint(std::fabs(Xb[d + 3] - Xb[d]) / D[d]) + 1;
    NN_bl[d] = ndum + 1;
    NN_bl[d + 3] = NN[d] - ndum;
  }
}

// define_sizes (source/vpm.f90:477-660), one block.  xp: XP(3,nvr).
void define_sizes(vpmg_handle* h, const double* xp, int nvr, int ntime, vpmg_sizes& s) {
  const vpmg_config& cfg = h->cfg;
  VPMG_CHECK(cfg.nbi >= 1 && cfg.nbj >= 1 && cfg.nbk >= 1, VPMG_ERR_ARG, "NBI, NBJ, NBK must be >= 1");
  const int nbd[3] = {cfg.nbi, cfg.nbj, cfg.nbk};
  const bool recompute = (ntime == 0 && cfg.idefine == 1) || cfg.idefine == 0 || !h->sized;
  if (recompute) {
    double Xb[6], Dpm[3] = {cfg.dpm[0], cfg.dpm[1], cfg.dpm[2]};
    int NN[3], NN_bl[6];
    if (cfg.use_box) {
      for (int d = 0; d < 6; ++d) Xb[d] = cfg.box[d];
      for (int d = 0; d < 3; ++d) {
        NN[d] = fnint(std::fabs(Xb[d + 3] - Xb[d]) / Dpm[d]) + 1;
        NN_bl[d] = 1;
        NN_bl[d + 3] = NN[d];
        VPMG_CHECK((NN[d] - 1) % (nbd[d] * cfg.ncoarse) == 0, VPMG_ERR_ARG,
                   "explicit box: cells must divide by the block count times ncoarse");
      }
    } else {
      VPMG_CHECK(nvr > 0 && xp, VPMG_ERR_ARG, "define_sizes needs particles to size the box");
      double mn[3] = {xp[0], xp[1], xp[2]}, mx[3] = {xp[0], xp[1], xp[2]};
      for (int p = 1; p < nvr; ++p)
        for (int d = 0; d < 3; ++d) {
          mn[d] = std::min(mn[d], xp[3 * (size_t)p + d]);
          mx[d] = std::max(mx[d], xp[3 * (size_t)p + d]);
        }
      for (int d = 0; d < 3; ++d) {
        Xb[d] = mn[d] - (double)cfg.interf_iproj * cfg.dpm[d];
        Xb[d + 3] = mx[d] + (double)cfg.interf_iproj * cfg.dpm[d];
      }
      const int nsiz[3] = {cfg.nbi * cfg.ncoarse, cfg.nbj * cfg.ncoarse, cfg.nbk * cfg.ncoarse};
      definepm(3, Xb, Dpm, 0, nsiz, NN, NN_bl);
    }
    for (int d = 0; d < 6; ++d) { s.xbound[d] = Xb[d]; s.nn_bl[d] = NN_bl[d]; }
    for (int d = 0; d < 3; ++d) { s.dpm[d] = Dpm[d]; s.nn[d] = NN[d]; }
  }
  const double* Xb = s.xbound;
  const double* D = s.dpm;
  const int NXbl = fnint((Xb[3] - Xb[0]) / D[0]) / cfg.nbi;
  const int NYbl = fnint((Xb[4] - Xb[1]) / D[1]) / cfg.nbj;
  const int NZbl = fnint((Xb[5] - Xb[2]) / D[2]) / cfg.nbk;
  double Xt[6] = {Xb[0] + (double)(0 * NXbl) * D[0], Xb[1] + (double)(0 * NYbl) * D[1], Xb[2] + (double)(0 * NZbl) * D[2],
                  Xb[0] + (double)(1 * NXbl) * D[0], Xb[1] + (double)(1 * NYbl) * D[1], Xb[2] + (double)(1 * NZbl) * D[2]};
  const int nsb[3] = {cfg.ncoarse, cfg.ncoarse, cfg.ncoarse};
  definepm(1, Xt, D, cfg.ncoarse, nsb, s.nnbl, s.nnbl_bl);
  for (int d = 0; d < 6; ++d) { s.xbound_bl[d] = Xt[d]; s.xbound_coarse[d] = Xb[d]; }
  for (int d = 0; d < 3; ++d) s.dpm_coarse[d] = (double)cfg.ncoarse * D[d];
  const int ns2 = 1 << std::max(cfg.ilevmax, 0);
  const int nsc[3] = {ns2, ns2, ns2};
  definepm(1, s.xbound_coarse, s.dpm_coarse, 4, nsc, s.nn_coarse, s.nn_bl_coarse);
  int ilev = cfg.ilevmax;
  for (int lev = 0; lev <= ilev; ++lev) {
    const int istep = 1 << lev;
    if ((s.nnbl_bl[3] - s.nnbl_bl[0]) / istep == 0 || (s.nnbl_bl[4] - s.nnbl_bl[1]) / istep == 0 ||
        (s.nnbl_bl[5] - s.nnbl_bl[2]) / istep == 0) {
      ilev = lev - 1;
      break;
    }
  }
  s.ilevmax = ilev;
  s.dvpm = D[0] * D[1] * D[2];
  s.defined = 1;
}

bool same_sizes(const vpmg_sizes& a, const vpmg_sizes& b) {
  return std::memcmp(&a, &b, sizeof(vpmg_sizes)) == 0;
}

Grid make_grid(const double xb[6], const double d[3], const int n[3]) {
  Grid g;
  for (int k = 0; k < 3; ++k) { g.xmin[k] = xb[k]; g.d[k] = d[k]; g.n[k] = n[k]; }
  return g;
}


void prepare(vpmg_handle* h) {
  const vpmg_sizes& s = h->sz;
  cudaStream_t st = h->stream;
  h->gglob = make_grid(s.xbound, s.dpm, s.nn);
  h->gbl = make_grid(s.xbound_bl, s.dpm, s.nnbl);
  h->gco = make_grid(s.xbound_coarse, s.dpm_coarse, s.nn_coarse);
  const size_t N = h->gglob.count(), NB = h->gbl.count(), NC = h->gco.count();
  h->nb3[0] = h->cfg.nbi; h->nb3[1] = h->cfg.nbj; h->nb3[2] = h->cfg.nbk;
  h->nblk = h->nb3[0] * h->nb3[1] * h->nb3[2];
  const size_t B = (size_t)h->nblk;
  h->rhs.ensure(3 * N); h->sol.ensure(3 * N); h->vel.ensure(3 * N); h->def.ensure(3 * N);
  if (h->arith == VPMG_ARITH_FF48) {  // float-float copies of the velocity and stretching for the gather
    h->vel_ff.ensure(3 * N); h->def_ff.ensure(3 * N);
    VPMG_CUDA(cudaMemsetAsync(h->vel_ff.p, 0, h->vel_ff.bytes(), h->stream));
    VPMG_CUDA(cudaMemsetAsync(h->def_ff.p, 0, h->def_ff.bytes(), h->stream));
  } else {
    h->vel_ff.release(); h->def_ff.release();
  }
  h->rhs_bl.ensure(B * 3 * NB); h->sol_bl.ensure(B * 3 * NB); h->sol0.ensure(NB);
  h->samp.ensure(B * 3 * NC); h->crhs.ensure(3 * NC); h->csol.ensure(3 * NC); h->csol0.ensure(NC);
  h->sampsum.ensure(3 * NC);
  for (DBuf<double>* b : {&h->rhs, &h->sol, &h->vel, &h->def, &h->rhs_bl, &h->sol_bl, &h->sol0, &h->samp, &h->crhs,
                          &h->csol, &h->csol0, &h->sampsum})
    fill_zero(b->p, b->n, st);
  // Dirichlet plans: whole block, inner block box, whole coarse grid
  const int bl_full[6] = {0, 0, 0, s.nnbl[0] - 1, s.nnbl[1] - 1, s.nnbl[2] - 1};
  const int bl_inner[6] = {s.nnbl_bl[0] - 1, s.nnbl_bl[1] - 1, s.nnbl_bl[2] - 1,
                           s.nnbl_bl[3] - 1, s.nnbl_bl[4] - 1, s.nnbl_bl[5] - 1};
  const int c_full[6] = {0, 0, 0, s.nn_coarse[0] - 1, s.nn_coarse[1] - 1, s.nn_coarse[2] - 1};
  dirichlet_prepare(h->dp_bl, s.nnbl, bl_full, s.dpm, st, h->arith);
  dirichlet_prepare(h->dp_inner, s.nnbl, bl_inner, s.dpm, st, h->arith);
  dirichlet_prepare(h->dp_c, s.nn_coarse, c_full, s.dpm_coarse, st, h->arith);
  size_t wmax = 0;
  for (DirichletPlan* p : {&h->dp_bl, &h->dp_inner, &h->dp_c}) wmax = std::max(wmax, (size_t)p->m[0] * p->m[1] * p->m[2]);
  h->work.ensure(wmax);
  if (h->nblk == 1) {
    h->bsolve.prepare(h->dp_bl, s.nnbl_bl, h->cfg.ncoarse);
    h->fsolve.prepare(h->dp_inner);
  }
  for (int d = 0; d < 3; ++d) {
    h->inner_lo[d] = s.nnbl_bl[d] - 1;
    h->inner_ext[d] = s.nnbl_bl[d + 3] - s.nnbl_bl[d] + 1;
  }
  // boundary operators: fine block (levels ilevmax), coarse (ilevmax-1); iyntree = 0 -> untreed sum
  const bool tree = h->cfg.iyntree == 1;
  boundary_prepare(h->bo_c, h->gco, tree ? std::max(s.ilevmax - 1, 0) : 0, h->op_budget, st, h->cfg.ibctyp, tree,
                   h->arith);
  if (h->nblk == 1) {
    boundary_prepare(h->bo_bl, h->gbl, tree ? std::max(s.ilevmax, 0) : 0, h->op_budget, st, h->cfg.ibctyp, tree,
                     h->arith);
    // YAPS maps
    YapsGeom Y;
    try {
      build_yaps_geometry(s.xbound_bl, s.dpm, s.nnbl, s.nnbl_bl, s.xbound_coarse, s.dpm_coarse, s.nn_coarse,
                          h->cfg.ncoarse, Y);
    } catch (const std::exception& e) {
      throw Error{VPMG_ERR_UNSUPPORTED, e.what()};
    }
    h->yaps.prepare(Y);
  } else {
    // several blocks: block boxes, one boundary operator each (the tree
    // geometry is built from each block's own coordinates), gather maps
    YapsMultiGeom Y;
    try {
      build_yaps_multi(h->nb3, s.xbound, s.dpm, h->cfg.ncoarse, s.nnbl, s.nnbl_bl, s.xbound_coarse, s.dpm_coarse,
                       s.nn_coarse, Y);
    } catch (const std::exception& e) {
      throw Error{VPMG_ERR_UNSUPPORTED, e.what()};
    }
    h->g_blk.assign(h->nblk, Grid{});
    h->bo_blk.clear();
    for (int b = 0; b < h->nblk; ++b) {
      h->g_blk[b] = make_grid(&Y.xbl[6 * (size_t)b], s.dpm, s.nnbl);
      h->bo_blk.push_back(std::make_unique<BoundaryOp>());
      boundary_prepare(*h->bo_blk[b], h->g_blk[b], tree ? std::max(s.ilevmax, 0) : 0, h->op_budget / h->nblk, st,
                       h->cfg.ibctyp, tree, h->arith);
    }
    h->ym.prepare(Y);
  }
  // particles: capacity for a full remesh of the global mesh
  h->parts.ensure((int)std::min<size_t>(N, (size_t)INT32_MAX / 16));
  h->parts.arith = h->arith;
  h->bins.ensure(N);
  VPMG_CUDA(cudaStreamSynchronize(st));
  h->prepared = true;
}

MeshDev mesh_dev(const Grid& g, int itype) {
  MeshDev m;
  for (int k = 0; k < 3; ++k) { m.xmin[k] = g.xmin[k]; m.d[k] = g.d[k]; m.inv[k] = 1.0 / g.d[k]; m.n[k] = g.n[k]; }
  m.itype = itype;
  m.ips = (itype == 2) ? 0 : 1;
  m.ipf = (itype == 2) ? 1 : 2;
  return m;
}

void ev_mark(vpmg_handle* h, int i) {
  if (h->profile) VPMG_CUDA(cudaEventRecord(h->ev[i], h->stream));
}

// pmesh(iynbc = 1) on a grid: zero-BC solve, panels, boundary values, BC solve.
void infinite_domain(vpmg_handle* h, DirichletPlan& dp, BoundaryOp& bo, const Grid& g, double* rhs3, double* sol3,
                     double* sol0, size_t n) {
  cudaStream_t st = h->stream;
  for (int c = 0; c < 3; ++c) {
    dirichlet_solve(dp, rhs3 + c * n, sol0, true, h->work.p, st);
    boundary_panels(bo, g, sol0, c, st);
  }
  double* sp[3] = {sol3, sol3 + n, sol3 + 2 * n};
  boundary_apply(bo, g, sp, st);
  for (int c = 0; c < 3; ++c) dirichlet_solve(dp, rhs3 + c * n, sol3 + c * n, false, h->work.p, st);
}

// The vector-potential solve: global RHS (h->rhs) -> global SOL (h->sol),
// i.e. rhsscat_3d, yaps3d (one block) and solget_3d.
// yaps3d with NBI x NBJ x NBK blocks (yaps_multi.cu): the blocks' solves run
// one after the other on the stream, every block solve in full.
void poisson_part_multi(vpmg_handle* h) {
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  const size_t N = h->gglob.count(), NB = h->gbl.count(), NC = h->gco.count();
  yaps_multi_rhsscat(h->ym, h->rhs.p, s.nn, s.nn_bl, s.nnbl, s.nnbl_bl, h->nb3, h->rhs_bl.p, st);
  fill_zero(h->sol_bl.p, (size_t)h->nblk * 3 * NB, st);
  ev_mark(h, 1);
  for (int b = 0; b < h->nblk; ++b) {
    double* RB = h->rhs_bl.p + (size_t)b * 3 * NB;
    double* SB[3] = {h->sol_bl.p + (size_t)b * 3 * NB, h->sol_bl.p + ((size_t)b * 3 + 1) * NB,
                     h->sol_bl.p + ((size_t)b * 3 + 2) * NB};
    BoundaryOp& bo = *h->bo_blk[b];
    for (int c = 0; c < 3; ++c) {
      dirichlet_solve(h->dp_bl, RB + c * NB, h->sol0.p, true, h->work.p, st);
      boundary_panels(bo, h->g_blk[b], h->sol0.p, c, st);
    }
    boundary_apply(bo, h->g_blk[b], SB, st);
    for (int c = 0; c < 3; ++c) dirichlet_solve(h->dp_bl, RB + c * NB, SB[c], false, h->work.p, st);
  }
  if (h->keep_intermediates) {
    h->bl_sol1_copy.ensure(3 * NB);
    VPMG_CUDA(cudaMemcpyAsync(h->bl_sol1_copy.p, h->sol_bl.p, sizeof(double) * 3 * NB, cudaMemcpyDeviceToDevice, st));
  }
  ev_mark(h, 4);
  fill_zero(h->csol.p, 3 * NC, st);
  yaps_multi_coarse(h->ym, h->sol_bl.p, NB, s.nn_coarse, s.dpm_coarse, h->samp.p, h->sampsum.p, h->crhs.p, st);
  infinite_domain(h, h->dp_c, h->bo_c, h->gco, h->crhs.p, h->csol.p, h->csol0.p, NC);
  yaps_multi_faces(h->ym, s.nn_coarse, h->csol.p, h->sampsum.p, h->samp.p, h->sol_bl.p, NB, st);
  ev_mark(h, 5);
  for (int b = 0; b < h->nblk; ++b)
    for (int c = 0; c < 3; ++c) {
      const size_t off = ((size_t)b * 3 + c) * NB;
      dirichlet_solve(h->dp_inner, h->rhs_bl.p + off, h->sol_bl.p + off, false, h->work.p, st);
    }
  yaps_multi_solget(h->sol_bl.p, s.nnbl, s.nnbl_bl, h->nb3, s.nn, s.nn_bl, h->sol.p, st);
  (void)N;
  ev_mark(h, 6);
}

// Single block, up to the fine block's boundary sources: rhsscat_3d and the
// zero-BC block solves with their normal-derivative panels.
void poisson_head(vpmg_handle* h) {
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  const size_t N = h->gglob.count(), NB = h->gbl.count();
  double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
  // rhsscat_3d: global interior -> block inner box; the block padding stays zero
  const int go[3] = {s.nn_bl[0] - 1, s.nn_bl[1] - 1, s.nn_bl[2] - 1};
  for (int c = 0; c < 3; ++c) box_copy(R[c], s.nn, go, comp(h->rhs_bl, NB, c), s.nnbl, h->inner_lo, h->inner_ext, st);
  fill_zero(h->sol_bl.p, 3 * NB, st);
  ev_mark(h, 1);
  // yaps3d (a): fine infinite-domain solve on the padded block.  By default
  // both block solves are evaluated only where the step reads them
  // (block_solve.cu); the full solves remain for parity checks.
  const bool full = h->full_block_solves || h->keep_intermediates;
  for (int c = 0; c < 3; ++c) {
    if (full) dirichlet_solve(h->dp_bl, comp(h->rhs_bl, NB, c), h->sol0.p, true, h->work.p, st);
    else block_solve_zero_bc(h->bsolve, h->dp_bl, comp(h->rhs_bl, NB, c), c, h->sol0.p, st);
    boundary_panels(h->bo_bl, h->gbl, h->sol0.p, c, st);
  }
  ev_mark(h, 2);
}

// Single block, from the fine block's boundary values on: BC solves,
// coarse grid, final inner-box solve and solget_3d.
void poisson_tail(vpmg_handle* h) {
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  const size_t N = h->gglob.count(), NB = h->gbl.count(), NC = h->gco.count();
  const int go[3] = {s.nn_bl[0] - 1, s.nn_bl[1] - 1, s.nn_bl[2] - 1};
  const bool full = h->full_block_solves || h->keep_intermediates;
  double* SB[3] = {comp(h->sol_bl, NB, 0), comp(h->sol_bl, NB, 1), comp(h->sol_bl, NB, 2)};
  ev_mark(h, 3);
  for (int c = 0; c < 3; ++c) {
    if (full) dirichlet_solve(h->dp_bl, comp(h->rhs_bl, NB, c), SB[c], false, h->work.p, st);
    else block_solve_bc(h->bsolve, h->dp_bl, c, SB[c], st);
  }
  if (h->keep_intermediates) {
    h->bl_sol1_copy.ensure(3 * NB);
    VPMG_CUDA(cudaMemcpyAsync(h->bl_sol1_copy.p, h->sol_bl.p, sizeof(double) * 3 * NB, cudaMemcpyDeviceToDevice, st));
  }
  ev_mark(h, 4);
  // (b)-(d): sample, coarse Laplacian, coarse infinite-domain solve, face interpolation
  fill_zero(h->samp.p, 3 * NC, st);
  fill_zero(h->crhs.p, 3 * NC, st);
  fill_zero(h->csol.p, 3 * NC, st);
  double* SM[3] = {comp(h->samp, NC, 0), comp(h->samp, NC, 1), comp(h->samp, NC, 2)};
  double* CR[3] = {comp(h->crhs, NC, 0), comp(h->crhs, NC, 1), comp(h->crhs, NC, 2)};
  double* CS[3] = {comp(h->csol, NC, 0), comp(h->csol, NC, 1), comp(h->csol, NC, 2)};
  yaps_sample(h->yaps, SB, SM, st);
  yaps_coarse_rhs(h->yaps, s.nn_coarse, s.dpm_coarse, SM, CR, st);
  infinite_domain(h, h->dp_c, h->bo_c, h->gco, h->crhs.p, h->csol.p, h->csol0.p, NC);
  yaps_face_interp(h->yaps, s.nn_coarse, CS, SM, SB, st);
  ev_mark(h, 5);
  // (e): final Dirichlet solve on the inner block box: the RHS (zero away
  // from the vorticity) transformed alone, the faces' values in DST space
  // (the block's transform scratch W is free by now)
  for (int c = 0; c < 3; ++c) {
    if (h->fsolve.ready && h->bsolve.ready)
      dirichlet_solve_faces(h->dp_inner, h->fsolve, comp(h->rhs_bl, NB, c), SB[c], h->work.p, h->bsolve.W.p, st);
    else
      dirichlet_solve(h->dp_inner, comp(h->rhs_bl, NB, c), SB[c], false, h->work.p, st);
  }
  // solget_3d
  double* S[3] = {comp(h->sol, N, 0), comp(h->sol, N, 1), comp(h->sol, N, 2)};
  for (int c = 0; c < 3; ++c) box_copy(SB[c], s.nnbl, h->inner_lo, S[c], s.nn, go, h->inner_ext, st);
  ev_mark(h, 6);
}

void poisson_part(vpmg_handle* h) {
  if (h->nblk > 1) {
    poisson_part_multi(h);
    return;
  }
  poisson_head(h);
  const size_t NB = h->gbl.count();
  double* SB[3] = {comp(h->sol_bl, NB, 0), comp(h->sol_bl, NB, 1), comp(h->sol_bl, NB, 2)};
  boundary_apply(h->bo_bl, h->gbl, SB, h->stream);
  poisson_tail(h);
}

// Field part of vpm(WhatToDo = 2) on binned particles (vpm.f90:171-314 + yaps3d).
void deposit_rhs(vpmg_handle* h) {
  const size_t N = h->gglob.count();
  const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
  double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
  deposit(h->parts, mg, h->bins, R, h->stream);
}

// The float-float copies of the velocity and stretching (float-float
// arithmetic only; null pointers otherwise).
void ff_fields(vpmg_handle* h, float2* VF[3], float2* GF[3]) {
  const size_t N = h->gglob.count();
  const bool ff = h->arith == VPMG_ARITH_FF48 && h->vel_ff.p && h->def_ff.p;
  for (int c = 0; c < 3; ++c) {
    VF[c] = ff ? h->vel_ff.p + c * N : nullptr;
    GF[c] = ff ? h->def_ff.p + c * N : nullptr;
  }
}

// calc_velocity_serial_3d(1) on h->sol and h->rhs
void field_velocity(vpmg_handle* h) {
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  const size_t N = h->gglob.count();
  double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
  double* S[3] = {comp(h->sol, N, 0), comp(h->sol, N, 1), comp(h->sol, N, 2)};
  // calc_velocity_serial_3d(1)
  double* V[3] = {comp(h->vel, N, 0), comp(h->vel, N, 1), comp(h->vel, N, 2)};
  double* G[3] = {comp(h->def, N, 0), comp(h->def, N, 1), comp(h->def, N, 2)};
  float2* VF[3], * GF[3];
  ff_fields(h, VF, GF);
  velocity_and_stretching(s.nn, s.dpm, S, R, V, G, st, 3, VF[0] ? VF : nullptr, GF[0] ? GF : nullptr);
  ev_mark(h, 7);
}

void field_step(vpmg_handle* h) {
  deposit_rhs(h);
  poisson_part(h);
  field_velocity(h);
}

// back_to_particles_3D(1): FP64 from the velocity and stretching fields, or
// float-float from their copies (written with them by
// velocity_and_stretching).
void m2p_fields(vpmg_handle* h, int up_mode, bool euler, double dt, const double uinf[3]) {
  const size_t N = h->gglob.count();
  const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
  if (h->arith == VPMG_ARITH_FF48) {
    const float2* V[3] = {h->vel_ff.p, h->vel_ff.p + N, h->vel_ff.p + 2 * N};
    const float2* G[3] = {h->def_ff.p, h->def_ff.p + N, h->def_ff.p + 2 * N};
    m2p(h->parts, mg, h->bins, V, G, up_mode, euler, dt, uinf, h->stream);
  } else {
    const double* V[3] = {comp(h->vel, N, 0), comp(h->vel, N, 1), comp(h->vel, N, 2)};
    const double* G[3] = {comp(h->def, N, 0), comp(h->def, N, 1), comp(h->def, N, 2)};
    m2p(h->parts, mg, h->bins, V, G, up_mode, euler, dt, uinf, h->stream);
  }
}
void m2p_step(vpmg_handle* h, int up_mode, bool euler, double dt, const double uinf[3]) {
  m2p_fields(h, up_mode, euler, dt, uinf);
  ev_mark(h, 8);
}

// remesh_particles_3d(1): deposit on the mesh with the recomputed spacing,
// emit one particle per node with |w| >= (REAL)1e-9 (vpm_remesh.f90:50-195).
void remesh(vpmg_handle* h) {
  cudaStream_t st = h->stream;
  const vpmg_sizes& s = h->sz;
  Grid gr = h->gglob;
  for (int d = 0; d < 3; ++d) gr.d[d] = (s.xbound[d + 3] - s.xbound[d]) / (double)(s.nn[d] - 1);
  const MeshDev mr = mesh_dev(gr, h->cfg.interf_iproj);
  const size_t N = gr.count();
  bin_particles(h->parts, mr, h->bins, st);
  double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
  deposit(h->parts, mr, h->bins, R, st);
  const int hh = h->cfg.interf_iproj / 2;
  const int lo[3] = {s.nn_bl[0] - 1 + hh, s.nn_bl[1] - 1 + hh, s.nn_bl[2] - 1 + hh};
  const int hi[3] = {s.nn_bl[3] - 1 - hh, s.nn_bl[4] - 1 - hh, s.nn_bl[5] - 1 - hh};
  const double thr = (double)1e-09f;  // default-REAL literal of vpm_remesh.f90:184
  remesh_emit(h->parts, mr, h->bins, R, lo, hi, thr, st);  // count stays on the device
  ev_mark(h, 9);
}

__global__ void k_set_int(int* __restrict__ d, int v) { *d = v; }

// Host mirror of the device particle count, and the errors flagged since
// the last sync (stencil outside the mesh, remesh over capacity).
void sync_np(vpmg_handle* h) {
  check_particle_errors(h->bins, h->stream);
  h->np = read_count(h->parts.d_np.p, h->stream);
}

__global__ void k_aos_to_soa(const double* __restrict__ xa, const double* __restrict__ qa, int n, double* x, double* y,
                             double* z, double* q0, double* q1, double* q2, double* vol) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  x[p] = xa[3 * (size_t)p]; y[p] = xa[3 * (size_t)p + 1]; z[p] = xa[3 * (size_t)p + 2];
  q0[p] = qa[4 * (size_t)p]; q1[p] = qa[4 * (size_t)p + 1]; q2[p] = qa[4 * (size_t)p + 2]; vol[p] = qa[4 * (size_t)p + 3];
}

__global__ void k_soa_to_aos(int n, const double* x, const double* y, const double* z, const double* q0,
                             const double* q1, const double* q2, const double* vol, double* __restrict__ xa,
                             double* __restrict__ qa) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  xa[3 * (size_t)p] = x[p]; xa[3 * (size_t)p + 1] = y[p]; xa[3 * (size_t)p + 2] = z[p];
  qa[4 * (size_t)p] = q0[p]; qa[4 * (size_t)p + 1] = q1[p]; qa[4 * (size_t)p + 2] = q2[p]; qa[4 * (size_t)p + 3] = vol[p];
}

void upload_particles(vpmg_handle* h, const double* xp, const double* qp, int n) {
  VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes (WhatToDo = 0) must come first");
  VPMG_CHECK(n >= 0 && n <= h->parts.capacity, VPMG_ERR_CAPACITY, "more particles than mesh nodes");
  h->stage.ensure(7 * (size_t)std::max(n, 1));
  if (n > 0) {
    VPMG_CUDA(cudaMemcpyAsync(h->stage.p, xp, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, h->stream));
    VPMG_CUDA(cudaMemcpyAsync(h->stage.p + 3 * (size_t)n, qp, sizeof(double) * 4 * n, cudaMemcpyHostToDevice, h->stream));
    Particles& P = h->parts;
    k_aos_to_soa<<<(n + 255) / 256, 256, 0, h->stream>>>(h->stage.p, h->stage.p + 3 * (size_t)n, n, P.x.p, P.y.p, P.z.p,
                                                        P.q0.p, P.q1.p, P.q2.p, P.vol.p);
    VPMG_LAUNCHED();
    VPMG_CUDA(cudaGetLastError());
  }
  k_set_int<<<1, 1, 0, h->stream>>>(h->parts.d_np.p, n);
  VPMG_LAUNCHED();
  h->np = n;
}

void download_particles(vpmg_handle* h, double* xp, double* qp, int n) {
  if (n <= 0) return;
  h->stage.ensure(7 * (size_t)n);
  Particles& P = h->parts;
  k_soa_to_aos<<<(n + 255) / 256, 256, 0, h->stream>>>(n, P.x.p, P.y.p, P.z.p, P.q0.p, P.q1.p, P.q2.p, P.vol.p,
                                                      h->stage.p, h->stage.p + 3 * (size_t)n);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaMemcpyAsync(xp, h->stage.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
  VPMG_CUDA(cudaMemcpyAsync(qp, h->stage.p + 3 * (size_t)n, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, h->stream));
  VPMG_CUDA(cudaStreamSynchronize(h->stream));
}

// The caller's UP(3, n) into the device UP array, which back_to_particles
// then adds to (source/vpm_time.f90:92-94).
void upload_up(vpmg_handle* h, const double* up, int n) {
  VPMG_CHECK(up, VPMG_ERR_ARG, "UP is null");
  if (n > 0)
    VPMG_CUDA(cudaMemcpyAsync(h->parts.up.p, up, sizeof(double) * 3 * (size_t)n, cudaMemcpyHostToDevice, h->stream));
}

void finish_phase_times(vpmg_handle* h) {
  if (!h->profile) return;
  VPMG_CUDA(cudaEventSynchronize(h->ev[9]));
  for (int i = 0; i < 9; ++i) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, h->ev[i], h->ev[i + 1]) != cudaSuccess) { cudaGetLastError(); ms = 0.f; }
    h->phase_ms[i] = ms;
  }
}

std::string trim_tokens(const std::string& line, int n, std::vector<std::string>& out) {
  std::string t = line;
  for (char& ch : t)
    if (ch == ',') ch = ' ';
  std::istringstream is(t);
  std::string w;
  for (int i = 0; i < n && (is >> w); ++i) out.push_back(w);
  return t;
}

}  // namespace

// ======================================================================
extern "C" {

const char* vpmg_status_string(int st) {
  switch (st) {
    case VPMG_OK: return "ok";
    case VPMG_ERR_ARG: return "bad argument";
    case VPMG_ERR_CUDA: return "CUDA error";
    case VPMG_ERR_NOMEM: return "device out of memory";
    case VPMG_ERR_OUTSIDE: return "particle stencil outside the mesh";
    case VPMG_ERR_CAPACITY: return "particle capacity exceeded";
    case VPMG_ERR_UNSUPPORTED: return "unsupported option";
    case VPMG_ERR_STATE: return "call out of order";
    case VPMG_ERR_TREE: return "quadtree inconsistency";
    default: return "unknown status";
  }
}

const char* vpmg_last_error(const vpmg_handle* h) { return h ? h->err.c_str() : "null handle"; }

int vpmg_read_pm_inp(const char* path, vpmg_config* c) {
  // Positional list-directed reads of source/vpm.f90:132-152: each READ
  // takes the leading values of its record and skips the rest.
  if (!path || !c) return VPMG_ERR_ARG;
  std::ifstream f(path);
  if (!f) return VPMG_ERR_ARG;
  std::memset(c, 0, sizeof(*c));
  std::string line;
  auto rec = [&](int n, std::vector<std::string>& v) -> bool {
    v.clear();
    while ((int)v.size() < n) {
      if (!std::getline(f, line)) return false;
      trim_tokens(line, n - (int)v.size(), v);
    }
    return true;
  };
  std::vector<std::string> v;
  try {
    if (!rec(3, v)) return VPMG_ERR_ARG;
    for (int d = 0; d < 3; ++d) c->dpm[d] = std::stod(v[d]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->interf_iproj = std::stoi(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->ibctyp = std::stoi(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->idvpm = std::stoi(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->epsvol = std::stod(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->ncoarse = std::stoi(v[0]);
    if (!rec(3, v)) return VPMG_ERR_ARG; c->nbi = std::stoi(v[0]); c->nbj = std::stoi(v[1]); c->nbk = std::stoi(v[2]);
    if (!rec(2, v)) return VPMG_ERR_ARG; c->nremesh = std::stoi(v[0]); c->ncell_rem = std::stoi(v[1]);
    if (!rec(2, v)) return VPMG_ERR_ARG; c->iyntree = std::stoi(v[0]); c->ilevmax = std::stoi(v[1]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->ompthreads = std::stoi(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->idefine = std::stoi(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG; c->iynslice = std::stoi(v[0]);
    if (!rec(1, v)) return VPMG_ERR_ARG;
    c->ipmwrite = std::stoi(v[0]);
    if (c->ipmwrite > 10) return VPMG_ERR_ARG;  // IPMWRITE > 10 stops the reference (vpm.f90:146)
    for (int i = 0; i < c->ipmwrite; ++i) {
      if (!rec(2, v)) return VPMG_ERR_ARG;
      c->ipmwstart[i] = std::stoi(v[0]);
      c->ipmwsteps[i] = std::stoi(v[1]);
    }
  } catch (...) {
    return VPMG_ERR_ARG;
  }
  return VPMG_OK;
}

int vpmg_create(const vpmg_config* cfg, int device, vpmg_handle** out) {
  if (!cfg || !out) return VPMG_ERR_ARG;
  *out = nullptr;
  if (cfg->interf_iproj < 2 || cfg->interf_iproj > 6) return VPMG_ERR_ARG;
  if (cfg->ibctyp != 2 && cfg->ibctyp != 3) return VPMG_ERR_UNSUPPORTED;
  if (cfg->idvpm != 1) return VPMG_ERR_UNSUPPORTED;
  if (cfg->ncell_rem != 1) return VPMG_ERR_UNSUPPORTED;
  if (cfg->ncoarse < 1 || cfg->dpm[0] <= 0 || cfg->dpm[1] <= 0 || cfg->dpm[2] <= 0) return VPMG_ERR_ARG;
  vpmg_handle* h = new vpmg_handle();
  h->cfg = *cfg;
  if (device < 0) {
    if (cudaGetDevice(&h->device) != cudaSuccess) { cudaGetLastError(); delete h; return VPMG_ERR_CUDA; }
  } else {
    h->device = device;
  }
  int rc = guarded(h, [&] {
    VPMG_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
    for (int i = 0; i < 10; ++i) VPMG_CUDA(cudaEventCreate(&h->ev[i]));
    size_t fr = 0, tot = 0;
    VPMG_CUDA(cudaMemGetInfo(&fr, &tot));
    h->op_budget = std::min<long long>(100LL << 30, (long long)(0.6 * (double)fr));
  });
  if (rc != VPMG_OK) { delete h; return rc; }
  *out = h;
  return VPMG_OK;
}

int vpmg_destroy(vpmg_handle* h) {
  if (!h) return VPMG_ERR_ARG;
  cudaSetDevice(h->device);
  if (h->stream) cudaStreamSynchronize(h->stream);
  if (h->graph.exec) cudaGraphExecDestroy(h->graph.exec);
  vpmg::hx::destroy_adjoint(h);
  for (int i = 0; i < 10; ++i)
    if (h->ev[i]) cudaEventDestroy(h->ev[i]);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
  return VPMG_OK;
}

int vpmg_define_sizes(vpmg_handle* h, const double* xp, int nvr, int ntime) {
  return guarded(h, [&] {
    vpmg_sizes s = h->sz;
    define_sizes(h, xp, nvr, ntime, s);
    if (!h->prepared || !same_sizes(s, h->sz)) {
      h->sz = s;
      h->sized = true;
      prepare(h);
    }
  });
}

int vpmg_get_sizes(const vpmg_handle* h, vpmg_sizes* out) {
  if (!h || !out) return VPMG_ERR_ARG;
  if (!h->sized) return VPMG_ERR_STATE;
  *out = h->sz;
  return VPMG_OK;
}

int vpmg_set_particles(vpmg_handle* h, const double* xp, const double* qp, int nvr, int capacity) {
  (void)capacity;
  return guarded(h, [&] {
    upload_particles(h, xp, qp, nvr);
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int vpmg_get_particles(vpmg_handle* h, double* xp, double* qp, int* nvr, int capacity) {
  return guarded(h, [&] {
    VPMG_CHECK(nvr, VPMG_ERR_ARG, "nvr is null");
    sync_np(h);
    *nvr = h->np;
    VPMG_CHECK(h->np <= capacity, VPMG_ERR_CAPACITY, "caller arrays too small");
    download_particles(h, xp, qp, h->np);
  });
}

int vpmg_get_particle_velocity(vpmg_handle* h, double* up, double* gp, int nvr) {
  return guarded(h, [&] {
    VPMG_CHECK(nvr <= h->parts.capacity && nvr >= 0, VPMG_ERR_ARG, "nvr out of range");
    if (nvr == 0) return;
    VPMG_CUDA(cudaMemcpyAsync(up, h->parts.up.p, sizeof(double) * 3 * nvr, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaMemcpyAsync(gp, h->parts.gp.p, sizeof(double) * 3 * nvr, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int vpmg_num_particles(const vpmg_handle* h, int* nvr) {
  if (!h || !nvr) return VPMG_ERR_ARG;
  *nvr = h->np;
  return VPMG_OK;
}

namespace {
// hist[(*counter)++] = particle count at the start of a step (graph node).
__global__ void k_log_count(int* __restrict__ hist, int* __restrict__ counter, const int* __restrict__ np, int cap) {
  const int c = *counter;
  if (c < cap) hist[c] = *np;
  *counter = c + 1;
}

constexpr int kHistCap = 1 << 16;

// A single-block step in two parts around the fine block's boundary
// operator (one_step = step_head, boundary_apply, step_tail), so that
// problems sharing an operator can meet at one apply.
void step_head(vpmg_handle* h) {
  ev_mark(h, 0);
  bin_particles(h->parts, mesh_dev(h->gglob, h->cfg.interf_iproj), h->bins, h->stream);
  deposit_rhs(h);
  poisson_head(h);
}
void step_tail(vpmg_handle* h, double dt, const double u0[3], int do_remesh) {
  poisson_tail(h);
  field_velocity(h);
  m2p_step(h, kUpSet, true, dt, u0);
  if (do_remesh) remesh(h);
  else ev_mark(h, 9);
}

void one_step(vpmg_handle* h, double dt, const double uinf[3], int do_remesh) {
  VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
  const double u0[3] = {uinf ? uinf[0] : 0.0, uinf ? uinf[1] : 0.0, uinf ? uinf[2] : 0.0};
  ev_mark(h, 0);
  bin_particles(h->parts, mesh_dev(h->gglob, h->cfg.interf_iproj), h->bins, h->stream);
  field_step(h);
  m2p_step(h, kUpSet, true, dt, u0);
  if (do_remesh) remesh(h);
  else ev_mark(h, 9);
}

// One step (field step + Euler + remesh, preceded by the count log) as a
// CUDA graph on the handle's stream.  Re-captured when dt, uinf or the
// remesh flag change.
void ensure_graph(vpmg_handle* h, double dt, const double uinf[3], int do_remesh) {
  VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
  VPMG_CHECK(!h->keep_intermediates, VPMG_ERR_STATE, "graph capture is off while intermediates are kept");
  const double u0[3] = {uinf ? uinf[0] : 0.0, uinf ? uinf[1] : 0.0, uinf ? uinf[2] : 0.0};
  auto& G = h->graph;
  if (G.exec && G.dt == dt && G.u[0] == u0[0] && G.u[1] == u0[1] && G.u[2] == u0[2] && G.remesh == do_remesh) return;
  if (G.exec) {
    cudaGraphExecDestroy(G.exec);
    G.exec = nullptr;
  }
  h->hist.ensure(kHistCap);
  h->hist_counter.ensure(1);
  const bool prof = h->profile;
  h->profile = false;
  const long long l0 = h->launches;
  cudaGraph_t g = nullptr;
  VPMG_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  try {
    k_log_count<<<1, 1, 0, h->stream>>>(h->hist.p, h->hist_counter.p, h->parts.d_np.p, kHistCap);
    VPMG_LAUNCHED();
    one_step(h, dt, u0, do_remesh);
  } catch (...) {
    cudaStreamEndCapture(h->stream, &g);
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    h->profile = prof;
    h->launches = l0;
    throw;
  }
  h->profile = prof;
  VPMG_CUDA(cudaStreamEndCapture(h->stream, &g));
  cudaError_t e = cudaGraphInstantiate(&G.exec, g, 0);
  cudaGraphDestroy(g);
  VPMG_CUDA(e);
  G.launches = h->launches - l0;  // counted per replay from now on
  h->launches = l0;
  G.dt = dt;
  for (int d = 0; d < 3; ++d) G.u[d] = u0[d];
  G.remesh = do_remesh;
}

long long read_hist(vpmg_handle* h, int n) {
  std::vector<int> v(std::max(n, 1));
  if (n > 0) VPMG_CUDA(cudaMemcpyAsync(v.data(), h->hist.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
  VPMG_CUDA(cudaStreamSynchronize(h->stream));
  long long s = 0;
  for (int i = 0; i < n; ++i) s += v[i];
  return s;
}
}  // namespace

int vpmg_step(vpmg_handle* h, double dt, const double uinf[3], int do_remesh) {
  return guarded(h, [&] {
    one_step(h, dt, uinf, do_remesh);
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
    sync_np(h);
    finish_phase_times(h);
  });
}

int vpmg_run(vpmg_handle* h, int nsteps, double dt, const double uinf[3], int do_remesh, double* ms,
             long long* particle_steps) {
  return guarded(h, [&] {
    VPMG_CHECK(nsteps >= 0, VPMG_ERR_ARG, "nsteps < 0");
    const bool use_graph = !h->keep_intermediates && !h->no_graphs;
    if (use_graph) ensure_graph(h, dt, uinf, do_remesh);
    cudaEvent_t a, b;
    VPMG_CUDA(cudaEventCreate(&a));
    VPMG_CUDA(cudaEventCreate(&b));
    const bool prof = h->profile;
    h->profile = false;
    long long ps = 0;
    float t = 0.f;
    try {
      for (int done = 0; done < nsteps || (nsteps == 0 && done == 0);) {
        const int chunk = std::min(nsteps - done, kHistCap);
        VPMG_CUDA(cudaStreamSynchronize(h->stream));
        if (use_graph) VPMG_CUDA(cudaMemsetAsync(h->hist_counter.p, 0, sizeof(int), h->stream));
        VPMG_CUDA(cudaEventRecord(a, h->stream));
        for (int k = 0; k < chunk; ++k) {
          if (use_graph) {
            VPMG_CUDA(cudaGraphLaunch(h->graph.exec, h->stream));
          } else {
            ps += h->np;
            one_step(h, dt, uinf, do_remesh);
            VPMG_CUDA(cudaStreamSynchronize(h->stream));
            sync_np(h);
          }
        }
        VPMG_CUDA(cudaEventRecord(b, h->stream));
        VPMG_CUDA(cudaEventSynchronize(b));
        float tc = 0.f;
        VPMG_CUDA(cudaEventElapsedTime(&tc, a, b));
        t += tc;
        if (use_graph) {
          ps += read_hist(h, chunk);
          h->launches += (long long)chunk * h->graph.launches;
        }
        done += chunk;
        if (nsteps == 0) break;
      }
      sync_np(h);
    } catch (...) {
      h->profile = prof;
      cudaEventDestroy(a);
      cudaEventDestroy(b);
      throw;
    }
    h->profile = prof;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t;
    if (particle_steps) *particle_steps = ps;
  });
}

int vpmg_batch_run(vpmg_handle* const* hs, int n, int nsteps, double dt, int do_remesh, double* ms,
                   long long* solves, long long* particle_steps) {
  if (!hs || n <= 0 || nsteps < 0) return VPMG_ERR_ARG;
  for (int i = 0; i < n; ++i)
    if (!hs[i]) return VPMG_ERR_ARG;
  // each problem: its own handle, stream and step graph; the graphs of all
  // problems are replayed step by step, interleaved, on their own streams
  for (int i = 0; i < n; ++i) {
    const int rc = guarded(hs[i], [&] {
      ensure_graph(hs[i], dt, nullptr, do_remesh);
      VPMG_CUDA(cudaMemsetAsync(hs[i]->hist_counter.p, 0, sizeof(int), hs[i]->stream));
      VPMG_CUDA(cudaStreamSynchronize(hs[i]->stream));
    });
    if (rc != VPMG_OK) return rc;
  }
  vpmg_handle* h0 = hs[0];
  return guarded(h0, [&] {
    VPMG_CHECK(nsteps <= kHistCap, VPMG_ERR_ARG, "too many steps for one batched run");
    cudaEvent_t start, stop;
    std::vector<cudaEvent_t> done(n);
    VPMG_CUDA(cudaEventCreateWithFlags(&start, cudaEventDefault));
    VPMG_CUDA(cudaEventCreateWithFlags(&stop, cudaEventDefault));
    for (int i = 0; i < n; ++i) VPMG_CUDA(cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming));
    VPMG_CUDA(cudaEventRecord(start, h0->stream));
    for (int i = 1; i < n; ++i) VPMG_CUDA(cudaStreamWaitEvent(hs[i]->stream, start, 0));
    for (int k = 0; k < nsteps; ++k)
      for (int i = 0; i < n; ++i) VPMG_CUDA(cudaGraphLaunch(hs[i]->graph.exec, hs[i]->stream));
    for (int i = 1; i < n; ++i) {
      VPMG_CUDA(cudaEventRecord(done[i], hs[i]->stream));
      VPMG_CUDA(cudaStreamWaitEvent(h0->stream, done[i], 0));
    }
    VPMG_CUDA(cudaEventRecord(stop, h0->stream));
    VPMG_CUDA(cudaEventSynchronize(stop));
    float t = 0.f;
    VPMG_CUDA(cudaEventElapsedTime(&t, start, stop));
    cudaEventDestroy(start);
    cudaEventDestroy(stop);
    for (int i = 0; i < n; ++i) cudaEventDestroy(done[i]);
    long long ps = 0;
    for (int i = 0; i < n; ++i) {
      ps += read_hist(hs[i], nsteps);
      hs[i]->launches += (long long)nsteps * hs[i]->graph.launches;
      LaunchScope ls(hs[i]);
      sync_np(hs[i]);
    }
    if (ms) *ms = t;
    if (solves) *solves = (long long)n * nsteps;
    if (particle_steps) *particle_steps = ps;
  });
}

// ---------------------------------------------------------------- batch ----
// Problems grouped by shared boundary operator.  A unit is one problem (its
// own step graph) or a group of up to kGroupMax problems whose fine-block
// operators are one recorded operator up to the mesh-spacing factor: the
// group's step is one graph in which every member runs its step head on its
// own stream, one launch applies the leader's operator to all members'
// sources (the weights stream from HBM once for the group), and the members
// run their step tails.  Units replay step by step on their leaders' streams.
struct vpmg_batch {
  struct Unit {
    std::vector<int> m;  // indices into hs; m[0] leads
    std::vector<double> ratio;
    std::vector<std::unique_ptr<GroupCorrection>> corr;  // per member (the leader's is empty)
    vpmg::DBuf<float2> gsrc;
    vpmg::DBuf<double> part;  // the dense block's partial sums per problem
    cudaGraphExec_t exec = nullptr;
    long long launches = 0;
    double dt = 0.0;
    int remesh = -1;
  };
  std::vector<vpmg_handle*> hs;
  std::vector<std::unique_ptr<Unit>> units;
  // replay order of the units within a step: 0 concurrent (each unit on its
  // leader's stream), 1 one after another on one stream, -1 chosen by timing
  // the first two steps of a call (one of each)
  int schedule = -1;
  float tuned_ms[2] = {0.f, 0.f};
  ~vpmg_batch() {
    for (auto& u : units)
      if (u->exec) cudaGraphExecDestroy(u->exec);
  }
};

namespace {
// CUDA events owned for the duration of one call (timed or not).
struct EventSet {
  std::vector<cudaEvent_t> e;
  EventSet(size_t n, bool timing) : e(n, nullptr) {
    try {
      for (auto& x : e) VPMG_CUDA(timing ? cudaEventCreate(&x) : cudaEventCreateWithFlags(&x, cudaEventDisableTiming));
    } catch (...) {
      release();  // a throwing constructor runs no destructor
      throw;
    }
  }
  ~EventSet() { release(); }
  void release() {
    for (auto& x : e)
      if (x) {
        cudaEventDestroy(x);
        x = nullptr;
      }
  }
  EventSet(const EventSet&) = delete;
  EventSet& operator=(const EventSet&) = delete;
};

// a follower whose recorded operator differs from the leader's in more than
// this fraction of the interactions keeps its own graph
constexpr double kGroupMaxCorrected = 0.02;

bool group_eligible(const vpmg_handle* h) {
  return h->prepared && h->nblk == 1 && h->bo_bl.precomputed && h->bo_bl.ibctyp == 2 && !h->keep_intermediates &&
         !h->no_graphs && !h->full_block_solves;
}

void capture_group(vpmg_batch* b, vpmg_batch::Unit& u, double dt, int do_remesh) {
  const double u0[3] = {0.0, 0.0, 0.0};
  const int n = (int)u.m.size();
  std::vector<vpmg_handle*> H(n);
  for (int k = 0; k < n; ++k) H[k] = b->hs[u.m[k]];
  vpmg_handle* L = H[0];
  cudaStream_t ls = L->stream;
  if (u.exec) {
    cudaGraphExecDestroy(u.exec);
    u.exec = nullptr;
  }
  GroupOut G{};
  for (int k = 0; k < n; ++k) {
    const size_t NB = H[k]->gbl.count();
    for (int c = 0; c < 3; ++c) G.o[k][c] = H[k]->sol_bl.p + c * NB;
    G.scale[k] = -u.ratio[k] / (4.0 * kPI);
    H[k]->hist.ensure(kHistCap);
    H[k]->hist_counter.ensure(1);
  }
  EventSet evs(2 * (size_t)n + 1, false);
  std::vector<cudaEvent_t>& ev = evs.e;
  std::vector<char> prof(n);
  std::vector<long long> l0(n);
  for (int k = 0; k < n; ++k) {
    prof[k] = H[k]->profile;
    H[k]->profile = false;
    l0[k] = H[k]->launches;
  }
  auto restore = [&] {
    for (int k = 0; k < n; ++k) H[k]->profile = prof[k];
  };
  const int lanes = n;
  cudaGraph_t g = nullptr;
  try {
    VPMG_CUDA(cudaStreamBeginCapture(ls, cudaStreamCaptureModeThreadLocal));
    try {
      VPMG_CUDA(cudaEventRecord(ev[0], ls));
      for (int k = 1; k < n; ++k) VPMG_CUDA(cudaStreamWaitEvent(H[k]->stream, ev[0], 0));
      for (int k = 0; k < n; ++k) {
        LaunchScope sc(H[k]);
        k_log_count<<<1, 1, 0, H[k]->stream>>>(H[k]->hist.p, H[k]->hist_counter.p, H[k]->parts.d_np.p, kHistCap);
        VPMG_LAUNCHED();
        step_head(H[k]);
        boundary_group_sources(H[k]->bo_bl, u.gsrc.p, k, lanes, H[k]->stream);
      }
      for (int k = 1; k < n; ++k) {
        VPMG_CUDA(cudaEventRecord(ev[k], H[k]->stream));
        VPMG_CUDA(cudaStreamWaitEvent(ls, ev[k], 0));
      }
      {
        LaunchScope sc(L);
        boundary_group_apply(L->bo_bl, u.gsrc.p, n, u.part.p, G, ls);
      }
      VPMG_CUDA(cudaEventRecord(ev[n], ls));
      for (int k = 1; k < n; ++k) VPMG_CUDA(cudaStreamWaitEvent(H[k]->stream, ev[n], 0));
      for (int k = 0; k < n; ++k) {
        LaunchScope sc(H[k]);
        const size_t NB = H[k]->gbl.count();
        double* SB[3] = {H[k]->sol_bl.p, H[k]->sol_bl.p + NB, H[k]->sol_bl.p + 2 * NB};
        boundary_group_correct(H[k]->bo_bl, *u.corr[k], SB, H[k]->stream);
        step_tail(H[k], dt, u0, do_remesh);
      }
      for (int k = 1; k < n; ++k) {
        VPMG_CUDA(cudaEventRecord(ev[n + k], H[k]->stream));
        VPMG_CUDA(cudaStreamWaitEvent(ls, ev[n + k], 0));
      }
    } catch (...) {
      cudaStreamEndCapture(ls, &g);
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();
      throw;
    }
    VPMG_CUDA(cudaStreamEndCapture(ls, &g));
    cudaError_t e = cudaGraphInstantiate(&u.exec, g, 0);
    cudaGraphDestroy(g);
    VPMG_CUDA(e);
  } catch (...) {
    for (int k = 0; k < n; ++k) H[k]->launches = l0[k];
    restore();
    throw;
  }
  u.launches = 0;
  for (int k = 0; k < n; ++k) {
    u.launches += H[k]->launches - l0[k];
    H[k]->launches = l0[k];
  }
  restore();
  u.dt = dt;
  u.remesh = do_remesh;
}
}  // namespace

int vpmg_batch_create(vpmg_handle* const* hs, int n, int flags, vpmg_batch** out) {
  if (!hs || n <= 0 || !out) return VPMG_ERR_ARG;
  *out = nullptr;
  for (int i = 0; i < n; ++i)
    if (!hs[i]) return VPMG_ERR_ARG;
  std::unique_ptr<vpmg_batch> b(new vpmg_batch);
  b->hs.assign(hs, hs + n);
  const int rc = guarded(hs[0], [&] {
    for (int i = 0; i < n; ++i) {
      vpmg_handle* h = hs[i];
      VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first (every problem of a batch)");
      VPMG_CHECK(h->device == hs[0]->device, VPMG_ERR_ARG, "a batch runs on one device");
      for (int j = 0; j < i; ++j) VPMG_CHECK(hs[j] != h, VPMG_ERR_ARG, "a problem appears twice in the batch");
      bool placed = false;
      if (group_eligible(h)) {
        for (auto& u : b->units) {
          vpmg_handle* L = hs[u->m[0]];
          double r = 1.0;
          if ((int)u->m.size() >= kGroupMax || !group_eligible(L)) continue;
          std::unique_ptr<GroupCorrection> c(new GroupCorrection);
          if (boundary_group_match(L->bo_bl, L->gbl, h->bo_bl, h->gbl, kGroupMaxCorrected, &r, *c, h->stream)) {
            u->m.push_back(i);
            u->ratio.push_back(r);
            u->corr.push_back(std::move(c));
            placed = true;
            break;
          }
        }
      }
      if (!placed) {
        b->units.emplace_back(new vpmg_batch::Unit);
        b->units.back()->m.push_back(i);
        b->units.back()->ratio.push_back(1.0);
        b->units.back()->corr.emplace_back(new GroupCorrection);
      }
    }
    for (auto& u : b->units) {
      if (u->m.size() < 2) continue;
      if (flags & VPMG_BATCH_RELEASE_SHARED) {
        for (size_t k = 1; k < u->m.size(); ++k) {
          vpmg_handle* f = hs[u->m[k]];
          if (f->graph.exec) {
            cudaGraphExecDestroy(f->graph.exec);
            f->graph.exec = nullptr;
          }
          vpmg::hx::destroy_adjoint(f);
          boundary_release_recorded(f->bo_bl);
        }
      }
      const BoundaryOp& L = hs[u->m[0]]->bo_bl;
      u->gsrc.ensure(4 * (size_t)L.ncell_total * u->m.size());
      const size_t np = boundary_group_partial_count(L, (int)u->m.size());
      if (np) u->part.ensure(np);
      VPMG_CUDA(cudaMemsetAsync(u->gsrc.p, 0, u->gsrc.bytes(), hs[u->m[0]]->stream));
      VPMG_CUDA(cudaStreamSynchronize(hs[u->m[0]]->stream));
    }
  });
  if (rc != VPMG_OK) return rc;
  *out = b.release();
  return VPMG_OK;
}

int vpmg_batch_info(const vpmg_batch* b, int* units, int* shared, long long* correction_rows) {
  if (!b) return VPMG_ERR_ARG;
  int s = 0;
  long long cr = 0;
  for (auto& u : b->units) {
    if (u->m.size() > 1) s += (int)u->m.size();
    for (auto& c : u->corr) cr += c->nrows;
  }
  if (units) *units = (int)b->units.size();
  if (shared) *shared = s;
  if (correction_rows) *correction_rows = cr;
  return VPMG_OK;
}

int vpmg_batch_step(vpmg_batch* b, int nsteps, double dt, int do_remesh, double* ms, long long* solves,
                    long long* particle_steps) {
  if (!b || nsteps < 0) return VPMG_ERR_ARG;
  vpmg_handle* h0 = b->hs[0];
  return guarded(h0, [&] {
    VPMG_CHECK(nsteps <= kHistCap, VPMG_ERR_ARG, "too many steps for one batched run");
    for (auto& u : b->units) {
      if (u->m.size() == 1) {
        vpmg_handle* h = b->hs[u->m[0]];
        LaunchScope sc(h);
        ensure_graph(h, dt, nullptr, do_remesh);
      } else if (!u->exec || u->dt != dt || u->remesh != do_remesh) {
        capture_group(b, *u, dt, do_remesh);
      }
    }
    for (vpmg_handle* h : b->hs) {
      VPMG_CUDA(cudaMemsetAsync(h->hist_counter.p, 0, sizeof(int), h->stream));
      VPMG_CUDA(cudaStreamSynchronize(h->stream));
    }
    const size_t nu = b->units.size();
    EventSet marks((size_t)nsteps + 1, true), dones(nu, false);  // destroyed on every exit path
    std::vector<cudaEvent_t>& mark = marks.e;
    std::vector<cudaEvent_t>& done = dones.e;
    auto lead = [&](size_t i) { return b->hs[b->units[i]->m[0]]; };
    auto exec_of = [&](size_t i) {
      const auto& u = *b->units[i];
      return (u.m.size() == 1) ? lead(i)->graph.exec : u.exec;
    };
    // one step of every unit, concurrent or in sequence, between two marks on h0's stream
    auto step = [&](int k, int mode) {
      if (mode == 1) {
        for (size_t i = 0; i < nu; ++i) VPMG_CUDA(cudaGraphLaunch(exec_of(i), h0->stream));
        VPMG_CUDA(cudaEventRecord(mark[k + 1], h0->stream));
        return;
      }
      for (size_t i = 0; i < nu; ++i)
        if (lead(i)->stream != h0->stream) VPMG_CUDA(cudaStreamWaitEvent(lead(i)->stream, mark[k], 0));
      for (size_t i = 0; i < nu; ++i) VPMG_CUDA(cudaGraphLaunch(exec_of(i), lead(i)->stream));
      for (size_t i = 0; i < nu; ++i) {
        if (lead(i)->stream == h0->stream) continue;
        VPMG_CUDA(cudaEventRecord(done[i], lead(i)->stream));
        VPMG_CUDA(cudaStreamWaitEvent(h0->stream, done[i], 0));
      }
      VPMG_CUDA(cudaEventRecord(mark[k + 1], h0->stream));
    };
    VPMG_CUDA(cudaEventRecord(mark[0], h0->stream));
    int k0 = 0;
    if (b->schedule < 0 && nsteps >= 2 && nu > 1) {
      for (int m = 0; m < 2; ++m) {
        step(m, m);
        VPMG_CUDA(cudaEventSynchronize(mark[m + 1]));
        VPMG_CUDA(cudaEventElapsedTime(&b->tuned_ms[m], mark[m], mark[m + 1]));
      }
      b->schedule = (b->tuned_ms[1] < b->tuned_ms[0]) ? 1 : 0;
      k0 = 2;
    }
    // the remaining steps: in sequence on h0's stream, or each unit running
    // through them on its own stream (joined at the end)
    if (b->schedule == 1) {
      for (int k = k0; k < nsteps; ++k)
        for (size_t i = 0; i < nu; ++i) VPMG_CUDA(cudaGraphLaunch(exec_of(i), h0->stream));
      VPMG_CUDA(cudaEventRecord(mark[nsteps], h0->stream));
    } else if (k0 < nsteps) {
      for (size_t i = 0; i < nu; ++i)
        if (lead(i)->stream != h0->stream) VPMG_CUDA(cudaStreamWaitEvent(lead(i)->stream, mark[k0], 0));
      for (int k = k0; k < nsteps; ++k)
        for (size_t i = 0; i < nu; ++i) VPMG_CUDA(cudaGraphLaunch(exec_of(i), lead(i)->stream));
      for (size_t i = 0; i < nu; ++i) {
        if (lead(i)->stream == h0->stream) continue;
        VPMG_CUDA(cudaEventRecord(done[i], lead(i)->stream));
        VPMG_CUDA(cudaStreamWaitEvent(h0->stream, done[i], 0));
      }
      VPMG_CUDA(cudaEventRecord(mark[nsteps], h0->stream));
    }
    VPMG_CUDA(cudaEventSynchronize(mark[nsteps]));
    float t = 0.f;
    VPMG_CUDA(cudaEventElapsedTime(&t, mark[0], mark[nsteps]));
    long long ps = 0;
    for (size_t i = 0; i < nu; ++i) {
      const auto& u = *b->units[i];
      const long long per = (u.m.size() == 1) ? lead(i)->graph.launches : u.launches;
      lead(i)->launches += (long long)nsteps * per;
    }
    for (vpmg_handle* h : b->hs) {
      ps += read_hist(h, nsteps);
      LaunchScope ls(h);
      sync_np(h);
    }
    if (ms) *ms = t;
    if (solves) *solves = (long long)b->hs.size() * nsteps;
    if (particle_steps) *particle_steps = ps;
  });
}

int vpmg_batch_set_schedule(vpmg_batch* b, int schedule) {
  if (!b || schedule < -1 || schedule > 1) return VPMG_ERR_ARG;
  b->schedule = schedule;
  return VPMG_OK;
}

int vpmg_batch_get_schedule(const vpmg_batch* b, int* schedule, float tuned_ms[2]) {
  if (!b) return VPMG_ERR_ARG;
  if (schedule) *schedule = b->schedule;
  if (tuned_ms) {
    tuned_ms[0] = b->tuned_ms[0];
    tuned_ms[1] = b->tuned_ms[1];
  }
  return VPMG_OK;
}

int vpmg_batch_destroy(vpmg_batch* b) {
  if (!b) return VPMG_ERR_ARG;
  delete b;
  return VPMG_OK;
}

int vpmg_bench_kernel(vpmg_handle* h, int which, int reps, double* ms, double* flops, double* bytes) {
  return guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
    VPMG_CHECK(reps >= 1, VPMG_ERR_ARG, "reps < 1");
    const size_t N = h->gglob.count(), NB = h->gbl.count();
    cudaStream_t st = h->stream;
    double fl = 0, by = 0;
    std::function<void()> f;
    if (which == 0) {
      h->bench_scratch.ensure(3 * NB);
      double* o[3] = {h->bench_scratch.p, h->bench_scratch.p + NB, h->bench_scratch.p + 2 * NB};
      BoundaryOp* bo = h->nblk > 1 ? h->bo_blk[0].get() : &h->bo_bl;
      const Grid* g = h->nblk > 1 ? &h->g_blk[0] : &h->gbl;
      f = [bo, g, o, st] { boundary_apply(*bo, *g, o, st); };
      const double nnz = (double)(bo->nnz + bo->ndense_acc);  // accepted interactions
      fl = 2.0 * 3.0 * nnz;  // three FMAs per interaction
      // streamed bytes: 12 per row entry (cell id + weight pair), 8 per slot of the dense block
      by = bo->precomputed ? (double)bo->nnz * (sizeof(int) + sizeof(float2)) + (double)bo->wtop.bytes() : 0.0;
      if (bo->ff.on) {
        // the coarsest level by FFT: the finer rows and the correction rows
        // at three FMAs per entry, plus the transforms' flops; bytes: both
        // row lists, the kernel spectra, and the transform arrays read and
        // written once per pass
        const FarField& F = bo->ff;
        fl = 6.0 * ((double)bo->nnz + (double)F.ncorr) + F.flops;
        by = 12.0 * ((double)bo->nnz + (double)F.ncorr) + (double)(F.kperp.bytes() + F.kpar.bytes()) +
             4.0 * (double)(F.S2.bytes() + F.X.bytes() + F.Z.bytes() + F.Sw.bytes() + F.T.bytes());
      }
    } else if (which == 1) {
      h->bench_scratch.ensure(NB);
      double* o = h->bench_scratch.p;
      f = [h, o, st] { dirichlet_solve(h->dp_inner, h->rhs_bl.p, o, true, h->work.p, st); };
      const DirichletPlan& P = h->dp_inner;
      const double nint = (double)P.m[0] * P.m[1] * P.m[2];
      fl = nint * (5.0 * std::log2(2.0 * (P.m[0] + 1)) + 5.0 * std::log2(2.0 * (P.m[1] + 1)) + 9.0);
      by = 16.0 * (double)NB;
    } else if (which == 2) {
      h->bench_scratch.ensure(3 * N);
      double* o[3] = {h->bench_scratch.p, h->bench_scratch.p + N, h->bench_scratch.p + 2 * N};
      const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
      // the last step ended with a remesh, which reuses the binning buffers
      // for its compaction: bin the current particles on the global mesh again
      bin_particles(h->parts, mg, h->bins, st);
      f = [h, o, mg, st] { deposit(h->parts, mg, h->bins, o, st); };
      const double P = (double)read_count(h->bins.nsorted_dev, st);
      const int w = mg.ips + mg.ipf + 1;
      fl = P * w * w * w * 7.0;  // per particle-node visit: 1 multiply + 3 FMAs
      by = 56.0 * P + 24.0 * (double)N;
    } else if (which == 3 || which == 4) {
      // calc_velocity_serial_3d: 3 = the curl (velocity), 4 = the stretching
      h->bench_scratch.ensure(6 * N);
      double* V[3] = {h->bench_scratch.p, h->bench_scratch.p + N, h->bench_scratch.p + 2 * N};
      double* G[3] = {h->bench_scratch.p + 3 * N, h->bench_scratch.p + 4 * N, h->bench_scratch.p + 5 * N};
      double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
      double* S[3] = {comp(h->sol, N, 0), comp(h->sol, N, 1), comp(h->sol, N, 2)};
      double* Vr[3] = {comp(h->vel, N, 0), comp(h->vel, N, 1), comp(h->vel, N, 2)};
      float2* VF[3], * GF[3];
      ff_fields(h, VF, GF);
      const vpmg_sizes s = h->sz;
      if (which == 3) {
        f = [s, S, R, V, G, st] { velocity_and_stretching(s.nn, s.dpm, S, R, V, G, st, 1); };
        fl = 15.0 * (double)N;  // 6 differences, 6 scalings, 3 combinations per node
        by = 48.0 * (double)N;  // psi read, u written
      } else {
        const bool ff = VF[0] != nullptr;
        float2* vf[3] = {VF[0], VF[1], VF[2]};
        float2* gf[3] = {GF[0], GF[1], GF[2]};
        f = [s, S, R, Vr, G, st, ff, vf, gf] {
          velocity_and_stretching(s.nn, s.dpm, S, R, const_cast<double* const*>(Vr), G, st, 2, ff ? vf : nullptr,
                                  ff ? gf : nullptr);
        };
        // 3 components x 3 directions x 4 flops + 2 sums where vorticity
        // surrounds the node (elsewhere the FP64 kernel writes zeros): RHS
        // read and stretching written everywhere, u read where computed
        const double act = ff ? (double)N : (double)count_vortical_nodes(s.nn, R, st);
        fl = 42.0 * act;
        by = 48.0 * (double)N + 24.0 * act;
      }
    } else if (which == 5) {
      // back_to_particles_3D(1) on the binned particles (UP/GP rewritten in place)
      const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
      bin_particles(h->parts, mg, h->bins, st);
      const double u0[3] = {0.0, 0.0, 0.0};
      f = [h, u0] { m2p_fields(h, kUpSet, false, 0.0, u0); };
      const double P = (double)read_count(h->bins.nsorted_dev, st);
      const int w = mg.ips + mg.ipf + 1;
      fl = P * w * w * w * 13.0;              // per visit: 1 multiply + 6 FMAs
      by = 80.0 * P + 48.0 * (double)N;        // X, vol read, UP/GP written; 6 fields read once
    } else if (which == 6) {
      // one component of the padded block's zero-BC solve, evaluated where it is read
      VPMG_CHECK(h->nblk == 1 && h->bsolve.ready, VPMG_ERR_UNSUPPORTED, "one-block handle needed");
      h->bench_scratch.ensure(NB);
      double* o = h->bench_scratch.p;
      f = [h, o, NB, st] { block_solve_zero_bc(h->bsolve, h->dp_bl, h->rhs_bl.p, 0, o, st); };
      const DirichletPlan& P = h->dp_bl;
      const double nint = (double)P.m[0] * P.m[1] * P.m[2];
      // forward x and y transforms, the Thomas sweep, 8 x-layer and 8 y-layer dot products
      fl = nint * (2.5 * std::log2(2.0 * (P.m[0] + 1)) + 2.5 * std::log2(2.0 * (P.m[1] + 1)) + 4.0 + 32.0);
      by = 8.0 * nint * 5.0;  // RHS read, transform written, sweep read + written, dots read
    } else if (which == 7) {
      // the remesh's |w| flags and their exclusive scan on the remesh grid
      const Grid gr = hx::remesh_grid(h);
      const MeshDev mr = mesh_dev(gr, h->cfg.interf_iproj);
      const vpmg_sizes s = h->sz;
      const int hh = h->cfg.interf_iproj / 2;
      const int lo[3] = {s.nn_bl[0] - 1 + hh, s.nn_bl[1] - 1 + hh, s.nn_bl[2] - 1 + hh};
      const int hi[3] = {s.nn_bl[3] - 1 - hh, s.nn_bl[4] - 1 - hh, s.nn_bl[5] - 1 - hh};
      double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
      std::array<int, 3> l{lo[0], lo[1], lo[2]}, u{hi[0], hi[1], hi[2]};
      f = [h, mr, R, l, u, st] { remesh_mask(mr, h->bins, R, l.data(), u.data(), (double)1e-09f, st); };
      fl = 5.0 * (double)N;
      by = 24.0 * (double)N + 4.0 * (double)N + 8.0 * (double)N;  // |w| read, flags written, scan
    } else if (which == 8) {
      // the sort by cell and the particle records on the global mesh
      // (k_keys, scan, k_scatter, k_cell_order, k_records64)
      const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
      f = [h, mg, st] { bin_particles(h->parts, mg, h->bins, st); };
      f();
      const double P = (double)read_count(h->bins.nsorted_dev, st);
      fl = 112.0 * P;  // 12 projection weights (offset + M4' polynomial, 8 flops each) + 16 y-z products
      // per particle: positions in, key and cursor, perm, strengths in, 24 record slots out; per node: counts,
      // starts and their scan
      by = 300.0 * P + 20.0 * (double)N;
    } else {
      throw Error{VPMG_ERR_ARG, "unknown kernel id"};
    }
    cudaEvent_t a, b;
    VPMG_CUDA(cudaEventCreate(&a));
    VPMG_CUDA(cudaEventCreate(&b));
    f();  // warm
    VPMG_CUDA(cudaStreamSynchronize(st));
    VPMG_CUDA(cudaEventRecord(a, st));
    for (int r = 0; r < reps; ++r) f();
    VPMG_CUDA(cudaEventRecord(b, st));
    VPMG_CUDA(cudaEventSynchronize(b));
    float t = 0.f;
    VPMG_CUDA(cudaEventElapsedTime(&t, a, b));
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (ms) *ms = t / reps;
    if (flops) *flops = fl;
    if (bytes) *bytes = by;
  });
}

double vpmg_projection_fun(int itype, double x) {
  // the projection kernels of pmproject.f90:391-431 on |x|, as the device
  // kernels evaluate them
  const double a = std::fabs(x);
  switch (itype) {
    case 2: return a > 1.0 ? 0.0 : 1.0 - a;
    case 3:
      if (a > 1.5) return 0.0;
      if (a >= 0.5) return 0.5 * (-a + 1.5) * (-a + 1.5);
      return 0.5 * (a + 1.5) * (a + 1.5) - 1.5 * (a + 0.5) * (a + 0.5);
    case 4:
      if (a > 2.0) return 0.0;
      if (a >= 1.0) return 0.5 * ((2.0 - a) * (2.0 - a)) * (1.0 - a);
      return 1.0 - 2.5 * (a * a) + 1.5 * (a * a * a);
    case 5:
    case 6: {
      const double lim = itype == 5 ? 0.5 : 1.0;
      if (a <= lim) return 1.0 - a * a;
      if (a <= lim + 1.0) return 0.5 * (1.0 - a) * (2.0 - a);
      return 0.0;
    }
    default: return 0.0;
  }
}

int vpmg_host_euler(double* xp, double* qp, const double* up, const double* gp, int n, double dt,
                    const double uinf[3]) {
  if (n < 0 || (n > 0 && (!xp || !qp || !up || !gp))) return VPMG_ERR_ARG;
  const double u0 = uinf ? uinf[0] : 0.0, u1 = uinf ? uinf[1] : 0.0, u2 = uinf ? uinf[2] : 0.0;
  for (int j = 0; j < n; ++j) {
    double* x = xp + 3 * (size_t)j;
    double* q = qp + 4 * (size_t)j;
    const double* u = up + 3 * (size_t)j;
    const double* g = gp + 3 * (size_t)j;
    x[0] = x[0] + (u[0] + u0) * dt;
    x[1] = x[1] + (u[1] + u1) * dt;
    x[2] = x[2] + (u[2] + u2) * dt;
    q[0] = q[0] - g[0] * dt;
    q[1] = q[1] - g[1] * dt;
    q[2] = q[2] - g[2] * dt;
  }
  return VPMG_OK;
}

int vpmg_remesh_device(vpmg_handle* h) {
  return guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
    remesh(h);
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
    sync_np(h);
  });
}

}  // extern "C"

namespace {
// writesol: the resident velocity and RHS (last field step) on the host.
void solution_file(vpmg_handle* h, const char* dir, int ntime) {
  VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
  const size_t N = h->gglob.count();
  std::vector<double> vel(3 * N), rhs(3 * N);
  VPMG_CUDA(cudaMemcpyAsync(vel.data(), h->vel.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, h->stream));
  VPMG_CUDA(cudaMemcpyAsync(rhs.data(), h->rhs.p, sizeof(double) * 3 * N, cudaMemcpyDeviceToHost, h->stream));
  VPMG_CUDA(cudaStreamSynchronize(h->stream));
  io::SolutionView v{};
  v.vel = vel.data();
  v.rhs = rhs.data();
  for (int d = 0; d < 3; ++d) { v.nn[d] = h->sz.nn[d]; v.xmin[d] = h->sz.xbound[d]; v.d[d] = h->sz.dpm[d]; }
  for (int d = 0; d < 6; ++d) v.nn_bl[d] = h->sz.nn_bl[d];
  const int st = io::write_solution(dir, ntime, v);
  VPMG_CHECK(st == VPMG_OK, st, "cannot write the solution file");
}

// writeline: the nine velocity lines along x of the block range.
void hist_file(vpmg_handle* h, const char* dir, int ntime) {
  VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes must come first");
  const vpmg_sizes& s = h->sz;
  int jk[9][2];
  io::hist_lines(s.nn_bl, jk);
  const int nl = s.nn_bl[3] - s.nn_bl[0] + 1;
  const size_t N = h->gglob.count();
  std::vector<double> lines((size_t)27 * nl);
  for (int l = 0; l < 9; ++l) {
    const int j = jk[l][0], k = jk[l][1];
    VPMG_CHECK(j >= 1 && j <= s.nn[1] && k >= 1 && k <= s.nn[2], VPMG_ERR_UNSUPPORTED,
               "mesh too small for the reference's hist lines");
    const size_t base = (size_t)(s.nn_bl[0] - 1) + (size_t)s.nn[0] * ((size_t)(j - 1) + (size_t)s.nn[1] * (k - 1));
    for (int c = 0; c < 3; ++c)
      VPMG_CUDA(cudaMemcpyAsync(lines.data() + ((size_t)l * 3 + c) * nl, h->vel.p + (size_t)c * N + base,
                                sizeof(double) * nl, cudaMemcpyDeviceToHost, h->stream));
  }
  VPMG_CUDA(cudaStreamSynchronize(h->stream));
  io::HistView v{};
  v.lines = lines.data();
  for (int d = 0; d < 3; ++d) { v.xmin[d] = s.xbound[d]; v.d[d] = s.dpm[d]; }
  for (int d = 0; d < 6; ++d) v.nn_bl[d] = s.nn_bl[d];
  const int st = io::write_hist(dir, ntime, v);
  VPMG_CHECK(st == VPMG_OK, st, "cannot write the hist files");
}

// The writers of vpm(WhatToDo = 2) after the velocity (vpm.f90:276-284).
void step_writers(vpmg_handle* h, int ntime) {
  const char* dir = h->out_dir.empty() ? nullptr : h->out_dir.c_str();
  if (h->out_flags & 1) {
    bool hit = false;
    for (int i = 0; i < h->cfg.ipmwrite && i < 10; ++i)
      hit = hit || (ntime >= h->cfg.ipmwstart[i] && ntime <= h->cfg.ipmwstart[i] + h->cfg.ipmwsteps[i]);
    if (hit) solution_file(h, dir, ntime);
  }
  if (h->out_flags & 2) hist_file(h, dir, ntime);
}
}  // namespace

extern "C" {

int vpmg_write_solution(vpmg_handle* h, const char* dir, int ntime) {
  return guarded(h, [&] { solution_file(h, dir, ntime); });
}

int vpmg_write_hist(vpmg_handle* h, const char* dir, int ntime) {
  return guarded(h, [&] { hist_file(h, dir, ntime); });
}

int vpmg_set_output(vpmg_handle* h, const char* dir, int flags) {
  if (!h || flags < 0 || flags > 3) return VPMG_ERR_ARG;
  h->out_dir = dir ? dir : "";
  h->out_flags = flags;
  return VPMG_OK;
}

int vpmg_vpm(vpmg_handle* h, double* xp, double* qp, double* up, double* gp, int* nvr, int neqpm, int whattodo,
             int ntime, double ni, int nvrm) {
  return guarded(h, [&] {
    VPMG_CHECK(nvr, VPMG_ERR_ARG, "NVR is null");
    VPMG_CHECK(neqpm == 3, VPMG_ERR_UNSUPPORTED, "neqpm must be 3");
    VPMG_CHECK(*nvr <= nvrm, VPMG_ERR_ARG, "NVR > NVRM");
    if (whattodo == 0) {
      vpmg_sizes s = h->sz;
      define_sizes(h, xp, *nvr, ntime, s);
      if (!h->prepared || !same_sizes(s, h->sz)) {
        h->sz = s;
        h->sized = true;
        prepare(h);
      }
      return;
    }
    VPMG_CHECK(whattodo == 1 || whattodo == 2 || whattodo == 4 || whattodo == 5, VPMG_ERR_UNSUPPORTED,
               "WhatToDo must be 0, 1, 2, 4 or 5");
    if (*nvr == 0) return;  // vpm.f90:171
    if (whattodo == 1 || whattodo == 4) {
      // 1 (vpm.f90:221-262): Poisson solve and the velocity field only
      //   (calc_velocity_serial_3d(0)); no particle output -- the field is
      //   read with vpmg_get_field.
      // 4 (vpm.f90:316-343): no solve; stretching from the new deposition
      //   and the resident velocity (calc_velocity_serial_3d(-1)), then UP
      //   and GP (back_to_particles_3D(itype = 1)).
      VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes (WhatToDo = 0) must come first");
      upload_particles(h, xp, qp, *nvr);
      const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
      bin_particles(h->parts, mg, h->bins, h->stream);
      const size_t N = h->gglob.count();
      double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
      double* S[3] = {comp(h->sol, N, 0), comp(h->sol, N, 1), comp(h->sol, N, 2)};
      double* Vv[3] = {comp(h->vel, N, 0), comp(h->vel, N, 1), comp(h->vel, N, 2)};
      double* G[3] = {comp(h->def, N, 0), comp(h->def, N, 1), comp(h->def, N, 2)};
      deposit(h->parts, mg, h->bins, R, h->stream);
      float2* VF[3], * GF[3];
      ff_fields(h, VF, GF);
      float2* const* vf = VF[0] ? VF : nullptr;
      float2* const* gf = GF[0] ? GF : nullptr;
      if (whattodo == 1) {
        poisson_part(h);
        velocity_and_stretching(h->sz.nn, h->sz.dpm, S, R, Vv, G, h->stream, 1, vf, gf);
      } else {
        VPMG_CHECK(up && gp, VPMG_ERR_ARG, "UP or GP is null");
        velocity_and_stretching(h->sz.nn, h->sz.dpm, S, R, Vv, G, h->stream, 2, vf, gf);
        const double u0[3] = {0.0, 0.0, 0.0};
        upload_up(h, up, *nvr);
        m2p_step(h, kUpAdd, false, 0.0, u0);
        VPMG_CUDA(cudaMemcpyAsync(up, h->parts.up.p, sizeof(double) * 3 * (size_t)*nvr, cudaMemcpyDeviceToHost,
                                  h->stream));
        VPMG_CUDA(cudaMemcpyAsync(gp, h->parts.gp.p, sizeof(double) * 3 * (size_t)*nvr, cudaMemcpyDeviceToHost,
                                  h->stream));
      }
      VPMG_CUDA(cudaStreamSynchronize(h->stream));
      check_particle_errors(h->bins, h->stream);
      return;
    }
    if (whattodo == 5) {
      // vpm.f90:345-372: deposition, diffuse_vort_3d, back_to_particles_3D(itype = 2)
      VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "define_sizes (WhatToDo = 0) must come first");
      VPMG_CHECK(gp, VPMG_ERR_ARG, "GP is null");
      upload_particles(h, xp, qp, *nvr);
      const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
      bin_particles(h->parts, mg, h->bins, h->stream);
      const size_t N = h->gglob.count();
      double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
      double* S[3] = {comp(h->sol, N, 0), comp(h->sol, N, 1), comp(h->sol, N, 2)};
      deposit(h->parts, mg, h->bins, R, h->stream);
      viscous_diffusion(h->sz.nn, h->sz.nn_bl, h->sz.dpm, ni, R, S, h->stream);
      const double* Vp[3] = {comp(h->vel, N, 0), comp(h->vel, N, 1), comp(h->vel, N, 2)};
      const double* Sp[3] = {S[0], S[1], S[2]};
      const double u0[3] = {0, 0, 0};
      m2p(h->parts, mg, h->bins, Vp, Sp, kUpSet, false, 0.0, u0, h->stream);  // GP = vol I(X) SOL; UP untouched
      VPMG_CUDA(cudaMemcpyAsync(gp, h->parts.gp.p, sizeof(double) * 3 * (size_t)*nvr, cudaMemcpyDeviceToHost,
                                h->stream));
      VPMG_CUDA(cudaStreamSynchronize(h->stream));
      check_particle_errors(h->bins, h->stream);
      return;
    }
    upload_particles(h, xp, qp, *nvr);
    const double u0[3] = {0, 0, 0};
    bin_particles(h->parts, mesh_dev(h->gglob, h->cfg.interf_iproj), h->bins, h->stream);
    field_step(h);
    if (h->out_flags) step_writers(h, ntime);
    upload_up(h, up, *nvr);
    m2p_step(h, kUpAdd, false, 0.0, u0);  // UP = UP + interpolated velocity, GP overwritten
    VPMG_CUDA(cudaMemcpyAsync(up, h->parts.up.p, sizeof(double) * 3 * (size_t)*nvr, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaMemcpyAsync(gp, h->parts.gp.p, sizeof(double) * 3 * (size_t)*nvr, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
    check_particle_errors(h->bins, h->stream);
  });
}

int vpmg_remesh_particles_3d(vpmg_handle* h, int iflag, double* xp, double* qp, int* nvr, int capacity) {
  return guarded(h, [&] {
    VPMG_CHECK(iflag == 1, VPMG_ERR_UNSUPPORTED, "remesh_particles_3d(iflag /= 1)");
    VPMG_CHECK(nvr, VPMG_ERR_ARG, "NVR is null");
    upload_particles(h, xp, qp, *nvr);
    remesh(h);
    sync_np(h);
    *nvr = h->np;
    VPMG_CHECK(h->np <= capacity, VPMG_ERR_CAPACITY, "remesh produced more particles than the caller's capacity");
    download_particles(h, xp, qp, h->np);
  });
}

int vpmg_pmesh(vpmg_handle* h, double* const sol[3], const double* const rhs[3], const double xbound[6],
               const double dpm[3], const int nn[3], const int nn_bl[6], int iynbc, int itree, int levmax) {

  return guarded(h, [&] {
    VPMG_CHECK(sol && rhs && xbound && dpm && nn && nn_bl, VPMG_ERR_ARG, "null argument");
    const Grid g = make_grid(xbound, dpm, nn);
    const size_t n = g.count();
    DBuf<double> r, s, s0, w;
    r.ensure(3 * n); s.ensure(3 * n); s0.ensure(n);
    for (int c = 0; c < 3; ++c) {
      VPMG_CUDA(cudaMemcpyAsync(r.p + c * n, rhs[c], sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
      VPMG_CUDA(cudaMemcpyAsync(s.p + c * n, sol[c], sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    }
    DirichletPlan dp;
    if (iynbc == 1) {
      const int full[6] = {0, 0, 0, nn[0] - 1, nn[1] - 1, nn[2] - 1};
      dirichlet_prepare(dp, nn, full, dpm, h->stream, h->arith);
      w.ensure((size_t)dp.m[0] * dp.m[1] * dp.m[2]);
      fill_zero(s0.p, n, h->stream);
      BoundaryOp bo;
      boundary_prepare(bo, g, itree == 1 ? levmax : 0, h->op_budget, h->stream, h->cfg.ibctyp, itree == 1, h->arith);
      for (int c = 0; c < 3; ++c) {
        dirichlet_solve(dp, r.p + c * n, s0.p, true, w.p, h->stream);
        boundary_panels(bo, g, s0.p, c, h->stream);
      }
      double* sp[3] = {s.p, s.p + n, s.p + 2 * n};
      boundary_apply(bo, g, sp, h->stream);
      for (int c = 0; c < 3; ++c) dirichlet_solve(dp, r.p + c * n, s.p + c * n, false, w.p, h->stream);
      VPMG_CUDA(cudaStreamSynchronize(h->stream));
    } else {
      const int box[6] = {nn_bl[0] - 1, nn_bl[1] - 1, nn_bl[2] - 1, nn_bl[3] - 1, nn_bl[4] - 1, nn_bl[5] - 1};
      dirichlet_prepare(dp, nn, box, dpm, h->stream, h->arith);
      w.ensure((size_t)dp.m[0] * dp.m[1] * dp.m[2]);
      for (int c = 0; c < 3; ++c) dirichlet_solve(dp, r.p + c * n, s.p + c * n, false, w.p, h->stream);
    }
    for (int c = 0; c < 3; ++c)
      VPMG_CUDA(cudaMemcpyAsync(sol[c], s.p + c * n, sizeof(double) * n, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int vpmg_project_particles_3d(vpmg_handle* h, const double* xp, const double* qp, int nvr, double* const rhs[3]) {
  return guarded(h, [&] {
    upload_particles(h, xp, qp, nvr);
    const MeshDev mg = mesh_dev(h->gglob, h->cfg.interf_iproj);
    bin_particles(h->parts, mg, h->bins, h->stream);
    const size_t N = h->gglob.count();
    double* R[3] = {comp(h->rhs, N, 0), comp(h->rhs, N, 1), comp(h->rhs, N, 2)};
    deposit(h->parts, mg, h->bins, R, h->stream);
    for (int c = 0; c < 3; ++c)
      VPMG_CUDA(cudaMemcpyAsync(rhs[c], R[c], sizeof(double) * N, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int vpmg_get_field(vpmg_handle* h, int which, double* out, size_t capacity, size_t* count) {
  return guarded(h, [&] {
    VPMG_CHECK(h->prepared, VPMG_ERR_STATE, "no mesh yet");
    const size_t N = h->gglob.count(), NB = h->gbl.count(), NC = h->gco.count();
    const double* src = nullptr;
    size_t n = 0;
    switch (which) {
      case VPMG_F_RHS: src = h->rhs.p; n = N; break;
      case VPMG_F_SOL: src = h->sol.p; n = N; break;
      case VPMG_F_VEL: src = h->vel.p; n = N; break;
      case VPMG_F_DEF: src = h->def.p; n = N; break;
      case VPMG_F_BL_SOL1:
        VPMG_CHECK(h->bl_sol1_copy.p, VPMG_ERR_STATE, "intermediates are kept only after vpmg_set_profiling(h, 2)");
        src = h->bl_sol1_copy.p; n = NB; break;
      case VPMG_F_COARSE_RHS: src = h->crhs.p; n = NC; break;
      case VPMG_F_COARSE_SOL: src = h->csol.p; n = NC; break;
      case VPMG_F_BL_FINAL: src = h->sol_bl.p; n = NB; break;
      default: throw Error{VPMG_ERR_ARG, "unknown field id"};
    }
    if (count) *count = n;
    if (!out) return;
    VPMG_CHECK(capacity >= 3 * n, VPMG_ERR_ARG, "output too small");
    VPMG_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
  });
}

long long vpmg_kernel_launches(const vpmg_handle* h) { return h ? h->launches : -1; }

int vpmg_phase_times(const vpmg_handle* h, double ms[9]) {
  if (!h || !ms) return VPMG_ERR_ARG;
  for (int i = 0; i < 9; ++i) ms[i] = h->phase_ms[i];
  return VPMG_OK;
}

int vpmg_tree_stats(const vpmg_handle* h, long long* interactions, long long* bytes, int* precomputed) {
  if (!h) return VPMG_ERR_ARG;
  const BoundaryOp& bo = h->nblk > 1 && !h->bo_blk.empty() ? *h->bo_blk[0] : h->bo_bl;
  if (interactions) *interactions = bo.nnz + bo.ndense_acc;
  if (bytes) *bytes = bo.bytes();
  if (precomputed) *precomputed = bo.precomputed ? 1 : 0;
  return VPMG_OK;
}

int vpmg_farfield_stats(const vpmg_handle* h, int* on, long long* corrections, double* flops) {
  if (!h) return VPMG_ERR_ARG;
  const BoundaryOp& bo = h->nblk > 1 && !h->bo_blk.empty() ? *h->bo_blk[0] : h->bo_bl;
  if (on) *on = bo.ff.on ? 1 : 0;
  if (corrections) *corrections = bo.ff.on ? bo.ff.ncorr : 0;
  if (flops) *flops = bo.ff.on ? bo.ff.flops : 0.0;
  return VPMG_OK;
}

int vpmg_set_profiling(vpmg_handle* h, int on) {
  if (!h) return VPMG_ERR_ARG;
  h->profile = on != 0;
  h->keep_intermediates = on >= 2;
  h->full_block_solves = on >= 3;
  return VPMG_OK;
}

int vpmg_fp64_peak(vpmg_handle* h, double* tflops) {
  return guarded(h, [&] {
    const double t = measure_fp64_peak(h->stream);
    if (tflops) *tflops = t;
  });
}

int vpmg_dst_tiles(const vpmg_handle* h, int pairs[6]) {
  if (!h || !pairs) return VPMG_ERR_ARG;
  if (!h->prepared) return VPMG_ERR_STATE;
  const vpmg::FFTPlan* p[6] = {&h->dp_bl.fx, &h->dp_bl.fy, &h->dp_inner.fx, &h->dp_inner.fy, &h->dp_c.fx, &h->dp_c.fy};
  for (int i = 0; i < 6; ++i) pairs[i] = p[i]->pairs;
  return VPMG_OK;
}

int vpmg_set_arithmetic(vpmg_handle* h, int arith) {
  if (!h) return VPMG_ERR_ARG;
  if (arith != VPMG_ARITH_FP64 && arith != VPMG_ARITH_FF48) return VPMG_ERR_ARG;
  if (arith == h->arith) return VPMG_OK;
  return guarded(h, [&] {
    VPMG_CUDA(cudaStreamSynchronize(h->stream));
    // captured graphs hold the other arithmetic's kernels and buffers
    if (h->graph.exec) {
      VPMG_CUDA(cudaGraphExecDestroy(h->graph.exec));
      h->graph.exec = nullptr;
    }
    vpmg::hx::destroy_adjoint(h);
    h->arith = arith;
    if (h->sized) {
      h->prepared = false;
      prepare(h);  // plans, recorded operators and particle records in the new arithmetic
    }
  });
}

int vpmg_get_arithmetic(const vpmg_handle* h, int* arith) {
  if (!h || !arith) return VPMG_ERR_ARG;
  *arith = h->arith;
  return VPMG_OK;
}

int vpmg_set_operator_budget(vpmg_handle* h, long long bytes) {
  if (!h) return VPMG_ERR_ARG;
  h->op_budget = bytes;
  return VPMG_OK;
}

}  // extern "C"

// ---- step helpers shared with adjoint.cu -------------------------------
namespace vpmg {
namespace hx {
MeshDev mesh_dev(const Grid& g, int itype) { return ::mesh_dev(g, itype); }
Grid remesh_grid(const vpmg_handle* h) {
  Grid gr = h->gglob;
  for (int d = 0; d < 3; ++d) gr.d[d] = (h->sz.xbound[d + 3] - h->sz.xbound[d]) / (double)(h->sz.nn[d] - 1);
  return gr;
}
void field_step(vpmg_handle* h) { ::field_step(h); }
void remesh(vpmg_handle* h) { ::remesh(h); }
void sync_np(vpmg_handle* h) { ::sync_np(h); }
void upload_particles(vpmg_handle* h, const double* xp, const double* qp, int n) { ::upload_particles(h, xp, qp, n); }
void download_particles(vpmg_handle* h, double* xp, double* qp, int n) { ::download_particles(h, xp, qp, n); }
void poisson_part(vpmg_handle* h) { ::poisson_part(h); }
void m2p_fields(vpmg_handle* h, int up_mode, bool euler, double dt, const double uinf[3]) {
  ::m2p_fields(h, up_mode, euler, dt, uinf);
}
void step_on_stream(vpmg_handle* h, double dt) {
  const double u0[3] = {0.0, 0.0, 0.0};
  if (h->keep_intermediates || h->no_graphs) {
    ::one_step(h, dt, u0, 1);
    return;
  }
  ensure_graph(h, dt, u0, 1);
  VPMG_CUDA(cudaMemsetAsync(h->hist_counter.p, 0, sizeof(int), h->stream));
  VPMG_CUDA(cudaGraphLaunch(h->graph.exec, h->stream));
  h->launches += h->graph.launches;
}
}  // namespace hx
}  // namespace vpmg
