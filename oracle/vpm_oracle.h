/*
 * vpm_oracle.h -- CPU restatement of vpm_free's particle-mesh time step.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * library in vpm_free_gb300/: only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference arm of bench.py may load it.  Nothing in the
 * product path links it.
 *
 * Parity status: the reference (Fortran 90 + MPI + Intel MKL Poisson
 * Library) cannot be compiled on either machine (no Fortran compiler, no
 * MPI, no MKL; MKL does not exist for aarch64).  This restatement is pinned
 * instead by
 *   - the reference's own analytic known-answer case, Hill's spherical
 *     vortex (source/test_applic.f90:2-179), at discretisation accuracy;
 *   - the discrete 7-point residual of its Dirichlet solver and a
 *     scipy.fft.dstn cross-check (the semantics of MKL d_Helmholtz_3D with
 *     'DDDDDD' boundaries and q = 0, source/pmsolve.f90:284-432);
 *   - a direct (non-tree) boundary sum bounding the tree error.
 * Bit-level parity with the Fortran binary is unpinned.
 *
 * Every routine follows the loop order and formulas of the reference file
 * cited beside it.  Single block only (NBI = NBJ = NBK = 1), 3-D only.
 * Fields are stored one array per component, x fastest, 1-based helpers.
 */
#ifndef VPM_ORACLE_H
#define VPM_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* pm.inp contents (source/vpm.f90:132-152) plus an optional explicit box. */
typedef struct vpmo_config {
  double dpm[3];
  int interf_iproj;
  int ibctyp;
  int idvpm;
  double epsvol;
  int ncoarse;
  int nbi, nbj, nbk;
  int nremesh, ncell_rem;
  int iyntree, ilevmax;
  int ompthreads;
  int idefine;
  int iynslice;
  int use_box;      /* 1: box[] is the global mesh, not the particle bounding box */
  double box[6];
} vpmo_config;

/* Mesh descriptors produced by define_sizes (source/vpm.f90:477-660). */
typedef struct vpmo_sizes {
  double xbound[6], dpm[3];
  int nn[3], nn_bl[6];
  double xbound_bl[6];
  int nnbl[3], nnbl_bl[6];
  double xbound_coarse[6], dpm_coarse[3];
  int nn_coarse[3], nn_bl_coarse[6];
  int ilevmax;
  double dvpm;
  int defined;
} vpmo_sizes;

/* source/pmlib.f90:216-432 */
void vpmo_definepm(int itype, double xbound[6], double dpm[3], int ndum, const int nsize[3],
                   int nn[3], int nn_bl[6]);

/* source/vpm.f90:477-660 (one block). xp is XP(3,nvr) column-major. */
int vpmo_define_sizes(const vpmo_config* cfg, const double* xp, int nvr, int ntime, vpmo_sizes* s);

/* source/pmproject.f90:391-431 */
double vpmo_projection_fun(int itype, double x);

/* source/pmproject.f90:43-98 + :110-153 (IDVPM = 1): rhs[c] (c = 0..2) are
 * NX*NY*NZ arrays; returns 0 or -1 if a stencil leaves the mesh. */
int vpmo_project_particles(const vpmo_sizes* s, int itype, const double* xp, const double* qp,
                           int nvr, double* rhs0, double* rhs1, double* rhs2, int nthreads);

/* Dirichlet 7-point solve on node box [s..f] (1-based, inclusive) of an
 * nx*ny*nz array: interior of sol <- solution of  Lap_h u = rhs  with the
 * boundary values already in sol (zero_bc = 0) or zero (zero_bc = 1).
 * Semantics of source/pmsolve.f90:284-432. */
void vpmo_dirichlet(int nx, int ny, int nz, const int box[6], const double d[3],
                    const double* rhs, double* sol, int zero_bc, int nthreads);

/* pmesh (source/pmlib.f90:69-192), 3-D, ibctyp = 2, components 0..2.
 * sol/rhs: 3 arrays each of nn[0]*nn[1]*nn[2]. */
int vpmo_pmesh(double* const sol[3], double* const rhs[3], const double xbound[6],
               const double dpm[3], const int nn[3], const int nn_bl[6], int iynbc, int itree,
               int levmax, int nthreads);
/* The same with the boundary type of pm.inp: ibctyp 2 (point sources,
 * calc_boundinf_3d[_lev]) or 3 (constant-source panels, FSOUR_A4,
 * calc_boundinf_3d[_lev]_s, source/pmbound.f90:520-648, 1255-1620). */
int vpmo_pmesh_bc(double* const sol[3], double* const rhs[3], const double xbound[6],
                  const double dpm[3], const int nn[3], const int nn_bl[6], int iynbc, int itree,
                  int levmax, int nthreads, int ibctyp);

/* vpmo_boundary_values (below) with the boundary type: 2 or 3. */
long vpmo_boundary_values_bc(double* const sol0[3], double* const bnd[3], const double xb[6],
                             const double D[3], const int nn[3], int levmax, int direct, int nthreads,
                             int ibctyp);

/* FSOUR_A4 (source/pmbound.f90:1540-1620) in the frame of target plane
 * iplane (+-1 Y, +-2 X, +-3 Z; negative on max faces). */
double vpmo_fsour_a4(const double xo[3], const double rg[3], int iplane, const double dpm[3], double area);

/* Full field step, WhatToDo = 2 (source/vpm.f90:171-314 with yaps3d) for
 * one block.  xp(3,nvr), qp(4,nvr) column-major; up/gp(3,nvr) outputs.
 * Intermediate fields are kept in a global scratch readable through
 * vpmo_get_field().  Returns 0 or a negative error. */
int vpmo_step_fields(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp,
                     const double* qp, double* up, double* gp, int nvr, int nthreads);

/* With NBI x NBJ x NBK > 1 blocks: the largest difference, relative to the
 * largest face value, between the boundary values that blocks sharing an
 * inner-face node assign to it in the last vpmo_step_fields (a check of
 * the neighbour transfers; 0 with one block). */
double vpmo_yaps_seam(void);

/* Field ids for vpmo_get_field / the CUDA library's vpmg_get_field. */
enum {
  VPMO_F_RHS = 0,      /* global RHS_pm(1:3) after project_vol3d      [3 x N]   */
  VPMO_F_SOL = 1,      /* global SOL_pm (psi) after solget_3d         [3 x N]   */
  VPMO_F_VEL = 2,      /* velvr[xyz]_pm                              [3 x N]   */
  VPMO_F_DEF = 3,      /* SOL_pm after calc_velocity (deformation)    [3 x N]   */
  VPMO_F_BL_SOL1 = 4,  /* block solution after the infinite-domain solve [3 x Nb] */
  VPMO_F_COARSE_RHS = 5,
  VPMO_F_COARSE_SOL = 6,
  VPMO_F_BL_FINAL = 7  /* block after the final Dirichlet solve        [3 x Nb] */
};
/* Copies field `which` (3 components back to back) into out; returns the
 * element count per component, or -1. */
long vpmo_get_field(int which, double* out, long capacity);

/* vpm(WhatToDo = 5): deposition, diffuse_vort_3d (SOL = -NI Lap_h RHS on the
 * block interior) and back_to_particles_3D(itype = 2): GP = vol sum W SOL.
 * The fields are kept for vpmo_get_field (RHS, SOL). */
// vpm(WhatToDo = 4) after vpmo_step_fields: stretching from these particles'
// deposition and the kept velocity; UP is added to, GP overwritten.
int vpmo_whattodo4(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, double* up,
                   double* gp, int nvr, int nthreads);
int vpmo_diffuse(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, double ni, double* gp,
                 int nvr, int nthreads);

/* Forward Euler of source/test.f90:104-117. */
void vpmo_euler(double* xp, double* qp, const double* up, const double* gp, int nvr, double dt,
                const double uinf[3]);

/* remesh_particles_3d(1) (source/vpm_remesh.f90:5-225), ncell_rem = 1.
 * Reads nvr particles, writes up to capacity new ones into xp_out/qp_out,
 * returns the new count (may exceed capacity: then nothing beyond capacity
 * is written). */
long vpmo_remesh(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp,
                 int nvr, double* xp_out, double* qp_out, long capacity, int nthreads);
/* The same with the |w| cut replaced by a node mask (N = NN1*NN2*NN3
 * ints): mode 1 records the cut's mask, mode 2 emits exactly the masked
 * nodes (the fixed-mask map whose derivative the reverse mode computes). */
long vpmo_remesh_masked(const vpmo_config* cfg, const vpmo_sizes* s, const double* xp, const double* qp, int nvr,
                        double* xp_out, double* qp_out, long capacity, int nthreads, int* mask, int mode);

/* Tree-accelerated boundary values alone (source/pinfdomain.f90:86-158
 * minus the final solve): given a zero-BC solution sol0 on an nn grid,
 * writes the infinite-domain boundary values into the faces of bnd (which
 * must be zero on entry).  direct = 1 uses the untreed panel sum instead
 * (source/pmbound.f90:415-515).  Returns the interaction count. */
long vpmo_boundary_values(double* const sol0[3], double* const bnd[3], const double xbound[6],
                          const double dpm[3], const int nn[3], int levmax, int direct,
                          int nthreads);

#ifdef __cplusplus
}
#endif
#endif
