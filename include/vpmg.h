/*
 * vpmg.h -- C-ABI of the GB300 (sm_103a) particle-mesh step library.
 *
 * Drop-in boundary for vpm_free's hot path: the Fortran host keeps its
 * `vpm(...)` driver call, pm.inp and particle arrays, and binds these entry
 * points through iso_c_binding (see vpm_free_gb300/fortran/).  Plain C
 * types only; every call returns an int status (0 = OK, < 0 = error, see
 * vpmg_status) and never aborts the process.  Arrays are FP64, and by
 * default every kernel computes in IEEE FP64, the reference's arithmetic.
 * vpmg_set_arithmetic selects float-float instead for the heavy kernels
 * (boundary operator, DST solves, projection weights, deposition,
 * mesh-to-particle, stretching): about 48 significant bits and FP32's
 * exponent range, on the FP32 pipes.  In either mode the fields match an
 * FP64 CPU restatement to relative L2 <= 1e-10.
 *
 * Array conventions follow the reference (Fortran column-major):
 *   XP(3,NVRM)  positions            -> double xp[ld*3], xp[3*p + d]
 *   QP(4,NVRM)  -omega*vol, volume   -> double qp[ld*4], qp[4*p + c]
 *   UP(3,NVRM), GP(3,NVRM) outputs
 *   fields (neq, NX, NY, NZ)         -> here one array per component,
 *                                       x fastest: f[c][i + NX*(j + NY*k)]
 * A handle owns one CUDA stream and its device memory; calls on one handle
 * must not overlap, calls on different handles may.
 */
#ifndef VPMG_H
#define VPMG_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef enum vpmg_status {
  VPMG_OK = 0,
  VPMG_ERR_ARG = -1,          /* bad argument / size                              */
  VPMG_ERR_CUDA = -2,         /* CUDA runtime error (message via vpmg_last_error) */
  VPMG_ERR_NOMEM = -3,        /* device allocation failed                          */
  VPMG_ERR_OUTSIDE = -4,      /* a particle stencil leaves the mesh                */
  VPMG_ERR_CAPACITY = -5,     /* remesh produced more particles than capacity      */
  VPMG_ERR_UNSUPPORTED = -6,  /* option outside the single-block 3-D path          */
  VPMG_ERR_STATE = -7,        /* call order (e.g. step before define_sizes)        */
  VPMG_ERR_TREE = -8          /* quadtree inconsistency (pinfdomain.f90:1516)      */
} vpmg_status;

/* pm.inp (source/vpm.f90:132-152 reads it positionally) + explicit box. */
typedef struct vpmg_config {
  double dpm[3];        /* DXpm DYpm DZpm                         pm.inp:1  */
  int interf_iproj;     /* projection function (2,3,4,5,6; 4=M4') pm.inp:2  */
  int ibctyp;           /* 2 point sources, 3 constant panels     pm.inp:3  */
  int idvpm;            /* 1: constant volume                     pm.inp:4  */
  double epsvol;        /*                                        pm.inp:5  */
  int ncoarse;          /* coarse/fine ratio of YAPS              pm.inp:6  */
  int nbi, nbj, nbk;    /* blocks (1 1 1 on one GPU)              pm.inp:7  */
  int nremesh, ncell_rem; /*                                      pm.inp:8  */
  int iyntree, ilevmax; /* quadtree on/off, levels                pm.inp:9  */
  int ompthreads;       /* ignored (host threads)                 pm.inp:10 */
  int idefine;          /* 1: box frozen after step 0             pm.inp:11 */
  int iynslice;         /* writer option (ignored)                pm.inp:12 */
  int use_box;          /* 1: box[] is the global mesh (no shrink-wrap)     */
  double box[6];        /* XMIN YMIN ZMIN XMAX YMAX ZMAX                    */
  int ipmwrite;         /* solution-file windows (<= 10)          pm.inp:13 */
  int ipmwstart[10];    /* window i: NTIME in [start, start + steps]        */
  int ipmwsteps[10];    /*                                        pm.inp:14+ */
} vpmg_config;

/* Mesh descriptors of define_sizes (source/vpm.f90:477-660), one block. */
typedef struct vpmg_sizes {
  double xbound[6], dpm[3];
  int nn[3], nn_bl[6];
  double xbound_bl[6];
  int nnbl[3], nnbl_bl[6];
  double xbound_coarse[6], dpm_coarse[3];
  int nn_coarse[3], nn_bl_coarse[6];
  int ilevmax;
  double dvpm;
  int defined;
} vpmg_sizes;

typedef struct vpmg_handle vpmg_handle;

/* ---- configuration ------------------------------------------------------ */
/* Parses pm.inp with the reference's positional reads (vpm.f90:132-152).   */
int vpmg_read_pm_inp(const char* path, vpmg_config* cfg);

/* ---- handle ------------------------------------------------------------- */
/* device < 0 keeps the current device.  Replaces the module state of
 * vpm_lib (source/vpm.f90:1-32) with an explicit handle.                   */
int vpmg_create(const vpmg_config* cfg, int device, vpmg_handle** out);
int vpmg_destroy(vpmg_handle* h);

/* Arithmetic of the heavy kernels (no counterpart in the reference, which
 * is REAL(8) throughout).  VPMG_ARITH_FP64 (default): IEEE FP64 everywhere.
 * VPMG_ARITH_FF48: boundary operator, DST solves, projection weights,
 * deposition, mesh-to-particle and stretching in float-float (hi + lo
 * floats, about 48 significant bits; magnitudes between about 1e-38 and
 * 3e38, smaller values flush to zero), the rest in FP64.  Changing it on a
 * sized handle rebuilds the plans and the recorded boundary operator.    */
enum { VPMG_ARITH_FP64 = 0, VPMG_ARITH_FF48 = 1 };
int vpmg_set_arithmetic(vpmg_handle* h, int arith);
int vpmg_get_arithmetic(const vpmg_handle* h, int* arith);
const char* vpmg_last_error(const vpmg_handle* h);
const char* vpmg_status_string(int status);

/* ---- the reference's driver call --------------------------------------- */
/* vpm(XP,QP,UP,GP,NVR,neqpm,WhatToDo,RHS_pm,velx,vely,velz,NTIME,NI,NVRM)
 * (source/vpm.f90:54-475).  WhatToDo 0 = read sizes (define_sizes, with
 * the pm.inp already given to vpmg_create), 1 = Poisson solve and velocity
 * field only (read it with vpmg_get_field; UP/GP untouched), 4 = stretching
 * from a new deposition and the resident velocity, then UP/GP (no solve),
 * 2 = field step: UP is
 * overwritten with the interpolated velocity and GP with the stretching
 * term times the particle volume (vpm_time.f90:62-107); 5 = viscous
 * diffusion (vpm.f90:345-372): GP = volume x interpolated -NI Lap_h RHS
 * (diffuse_vort_3d, vpm_gcalc.f90:138-210), UP untouched.  neqpm must be 3.
 * Host pointers; the copies to and from the device happen inside.          */
int vpmg_vpm(vpmg_handle* h, double* xp, double* qp, double* up, double* gp, int* nvr, int neqpm,
             int whattodo, int ntime, double ni, int nvrm);

/* remesh_particles_3d(1) (source/vpm_remesh.f90:5-225), ncell_rem = 1.
 * Reads *nvr particles from xp/qp (leading dimension = capacity) and
 * overwrites them with the new set; *nvr = new count.  If the new count
 * exceeds capacity nothing is written, *nvr holds the required count and
 * VPMG_ERR_CAPACITY is returned (the reference reallocates XPR/QPR).       */
int vpmg_remesh_particles_3d(vpmg_handle* h, int iflag, double* xp, double* qp, int* nvr, int capacity);

/* ---- the reference's single-block library calls ------------------------ */
/* pmesh(SOL,RHS,...,Xbound,Dpm,NN,NN_bl,...,ibctyp,neqs,neqf,iynbc,NVR,itree,levmax)
 * (source/pmlib.f90:69-192), 3-D, neqs = 1, neqf = 3; ibctyp is the
 * handle's (pm.inp): 2 point-source or 3 constant-source panel boundary.
 * sol/rhs: 3 host arrays of NN[0]*NN[1]*NN[2] doubles each.              */
int vpmg_pmesh(vpmg_handle* h, double* const sol[3], const double* const rhs[3], const double xbound[6],
               const double dpm[3], const int nn[3], const int nn_bl[6], int iynbc, int itree, int levmax);

/* project_particles_3D + project_vol3d(IDVPM=1) (source/pmproject.f90:43-153)
 * on the mesh of the last define_sizes: rhs[c] = sum_p W(x)W(y)W(z) QP(c,p) / DVpm. */
int vpmg_project_particles_3d(vpmg_handle* h, const double* xp, const double* qp, int nvr,
                              double* const rhs[3]);

/* projection_fun(itype, x) of module projlib (source/pmproject.f90:391-431):
 * the 1-D projection kernels, 2 linear, 3 TSC, 4 M4', 5 and 6 the
 * reference's two others, evaluated on |x| (0 for other itype).  Host
 * code, no GPU; for host programs that `use projlib`.                    */
double vpmg_projection_fun(int itype, double x);

/* ---- allocation-free Dirichlet solve ----------------------------------
 * No counterpart in the reference: an extra entry point of this library.
 * The Dirichlet 7-point solve of vpmg_pmesh(iynbc = 0), for callers that
 * cannot let a library allocate device memory -- a host code that hands
 * the whole GPU to its own pool allocator, or one that runs inside a fixed
 * memory budget where an extra cudaMalloc would fail.  This call makes no
 * cudaMalloc, cudaFree or allocating library call: its temporaries live in
 * one static device array of 33.6 MB that every GPU which loads this
 * library holds until the process exits.
 *   rhs, sol  device pointers to dims[0]*dims[1]*dims[2] doubles, x fastest;
 *             the interior of the 0-based inclusive node box `box` of sol
 *             receives the solution of Lap_h u = rhs; the box faces of sol
 *             are the Dirichlet values (zero_bc = 0) or are zeroed (1);
 *   h         mesh spacings;  stream: a cudaStream_t (NULL = default
 *             stream); the call is asynchronous on that stream.
 * Limits: at most 2^21 interior nodes and 900 along x and along y; larger
 * boxes return VPMG_ERR_ARG before any GPU work.  2*(cells) along x and y
 * must have no prime factor above 17 (else VPMG_ERR_UNSUPPORTED).
 * The first call on a device does that device's set-up (looks up the
 * array's device address, loads constant tables): make it from one thread,
 * and before any stream capture.  Every call shares the one array, which
 * keeps the last call's contents; each call rebuilds what it reads, but
 * calls whose GPU work overlaps (other streams, threads) race on it.     */
int vpmg_dirichlet_static(const double* rhs, double* sol, const int dims[3], const int box[6], const double h[3],
                          int zero_bc, void* stream);

/* ---- device-resident loop (test.f90:83-150 without the AVATAR inflow) -- */
int vpmg_define_sizes(vpmg_handle* h, const double* xp, int nvr, int ntime);
int vpmg_get_sizes(const vpmg_handle* h, vpmg_sizes* out);
/* Upload particles to the handle's device arrays (capacity particles).    */
int vpmg_set_particles(vpmg_handle* h, const double* xp, const double* qp, int nvr, int capacity);
int vpmg_get_particles(vpmg_handle* h, double* xp, double* qp, int* nvr, int capacity);
int vpmg_get_particle_velocity(vpmg_handle* h, double* up, double* gp, int nvr);
/* One device-resident step on the uploaded particles: field step
 * (WhatToDo = 2), forward Euler (test.f90:104-117) and, if remesh != 0,
 * remesh_particles_3d(1).  No host copies of particle data.             */
int vpmg_step(vpmg_handle* h, double dt, const double uinf[3], int remesh);
int vpmg_remesh_device(vpmg_handle* h);
int vpmg_num_particles(const vpmg_handle* h, int* nvr);

/* Field ids for vpmg_get_field. */
enum {
  VPMG_F_RHS = 0,      /* RHS_pm(1:3) after project_vol3d            3 x N  */
  VPMG_F_SOL = 1,      /* SOL_pm (vector potential) after solget_3d  3 x N  */
  VPMG_F_VEL = 2,      /* velvr[xyz]_pm                             3 x N  */
  VPMG_F_DEF = 3,      /* stretching (SOL_pm after calc_velocity)   3 x N  */
  VPMG_F_BL_SOL1 = 4,  /* block after the infinite-domain solve     3 x Nb */
  VPMG_F_COARSE_RHS = 5,
  VPMG_F_COARSE_SOL = 6,
  VPMG_F_BL_FINAL = 7  /* block after the final Dirichlet solve     3 x Nb */
};
/* Copies 3 components (back to back) of a resident field into out.
 * *count = elements per component.                                      */
int vpmg_get_field(vpmg_handle* h, int which, double* out, size_t capacity, size_t* count);

/* ---- instrumentation --------------------------------------------------- */
/* Number of kernels launched by this handle since creation.              */
long long vpmg_kernel_launches(const vpmg_handle* h);
/* Per-phase device milliseconds of the last vpmg_step (CUDA events):
 * [0] deposit, [1] fine zero-BC solve, [2] boundary values, [3] fine BC
 * solve, [4] coarse, [5] final solve, [6] FD, [7] M2P+Euler, [8] remesh. */
int vpmg_phase_times(const vpmg_handle* h, double ms[9]);
/* Boundary-operator statistics: interactions per fine solve, bytes held. */
int vpmg_tree_stats(const vpmg_handle* h, long long* interactions, long long* bytes, int* precomputed);
/* Whether the fine block's operator evaluates its coarsest tree level by
 * FFT convolutions on the face lattices (FP64 handles whose coarsest cells
 * form uniform lattices; VPMG_FARFIELD=0 at set-up keeps the dense block),
 * its correction entries (the coarsest cells the walk opened) and the
 * FP64 flops of one apply of the FFT part.  Instrumentation; no counterpart
 * in the reference.                                                     */
int vpmg_farfield_stats(const vpmg_handle* h, int* on, long long* corrections, double* flops);
/* Per-phase event timing: 0 off (default), 1 on; 2 also keeps the
 * intermediate block fields readable by vpmg_get_field and evaluates the
 * block solves on the whole block (as the reference does) instead of only
 * where the step reads them; 3 = 2. */
int vpmg_set_profiling(vpmg_handle* h, int on);
/* Runs nsteps device-resident steps (as vpmg_step) between two CUDA events
 * on the handle's stream; *ms = elapsed device time, *particle_steps = sum
 * of the particle counts at the start of each step.  The step is captured
 * once as a CUDA graph (counts stay on the device) and replayed.         */
int vpmg_run(vpmg_handle* h, int nsteps, double dt, const double uinf[3], int remesh, double* ms,
             long long* particle_steps);
/* Batched problems: n independent handles (each its own mesh, particles,
 * stream) advance nsteps device-resident steps.  Each handle's step is
 * captured once as a CUDA graph; the graphs of all problems are replayed
 * step by step on their own streams so that small problems run
 * concurrently.  *ms = device time of the whole batch, *solves = n*nsteps,
 * *particle_steps = sum over problems and steps of the particle count.   */
int vpmg_batch_run(vpmg_handle* const* hs, int n, int nsteps, double dt, int remesh, double* ms,
                   long long* solves, long long* particle_steps);
/* Host helper: the forward Euler of the reference's time loop
 * (source/test.f90:104-117, FACDEF = 1) on host arrays, one pass:
 *   XP(:,j) = XP(:,j) + (UP(:,j) + UINF) * dt,  QP(1:3,j) = QP(1:3,j) - GP(:,j) * dt
 * for j < n (uinf may be NULL).  The compiled loop a Fortran host runs,
 * for C and Python hosts; no GPU work.                                  */
int vpmg_host_euler(double* xp, double* qp, const double* up, const double* gp, int n, double dt,
                    const double uinf[3]);
/* Batch object: the same n problems, grouped at creation by shared
 * boundary operator.  Single-block problems (ibctyp 2) whose fine-block
 * operators agree up to the mesh-spacing factor (same index geometry and
 * tree; weights within 1e-12 of the leader's scaled ones; the cells that
 * the two tree walks decided differently, at most 2 % of the
 * interactions, kept as per-problem correction rows) form groups of up to
 * 16; a group's step is one
 * CUDA graph that applies the leader's recorded operator to all members'
 * sources in one launch, so the operator streams from HBM once per group
 * and step.  Other problems keep their own step graphs.  The handles must
 * outlive the batch and take no other calls while it runs.
 * Replaces: the loop over independent problems a host runs around vpm()
 * (source/test.f90:83-150), one problem after another.                  */
typedef struct vpmg_batch vpmg_batch;
/* flags: VPMG_BATCH_RELEASE_SHARED frees the followers' own recorded
 * operators (the group reads only the leader's); on their own, those
 * handles then walk the tree at every apply.                            */
#define VPMG_BATCH_RELEASE_SHARED 1
int vpmg_batch_create(vpmg_handle* const* hs, int n, int flags, vpmg_batch** out);
/* *units = graphs replayed per step; *shared = problems in groups of >= 2;
 * *correction_rows = boundary nodes whose recorded row differs from the
 * group leader's scaled row (a cell exactly on the tree's opening radius in
 * index units, decided by each problem's own rounding): their differences
 * are added per problem after the group's apply.                          */
int vpmg_batch_info(const vpmg_batch* b, int* units, int* shared, long long* correction_rows);
/* nsteps device-resident steps of every problem (as vpmg_batch_run);
 * errors are reported through the first handle (vpmg_last_error).       */
int vpmg_batch_step(vpmg_batch* b, int nsteps, double dt, int remesh, double* ms, long long* solves,
                    long long* particle_steps);
/* Replay order of the batch's graphs within a step: 0 concurrent (each on
 * its own stream), 1 one after another on one stream, -1 (default) chosen
 * by timing the first two steps of the next call with nsteps >= 2 (one
 * step each way; tuned_ms gives the two times).  Results do not depend on
 * the order.                                                             */
int vpmg_batch_set_schedule(vpmg_batch* b, int schedule);
int vpmg_batch_get_schedule(const vpmg_batch* b, int* schedule, float tuned_ms[2]);
int vpmg_batch_destroy(vpmg_batch* b);
/* Replays one kernel of the last step `reps` times between CUDA events on
 * the handle's stream (instrumentation for roofline figures).
 *   which = 0: boundary operator apply on the fine block (recorded operator
 *              or the tree walk), 1: one inner-box Dirichlet solve (5
 *              kernels), 2: deposition gather, 3: velocity curl, 4:
 *              stretching, 5: mesh-to-particle gather, 6: one component of
 *              the padded block's zero-BC solve evaluated where it is read,
 *              7: the remesh's |w| flags and their scan, 8: the sort by
 *              cell and the particle records on the global mesh.
 * Outputs: mean device ms per replay, algorithmic FP64 flops (an FMA
 * counts 2) and DRAM bytes per replay (figures of the algorithm, not
 * counters).  The replay writes only scratch buffers, the particles'
 * UP/GP and the binning arrays, all rewritten by the next step.          */
int vpmg_bench_kernel(vpmg_handle* h, int which, int reps, double* ms, double* flops, double* bytes);
/* FP64 FMA throughput of this GPU (TFLOP/s, FMA = 2 flops) from a
 * register-resident DFMA loop: the roofline peak of the FP64-bound kernels. */
int vpmg_fp64_peak(vpmg_handle* h, double* tflops);
/* DST tile shapes chosen by the set-up autotuner (line pairs per CTA, 2, 4
 * or 8) of the padded block's x and y transforms, the inner box's and the
 * coarse grid's, in that order.                                         */
int vpmg_dst_tiles(const vpmg_handle* h, int pairs[6]);
/* Memory limit (bytes) for the precomputed boundary operator; 0 = never
 * precompute (walk the tree every step).  Default: 100 GiB.              */
int vpmg_set_operator_budget(vpmg_handle* h, long long bytes);

/* ---- the reference's files ------------------------------------------- */
/* particles.bin of source/test.f90:24-37 (Fortran sequential unformatted:
 * NVR, Vref, then NVR records X Y Z w1 w2 w3).  Returns XP(3,NVR) and
 * QP(4,NVR) with QP(1:3) = -w*Vref and QP(4) = Vref.  With xp = qp = NULL
 * only *nvr and *vref are read (size query).  No GPU needed.              */
int vpmg_read_particles_bin(const char* path, int* nvr, double* vref, double* xp, double* qp, int capacity);
/* The inverse: writes XP/QP so that vpmg_read_particles_bin returns them.  */
int vpmg_write_particles_bin(const char* path, int nvr, double vref, const double* xp, const double* qp);
/* writesol (source/vpm.f90:662-709): <dir>/NNNNNsolution.bin of the block
 * range with X Y Z U V W and the vorticity -RHS of the last field step.   */
int vpmg_write_solution(vpmg_handle* h, const char* dir, int ntime);
/* writeline (source/vpm.f90:789-833): appends the nine velocity lines to
 * <dir>/01hist.bin .. 09hist.bin (NTIME = 1 restarts them with a header). */
int vpmg_write_hist(vpmg_handle* h, const char* dir, int ntime);
/* The writers vpm(..., WhatToDo = 2, ...) calls, as the reference does
 * after the velocity (vpm.f90:276-284): flags bit 0 = solution files in
 * the pm.inp windows (NTIME in [IPMWSTART, IPMWSTART + IPMWSTEPS]), bit 1 =
 * the hist lines every field step.  Default: off.  dir NULL = cwd.        */
int vpmg_set_output(vpmg_handle* h, const char* dir, int flags);

/* ---- reverse mode (no counterpart in the reference) -------------------- */
/* The vector-potential solve alone (rhsscat_3d, yaps3d, solget_3d of
 * source/vpm.f90:171-314) on host arrays: psi = L r, both 3 x NN
 * components back to back, node (i,j,k) at i + NN1 (j + NN2 k).         */
int vpmg_apply_poisson(vpmg_handle* h, const double* r, double* psi);
/* Its exact transpose: rbar = L^T psibar (same layout).                  */
int vpmg_adjoint_poisson(vpmg_handle* h, const double* psibar, double* rbar);
/* Vector-Jacobian product of the field step vpm(..., WhatToDo = 2, ...):
 * with (UP, GP) = F(XP, QP), returns xbar (3, nvr) and qbar (3, nvr; for
 * QP(1:3)) = (dF / d(XP, QP(1:3)))^T (upbar, gpbar).  The handle's
 * particles become XP/QP, as vpm(...) leaves them.  M4' projection only.  */
int vpmg_vjp_fields(vpmg_handle* h, const double* xp, const double* qp, int nvr, const double* upbar,
                    const double* gpbar, double* xbar, double* qbar);
/* Vector-Jacobian product of remesh_particles_3d(1) (source/vpm_remesh.f90:
 * 5-225) with respect to the input XP and QP(1:3): qbar_new (3, nnew) is
 * the adjoint of the emitted strengths, nnew the count the remesh emits
 * (VPMG_ERR_ARG otherwise); the |w| cut is a fixed mask.                  */
int vpmg_vjp_remesh(vpmg_handle* h, const double* xp, const double* qp, int nvr, const double* qbar_new, int nnew,
                    double* xbar, double* qbar);
/* Loss of nsteps steps (field step, Euler push with uinf = 0, remesh)
 * from the handle's particles, evaluated on the velocity field of the
 * final particles:
 *   loss = sum_p |u(probe_p)|^2 + ke_weight * 0.5 * DV * sum_nodes |u|^2
 * with u(probe) the M4' interpolation.  probes: (3, nprobe) like XP.
 * mask_mode 0: the reference's remesh |w| cut; 1: the cut, recording each
 * step's node mask; 2: the masks recorded by the last vpmg_adjoint_run (or
 * mode-1 call): the fixed-mask map that the gradient differentiates.
 * The handle's particles are left as they were.  M4' projection only.   */
int vpmg_adjoint_loss(vpmg_handle* h, int nsteps, double dt, const double* probes, int nprobe, double ke_weight,
                      int mask_mode, double* loss);
/* The same loss and its gradient with respect to the initial particle
 * positions xbar (3, NVR) and strengths qbar (3, NVR; QP(1:3)), by the
 * exact transpose of every step, with the particle states checkpointed on
 * the forward pass (7 doubles per mesh node and step of device memory)
 * and each step's remesh mask recorded (the |w| cut is held fixed).
 * ms_forward / ms_backward: device milliseconds of the two passes.       */
int vpmg_adjoint_run(vpmg_handle* h, int nsteps, double dt, const double* probes, int nprobe, double ke_weight,
                     double* loss, double* xbar, double* qbar, double* ms_forward, double* ms_backward);

#ifdef __cplusplus
}
#endif
#endif
