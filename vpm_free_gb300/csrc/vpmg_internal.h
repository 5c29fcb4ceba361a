// vpmg_internal.h -- shared declarations of the sm_103a particle-mesh library.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/vpmg.h"

namespace vpmg {

constexpr double kPI = 3.14159265358979323846264338327950288;

// ------------------------------------------------------------ errors ----
struct Error {
  int status;
  std::string msg;
};
#define VPMG_CUDA(x)                                                                      \
  do {                                                                                    \
    cudaError_t e_ = (x);                                                                 \
    if (e_ != cudaSuccess)                                                                \
      throw ::vpmg::Error{VPMG_ERR_CUDA, std::string(#x) + ": " + cudaGetErrorString(e_)}; \
  } while (0)
#define VPMG_CHECK(cond, code, text)                                  \
  do {                                                                \
    if (!(cond)) throw ::vpmg::Error{(code), std::string(text)};      \
  } while (0)

// Kernel launch counter shared by every launch site (instrumentation).
extern thread_local long long* g_launch_counter;
inline void count_launch(int n = 1) {
  if (g_launch_counter) *g_launch_counter += n;
}
#define VPMG_LAUNCHED() ::vpmg::count_launch()

// ---------------------------------------------------- device buffers ----
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void ensure(size_t count) {
    if (count <= n && p) return;
    release();
    if (count == 0) return;
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      throw Error{VPMG_ERR_NOMEM, "cudaMalloc of " + std::to_string(count * sizeof(T)) + " bytes failed"};
    }
    n = count;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// ------------------------------------------------------------- grids ----
// A node grid: origin, spacing and node counts (1-based node i sits at
// xmin + (i-1)*d, as everywhere in the reference).
struct Grid {
  double xmin[3], d[3];
  int n[3];
  size_t count() const { return (size_t)n[0] * n[1] * n[2]; }
};

// --------------------------------------------------- Dirichlet solver ----
// FFT plan for a DST-I of n = N-1 points.  N even: real-symmetric form,
// two real lines packed in one complex FFT of length M = N (rs = 1);
// N odd: the odd extension, complex length M = 2N (rs = 0).
struct FFTPlan {
  int n = 0, N = 0, M = 0;
  int rs = 0;
  int pairs = 4;     // line pairs per CTA of the DST kernels (tuned per plan)
  int arith = VPMG_ARITH_FP64;  // arithmetic of the transforms
  int nst = 0;
  int radix[24];
  DBuf<double2> twd; // e^{-2 pi i t / M}, t = 0..M-1, FP64
  DBuf<float4> tw;   // the same as float-float (re.hi, re.lo, im.hi, im.lo)
  DBuf<double> sn;   // sin(pi j / N), j = 0..N-1 (rs only)
};
void make_fft_plan(FFTPlan& p, int n, int arith);

// A Dirichlet box inside a node array of dims dims[3]: nodes box[0..2] to
// box[3..5] (0-based, inclusive).  Interior m[d] = box[d+3]-box[d]-1.
struct DirichletPlan {
  int dims[3] = {0, 0, 0};
  int box[6] = {0, 0, 0, 0, 0, 0};
  int m[3] = {0, 0, 0};
  double h[3] = {0, 0, 0};
  int arith = VPMG_ARITH_FP64;  // arithmetic of the transforms and sweeps
  FFTPlan fx, fy;
  DBuf<float2> rinv;  // reciprocal Thomas pivots, [k][q][p], float-float pairs
  DBuf<double> rinvd; // the same in FP64
  bool ready = false;
};
void dirichlet_prepare(DirichletPlan& P, const int dims[3], const int box[6], const double h[3], cudaStream_t s,
                       int arith);
// Interior of sol <- solution of Lap_h u = rhs with the box faces of sol as
// boundary values (zero_bc = false) or zero (true; then the box faces of
// sol are zeroed).  work: >= m0*m1*m2 doubles.
void dirichlet_solve(DirichletPlan& P, const double* rhs, double* sol, bool zero_bc, double* work, cudaStream_t s);
// Pieces of a partially evaluated solve (block_solve.cu).
double dirichlet_scale(const DirichletPlan& P);  // factor applied in the forward x pass
void dst_forward_xy(DirichletPlan& P, const double* rhs, const double* sol, bool zero_bc, double* ghat,
                    cudaStream_t s);
void dst_lines_y(const FFTPlan& p, double* data, int m0, int m1, int m2, cudaStream_t s);
void dst_x_inv_to_box(const FFTPlan& p, const double* data, double* sol, const int dims[3], const int o[3],
                      const int m[3], cudaStream_t s);
// Up to 8 of the above in one launch (each job with its own plan and arrays;
// the plans share one arithmetic).  Results equal the single launches'.
struct DstYLines {
  const FFTPlan* plan;
  double* data;
  int m0, m1, m2;
};
void dst_lines_y_jobs(const DstYLines* jobs, int n, cudaStream_t s);
struct DstXInvLines {
  const FFTPlan* plan;
  const double* data;
  double* sol;
  int dims[3], o[3], m[3];
};
void dst_x_inv_jobs(const DstXInvLines* jobs, int n, cudaStream_t s);

// ------------------------------------------------- boundary operator ----
struct TreeGeom;  // host-built quadtree of one grid (tree_host.cpp)
// Frame of one boundary plane for the constant-source panel potential
// (FSOUR_A4): unit vectors E1..E3, corner offsets S/T, side lengths D,
// diagonal and area of one cell of that plane.
struct PanelFrame {
  double E1[3], E2[3], E3[3], S[4], T[4], D[4], diag, area;
};

// The coarsest tree level of a recorded operator evaluated as convolutions
// on the face lattices (farfield.cu).  Every target sums every coarsest cell
// (the opened ones included) by FFTs: between parallel faces a 2-D
// convolution, between perpendicular faces a 1-D convolution along their
// shared axis and a dense sum over the other two; the cells each target
// opened are then subtracted as sparse correction rows.
struct FarFieldAxis {    // complex FFT of length P = 2^a 3^b along one axis
  int P = 0, nst = 0, npair = 1;
  int radix[16];
  DBuf<double2> tw;      // e^{-2 pi i t / P}
};
struct FarField {
  bool on = false;
  int istep = 0;                      // panels per coarsest cell side
  int N[3] = {0, 0, 0};               // grid nodes per axis
  double h[3] = {0, 0, 0};            // grid spacing per axis
  double dS[6] = {0, 0, 0, 0, 0, 0};  // area of a coarsest cell of each face
  int cell0[6] = {0, 0, 0, 0, 0, 0};  // first coarsest cell of each face (within the level)
  FarFieldAxis ax[3];
  long long kpar_off[3][2] = {{0, 0}, {0, 0}, {0, 0}};  // [normal axis][same face, opposite face]
  long long kperp_off[24] = {};       // [target face * 4 + perpendicular source slot]
  long long t_off[6][2] = {}, s2_off[6][2] = {}, sw_off[6][2] = {}, z_off[6][2] = {};
  DBuf<double> kpar, kperp;           // kernel spectra (real), the inverse scalings folded in
  DBuf<double2> T, S2, X, Sw, Z;      // transform work arrays
  double flops = 0.0;                 // FP64 flops of one apply (FFTs 5 P log2 P per line, products, sums)
  long long ncorr = 0;                // correction rows: the opened coarsest cells, weight -dS/r
  DBuf<long long> crow;
  DBuf<int> ccol;
  DBuf<double> cw;
  long long bytes() const;
};

struct BoundaryOp {
  // panels (level 0) and aggregated levels, device copies
  int nbound = 0, levmax = 0, ncell_total = 0, ntarget = 0;
  int ibctyp = 2;     // 2: point sources -dS/(4 pi r); 3: constant-source panels
  int arith = VPMG_ARITH_FP64;  // recorded weights and their products: FP64 or float-float
  bool tree = true;   // Bounds3d_lev (tree) or the untreed Bounds3d
  PanelFrame frame[6];                  // ibctyp 3: one per target plane
  std::vector<int> lev_off;    // flat offset of each level's cells
  std::vector<int> nbound_lev; // cumulative cells per level (all faces)
  DBuf<double> cx, cy, cz, cds, cthr;   // per flat cell: centre, area, 10*sqrt(ds)
  DBuf<int> child;                      // per flat cell: 4 flat child ids (-1 unused)
  DBuf<int> flags;                      // per flat cell: ilev_t(.,.,6)
  DBuf<int> agg_leaf0;                  // per flat cell: first leaf (flat) or -1 (dummy)
  DBuf<int> agg_rowlen;                 // per flat cell: fast-axis leaf count of its face
  DBuf<int> agg_istep;
  DBuf<int> anc;                        // [(lev-1)*nbound + leaf]: flat ancestor cell or -1
  DBuf<double> csrc;                    // 3 * ncell_total aggregated sources
  DBuf<float2> csrc_ff;                 // the same packed [cell][s0 s1 s2 0] in 8-byte words (doubles or float-float pairs)
  // panels: face geometry for the normal derivative
  DBuf<int> pan_face, pan_i, pan_j, pan_k;  // lower-corner node (0-based) of each panel
  // targets
  DBuf<int> tgt_node;                   // linear node index of each boundary node
  DBuf<double> tx, ty, tz;
  DBuf<int> tgt_frame;                  // ibctyp 3: frame slot of each target's plane
  // precomputed operator (CSR over targets)
  bool precomputed = false;
  long long nnz = 0;
  DBuf<long long> rowptr;
  DBuf<int> col;
  DBuf<float2> w;                       // weights dS/r, 8-byte words: doubles, or float-float pairs (hi + lo = dS/r to 2^-48)
  // the coarsest level, which every target walks in full, as a dense block:
  // [target / 32][cell][target % 32] weight words (as w), zero where the
  // cell was opened; the rows above then hold only the finer levels
  bool dense = false;
  int ntopd = 0;                        // cells of the coarsest level
  long long ndense_acc = 0;             // accepted interactions in the block
  DBuf<float2> wtop;
  int dseg = 1;                         // segments of the coarsest cells (k_apply_dense grid y)
  DBuf<double> dsum;                    // [segment][3][ntarget] partial sums of the block
  DBuf<unsigned long long> dcount;
  // its transpose (CSR over cells, for the reverse mode), built on first use
  bool transposed = false;
  DBuf<long long> colptr;
  DBuf<int> trow;
  DBuf<float2> tw;                      // weight words of the transposed list
  DBuf<float2> vff;                     // per target: the boundary-value adjoint in the operator's arithmetic
  DBuf<double> dpart;                   // dense transpose: partial sums [chunk group][cell]
  FarField ff;                          // the dense block's sums by FFT (FP64, uniform coarsest lattices)
  long long bytes() const;
};
void boundary_prepare(BoundaryOp& B, const Grid& g, int levmax, long long budget_bytes, cudaStream_t s,
                      int ibctyp, bool tree, int arith);
// Sets B.ff up when the recorded operator's coarsest level is a uniform
// lattice on every face (FP64, ibctyp 2, tree, dense block recorded) and
// VPMG_FARFIELD is not "0"; set-up time, outside stream capture.
void farfield_prepare(BoundaryOp& B, const Grid& g, cudaStream_t s);
// dsum[comp][target] = sum over every coarsest cell of dS/r times its source.
void farfield_apply(BoundaryOp& B, double* dsum, cudaStream_t s);
void farfield_release(BoundaryOp& B);
// Per component: normal-derivative panels from the zero-BC solution sol0,
// aggregate, then add the boundary values into the faces of sol.
void boundary_panels(BoundaryOp& B, const Grid& g, const double* sol0, int comp, cudaStream_t s);
void boundary_apply(BoundaryOp& B, const Grid& g, double* const sol[3], cudaStream_t s);
// Problems that share one recorded operator (same index geometry, weights
// in proportion to the mesh spacing): each problem's sources go to its slot
// of an interleaved buffer [cell][slot][4] (float2, nprob slots per cell),
// then one launch adds
// every problem's boundary values (o[p][c] at the target nodes, times scale[p]).
constexpr int kGroupMax = 16;
struct GroupOut {
  double* o[kGroupMax][3];
  double scale[kGroupMax];
};
// Rows of a follower's operator that are not the leader's times the ratio
// (ties of the opening test broken by each problem's rounding): the
// follower's row minus the scaled leader's row, applied after the group.
struct GroupCorrection {
  int nrows = 0;
  long long nnz = 0;
  DBuf<int> rows;
  DBuf<long long> rowptr;
  DBuf<int> col;
  DBuf<double> w;
};
// true when F can share L's recorded operator: same index geometry and
// tree, weights L's times *ratio except for the cells where the two walks
// decided differently, which C holds (at most max_frac of the interactions)
bool boundary_group_match(const BoundaryOp& L, const Grid& gl, const BoundaryOp& F, const Grid& gf, double max_frac,
                          double* ratio, GroupCorrection& C, cudaStream_t s);
void boundary_group_correct(const BoundaryOp& F, const GroupCorrection& C, double* const sol[3], cudaStream_t s);
// Frees the recorded operator (and its transpose): applies walk the tree again.
void boundary_release_recorded(BoundaryOp& B);
void boundary_group_sources(BoundaryOp& B, float2* gsrc, int slot, int lanes, cudaStream_t s);
// doubles of the dense block's partial sums for a group of nprob problems
size_t boundary_group_partial_count(const BoundaryOp& L, int nprob);
void boundary_group_apply(const BoundaryOp& L, const float2* gsrc, int nprob, double* part, const GroupOut& G,
                          cudaStream_t s);
// Transposes (one component): boundary-value adjoint (grid node array) ->
// cell adjoints -> panel adjoints -> accumulated into the sol0 adjoint.
void boundary_apply_T(BoundaryOp& B, const double* bcbar, double* cellbar, cudaStream_t s);
// Builds the transposed interaction list when the operator is recorded and
// the copy fits in half of the free device memory (set-up time, outside
// stream capture); boundary_apply_T then gathers per cell instead of
// scattering with atomics.
void boundary_transpose_prepare(BoundaryOp& B, cudaStream_t s);
void boundary_agg_T(BoundaryOp& B, const double* cellbar, double* panelbar, cudaStream_t s);
void boundary_panels_T(BoundaryOp& B, const Grid& g, const double* panelbar, double* sol0bar, cudaStream_t s);

// ---------------------------------------------------- small kernels ----
void fill_zero(double* p, size_t n, cudaStream_t s);
void exclusive_scan_int(const int* in, int* out, size_t n, int* block_sums, cudaStream_t s);
size_t scan_block_sums_needed(size_t n);
double measure_fp64_peak(cudaStream_t s);  // TFLOP/s of a DFMA loop

}  // namespace vpmg
