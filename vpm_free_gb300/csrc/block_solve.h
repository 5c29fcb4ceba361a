// block_solve.h -- the padded YAPS block's two infinite-domain solves,
// evaluated only where the step reads them (block_solve.cu).
#pragma once
#include "vpmg_internal.h"

namespace vpmg {

struct BlockSolve {
  bool ready = false;
  int dims[3] = {0, 0, 0};  // block node counts
  int m[3] = {0, 0, 0};     // interior counts
  int nsx = 0, nsy = 0, nsz = 0;
  DBuf<double> ghat;        // 3 * interior: forward transforms of the RHS
  DBuf<double> W;           // interior: Thomas output
  int arith = VPMG_ARITH_FP64;  // the plan's arithmetic
  // sine rows sin(pi (i+1)(p+1)/N) of the selected interior indices, one
  // 8-byte word each: a double, or a float-float pair (arith)
  DBuf<double> S_fx, S_fy_lo, S_fy_hi, S_ix, S_iy_lo, S_iy_hi, S_sx, S_sy;
  DBuf<double> e_x1, e_y1;  // sines of the first interior layer along x and y
  DBuf<int> l_fx, l_ix, l_sx, l_sy, l_sz, l_idy, l_idz;  // node lists for scatters / plane lists
  DBuf<double> X8, Y4, X2, Y1, Ys, XS;  // compact partial results
  // Dirichlet face values -> their transforms: the x and y pairs as (sum,
  // difference), the z faces as they are
  DBuf<double> fxs, fxd, fys, fyd, fz0, fzN;
  int inner_lo[3] = {0, 0, 0}, inner_hi[3] = {0, 0, 0};  // interior indices of the inner-box faces
  void prepare(const DirichletPlan& P, const int nnbl_bl[6], int ncoarse);
};

// A whole box's Dirichlet solve with its face values entering in DST space
// (as the block's BC solve does): forward x/y transforms of the RHS alone,
// so vorticity-free tiles skip their FFTs; the faces of sol, transformed
// along their own axes, join the Thomas sweep; full inverse transforms into
// sol's interior.  work and out: interior-size scratch arrays.
struct FaceSolve {
  bool ready = false;
  DBuf<double> f;   // the six faces' values, then their transforms
  DBuf<double> e;   // sines of the first interior layer along x and y
  void prepare(const DirichletPlan& P);
};
void dirichlet_solve_faces(DirichletPlan& P, FaceSolve& F, const double* rhs, double* sol, double* work,
                           double* out, cudaStream_t s);

// Zero-BC solve of component c: forward transform kept in ghat, u near the
// six faces (4 interior layers) written into sol0.
void block_solve_zero_bc(BlockSolve& B, DirichletPlan& P, const double* rhs_c, int c, double* sol0, cudaStream_t s);
// Solve with the boundary values already on the faces of sol_c: writes the
// inner-box faces and the every-ncoarse-th interior samples of sol_c.
void block_solve_bc(BlockSolve& B, DirichletPlan& P, int c, double* sol_c, cudaStream_t s);

}  // namespace vpmg
