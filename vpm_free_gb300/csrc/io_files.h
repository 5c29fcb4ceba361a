// io_files.h -- the reference's particle and solution file formats (io_files.cpp).
#pragma once
#include "../../include/vpmg.h"

namespace vpmg {
namespace io {

// Host copies of the fields a solution file reads (3 components of nn
// nodes each, back to back, x fastest) and the mesh they live on.
struct SolutionView {
  const double* vel;
  const double* rhs;
  int nn[3], nn_bl[6];
  double xmin[3], d[3];
};
// The nine velocity lines of writeline: lines[(l*3 + c)*nl + i], i over
// NXs_bl..NXf_bl, at the (J, K) of hist_lines(l).
struct HistView {
  const double* lines;
  int nn_bl[6];
  double xmin[3], d[3];
};

int read_particles(const char* path, int* nvr, double* vref, double* xp, double* qp, int capacity);
int write_particles(const char* path, int nvr, double vref, const double* xp, const double* qp);
int write_solution(const char* dir, int ntime, const SolutionView& s);
void hist_lines(const int nn_bl[6], int jk[9][2]);  // 1-based global (J, K) of the nine lines
int write_hist(const char* dir, int ntime, const HistView& h);

}  // namespace io
}  // namespace vpmg
