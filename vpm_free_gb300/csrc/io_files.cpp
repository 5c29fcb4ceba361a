// io_files.cpp -- the reference's on-disk formats either side of the step.
//
//  * particles.bin (source/test.f90:24-37): record 1 NVR (int32), record 2
//    Vref (float64), then NVR records of 6 float64 (X, Y, Z, w1, w2, w3);
//    the reader forms QP(1:3) = -w Vref and QP(4) = Vref.
//  * NNNNNsolution.bin (writesol, source/vpm.f90:662-709): a VARIABLES
//    record, a ZONE record, then one record of 9 float64 per node of the
//    block range (X, Y, Z, U, V, W, -RHS(1:3)), i fastest.
//  * NNhist.bin (writeline, source/vpm.f90:789-833): nine files of
//    velocity lines along x, appended every field step, with a header
//    written (and the file restarted) when NTIME = 1.
//
// All three are Fortran sequential unformatted files: every record is
// framed by its byte length as a 4-byte little-endian integer before and
// after the payload (the default record marker of gfortran and ifort).
// Compiled with -ffp-contract=off like the rest of the host code.
#include "io_files.h"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace vpmg {
namespace io {

namespace {

struct Record {
  std::vector<unsigned char> b;
  template <class T>
  Record& put(const T& v) {
    const unsigned char* p = reinterpret_cast<const unsigned char*>(&v);
    b.insert(b.end(), p, p + sizeof(T));
    return *this;
  }
  Record& put_text(const char* s) {
    b.insert(b.end(), s, s + std::strlen(s));
    return *this;
  }
};

bool write_record(FILE* f, const Record& r) {
  const uint32_t n = (uint32_t)r.b.size();
  return std::fwrite(&n, 4, 1, f) == 1 && (n == 0 || std::fwrite(r.b.data(), 1, n, f) == n) &&
         std::fwrite(&n, 4, 1, f) == 1;
}

// Reads one record; false at end of file or on a malformed frame.
bool read_record(FILE* f, std::vector<unsigned char>& out) {
  uint32_t n = 0, m = 0;
  if (std::fread(&n, 4, 1, f) != 1) return false;
  out.resize(n);
  if (n && std::fread(out.data(), 1, n, f) != n) return false;
  if (std::fread(&m, 4, 1, f) != 1 || m != n) return false;
  return true;
}

std::string join(const char* dir, const std::string& name) {
  if (!dir || !*dir) return name;
  std::string d(dir);
  if (d.back() != '/') d += '/';
  return d + name;
}

}  // namespace

int read_particles(const char* path, int* nvr, double* vref, double* xp, double* qp, int capacity) {
  if (!path || !nvr) return VPMG_ERR_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return VPMG_ERR_ARG;
  std::vector<unsigned char> r;
  int status = VPMG_OK;
  int32_t n = 0;
  double v = 0.0;
  if (!read_record(f, r) || r.size() < 4) status = VPMG_ERR_ARG;
  if (status == VPMG_OK) {
    std::memcpy(&n, r.data(), 4);
    if (n < 0 || !read_record(f, r) || r.size() < 8) status = VPMG_ERR_ARG;
  }
  if (status == VPMG_OK) {
    std::memcpy(&v, r.data(), 8);
    *nvr = n;
    if (vref) *vref = v;
    if (xp || qp) {
      if (!xp || !qp) status = VPMG_ERR_ARG;
      else if (n > capacity) status = VPMG_ERR_CAPACITY;
      else
        for (int32_t i = 0; i < n && status == VPMG_OK; ++i) {
          double rec[6];
          if (!read_record(f, r) || r.size() < sizeof(rec)) {
            status = VPMG_ERR_ARG;
            break;
          }
          std::memcpy(rec, r.data(), sizeof(rec));
          for (int d = 0; d < 3; ++d) xp[3 * (size_t)i + d] = rec[d];
          // test.f90:34-36: QPR(1:3) = -QPR(1:3)*Vref; QPR(4) = QPR(4)*Vref (= 0); QPR(4) = Vref
          for (int d = 0; d < 3; ++d) qp[4 * (size_t)i + d] = -rec[3 + d] * v;
          qp[4 * (size_t)i + 3] = v;
        }
    }
  }
  std::fclose(f);
  return status;
}

int write_particles(const char* path, int nvr, double vref, const double* xp, const double* qp) {
  if (!path || nvr < 0 || (nvr > 0 && (!xp || !qp)) || !(vref != 0.0)) return VPMG_ERR_ARG;
  FILE* f = std::fopen(path, "wb");
  if (!f) return VPMG_ERR_ARG;
  bool ok = write_record(f, Record().put((int32_t)nvr)) && write_record(f, Record().put(vref));
  for (int i = 0; i < nvr && ok; ++i) {
    Record r;
    for (int d = 0; d < 3; ++d) r.put(xp[3 * (size_t)i + d]);
    for (int d = 0; d < 3; ++d) r.put(-qp[4 * (size_t)i + d] / vref);
    ok = write_record(f, r);
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? VPMG_OK : VPMG_ERR_ARG;
}

int write_solution(const char* dir, int ntime, const SolutionView& s) {
  char name[64];
  std::snprintf(name, sizeof(name), "%05dsolution.bin", ntime);
  FILE* f = std::fopen(join(dir, name).c_str(), "wb");
  if (!f) return VPMG_ERR_ARG;
  const int i0 = s.nn_bl[0], j0 = s.nn_bl[1], k0 = s.nn_bl[2];  // 1-based NXs_bl ..
  const int i1 = s.nn_bl[3], j1 = s.nn_bl[4], k1 = s.nn_bl[5];  // .. NXf_bl
  bool ok = write_record(f, Record().put_text("VARIABLES = \"X\" \"Y\" \"Z\" \"U\" \"V\" \"W\" \"VORTX\" \"VORTY\" \"VORTZ\""));
  ok = ok && write_record(f, Record()
                                 .put_text("ZONE I=")
                                 .put((int32_t)(i1 - i0 + 1))
                                 .put_text(" J=")
                                 .put((int32_t)(j1 - j0 + 1))
                                 .put_text(" K=")
                                 .put((int32_t)(k1 - k0 + 1))
                                 .put_text(" F=POINT"));
  const size_t NX = s.nn[0], NY = s.nn[1], N = NX * NY * (size_t)s.nn[2];
  for (int k = k0; k <= k1 && ok; ++k)
    for (int j = j0; j <= j1 && ok; ++j)
      for (int i = i0; i <= i1 && ok; ++i) {
        const size_t id = (size_t)(i - 1) + NX * ((size_t)(j - 1) + NY * (size_t)(k - 1));
        Record r;
        r.put(s.xmin[0] + (double)(i - 1) * s.d[0]);
        r.put(s.xmin[1] + (double)(j - 1) * s.d[1]);
        r.put(s.xmin[2] + (double)(k - 1) * s.d[2]);
        for (int c = 0; c < 3; ++c) r.put(s.vel[(size_t)c * N + id]);
        for (int c = 0; c < 3; ++c) r.put(-s.rhs[(size_t)c * N + id]);
        ok = write_record(f, r);
      }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? VPMG_OK : VPMG_ERR_ARG;
}

void hist_lines(const int nn_bl[6], int jk[9][2]) {
  // writeline (vpm.f90:800-818): jmat = 0.5*NNJ etc. with default-REAL
  // literals, truncated on assignment to an integer; the results are used
  // directly as global indices J, K.
  const int NNJ = nn_bl[4] - nn_bl[1] + 1, NNK = nn_bl[5] - nn_bl[2] + 1;
  const float fj[9] = {0.5f, 0.25f, 0.25f, 0.75f, 0.75f, 0.5f, 0.5f, 0.25f, 0.75f};
  const float fk[9] = {0.5f, 0.25f, 0.75f, 0.25f, 0.75f, 0.25f, 0.75f, 0.5f, 0.5f};
  for (int i = 0; i < 9; ++i) {
    jk[i][0] = (int)(fj[i] * (float)NNJ);
    jk[i][1] = (int)(fk[i] * (float)NNK);
  }
}

int write_hist(const char* dir, int ntime, const HistView& h) {
  int jk[9][2];
  hist_lines(h.nn_bl, jk);
  const int i0 = h.nn_bl[0], i1 = h.nn_bl[3], nl = i1 - i0 + 1;
  for (int l = 0; l < 9; ++l) {
    char name[32];
    std::snprintf(name, sizeof(name), "%02dhist.bin", l + 1);
    // access='APPEND'; NTIME = 1 rewinds, and a sequential write after a
    // rewind ends the file there
    FILE* f = std::fopen(join(dir, name).c_str(), ntime == 1 ? "wb" : "ab");
    if (!f) return VPMG_ERR_ARG;
    bool ok = true;
    if (ntime == 1) {
      ok = write_record(f, Record().put(h.xmin[0]).put(h.xmin[1]).put(h.xmin[2])) &&
           write_record(f, Record().put(h.d[0]).put(h.d[1]).put(h.d[2])) &&
           write_record(f, Record().put((int32_t)i0).put((int32_t)i1).put((int32_t)jk[l][0]).put((int32_t)jk[l][1]));
    }
    Record r;
    r.put((int32_t)ntime);
    for (int c = 0; c < 3; ++c)
      for (int i = 0; i < nl; ++i) r.put(h.lines[((size_t)l * 3 + c) * nl + i]);
    ok = ok && write_record(f, r);
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return VPMG_ERR_ARG;
  }
  return VPMG_OK;
}

}  // namespace io
}  // namespace vpmg

extern "C" {

int vpmg_read_particles_bin(const char* path, int* nvr, double* vref, double* xp, double* qp, int capacity) {
  return vpmg::io::read_particles(path, nvr, vref, xp, qp, capacity);
}

int vpmg_write_particles_bin(const char* path, int nvr, double vref, const double* xp, const double* qp) {
  return vpmg::io::write_particles(path, nvr, vref, xp, qp);
}

}  // extern "C"
