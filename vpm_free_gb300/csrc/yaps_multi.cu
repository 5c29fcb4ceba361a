// yaps_multi.cu -- YAPS with NBI x NBJ x NBK blocks on one GPU.
//
// The reference runs one block per MPI rank (source/yaps3d.f90:1-453 with
// rhsscat_3d / solget_3d, source/vpm_mpi.f90:199-328).  Here every block's
// fields live in HBM side by side ([block][component][node]) and the
// exchanges become gathers:
//   * rhsscat: each block's inner box takes the global RHS; a block that is
//     not first along an axis leaves its lower inner plane at zero
//     (vpm_mpi.f90:232-234), so a shared plane is deposited once;
//   * sampling every nc-th node of each block onto its own coarse array
//     (yaps3d.f90:104-138) and the coarse RHS as the sum over blocks, in
//     block order, of the 7-point Laplacian inside each block's map
//     (:254-261, :1990-2016);
//   * interp_stencil (:1914-1983): each inner-face node takes
//     sum TSC * (SOL_coarse - sum_b sample_b + sum_{nnb_b = 1} sample_b)
//     plus the first solution of every neighbour block whose map covers
//     the node's stencil, read at the same position in that block (the
//     BBound arrays that mapnodes_bl, :457-1912, fills by messages);
//   * solget: the global SOL takes each block's inner box in block order,
//     so the higher block wins on a shared plane.
// Face values are written to a separate array first because neighbours
// read the first solutions at nodes that are other blocks' faces.
#include <algorithm>

#include "yaps_multi.h"

namespace vpmg {

namespace {

template <class T>
void upload(DBuf<T>& b, const std::vector<T>& h) {
  b.ensure(std::max<size_t>(h.size(), 1));
  if (!h.empty()) VPMG_CUDA(cudaMemcpy(b.p, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice));
}

unsigned blocks_for(size_t n, int threads) {
  return (unsigned)std::min<size_t>(std::max<size_t>(1, (n + threads - 1) / threads), 152 * 64);
}

// rhs_bl[b][c][node] for every block node: the global value inside the inner
// box (zero on a non-first block's lower inner planes), zero in the padding.
__global__ void k_rhsscat(const double* __restrict__ rhs, size_t N, int NX, int NY, int BX, int BY, int BZ, int lo0,
                          int lo1, int lo2, int hi0, int hi1, int hi2, int g0, int g1, int g2, int NBI, int NBJ,
                          int nblk, double* __restrict__ rhs_bl) {
  const size_t NB = (size_t)BX * BY * BZ;
  const size_t total = (size_t)nblk * 3 * NB;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t node = t % NB;
    const int c = (int)((t / NB) % 3);
    const int b = (int)(t / (3 * NB));
    const int i = (int)(node % BX), j = (int)((node / BX) % BY), k = (int)(node / ((size_t)BX * BY));
    const int bi = b % NBI, bj = (b / NBI) % NBJ, bk = b / (NBI * NBJ);
    double v = 0.0;
    if (i >= lo0 && i <= hi0 && j >= lo1 && j <= hi1 && k >= lo2 && k <= hi2 && !(bi > 0 && i == lo0) &&
        !(bj > 0 && j == lo1) && !(bk > 0 && k == lo2)) {
      const int gi = g0 + bi * (hi0 - lo0) + (i - lo0), gj = g1 + bj * (hi1 - lo1) + (j - lo1),
                gk = g2 + bk * (hi2 - lo2) + (k - lo2);
      v = rhs[(size_t)c * N + (size_t)gi + (size_t)NX * ((size_t)gj + (size_t)NY * gk)];
    }
    rhs_bl[t] = v;
  }
}

__global__ void k_sample(const double* __restrict__ sol_bl, size_t NB, const long long* __restrict__ src,
                         const long long* __restrict__ dst, int nsamp, int nblk, size_t NC, double* __restrict__ samp) {
  const size_t total = (size_t)nblk * 3 * nsamp;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const int m = (int)(t % nsamp);
    const int c = (int)((t / nsamp) % 3);
    const int b = (int)(t / (3 * (size_t)nsamp));
    samp[((size_t)b * 3 + c) * NC + dst[(size_t)b * nsamp + m]] = sol_bl[((size_t)b * 3 + c) * NB + src[m]];
  }
}

// Per coarse node and component: the sum of the samples over blocks (in
// block order, as interp_stencil's add_sample) and the coarse RHS, the sum
// over blocks of the Laplacian where the node is strictly inside the
// block's map.
__global__ void k_coarse(const double* __restrict__ samp, const int* __restrict__ maps, int nblk, int CX, int CY, int CZ,
                         double i2x, double i2y, double i2z, double* __restrict__ sampsum, double* __restrict__ crhs) {
  const size_t NC = (size_t)CX * CY * CZ;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < 3 * NC; t += (size_t)gridDim.x * blockDim.x) {
    const size_t id = t % NC;
    const int c = (int)(t / NC);
    const int i = (int)(id % CX) + 1, j = (int)((id / CX) % CY) + 1, k = (int)(id / ((size_t)CX * CY)) + 1;
    double ss = 0.0, rr = 0.0;
    for (int b = 0; b < nblk; ++b) {
      const double* S = samp + ((size_t)b * 3 + c) * NC;
      ss = S[id] + ss;
      const int* mp = maps + 6 * b;
      if (i > mp[0] && i < mp[3] && j > mp[1] && j < mp[4] && k > mp[2] && k < mp[5]) {
        const size_t sy = CX, sz = (size_t)CX * CY;
        const double s0 = S[id];
        const double l = ((S[id + 1] - 2.0 * s0) + S[id - 1]) * i2x + ((S[id + sy] - 2.0 * s0) + S[id - sy]) * i2y +
                         ((S[id + sz] - 2.0 * s0) + S[id - sz]) * i2z;
        rr = rr + l;
      }
    }
    sampsum[t] = ss;
    crhs[t] = rr;
  }
}

// interp_stencil for every inner-face node of every block -> face_val.
__global__ void k_face(const int* __restrict__ fblock, const long long* __restrict__ fnode,
                       const long long* __restrict__ fcbase, const double* __restrict__ fw,
                       const int* __restrict__ flag_off, const int* __restrict__ flag_blk,
                       const int* __restrict__ bb_off, const int* __restrict__ bb_blk,
                       const long long* __restrict__ bb_node, int nface, const double* __restrict__ csol,
                       const double* __restrict__ sampsum, const double* __restrict__ samp, size_t NC, int CX, int CY,
                       const double* __restrict__ sol_bl, size_t NB, double* __restrict__ face_val) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nface) return;
  const int b = fblock[t];
  const long long cb = fcbase[t];
  const double* w = fw + 9 * (size_t)t;
  const int f0 = flag_off[t], f1 = flag_off[t + 1];
  const int q0 = bb_off[t], q1 = bb_off[t + 1];
  for (int c = 0; c < 3; ++c) {
    double v = sol_bl[((size_t)b * 3 + c) * NB + fnode[t]];
    for (int kc = 0; kc < 3; ++kc)
      for (int jc = 0; jc < 3; ++jc)
        for (int ic = 0; ic < 3; ++ic) {
          const size_t ci = (size_t)cb + ic + (size_t)CX * (jc + (size_t)CY * kc);
          double add = 0.0;
          for (int f = f0; f < f1; ++f) add = samp[((size_t)flag_blk[f] * 3 + c) * NC + ci] + add;
          const double f = (w[ic] * w[3 + jc]) * w[6 + kc];
          v = v + f * ((csol[(size_t)c * NC + ci] - sampsum[(size_t)c * NC + ci]) + add);
        }
    for (int q = q0; q < q1; ++q) v = v + sol_bl[((size_t)bb_blk[q] * 3 + c) * NB + bb_node[q]];
    face_val[(size_t)c * nface + t] = v;
  }
}

__global__ void k_face_store(const int* __restrict__ fblock, const long long* __restrict__ fnode, int nface,
                             const double* __restrict__ face_val, size_t NB, double* __restrict__ sol_bl) {
  const size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
  if (t >= 3 * (size_t)nface) return;
  const int f = (int)(t % nface), c = (int)(t / nface);
  sol_bl[((size_t)fblock[f] * 3 + c) * NB + fnode[f]] = face_val[t];
}

// solget_3d: every global node of the blocks' union takes the value of the
// last block (in block order) whose inner box holds it.
__global__ void k_solget(const double* __restrict__ sol_bl, size_t NB, int BX, int BY, int lo0, int lo1, int lo2,
                         int c0, int c1, int c2, int NBI, int NBJ, int NBK, int g0, int g1, int g2, int NX, int NY,
                         size_t N, double* __restrict__ sol) {
  const size_t e0 = (size_t)NBI * c0 + 1, e1 = (size_t)NBJ * c1 + 1, e2 = (size_t)NBK * c2 + 1;
  const size_t total = 3 * e0 * e1 * e2;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < total; t += (size_t)gridDim.x * blockDim.x) {
    const size_t u = t % (e0 * e1 * e2);
    const int c = (int)(t / (e0 * e1 * e2));
    const int x = (int)(u % e0), y = (int)((u / e0) % e1), z = (int)(u / (e0 * e1));
    const int bi = min(x / c0, NBI - 1), bj = min(y / c1, NBJ - 1), bk = min(z / c2, NBK - 1);
    const int b = (bk * NBJ + bj) * NBI + bi;
    const size_t ln = (size_t)(lo0 + x - bi * c0) + (size_t)BX * ((size_t)(lo1 + y - bj * c1) + (size_t)BY * (lo2 + z - bk * c2));
    sol[(size_t)c * N + (size_t)(g0 + x) + (size_t)NX * ((size_t)(g1 + y) + (size_t)NY * (g2 + z))] =
        sol_bl[((size_t)b * 3 + c) * NB + ln];
  }
}

}  // namespace

void YapsMultiDev::prepare(const YapsMultiGeom& Y) {
  nblk = Y.nblk;
  nsamp = Y.nsamp;
  nface = (int)Y.faces.size();
  std::vector<int> fb(nface), foff(nface + 1), boff(nface + 1);
  std::vector<long long> fn(nface), fc(nface);
  std::vector<double> fw(9 * (size_t)nface);
  for (int t = 0; t < nface; ++t) {
    const MultiFace& F = Y.faces[t];
    fb[t] = F.block; fn[t] = F.node; fc[t] = F.cbase;
    for (int m = 0; m < 9; ++m) fw[9 * (size_t)t + m] = F.w[m];
    foff[t] = F.flag0; boff[t] = F.bb0;
  }
  foff[nface] = (int)Y.flag_blocks.size();
  boff[nface] = (int)Y.bb_block.size();
  upload(face_block, fb); upload(face_node, fn); upload(face_cbase, fc); upload(face_w, fw);
  upload(flag_off, foff); upload(flag_blk, Y.flag_blocks);
  upload(bb_off, boff); upload(bb_blk, Y.bb_block); upload(bb_node, Y.bb_node);
  upload(samp_src, Y.samp_src); upload(samp_dst, Y.samp_dst); upload(maps, Y.maps);
  face_val.ensure(3 * (size_t)std::max(nface, 1));
}

void yaps_multi_rhsscat(const YapsMultiDev& Y, const double* rhs, const int nn[3], const int nn_bl[6],
                        const int nbl[3], const int nnbl_bl[6], const int nblocks[3], double* rhs_bl, cudaStream_t s) {
  const size_t N = (size_t)nn[0] * nn[1] * nn[2];
  const size_t total = (size_t)Y.nblk * 3 * nbl[0] * nbl[1] * nbl[2];
  k_rhsscat<<<blocks_for(total, 256), 256, 0, s>>>(rhs, N, nn[0], nn[1], nbl[0], nbl[1], nbl[2], nnbl_bl[0] - 1,
                                                   nnbl_bl[1] - 1, nnbl_bl[2] - 1, nnbl_bl[3] - 1, nnbl_bl[4] - 1,
                                                   nnbl_bl[5] - 1, nn_bl[0] - 1, nn_bl[1] - 1, nn_bl[2] - 1,
                                                   nblocks[0], nblocks[1], Y.nblk, rhs_bl);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void yaps_multi_coarse(YapsMultiDev& Y, const double* sol_bl, size_t NB, const int cdims[3], const double dc[3],
                       double* samp, double* sampsum, double* crhs, cudaStream_t s) {
  const size_t NC = (size_t)cdims[0] * cdims[1] * cdims[2];
  fill_zero(samp, (size_t)Y.nblk * 3 * NC, s);
  const size_t ns = (size_t)Y.nblk * 3 * Y.nsamp;
  k_sample<<<blocks_for(ns, 256), 256, 0, s>>>(sol_bl, NB, Y.samp_src.p, Y.samp_dst.p, Y.nsamp, Y.nblk, NC, samp);
  VPMG_LAUNCHED();
  k_coarse<<<blocks_for(3 * NC, 256), 256, 0, s>>>(samp, Y.maps.p, Y.nblk, cdims[0], cdims[1], cdims[2],
                                                   1.0 / (dc[0] * dc[0]), 1.0 / (dc[1] * dc[1]),
                                                   1.0 / (dc[2] * dc[2]), sampsum, crhs);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void yaps_multi_faces(YapsMultiDev& Y, const int cdims[3], const double* csol, const double* sampsum,
                      const double* samp, double* sol_bl, size_t NB, cudaStream_t s) {
  if (Y.nface == 0) return;
  const size_t NC = (size_t)cdims[0] * cdims[1] * cdims[2];
  k_face<<<(Y.nface + 127) / 128, 128, 0, s>>>(Y.face_block.p, Y.face_node.p, Y.face_cbase.p, Y.face_w.p,
                                               Y.flag_off.p, Y.flag_blk.p, Y.bb_off.p, Y.bb_blk.p, Y.bb_node.p,
                                               Y.nface, csol, sampsum, samp, NC, cdims[0], cdims[1], sol_bl, NB,
                                               Y.face_val.p);
  VPMG_LAUNCHED();
  k_face_store<<<(unsigned)((3 * (size_t)Y.nface + 255) / 256), 256, 0, s>>>(Y.face_block.p, Y.face_node.p, Y.nface,
                                                                            Y.face_val.p, NB, sol_bl);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

void yaps_multi_solget(const double* sol_bl, const int nbl[3], const int nnbl_bl[6], const int nblocks[3],
                       const int nn[3], const int nn_bl[6], double* sol, cudaStream_t s) {
  const int c0 = nnbl_bl[3] - nnbl_bl[0], c1 = nnbl_bl[4] - nnbl_bl[1], c2 = nnbl_bl[5] - nnbl_bl[2];
  const size_t total = 3 * ((size_t)nblocks[0] * c0 + 1) * ((size_t)nblocks[1] * c1 + 1) * ((size_t)nblocks[2] * c2 + 1);
  const size_t NB = (size_t)nbl[0] * nbl[1] * nbl[2], N = (size_t)nn[0] * nn[1] * nn[2];
  k_solget<<<blocks_for(total, 256), 256, 0, s>>>(sol_bl, NB, nbl[0], nbl[1], nnbl_bl[0] - 1, nnbl_bl[1] - 1,
                                                  nnbl_bl[2] - 1, c0, c1, c2, nblocks[0], nblocks[1], nblocks[2],
                                                  nn_bl[0] - 1, nn_bl[1] - 1, nn_bl[2] - 1, nn[0], nn[1], N, sol);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaGetLastError());
}

}  // namespace vpmg
