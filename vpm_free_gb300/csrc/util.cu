// util.cu -- fills and an exclusive prefix sum over int counts.
#include <algorithm>
#include "vpmg_internal.h"

namespace vpmg {

thread_local long long* g_launch_counter = nullptr;

namespace {
constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

__global__ void k_fill_zero(double* __restrict__ p, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) p[i] = 0.0;
}

__device__ __forceinline__ int warp_incl_scan(int v) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int t = __shfl_up_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) >= o) v += t;
  }
  return v;
}

// Block-wide exclusive scan of one value per thread; returns the block total.
__device__ int block_excl_scan(int v, int& total) {
  __shared__ int wsum[kScanThreads / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int inc = warp_incl_scan(v);
  if (lane == 31) wsum[wid] = inc;
  __syncthreads();
  if (wid == 0) {
    int s = (lane < kScanThreads / 32) ? wsum[lane] : 0;
    s = warp_incl_scan(s);
    if (lane < kScanThreads / 32) wsum[lane] = s;
  }
  __syncthreads();
  const int before = (wid > 0) ? wsum[wid - 1] : 0;
  total = wsum[kScanThreads / 32 - 1];
  __syncthreads();
  return before + inc - v;
}

__global__ void __launch_bounds__(kScanThreads) k_tile_sums(const int* __restrict__ in, size_t n, int* __restrict__ sums) {
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i)
    if (base + i < n) s += in[base + i];
  int total;
  block_excl_scan(s, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(int* __restrict__ sums, int nt) {
  int carry = 0;
  for (int base = 0; base < nt; base += kScanThreads) {
    const int i = base + threadIdx.x;
    const int v = (i < nt) ? sums[i] : 0;
    int total;
    const int ex = block_excl_scan(v, total);
    if (i < nt) sums[i] = carry + ex;
    carry += total;
  }
}

__global__ void __launch_bounds__(kScanThreads) k_tile_scan(const int* __restrict__ in, int* __restrict__ out, size_t n,
                                                            const int* __restrict__ sums) {
  const size_t base = (size_t)blockIdx.x * kScanTile + (size_t)threadIdx.x * kScanItems;
  int v[kScanItems];
  int s = 0;
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    s += v[i];
  }
  int total;
  int run = block_excl_scan(s, total) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = run;
    run += v[i];
  }
}

// Dependent-chain DFMA loop: 8 independent chains per thread.
__global__ void k_dfma_peak(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-3, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6,
         x7 = x0 + 7;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
}
}  // namespace

double measure_fp64_peak(cudaStream_t s) {
  int dev = 0, sms = 0;
  VPMG_CUDA(cudaGetDevice(&dev));
  VPMG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int blocks = sms * 8, threads = 256, iters = 4000;
  DBuf<double> o;
  o.ensure((size_t)blocks * threads);
  k_dfma_peak<<<blocks, threads, 0, s>>>(o.p, 100, 0.999, 1e-3);
  VPMG_LAUNCHED();
  cudaEvent_t a, b;
  VPMG_CUDA(cudaEventCreate(&a));
  VPMG_CUDA(cudaEventCreate(&b));
  VPMG_CUDA(cudaEventRecord(a, s));
  k_dfma_peak<<<blocks, threads, 0, s>>>(o.p, iters, 0.999, 1e-3);
  VPMG_LAUNCHED();
  VPMG_CUDA(cudaEventRecord(b, s));
  VPMG_CUDA(cudaEventSynchronize(b));
  float ms = 0.f;
  VPMG_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return (double)blocks * threads * iters * 8 * 2 / (ms * 1e-3) / 1e12;
}

void fill_zero(double* p, size_t n, cudaStream_t s) {
  if (!n) return;
  const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
  k_fill_zero<<<blocks, 256, 0, s>>>(p, n);
  VPMG_LAUNCHED();
}

size_t scan_block_sums_needed(size_t n) { return (n + kScanTile - 1) / kScanTile + 1; }

// out[i] = sum_{j<i} in[j]; out[n] is NOT written (callers read the total
// from the tile sums: block_sums[ntiles] receives it).
void exclusive_scan_int(const int* in, int* out, size_t n, int* block_sums, cudaStream_t s) {
  const int nt = (int)((n + kScanTile - 1) / kScanTile);
  k_tile_sums<<<nt, kScanThreads, 0, s>>>(in, n, block_sums);
  k_scan_sums<<<1, kScanThreads, 0, s>>>(block_sums, nt + 1);  // entry nt (zero) becomes the grand total
  k_tile_scan<<<nt, kScanThreads, 0, s>>>(in, out, n, block_sums);
  count_launch(3);
}

}  // namespace vpmg
