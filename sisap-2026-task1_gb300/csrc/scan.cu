// scan.cu -- device-wide exclusive prefix sum of int32 counts.
//
// Used by the forest (tile and node compaction) and the leaf table.  Three
// passes per level: block sums, a recursive scan of the sums, and a block-local
// scan plus the scanned block offset.  Each block covers 2048 values (256
// threads x 8); inputs are small next to the graph data, so this is simple
// rather than single-pass.
#include "knng_internal.cuh"

namespace knng {
namespace {

constexpr int kThreads = 256;
constexpr int kItems = 8;
constexpr int kTile = kThreads * kItems;

__device__ __forceinline__ int32_t block_exclusive(int32_t v, int32_t* warp_tot, int32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int32_t inc = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
    if (lane >= o) inc += t;
  }
  if (lane == 31) warp_tot[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    int32_t w = lane < kThreads / 32 ? warp_tot[lane] : 0;
    int32_t wi = w;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t t = __shfl_up_sync(0xffffffffu, wi, o);
      if (lane >= o) wi += t;
    }
    if (lane < kThreads / 32) warp_tot[lane] = wi - w;
    if (lane == kThreads / 32 - 1) *total = wi;
  }
  __syncthreads();
  int32_t r = inc - v + warp_tot[warp];
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(kThreads) block_sums(const int32_t* __restrict__ in, int64_t n,
                                                        int32_t* __restrict__ sums) {
  __shared__ int32_t wt[kThreads / 32];
  __shared__ int32_t tot;
  const int64_t base = int64_t(blockIdx.x) * kTile + int64_t(threadIdx.x) * kItems;
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k)
    if (base + k < n) s += in[base + k];
  block_exclusive(s, wt, &tot);
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kThreads) block_scan(const int32_t* in, int64_t n,
                                                        const int32_t* __restrict__ offs, int32_t* out,
                                                        int64_t* total) {
  __shared__ int32_t wt[kThreads / 32];
  __shared__ int32_t tot;
  const int64_t base = int64_t(blockIdx.x) * kTile + int64_t(threadIdx.x) * kItems;
  int32_t v[kItems];
  int32_t s = 0;
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    v[k] = base + k < n ? in[base + k] : 0;
    s += v[k];
  }
  int32_t run = block_exclusive(s, wt, &tot) + (offs ? offs[blockIdx.x] : 0);
#pragma unroll
  for (int k = 0; k < kItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (total && blockIdx.x == gridDim.x - 1 && threadIdx.x == kThreads - 1) *total = run;
}

int64_t nblocks(int64_t n) { return (n + kTile - 1) / kTile; }

}  // namespace

size_t scan_tmp_bytes(int64_t n) {
  size_t b = 0;
  for (int64_t m = nblocks(n); m > 1; m = nblocks(m)) b += size_t(m) * sizeof(int32_t);
  return b + 256;
}

cudaError_t exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int64_t* total, void* tmp,
                               cudaStream_t s) {
  if (n <= 0) {
    if (total) KNNG_CUDA_TRY(cudaMemsetAsync(total, 0, sizeof(int64_t), s));
    return cudaSuccess;
  }
  const int64_t nb = nblocks(n);
  if (nb == 1) {
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    block_scan<<<1, kThreads, 0, s>>>(in, n, nullptr, out, total);
    note_launch();
    return cudaGetLastError();
  }
  int32_t* sums = static_cast<int32_t*>(tmp);
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  block_sums<<<unsigned(nb), kThreads, 0, s>>>(in, n, sums);
  note_launch();
  KNNG_CUDA_TRY(cudaGetLastError());
  KNNG_CUDA_TRY(exclusive_scan_i32(sums, sums, nb, nullptr, sums + nb, s));
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  block_scan<<<unsigned(nb), kThreads, 0, s>>>(in, n, sums, out, total);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
