// hyperplane.cu -- optional sketch: 128 seeded random hyperplanes (K1b).
//
// The reference's README describes "128-bit random-hyperplane sketches"
// (README.md:33-34), but src/main.cpp:182-190 keeps one sign bit per
// coordinate (d bits), which stays the default.  This mode projects each
// row's int8 codes onto 128 seeded integer hyperplanes:
//   plane k, coordinate j: h = SplitMix64((seed << 32) ^ (k << 10 | j)),
//     g_kj = sum over the 4 low bytes b of h of (b >> 2) - 32, in [-128, 124]
//     (a sum of four uniforms, close to a Gaussian);
//   bit k = (sum_j q_j * g_kj > 0), exact in int32 (|sum| <= 1024 * 128 * 128);
//   bit k % 64 of word k / 64, two words per row.
// Integer arithmetic throughout, so the bits equal the oracle's restatement
// bit for bit.  The NN-Descent join then scores candidates with
// 1024 - popcount over the 2 words (the same formula the reference applies
// to its 16 words, src/main.cpp:354-370): 16 bytes gathered per candidate
// instead of 128.
//
// One persistent CTA per SM: the planes are generated into shared memory
// (128 x (d/4 + 1) words; the pad keeps the 32 lanes' plane reads on distinct
// banks), then tiles of 64 code rows are staged with 16-byte loads and each
// warp projects 8 rows onto the 128 planes (lane l owns planes l, l+32, l+64,
// l+96) with dp4a; a ballot per plane group assembles the bits.  About
// n * 128 * d / 4 dp4a: ~7 ms at 6.35M x 1024.
#include "knng_internal.cuh"

#include <algorithm>

namespace knng {
namespace {

constexpr int kHpThreads = 256;
constexpr int kHpTile = 64;  // rows per tile: 8 warps x 8 rows
constexpr int kPlanes = 128;

__device__ __forceinline__ uint64_t mix64(uint64_t x) {  // SplitMix64 finaliser (Steele, Lea, Flood 2014)
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__device__ __forceinline__ int plane_value(uint32_t seed, int k, int j) {
  const uint64_t h = mix64((uint64_t(seed) << 32) ^ uint64_t((uint32_t(k) << 10) | uint32_t(j)));
  int v = 0;
#pragma unroll
  for (int b = 0; b < 4; ++b) v += int((h >> (8 * b)) & 0xffu) >> 2;
  return v - 128;
}

__global__ void __launch_bounds__(kHpThreads, 1) hyperplane_kernel(const int8_t* __restrict__ codes, int64_t n, int d,
                                                                  uint32_t seed, uint64_t* __restrict__ sketch) {
  extern __shared__ __align__(16) int32_t hp_smem[];
  const int dw = d / 4, ps = dw + 1;
  int32_t* planes = hp_smem;                  // [kPlanes][ps]
  int32_t* rows = hp_smem + kPlanes * ps;     // [kHpTile][dw]; 512 * ps bytes in: 16-byte aligned
  for (int t = threadIdx.x; t < kPlanes * dw; t += kHpThreads) {
    const int k = t / dw, w = t - (t / dw) * dw;
    uint32_t packed = 0;
#pragma unroll
    for (int b = 0; b < 4; ++b) packed |= uint32_t(uint8_t(int8_t(plane_value(seed, k, 4 * w + b)))) << (8 * b);
    planes[k * ps + w] = int32_t(packed);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tiles = (n + kHpTile - 1) / kHpTile;
  const int rb = warp * 8;
  for (int64_t t = blockIdx.x; t < tiles; t += gridDim.x) {
    __syncthreads();  // the planes are written; the previous tile's rows are consumed
    const int64_t r0 = t * kHpTile;
    const int nr = int(n - r0 < kHpTile ? n - r0 : int64_t(kHpTile));
    const int chunks = nr * (d / 16);
    const uint4* src = reinterpret_cast<const uint4*>(codes + r0 * d);
    for (int c = threadIdx.x; c < chunks; c += kHpThreads) reinterpret_cast<uint4*>(rows)[c] = __ldg(src + c);
    __syncthreads();
    if (rb >= nr) continue;  // warp-uniform; rows past nr below read stale words whose results are dropped
    int acc[8][4];
#pragma unroll
    for (int r = 0; r < 8; ++r)
#pragma unroll
      for (int m = 0; m < 4; ++m) acc[r][m] = 0;
    for (int w = 0; w < dw; ++w) {
      int pv[4];
#pragma unroll
      for (int m = 0; m < 4; ++m) pv[m] = planes[(lane + 32 * m) * ps + w];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int rv = rows[(rb + r) * dw + w];
#pragma unroll
        for (int m = 0; m < 4; ++m) acc[r][m] = __dp4a(rv, pv[m], acc[r][m]);
      }
    }
#pragma unroll
    for (int r = 0; r < 8; ++r) {
      if (rb + r >= nr) break;  // uniform across the warp
      const unsigned b0 = __ballot_sync(0xffffffffu, acc[r][0] > 0), b1 = __ballot_sync(0xffffffffu, acc[r][1] > 0);
      const unsigned b2 = __ballot_sync(0xffffffffu, acc[r][2] > 0), b3 = __ballot_sync(0xffffffffu, acc[r][3] > 0);
      if (lane == 0) {
        uint64_t* o = sketch + (r0 + rb + r) * 2;
        o[0] = uint64_t(b0) | (uint64_t(b1) << 32);
        o[1] = uint64_t(b2) | (uint64_t(b3) << 32);
      }
    }
  }
}

}  // namespace

cudaError_t launch_hyperplane_sketch(const int8_t* codes, int64_t n, int d, uint32_t seed, uint64_t* sketch,
                                     int num_sms, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (!dim_ok(d)) return cudaErrorInvalidValue;
  const int dw = d / 4;
  const size_t smem = size_t(kPlanes) * (dw + 1) * 4 + size_t(kHpTile) * dw * 4;
  KNNG_CUDA_TRY(ensure_smem_attr(reinterpret_cast<const void*>(hyperplane_kernel), smem));
  const int64_t tiles = (n + kHpTile - 1) / kHpTile;
  const unsigned grid = unsigned(std::min<int64_t>(tiles, num_sms));
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  hyperplane_kernel<<<grid, kHpThreads, smem, s>>>(codes, n, d, seed, sketch);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
