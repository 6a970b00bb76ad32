// quantize.cu -- K1: float32 rows -> int8 codes + sign-bit sketches, one pass.
//
// Reference: src/main.cpp:179-192.  For every coordinate
//   scaled  = x * 127.0f
//   clamped = max(-128.0f, min(127.0f, scaled))    (std::min/max operand order,
//                                                   so NaN -> 127)
//   code    = (int8) clamped                       (truncation toward zero)
//   sketch bit k%64 of word k/64 = clamped > 0
// Subnormal inputs are read as zero, as the reference's -ffast-math build does.
// KNNG_QUANT_ROUND clamps to [-127, 127] and rounds half away from zero.
//
// Layout: one thread owns 16 consecutive floats of a row (four 16-byte loads,
// one 16-byte code store); the four threads of a 64-coordinate sketch word sit
// in adjacent lanes and assemble it with shuffles.  d % 64 == 0 keeps every
// quad inside one row.  HBM-bound: 4d + d + d/8 bytes per row.
#include "knng_internal.cuh"

namespace knng {
namespace {

__device__ __forceinline__ int quant1(float v, int mode, unsigned& bit) {
  if (fabsf(v) < 1.17549435e-38f) v = 0.0f;  // FLT_MIN: subnormals read as zero
  float s = v * 127.0f;
  float c;
  int q;
  if (mode == KNNG_QUANT_ROUND) {
    c = (s < 127.0f) ? s : 127.0f;
    c = (-127.0f < c) ? c : -127.0f;
    q = __float2int_rz(roundf(c));
  } else {
    c = (s < 127.0f) ? s : 127.0f;
    c = (-128.0f < c) ? c : -128.0f;
    q = __float2int_rz(c);
  }
  bit = c > 0.0f ? 1u : 0u;
  return q;
}

__global__ void __launch_bounds__(256) quantize_kernel(const float4* __restrict__ x, int64_t chunks,
                                                       int mode, uint4* __restrict__ codes,
                                                       uint64_t* __restrict__ sketch) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  // chunks is a multiple of 4 (d % 64 == 0), so every quad of lanes stays active together
  for (int64_t c = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; c - (threadIdx.x & 31) < chunks;
       c += stride) {
    const bool live = c < chunks;
    unsigned bits = 0;
    if (live) {
      float4 v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) v[u] = __ldcs(x + c * 4 + u);
      unsigned w[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        unsigned b0, b1, b2, b3;
        int q0 = quant1(v[u].x, mode, b0), q1 = quant1(v[u].y, mode, b1);
        int q2 = quant1(v[u].z, mode, b2), q3 = quant1(v[u].w, mode, b3);
        w[u] = (unsigned(q0) & 0xffu) | ((unsigned(q1) & 0xffu) << 8) | ((unsigned(q2) & 0xffu) << 16) |
               ((unsigned(q3) & 0xffu) << 24);
        bits |= (b0 | (b1 << 1) | (b2 << 2) | (b3 << 3)) << (4 * u);
      }
      codes[c] = make_uint4(w[0], w[1], w[2], w[3]);
    }
    // assemble a 64-bit word from 4 adjacent lanes (16 bits each)
    const unsigned lane = threadIdx.x & 31;
    unsigned b1 = __shfl_down_sync(0xffffffffu, bits, 1);
    unsigned b2 = __shfl_down_sync(0xffffffffu, bits, 2);
    unsigned b3 = __shfl_down_sync(0xffffffffu, bits, 3);
    if (live && (lane & 3) == 0) {
      uint64_t word = uint64_t(bits) | (uint64_t(b1) << 16) | (uint64_t(b2) << 32) | (uint64_t(b3) << 48);
      sketch[c >> 2] = word;
    }
  }
}

}  // namespace

cudaError_t launch_quantize(const float* x, int64_t n, int d, int quant_mode, int8_t* codes,
                            uint64_t* sketch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t chunks = n * int64_t(d / 16);
  int dev = 0, sms = 0;
  KNNG_CUDA_TRY(cudaGetDevice(&dev));
  KNNG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  int64_t want = (chunks + 255) / 256;
  int64_t cap = int64_t(sms) * 8;
  int blocks = int(want < cap ? want : cap);
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  quantize_kernel<<<blocks, 256, 0, s>>>(reinterpret_cast<const float4*>(x), chunks, quant_mode,
                                         reinterpret_cast<uint4*>(codes), sketch);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
