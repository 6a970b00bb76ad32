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
// Layout: the rows are one stream of float4; every warp load instruction
// reads 32 consecutive float4 (512 contiguous bytes) and each lane stores the
// 4-byte code word of its float4, so both the HBM path and host rows read
// directly over the CPU link stay coalesced.  A sketch word covers 16
// consecutive float4 of one row (d % 64 == 0), combined across lanes by shuffles.
// Bound by the input stream: 4d + d + d/8 bytes per row.
#include "knng_internal.cuh"

namespace knng {
namespace {

// x * 127 with subnormal inputs read as zero.  The flush-to-zero multiply
// gives exactly that for every input: a subnormal x becomes a signed zero, and
// a normal x has a normal product, so nothing else is flushed.
__device__ __forceinline__ float scale127_daz(float v) {
  float s;
  asm("mul.ftz.f32 %0, %1, %2;" : "=f"(s) : "f"(v), "f"(127.0f));
  return s;
}

// The reference's std::max(lo, std::min(127.0f, s)): fminf/fmaxf return the
// non-NaN operand, so NaN becomes 127 as in std::min(127.0f, NaN).
template <int kMode>
__device__ __forceinline__ int quant1(float v, unsigned& bit) {
  const float s = scale127_daz(v);
  const float c = fmaxf(fminf(s, 127.0f), kMode == KNNG_QUANT_ROUND ? -127.0f : -128.0f);
  bit = c > 0.0f ? 1u : 0u;
  return kMode == KNNG_QUANT_ROUND ? __float2int_rz(roundf(c)) : __float2int_rz(c);
}

// A warp covers 128 consecutive float4 per step and each of its load
// instructions reads 32 consecutive float4 (512 contiguous bytes), which
// host memory read over the CPU link needs as much as HBM does.  Lane l
// quantises float4 base + 32u + l (u = 0..3) into one 4-byte code word and a
// 4-bit sign nibble; the sketch word of 16 consecutive float4 (64 floats,
// bit j = float j > 0) takes lane l's nibble at bit 4 (l % 16), combined by
// three xor-shuffle ORs within 8 lanes and one shuffle for the upper half.
template <int kMode>
__global__ void __launch_bounds__(256) quantize_kernel(const float4* __restrict__ x, int64_t nf4,
                                                       uint32_t* __restrict__ codes, uint64_t* __restrict__ sketch) {
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int64_t warp = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = (int64_t(gridDim.x) * blockDim.x) >> 5;
  for (int64_t base = warp * 128; base < nf4; base += nwarps * 128) {
    float4 v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t f = base + 32 * u + lane;
      v[u] = f < nf4 ? __ldcs(x + f) : make_float4(0.f, 0.f, 0.f, 0.f);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t f = base + 32 * u + lane;
      unsigned b0, b1, b2, b3;
      const int q0 = quant1<kMode>(v[u].x, b0), q1 = quant1<kMode>(v[u].y, b1);
      const int q2 = quant1<kMode>(v[u].z, b2), q3 = quant1<kMode>(v[u].w, b3);
      if (f < nf4)
        codes[f] = (unsigned(q0) & 0xffu) | ((unsigned(q1) & 0xffu) << 8) | ((unsigned(q2) & 0xffu) << 16) |
                   ((unsigned(q3) & 0xffu) << 24);
      unsigned w = (b0 | (b1 << 1) | (b2 << 2) | (b3 << 3)) << (4 * (lane & 7));
      w |= __shfl_xor_sync(full, w, 1);
      w |= __shfl_xor_sync(full, w, 2);
      w |= __shfl_xor_sync(full, w, 4);  // lanes 8g..8g+7: their 32 sign bits
      const unsigned hi = __shfl_down_sync(full, w, 8);
      // nf4 is a multiple of 16, so a 16-lane group is wholly in range or out
      if ((lane & 15) == 0 && f < nf4) sketch[f >> 4] = uint64_t(w) | (uint64_t(hi) << 32);
    }
  }
}

}  // namespace

cudaError_t launch_quantize(const float* x, int64_t n, int d, int quant_mode, int8_t* codes,
                            uint64_t* sketch, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int64_t nf4 = n * int64_t(d / 4);  // a multiple of 16: d % 64 == 0
  int dev = 0, sms = 0;
  KNNG_CUDA_TRY(cudaGetDevice(&dev));
  KNNG_CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const int64_t want = (nf4 + 1023) / 1024;  // 8 warps x 128 float4 per block step
  const int64_t cap = int64_t(sms) * 8;
  const int blocks = int(want < cap ? want : cap);
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  const float4* x4 = reinterpret_cast<const float4*>(x);
  uint32_t* c4 = reinterpret_cast<uint32_t*>(codes);
  if (quant_mode == KNNG_QUANT_ROUND) quantize_kernel<KNNG_QUANT_ROUND><<<blocks, 256, 0, s>>>(x4, nf4, c4, sketch);
  else quantize_kernel<KNNG_QUANT_TRUNC><<<blocks, 256, 0, s>>>(x4, nf4, c4, sketch);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
