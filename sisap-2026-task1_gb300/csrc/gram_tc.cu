// gram_tc.cu -- K3 on the 5th-generation tensor cores: leaf Gram blocks with
// tcgen05.mma (bf16 operands, fp32 accumulation in tensor memory).
//
// Reference: the dots of src/main.cpp:261-269 (every pair of members of a
// leaf).  ptxas rejects tcgen05.mma.kind::i8 for sm_103a, so the int8 codes are
// widened to bf16 (exact: |q| <= 128 needs 8 significant bits) and multiplied
// with kind::f16 into fp32 accumulators.  Every partial sum is an integer of
// magnitude <= d * 128 * 128 <= 2^24, which fp32 represents exactly, so the
// result equals the int32 dot bit for bit (checked against the dp4a kernel).
//
// Tile: two leaves (<= 64 members each) stacked as one 128-row operand X;
// one MMA chain computes D = X * X^T (M = N = 128) and the two 64 x 64
// diagonal blocks are the two leaves' Gram blocks.  X is staged 128 columns of
// d at a time into one of two shared-memory stages in the K-major core-matrix
// layout (8 rows x 16 bytes per core matrix, no swizzle; LBO = 128 B between
// core matrices along K, SBO = 2048 B between 8-row groups), converting int8
// to bf16 on the way (TMA cannot convert).  One thread issues 8 MMAs (K = 16
// each) per stage and commits them to the stage's mbarrier; the stage is
// refilled only after that barrier flips.  D lives in 128 TMEM columns; warp w
// reads lanes 32w..32w+31 with tcgen05.ld.  Every mbarrier wait is bounded (the
// limit is a launch argument): on timeout the kernel records kErrTimeout, the
// whole block stops issuing work at the next barrier, thread 0 waits with the
// full limit for every MMA it committed and the tensor memory is freed before
// the kernel returns.
#include "knng_internal.cuh"

#include <algorithm>

namespace knng {
namespace {

constexpr int kTcThreads = 128;
constexpr int kChunk = 128;                     // d columns per stage
constexpr int kStageBytes = 128 * kChunk * 2;   // 128 rows x 128 bf16 = 32 KB
constexpr uint32_t kTmemCols = 128;
constexpr long long kSpinLimit = 1ll << 26;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit) {
  for (long long i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// Shared-memory matrix descriptor: K-major, no swizzle, descriptor version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = 0;
  d |= uint64_t((addr >> 4) & 0x3fff);
  d |= uint64_t((lbo >> 4) & 0x3fff) << 16;
  d |= uint64_t((sbo >> 4) & 0x3fff) << 32;
  d |= uint64_t(1) << 46;
  return d;
}

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major, N, M.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

__device__ __forceinline__ uint32_t bf16x2(int a, int b) {
  // int8 values widened exactly: bf16 of a float integer in [-128, 127]
  const uint32_t lo = __float_as_uint(float(a)) >> 16;
  const uint32_t hi = __float_as_uint(float(b)) >> 16;
  return lo | (hi << 16);
}

__global__ void __launch_bounds__(kTcThreads, 1) leaf_gram_tc(const int8_t* __restrict__ codes, int d,
                                                             const int32_t* __restrict__ perm,
                                                             const int32_t* __restrict__ leaf_start,
                                                             int64_t nleaves, int64_t total,
                                                             int32_t* __restrict__ gram, unsigned* err,
                                                             long long spin_limit) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_base;
  unsigned char* stage[2] = {smem, smem + kStageBytes};
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;

  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&mbar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = tmem_base;
  const uint32_t idesc = instr_desc(128, 128);
  const int nchunks = d / kChunk;
  uint32_t phase[2] = {0, 0};
  int pending[2] = {0, 0};  // commits issued on a stage and not yet waited for
  const int64_t npairs = (nleaves + 1) / 2;
  // Aborting is decided only from __syncthreads_or over every thread's wait
  // outcome, so every thread takes the same path to the drain (a flag in
  // shared memory written by one thread and read by another without a barrier
  // in between would split the block across different barriers).
  bool aborted = false;

  for (int64_t pr = blockIdx.x; pr < npairs && !aborted; pr += gridDim.x) {
    int64_t ls[2], lm[2];
    for (int h = 0; h < 2; ++h) {
      const int64_t l = 2 * pr + h;
      if (l < nleaves) {
        ls[h] = leaf_start[l];
        lm[h] = (l + 1 < nleaves ? leaf_start[l + 1] : total) - ls[h];
      } else {
        ls[h] = 0;
        lm[h] = 0;
      }
    }
    // this thread stages row r = tid of X: leaf tid/64, member tid%64
    const int hrow = tid >> 6, mrow = tid & 63;
    const bool live_row = mrow < lm[hrow];
    const int8_t* src = live_row ? codes + int64_t(perm[ls[hrow] + mrow]) * d : nullptr;
    for (int c = 0; c < nchunks; ++c) {
      const int st = c & 1;
      int gave_up = 0;
      if (pending[st]) {  // the MMAs that read this stage two chunks ago must be done
        if (mbar_wait(smem_u32(&mbar[st]), phase[st], spin_limit)) {
          phase[st] ^= 1;
          pending[st] = 0;
        } else {
          gave_up = 1;  // pending stays set, so the drain below still waits for this commit
        }
      }
      if (__syncthreads_or(gave_up)) {
        aborted = true;
        break;
      }
      // row tid, 128 codes -> 16 core-matrix rows of 8 bf16 (16 bytes each)
      unsigned char* base = stage[st] + (tid >> 3) * 2048 + (tid & 7) * 16;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        int4 v = make_int4(0, 0, 0, 0);
        if (live_row) v = __ldg(reinterpret_cast<const int4*>(src + c * kChunk) + q);
        const int w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint4 o;
          const int a = w[2 * h], b = w[2 * h + 1];
          o.x = bf16x2(int(int8_t(a)), int(int8_t(a >> 8)));
          o.y = bf16x2(int(int8_t(a >> 16)), int(int8_t(a >> 24)));
          o.z = bf16x2(int(int8_t(b)), int(int8_t(b >> 8)));
          o.w = bf16x2(int(int8_t(b >> 16)), int(int8_t(b >> 24)));
          *reinterpret_cast<uint4*>(base + (2 * q + h) * 128) = o;
        }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncthreads();
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const uint32_t sa = smem_u32(stage[st]);
#pragma unroll
        for (int kk = 0; kk < kChunk / 16; ++kk) {
          const uint64_t desc = smem_desc(sa + kk * 256, 128, 2048);
          const uint32_t acc = (c > 0 || kk > 0) ? 1u : 0u;
          asm volatile(
              "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
              "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(taddr),
              "l"(desc), "l"(desc), "r"(idesc), "r"(acc)
              : "memory");
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                         smem_u32(&mbar[st]))
                     : "memory");
      }
      pending[st] = 1;
    }
    if (aborted) break;
    // the last commit covers every MMA of this tile
    const int last = (nchunks - 1) & 1;
    int gave_up = 0;
    if (mbar_wait(smem_u32(&mbar[last]), phase[last], spin_limit)) {
      phase[last] ^= 1;
      pending[last] = 0;
    } else {
      gave_up = 1;
    }
    if (__syncthreads_or(gave_up)) {
      aborted = true;
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    // warp w reads TMEM lanes 32w..32w+31 = rows of X; warps 0-1 hold leaf 0
    // (columns 0-63), warps 2-3 leaf 1 (columns 64-127)
    const int h = warp >> 1, mi = (warp & 1) * 32 + lane;
    const uint32_t lane_addr = taddr + (uint32_t(warp * 32) << 16) + uint32_t(h * 64);
    int32_t* out = (mi < lm[h]) ? gram + (ls[h] + mi) * int64_t(kMaxLeaf) : nullptr;
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      uint32_t r[16];
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(lane_addr + q * 16)
          : "memory");
      asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
      if (out) {
#pragma unroll
        for (int j = 0; j < 16; ++j)
          if (q * 16 + j < lm[h]) out[q * 16 + j] = __float2int_rn(__uint_as_float(r[j]));
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();  // D is read before the next tile's first MMA overwrites it
  }
  // drain: wait for any commit still outstanding (thread 0 issued them and
  // knows which), always with the full limit, so tensor memory is never freed
  // under an MMA in flight; then free it
  if (aborted && tid == 0) atomicOr(err, kErrTimeout);
  if (tid == 0)
    for (int st = 0; st < 2; ++st)
      if (pending[st]) mbar_wait(smem_u32(&mbar[st]), phase[st], kSpinLimit);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  if (warp == 0)
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(kTmemCols) : "memory");
}

}  // namespace

cudaError_t launch_leaf_gram_tc(const int8_t* codes, int d, const int32_t* perm, const int32_t* leaf_start,
                                int64_t nleaves, int64_t total, int32_t* gram, unsigned* err, int num_sms,
                                cudaStream_t s, int wait_limit) {
  if (d % kChunk != 0) return cudaErrorInvalidValue;
  const size_t smem = 2 * size_t(kStageBytes) + 1024;
  KNNG_CUDA_TRY(ensure_smem_attr(reinterpret_cast<const void*>(leaf_gram_tc), smem));
  const int64_t pairs = (nleaves + 1) / 2;
  // two CTAs per SM at most: 2 x 128 TMEM columns of the 512, and ~65 KB shared memory each
  const int64_t blocks = std::min<int64_t>(pairs, int64_t(num_sms) * 2);
  if (blocks <= 0) return cudaSuccess;
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  // wait_limit > 0: polls per wait; 0: the default; < 0: every wait in the
  // main loop gives up at once (the drain keeps the full limit)
  const long long spins = wait_limit > 0 ? (long long)wait_limit : wait_limit < 0 ? 0ll : kSpinLimit;
  leaf_gram_tc<<<unsigned(blocks), kTcThreads, smem, s>>>(codes, d, perm, leaf_start, nleaves, total, gram, err,
                                                          spins);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
