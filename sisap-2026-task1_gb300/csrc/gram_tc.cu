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
// diagonal blocks are the two leaves' Gram blocks.  X moves through a
// software pipeline of 64-column steps (d/64 per tile, continuing across the
// CTA's tiles):
//   * cp.async copies step g + 3's int8 chunk (128 rows x 64 bytes, gathered
//     through the leaf permutation) into a 4-slot ring, so the loads of three
//     steps are in flight while step g is converted and multiplied;
//   * 256 threads widen step g's int8 chunk to bf16 (exact: |q| <= 128)
//     in shared memory, into the K-major core-matrix layout the MMA reads
//     (8 rows x 16 bytes per core matrix, no swizzle; LBO = 128 B between
//     core matrices along K, SBO = 1024 B between 8-row groups), in one of two
//     bf16 stages (TMA cannot convert);
//   * one thread issues the step's 4 MMAs (K = 16 each) and commits them to
//     the stage's mbarrier; a stage is rewritten only after its barrier flips.
// At a tile's last step D (128 TMEM columns) is read with tcgen05.ld: warps w
// and w + 4 share lane quadrant w % 4 and read half of its leaf's 64 columns
// each.  Three CTAs per SM (65 KB of shared memory, 128 TMEM columns each).
// Every mbarrier wait is bounded (the limit is a launch argument).  Giving up
// is decided by __syncthreads_or over every thread's wait outcome, so the
// whole block leaves together; the kernel then records kErrTimeout, waits for
// its copies, lets thread 0 wait with the full limit for every MMA it
// committed, and frees its tensor memory before returning.
#include "knng_internal.cuh"

#include <algorithm>

namespace knng {
namespace {

constexpr int kTcThreads = 256;
constexpr int kCtasPerSm = 3;
constexpr int kChunk = 64;                      // d columns per pipeline step
constexpr int kRing = 4;                        // int8 ring slots: copies issued 3 steps ahead
constexpr int kAhead = kRing - 1;
constexpr int kRowBufs = 4;                     // tiles whose row ids are resident
constexpr int kI8Bytes = 128 * kChunk;          // 8 KB: a step's 128 rows of int8
constexpr int kStageBytes = 128 * kChunk * 2;   // 16 KB: the same rows widened to bf16
constexpr int kSbo = (kChunk / 8) * 128;        // 1024 B between 8-row groups of a stage
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

// Two int8 values widened to a bf16 pair (lo in the low half): exact, every
// integer in [-128, 127] has at most 8 significant bits.
__device__ __forceinline__ uint32_t bf16x2(int lo, int hi) {
  uint32_t r;
  asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(r) : "f"(float(hi)), "f"(float(lo)));
  return r;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

__global__ void __launch_bounds__(kTcThreads, kCtasPerSm) leaf_gram_tc(const int8_t* __restrict__ codes, int d,
                                                                      const int32_t* __restrict__ perm,
                                                                      const int32_t* __restrict__ leaf_start,
                                                                      int64_t nleaves, int64_t total,
                                                                      int32_t* __restrict__ gram, unsigned* err,
                                                                      long long spin_limit) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ __align__(8) uint64_t mbar[2];
  __shared__ uint32_t tmem_base;
  __shared__ int32_t row_id[kRowBufs][128];            // id of X's row r in a tile, -1 past a leaf's end
  __shared__ int32_t tile_ls[kRowBufs][2], tile_lm[kRowBufs][2];  // start and size of the tile's two leaves
  unsigned char* stage[2] = {smem, smem + kStageBytes};
  unsigned char* ring = smem + 2 * kStageBytes;
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
  const int nchunks = d / kChunk;
  const int64_t npairs = (nleaves + 1) / 2;
  const int64_t ntiles = int64_t(blockIdx.x) < npairs ? (npairs - 1 - int64_t(blockIdx.x)) / gridDim.x + 1 : 0;
  const int64_t nsteps = ntiles * nchunks;

  // tile q of this CTA is the leaf pair blockIdx.x + q * gridDim.x; its row
  // ids and leaf extents go to row buffer q % kRowBufs
  auto fill_rows = [&](int64_t q) {
    if (q >= ntiles || tid >= 128) return;
    const int64_t pr = int64_t(blockIdx.x) + q * gridDim.x;
    const int b = int(q % kRowBufs), h = tid >> 6, m = tid & 63;
    const int64_t l = 2 * pr + h;
    int64_t s0 = 0, len = 0;
    if (l < nleaves) {
      s0 = leaf_start[l];
      len = (l + 1 < nleaves ? leaf_start[l + 1] : total) - s0;
    }
    row_id[b][tid] = m < len ? perm[s0 + m] : -1;
    if (m == 0) {
      tile_ls[b][h] = int32_t(s0);
      tile_lm[b][h] = int32_t(len);
    }
  };
  // step g's copies (int8 chunk c of tile q) into ring slot g % kRing: one
  // commit group per step, empty past the last step
  auto issue = [&](int64_t g) {
    if (g < nsteps) {
      const int64_t q = g / nchunks;
      const int c = int(g - q * nchunks);
      const int b = int(q % kRowBufs);
      unsigned char* dst = ring + (g % kRing) * kI8Bytes;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int idx = tid + kTcThreads * u;  // 512 pieces of 16 bytes: row idx / 4, piece idx % 4
        const int r = idx >> 2, pc = idx & 3;
        const int32_t id = row_id[b][r];
        if (id >= 0) cp_async16(dst + r * kChunk + pc * 16, codes + int64_t(id) * d + c * kChunk + pc * 16);
      }
    }
    cp_async_commit();
  };

  for (int q = 0; q < kRowBufs; ++q) fill_rows(q);
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = tmem_base;
  const uint32_t idesc = instr_desc(128, 128);
  uint32_t phase[2] = {0, 0};
  int pending[2] = {0, 0};  // commits issued on a stage and not yet waited for (thread 0's view counts)
  bool aborted = false;     // block-uniform: set only from __syncthreads_or
  for (int g = 0; g < kAhead; ++g) issue(g);

  for (int64_t g = 0; g < nsteps; ++g) {
    const int64_t q = g / nchunks;
    const int c = int(g - q * nchunks);
    const int st = int(g & 1);
    const int b = int(q % kRowBufs);
    // the buffer of tile q - 1, whose epilogue ended at the last barrier; its
    // new tile's first copies are issued at least 3 steps from now
    if (c == 0 && q >= 1) fill_rows(q + kRowBufs - 1);
    issue(g + kAhead);  // into the slot of step g - 1, converted before the last barrier
    cp_async_wait<kAhead>();  // this thread's copies of step g have landed
    int gave_up = 0;
    if (pending[st]) {  // the MMAs of step g - 2 read this stage
      if (mbar_wait(smem_u32(&mbar[st]), phase[st], spin_limit)) {
        phase[st] ^= 1;
        pending[st] = 0;
      } else {
        gave_up = 1;  // pending stays set: the drain waits for that commit
      }
    }
    if (__syncthreads_or(gave_up)) {  // also publishes every thread's copies of step g
      aborted = true;
      break;
    }
    {  // thread t widens 32 codes of X's row t / 2 into the core-matrix layout
      const int r = tid >> 1, half = tid & 1;
      const bool live = row_id[b][r] >= 0;
      const unsigned char* src = ring + (g % kRing) * kI8Bytes + r * kChunk + half * 32;
      unsigned char* dst = stage[st] + (r >> 3) * kSbo + (r & 7) * 16 + half * 4 * 128;
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const uint4 v = live ? *reinterpret_cast<const uint4*>(src + 16 * p) : make_uint4(0, 0, 0, 0);
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const uint32_t a = w[2 * e], bb = w[2 * e + 1];
          uint4 o;
          o.x = bf16x2(int(int8_t(a)), int(int8_t(a >> 8)));
          o.y = bf16x2(int(int8_t(a >> 16)), int(int8_t(a >> 24)));
          o.z = bf16x2(int(int8_t(bb)), int(int8_t(bb >> 8)));
          o.w = bf16x2(int(int8_t(bb >> 16)), int(int8_t(bb >> 24)));
          *reinterpret_cast<uint4*>(dst + (2 * p + e) * 128) = o;
        }
      }
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const uint32_t sa = smem_u32(stage[st]);
#pragma unroll
      for (int kk = 0; kk < kChunk / 16; ++kk) {
        const uint64_t desc = smem_desc(sa + kk * 256, 128, kSbo);
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
    if (c == nchunks - 1) {  // the tile's last step: its commit covers every MMA of the tile
      gave_up = 0;
      if (mbar_wait(smem_u32(&mbar[st]), phase[st], spin_limit)) {
        phase[st] ^= 1;
        pending[st] = 0;
      } else {
        gave_up = 1;
      }
      if (__syncthreads_or(gave_up)) {
        aborted = true;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      // warp w reads TMEM lanes 32 (w % 4) .. + 31 = rows of X: leaf h = (w % 4) / 2,
      // member (w % 2) * 32 + lane; warps w < 4 take the leaf's first 32 columns
      const int quad = warp & 3, h = quad >> 1, mi = (quad & 1) * 32 + lane, j0 = 32 * (warp >> 2);
      const int lm = tile_lm[b][h];
      int32_t* out = mi < lm ? gram + (int64_t(tile_ls[b][h]) + mi) * int64_t(kMaxLeaf) : nullptr;
      const uint32_t lane_addr = taddr + (uint32_t(quad * 32) << 16) + uint32_t(64 * h + j0);
#pragma unroll
      for (int hq = 0; hq < 2; ++hq) {
        uint32_t rr[16];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
            : "=r"(rr[0]), "=r"(rr[1]), "=r"(rr[2]), "=r"(rr[3]), "=r"(rr[4]), "=r"(rr[5]), "=r"(rr[6]),
              "=r"(rr[7]), "=r"(rr[8]), "=r"(rr[9]), "=r"(rr[10]), "=r"(rr[11]), "=r"(rr[12]), "=r"(rr[13]),
              "=r"(rr[14]), "=r"(rr[15])
            : "r"(lane_addr + hq * 16)
            : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if (out) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int jj = j0 + 16 * hq + j;
            if (jj < lm) out[jj] = __float2int_rn(__uint_as_float(rr[j]));
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();  // D is read before the next tile's first MMA overwrites it
    }
  }
  // drain: no copy may land after the exit, every committed MMA must be done
  // before the tensor memory is freed (thread 0 issued them and knows which;
  // always the full limit), then free it
  cp_async_wait<0>();
  if (aborted && tid == 0) atomicOr(err, kErrTimeout);
  if (tid == 0)
    for (int s2 = 0; s2 < 2; ++s2)
      if (pending[s2]) mbar_wait(smem_u32(&mbar[s2]), phase[s2], kSpinLimit);
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
  const size_t smem = 2 * size_t(kStageBytes) + size_t(kRing) * kI8Bytes + 1024;  // + alignment slack
  KNNG_CUDA_TRY(ensure_smem_attr(reinterpret_cast<const void*>(leaf_gram_tc), smem));
  const int64_t pairs = (nleaves + 1) / 2;
  // three CTAs per SM: 3 x 128 TMEM columns of the 512, ~67 KB of shared memory each
  const int64_t blocks = std::min<int64_t>(pairs, int64_t(num_sms) * kCtasPerSm);
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
