// gram_tc.cu -- K3 on the 5th-generation tensor cores: leaf Gram blocks with
// tcgen05.mma (f16 operands, fp32 accumulation in tensor memory).
//
// Reference: the dots of src/main.cpp:261-269 (every pair of members of a
// leaf).  ptxas rejects tcgen05.mma.kind::i8 for sm_103a, so the int8 codes are
// widened to f16 (exact: every integer in [-128, 127] is an f16) and
// multiplied with kind::f16 into fp32 accumulators.  Every partial sum is an integer of
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
//   * 256 threads widen step g's int8 chunk to f16 in shared memory (two
//     integer ops and one packed half add per four codes), into the K-major
//     core-matrix layout the MMA reads (8 rows x 16 bytes per core matrix, no
//     swizzle; LBO = 128 B between core matrices along K, SBO = 1024 B between
//     8-row groups), in one of two f16 stages (TMA cannot convert);
//   * one thread issues the step's 4 MMAs (K = 16 each) and commits them to
//     the stage's mbarrier; a stage is rewritten only after its barrier flips.
// At a tile's last step D (128 TMEM columns) is read with tcgen05.ld: warps w
// and w + 4 share lane quadrant w % 4 and read half of its leaf's 64 columns
// each.  Three CTAs per SM (65 KB of shared memory, 128 TMEM columns each).
// Each thread waits for the next step's copies before the step's single
// barrier, so one barrier per step publishes both the f16 stage the MMAs
// read and the int8 chunk the next step widens.
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
constexpr int kRowBufs = 8;                     // tiles whose row ids are resident (refilled 7 tiles ahead)
constexpr int kI8Bytes = 128 * kChunk;          // 8 KB: a step's 128 rows of int8
constexpr int kStageBytes = 128 * kChunk * 2;   // 16 KB: the same rows widened to f16
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

// Instruction descriptor, kind::f16: D f32, A and B f16 (type 0), both K-major, N, M.
__host__ __device__ constexpr uint32_t instr_desc(int M, int N) {
  return (1u << 4) | (uint32_t(N >> 3) << 17) | (uint32_t(M >> 4) << 24);
}

// Four int8 codes (one 32-bit word) widened to two f16 pairs, exactly and in
// integer/packed-half steps: u = code + 128 (xor 0x80 per byte) becomes the f16
// 1024 + u by placing 0x64 above each byte (0x6400 is 1024.0, whose unit in the
// last place is 1), and one packed add of -1152 leaves code = u - 128.
__device__ __forceinline__ void widen4(uint32_t w, uint32_t& lo, uint32_t& hi) {
  const uint32_t u = w ^ 0x80808080u;
  const uint32_t a = __byte_perm(u, 0x64646464u, 0x4140);  // codes 0, 1
  const uint32_t b = __byte_perm(u, 0x64646464u, 0x4342);  // codes 2, 3
  asm("add.f16x2 %0, %1, %2;" : "=r"(lo) : "r"(a), "r"(0xE480E480u));
  asm("add.f16x2 %0, %1, %2;" : "=r"(hi) : "r"(b), "r"(0xE480E480u));
}

// Byte offset of 16-byte piece pc (0..3) of row r in a ring slot: rows are
// 64 bytes apart and the pieces of a row are permuted by (r / 2) % 4, so 8
// consecutive rows' pieces of one index fall in 8 distinct bank groups.
__device__ __forceinline__ int ring_offset(int r, int pc) { return r * kChunk + ((pc ^ ((r >> 1) & 3)) << 4); }

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(void* dst, const void* src) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem_u32(dst)), "l"(src) : "memory");
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
                                                                      int32_t* __restrict__ gram, int64_t gram_pos0,
                                                                      unsigned* err, long long spin_limit,
                                                                      int64_t n_rows) {
  (void)n_rows;
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
  const int ntiles = int64_t(blockIdx.x) < npairs ? int((npairs - 1 - int64_t(blockIdx.x)) / gridDim.x) + 1 : 0;

  // tile q of this CTA is the leaf pair blockIdx.x + q * gridDim.x; its row
  // ids and leaf extents go to row buffer q % kRowBufs.  Thread t < 128
  // handles X's row t: leaf h = t / 64, member m = t % 64.
  auto leaf_extent = [&](int q, int64_t& s0, int64_t& len) {
    s0 = 0;
    len = 0;
    if (q >= ntiles || tid >= 128) return;
    const int64_t l = 2 * (int64_t(blockIdx.x) + int64_t(q) * gridDim.x) + (tid >> 6);
    if (l < nleaves) {
      s0 = leaf_start[l];
      len = (l + 1 < nleaves ? leaf_start[l + 1] : total) - s0;
    }
  };
  // the row id arrives by cp.async (in the caller's next commit group) or,
  // for the initial tiles, by a plain load
  auto fill_rows = [&](int q, int64_t s0, int64_t len, bool async) {
    if (q >= ntiles || tid >= 128) return;
    const int b = q & (kRowBufs - 1), h = tid >> 6, m = tid & 63;
    if (m < len) {
      if (async) cp_async4(&row_id[b][tid], perm + s0 + m);
      else row_id[b][tid] = perm[s0 + m];
    } else {
      row_id[b][tid] = -1;
    }
    if (m == 0) {
      tile_ls[b][h] = int32_t(s0);
      tile_lm[b][h] = int32_t(len);
    }
  };
  // The copy stream runs kAhead steps ahead of the compute: (iq, ic) is the
  // tile and chunk of the next step to copy, islot its ring slot.  One commit
  // group per step, empty past the last tile.
  int iq = 0, ic = 0, islot = 0;
  auto issue_next = [&]() {
    if (iq < ntiles) {
      const int b = iq & (kRowBufs - 1);
      unsigned char* dst = ring + islot * kI8Bytes;
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        const int idx = tid + kTcThreads * u;  // 512 pieces of 16 bytes: row idx / 4, piece idx % 4
        const int r = idx >> 2, pc = idx & 3;
        const int32_t id = row_id[b][r];
        // (bounds-checked build) -1 marks a row past its leaf's end; any other
        // id must be a row of `codes`
        if (id >= 0 && KNNG_GUARD(err, id < n_rows))
          cp_async16(dst + ring_offset(r, pc), codes + int64_t(id) * d + ic * kChunk + pc * 16);
        else
          KNNG_FLAG_IF(err, id < -1);
      }
      if (++ic == nchunks) {
        ic = 0;
        ++iq;
      }
    }
    cp_async_commit();
    islot = (islot + 1) & (kRing - 1);
  };

  for (int q = 0; q < kRowBufs; ++q) {
    int64_t s0, len;
    leaf_extent(q, s0, len);
    fill_rows(q, s0, len, false);
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const uint32_t taddr = tmem_base;
  const uint32_t idesc = instr_desc(128, 128);
  uint32_t phase[2] = {0, 0};
  int pending[2] = {0, 0};  // commits issued on a stage and not yet waited for (thread 0's view counts)
  bool aborted = false;     // block-uniform: set only from __syncthreads_or
  for (int g = 0; g < kAhead; ++g) issue_next();
  cp_async_wait<kAhead - 1>();  // the first step's copies
  __syncthreads();

  // Invariant at the top of a step: its int8 chunk is in ring slot `slot`,
  // visible to every thread.  One barrier per step: each thread waits for
  // the next step's copies before it, so the barrier publishes both this
  // step's f16 stage and the next step's int8 chunk.
  int q = 0, c = 0, st = 0, slot = 0;
  int64_t f_s0 = 0, f_len = 0;  // extent of the tile being refilled, loaded one step ahead
  while (q < ntiles) {
    const int b = q & (kRowBufs - 1);
    // Tile q + 7 reuses the buffer of tile q - 1, whose epilogue ended at a
    // barrier: its leaf extent is loaded at the tile's first step (used a
    // step later, so the load does not stall the barrier) and its row ids
    // are copied at the second step, in that step's commit group, which is
    // waited for a dozen steps before the first copy that reads them.
    if (q >= 1 && c == 0) leaf_extent(q + kRowBufs - 1, f_s0, f_len);
    if (q >= 1 && c == 1) fill_rows(q + kRowBufs - 1, f_s0, f_len, true);
    int gave_up = 0;
    if (pending[st]) {  // the MMAs of two steps ago read this stage
      if (mbar_wait(smem_u32(&mbar[st]), phase[st], spin_limit)) {
        phase[st] ^= 1;
        pending[st] = 0;
      } else {
        gave_up = 1;  // pending stays set: the drain waits for that commit
      }
    }
    if (!gave_up) {
      // the warp widens 32 codes of each of 16 rows into the core-matrix
      // layout: lanes 8h..8h+7 take rows 0-7 (h = 0, 1) or 8-15 (h = 2, 3)
      // of the warp's 16 and the half h & 1 of the row's 64 codes, so the 8
      // lanes of every 16-byte access phase touch 8 distinct bank groups in
      // both the ring and the stage
      const int r = warp * 16 + (lane & 7) + 8 * (lane >> 4), half = (lane >> 3) & 1;
      const bool live = row_id[b][r] >= 0;
      const unsigned char* src = ring + slot * kI8Bytes;
      unsigned char* dst = stage[st] + (r >> 3) * kSbo + (r & 7) * 16 + half * 4 * 128;
#pragma unroll
      for (int p = 0; p < 2; ++p) {
        const uint4 v =
            live ? *reinterpret_cast<const uint4*>(src + ring_offset(r, 2 * half + p)) : make_uint4(0, 0, 0, 0);
        uint4 o0, o1;
        widen4(v.x, o0.x, o0.y);
        widen4(v.y, o0.z, o0.w);
        widen4(v.z, o1.x, o1.y);
        widen4(v.w, o1.z, o1.w);
        *reinterpret_cast<uint4*>(dst + (2 * p) * 128) = o0;
        *reinterpret_cast<uint4*>(dst + (2 * p + 1) * 128) = o1;
      }
    }
    issue_next();               // into the slot of the previous step, converted before the last barrier
    cp_async_wait<kAhead - 1>();  // this thread's copies of the next step have landed
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    if (__syncthreads_or(gave_up)) {
      aborted = true;
      break;
    }
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
      int32_t* out = mi < lm ? gram + (int64_t(tile_ls[b][h]) - gram_pos0 + mi) * int64_t(kMaxLeaf) : nullptr;
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
    st ^= 1;
    slot = (slot + 1) & (kRing - 1);
    if (++c == nchunks) {
      c = 0;
      ++q;
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
                                int64_t nleaves, int64_t total, int32_t* gram, int64_t gram_pos0, unsigned* err,
                                int num_sms, cudaStream_t s, int wait_limit, int64_t n_rows) {
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
  leaf_gram_tc<<<unsigned(blocks), kTcThreads, smem, s>>>(codes, d, perm, leaf_start, nleaves, total, gram, gram_pos0,
                                                          err, spins, n_rows);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
