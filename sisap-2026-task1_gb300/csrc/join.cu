// join.cu -- K5: one NN-Descent iteration, one CTA (8 warps) per row at a time.
//
// Reference: src/main.cpp:324-430.  For row i:
//   candidates c_j = G[G[i][k]][k2], j = k*K + k2, minus i;
//   h_j = 1024 - sum_w popcount(b_i[w] ^ b_c[w]);
//   the R = K*rerank_mult best by h are visited in order, skipped when the id
//   is in the row's current pool, otherwise scored by exact int8 dot and
//   shift-inserted when dot > pool[K-1].score (existing entries keep ties);
//   positions whose id changed are written back and counted.
// The reference picks the R best with std::nth_element (ties unspecified) and
// visits them in the order it leaves.  Here the R best are taken by
// (h desc, j asc) and visited in that order, which the oracle's TIE_STABLE
// mode reproduces; every other step is the reference's sequential semantics.
//
// Only visits that can change the pool need work: a candidate whose id sits
// in the starting pool with a real score is either still there (skipped) or
// was evicted with a score <= the rising threshold (rejected), and a
// candidate whose dot is <= the starting pool[K-1].score is always rejected.
// So the kernel computes dots for the selected candidates not in the starting
// pool, keeps those above the starting threshold ("promising"), sorts them by
// (h desc, j asc) and replays the reference's insertion loop over them in one
// warp, with the pool held two entries per lane.
//
// Stages per row (shared memory, K = 50, R = 400, d = 1024: ~27 KB):
//   A  own list, sketch, code row; clear the h histogram
//   B  gather the K*K two-hop ids (K rows of K ids, contiguous per row)
//   C  Hamming: 8 lanes per candidate, one 16-byte sketch chunk per lane
//      (128-byte rows = one coalesced line per candidate), warp __popc
//   D  threshold h_t from the histogram (warp scan over 1025 bins)
//   E  selection: all h > h_t plus the first R - count(h > h_t) with h == h_t
//      in j order (one block scan of per-thread tie counts)
//   F  drop ids in the starting pool; dp4a dots, 8 lanes per candidate
//   G  rank-sort the promising candidates by (h desc, j asc)
//   H  sequential insertion + write-back + update count (warp 0)
// HBM-bound: per row K*4*K (ids) + K*K*d/8 (sketches) + <= R*d (code rows).
#include "knng_internal.cuh"

#include <algorithm>

namespace knng {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kGroups = kThreads / 8;  // 8-lane groups per CTA
constexpr int kHBins = 1025;

struct JoinSmem {
  int K, R, KK, d, W;
  size_t bytes;
  size_t o_cand_id, o_cand_h, o_hist, o_sel, o_need, o_pkey, o_pid, o_pdot, o_order, o_pool_id, o_pool_sc,
      o_code, o_sk;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline JoinSmem join_smem(int K, int R, int d) {
  JoinSmem s;
  s.K = K;
  s.R = R;
  s.KK = K * K;
  s.d = d;
  s.W = d / 64;
  size_t o = 0;
  s.o_code = o;    o = align16(o + size_t(d));
  s.o_sk = o;      o = align16(o + size_t(s.W) * 8);
  s.o_cand_id = o; o = align16(o + size_t(s.KK) * 4);
  s.o_cand_h = o;  o = align16(o + size_t(s.KK) * 2);
  s.o_hist = o;    o = align16(o + size_t(kHBins) * 4);
  s.o_sel = o;     o = align16(o + size_t(R) * 2);
  s.o_need = o;    o = align16(o + size_t(R) * 2);
  s.o_pkey = o;    o = align16(o + size_t(R) * 4);
  s.o_pid = o;     o = align16(o + size_t(R) * 4);
  s.o_pdot = o;    o = align16(o + size_t(R) * 4);
  s.o_order = o;   o = align16(o + size_t(R) * 2);
  s.o_pool_id = o; o = align16(o + size_t(K) * 4);
  s.o_pool_sc = o; o = align16(o + size_t(K) * 4);
  s.bytes = o;
  return s;
}

__device__ __forceinline__ int popc_u4(uint4 a, uint4 b) {
  return __popc(a.x ^ b.x) + __popc(a.y ^ b.y) + __popc(a.z ^ b.z) + __popc(a.w ^ b.w);
}

__device__ __forceinline__ int dot_u4(uint4 a, uint4 b, int acc) {
  acc = __dp4a(int(a.x), int(b.x), acc);
  acc = __dp4a(int(a.y), int(b.y), acc);
  acc = __dp4a(int(a.z), int(b.z), acc);
  return __dp4a(int(a.w), int(b.w), acc);
}

__global__ void __launch_bounds__(kThreads, 4) join_kernel(
    const int8_t* __restrict__ codes, const uint64_t* __restrict__ sketch, int64_t n, int d, int K, int R,
    const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out, int32_t* scores_out,
    const int32_t* __restrict__ row_order, unsigned long long* __restrict__ counters) {
  extern __shared__ __align__(16) unsigned char smem[];
  const JoinSmem L = join_smem(K, R, d);
  uint4* my_code = reinterpret_cast<uint4*>(smem + L.o_code);
  uint4* my_sk = reinterpret_cast<uint4*>(smem + L.o_sk);
  int32_t* cand_id = reinterpret_cast<int32_t*>(smem + L.o_cand_id);
  uint16_t* cand_h = reinterpret_cast<uint16_t*>(smem + L.o_cand_h);
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem + L.o_hist);
  uint16_t* sel = reinterpret_cast<uint16_t*>(smem + L.o_sel);
  uint16_t* need = reinterpret_cast<uint16_t*>(smem + L.o_need);
  uint32_t* pkey = reinterpret_cast<uint32_t*>(smem + L.o_pkey);
  int32_t* pid = reinterpret_cast<int32_t*>(smem + L.o_pid);
  int32_t* pdot = reinterpret_cast<int32_t*>(smem + L.o_pdot);
  uint16_t* order = reinterpret_cast<uint16_t*>(smem + L.o_order);
  int32_t* pool_id = reinterpret_cast<int32_t*>(smem + L.o_pool_id);
  int32_t* pool_sc = reinterpret_cast<int32_t*>(smem + L.o_pool_sc);
  __shared__ int s_cnt, s_ht, s_gt, s_nsel, s_nneed, s_nprom;
  __shared__ int32_t s_wsum[kWarps];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, sub = lane & 7;
  const int KK = L.KK, W = L.W, nchunk = d / 16, sk_chunks = W / 2;
  const bool inplace = ids_out == ids_in;
  unsigned long long my_updates = 0, my_cands = 0, my_dots = 0;

  for (int64_t r = blockIdx.x; r < n; r += gridDim.x) {
    const int64_t i = row_order ? int64_t(row_order[r]) : r;
    // ---- A
    for (int k = tid; k < K; k += kThreads) {
      pool_id[k] = ids_in[i * K + k];
      pool_sc[k] = scores_in[i * K + k];
    }
    for (int c = tid; c < nchunk; c += kThreads) my_code[c] = reinterpret_cast<const uint4*>(codes + i * d)[c];
    for (int c = tid; c < sk_chunks; c += kThreads) my_sk[c] = reinterpret_cast<const uint4*>(sketch + i * W)[c];
    for (int h = tid; h < kHBins; h += kThreads) hist[h] = 0;
    if (tid == 0) {
      s_cnt = 0;
      s_nsel = 0;
      s_nneed = 0;
      s_nprom = 0;
    }
    __syncthreads();
    // ---- B
    for (int j = tid; j < KK; j += kThreads) {
      const int k = j / K, k2 = j - k * K;
      const int32_t n1 = pool_id[k];
      const int32_t n2 = (n1 >= 0 && n1 < n) ? ids_in[int64_t(n1) * K + k2] : -1;
      cand_id[j] = (n2 == i || n2 < 0 || n2 >= n) ? -1 : n2;
    }
    __syncthreads();
    // ---- C  (groups of 8 lanes; 4 candidates in flight per group)
    {
      const uint4 mine = sub < sk_chunks ? my_sk[sub] : make_uint4(0, 0, 0, 0);
      int local_cnt = 0;
      const int slot = lane >> 3;
      // the loop bound is warp-uniform so every lane reaches the shuffles
      for (int wbase = warp * 4; wbase < KK; wbase += 4 * kGroups) {
        const int base = wbase + slot;
        uint4 v[4];
        int cj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int j = base + u * kGroups;
          cj[u] = j < KK ? cand_id[j] : -1;
          v[u] = make_uint4(0, 0, 0, 0);
          if (cj[u] >= 0 && sub < sk_chunks)
            v[u] = __ldg(reinterpret_cast<const uint4*>(sketch + int64_t(cj[u]) * W) + sub);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          int pc = (cj[u] >= 0 && sub < sk_chunks) ? popc_u4(v[u], mine) : 0;
          pc += __shfl_xor_sync(0xffffffffu, pc, 1);
          pc += __shfl_xor_sync(0xffffffffu, pc, 2);
          pc += __shfl_xor_sync(0xffffffffu, pc, 4);
          const int j = base + u * kGroups;
          if (sub == 0 && j < KK) {
            if (cj[u] >= 0) {
              const int h = 1024 - pc;
              cand_h[j] = uint16_t(h);
              atomicAdd(&hist[h], 1u);
              ++local_cnt;
            } else {
              cand_h[j] = 0xffff;
            }
          }
        }
      }
      if (local_cnt) atomicAdd(&s_cnt, local_cnt);
    }
    __syncthreads();
    // ---- D
    const int cnt = s_cnt;
    my_cands += unsigned(cnt);
    if (cnt > R) {
      if (warp == 0) {
        const int per = (kHBins + 31) / 32;
        const int lo = lane * per, hi = min(kHBins, lo + per);
        int sum = 0;
        for (int x = lo; x < hi; ++x) sum += int(hist[1024 - x]);
        int incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        const int excl = incl - sum;
        if (excl < R && R <= incl) {
          int run = excl;
          for (int x = lo; x < hi; ++x) {
            const int c = int(hist[1024 - x]);
            if (run + c >= R) {
              s_ht = 1024 - x;
              s_gt = run;
              break;
            }
            run += c;
          }
        }
      }
    } else if (tid == 0) {
      s_ht = -1;  // everything valid is selected
      s_gt = cnt;
    }
    __syncthreads();
    // ---- E  (thread-contiguous segments keep the j order for the tie ranks)
    {
      const int ht = s_ht, need_eq = R - s_gt;
      const int seg = (KK + kThreads - 1) / kThreads;
      const int j0 = tid * seg, j1 = min(KK, j0 + seg);
      int eq = 0;
      if (ht >= 0)
        for (int j = j0; j < j1; ++j) eq += (cand_h[j] == ht) ? 1 : 0;
      int incl = eq;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      int rank = incl - eq;
      for (int w = 0; w < warp; ++w) rank += s_wsum[w];
      for (int j = j0; j < j1; ++j) {
        const int h = cand_h[j];
        if (h == 0xffff) continue;
        bool take;
        if (ht < 0) {
          take = true;
        } else if (h > ht) {
          take = true;
        } else if (h == ht) {
          take = rank < need_eq;
          ++rank;
        } else {
          take = false;
        }
        if (take) sel[atomicAdd(&s_nsel, 1)] = uint16_t(j);
      }
    }
    __syncthreads();
    // ---- F1  drop ids present in the starting pool with a real score
    const int nsel = s_nsel;
    for (int s = tid; s < nsel; s += kThreads) {
      const int j = sel[s];
      const int32_t id = cand_id[j];
      bool skip = false;
      for (int k = 0; k < K; ++k)
        if (pool_id[k] == id && pool_sc[k] != kScoreMinI) skip = true;
      if (!skip) need[atomicAdd(&s_nneed, 1)] = uint16_t(j);
    }
    __syncthreads();
    // ---- F2  dots (8 lanes per candidate; a lane keeps up to eight 16-byte
    //           loads of the candidate row in flight; own row from shared memory)
    {
      const int nneed = s_nneed;
      my_dots += unsigned(nneed);
      const int32_t thr0 = pool_sc[K - 1];
      const int per_lane = d / 128;
      for (int wbase = warp * 4; wbase < nneed; wbase += kGroups) {
        const int q = wbase + (lane >> 3);
        const int j = q < nneed ? int(need[q]) : -1;
        int acc = 0;
        if (j >= 0) {
          const uint4* row = reinterpret_cast<const uint4*>(codes + int64_t(cand_id[j]) * d);
          uint4 v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (u < per_lane) v[u] = __ldg(row + sub + 8 * u);
#pragma unroll
          for (int u = 0; u < 8; ++u)
            if (u < per_lane) acc = dot_u4(v[u], my_code[sub + 8 * u], acc);
        }
        acc += __shfl_xor_sync(0xffffffffu, acc, 1);
        acc += __shfl_xor_sync(0xffffffffu, acc, 2);
        acc += __shfl_xor_sync(0xffffffffu, acc, 4);
        if (sub == 0 && j >= 0 && acc > thr0) {
          const int slot = atomicAdd(&s_nprom, 1);
          pkey[slot] = (uint32_t(cand_h[j]) << 12) | uint32_t(4095 - j);
          pid[slot] = cand_id[j];
          pdot[slot] = acc;
        }
      }
    }
    __syncthreads();
    // ---- G  rank sort (keys are distinct)
    const int P = s_nprom;
    for (int p = tid; p < P; p += kThreads) {
      const uint32_t kp = pkey[p];
      int rank = 0;
      for (int q = 0; q < P; ++q) rank += pkey[q] > kp ? 1 : 0;
      order[rank] = uint16_t(p);
    }
    __syncthreads();
    // ---- H  sequential insertion in warp 0, then write-back
    if (warp == 0) {
      int32_t idA = lane < K ? pool_id[lane] : -1, scA = lane < K ? pool_sc[lane] : kScoreMinI;
      int32_t idB = 32 + lane < K ? pool_id[32 + lane] : -1, scB = 32 + lane < K ? pool_sc[32 + lane] : kScoreMinI;
      const unsigned full = 0xffffffffu;
      for (int rr = 0; rr < P; ++rr) {
        const int p = order[rr];
        const int32_t id = pid[p], dot = pdot[p];
        if (__any_sync(full, idA == id || idB == id)) continue;
        const int32_t last = (K - 1) < 32 ? __shfl_sync(full, scA, K - 1) : __shfl_sync(full, scB, K - 33);
        if (!(dot > last)) continue;
        const int pos = __popc(__ballot_sync(full, lane < K - 1 && scA >= dot)) +
                        __popc(__ballot_sync(full, 32 + lane < K - 1 && scB >= dot));
        const int32_t upIdA = __shfl_up_sync(full, idA, 1), upScA = __shfl_up_sync(full, scA, 1);
        const int32_t upIdB = __shfl_up_sync(full, idB, 1), upScB = __shfl_up_sync(full, scB, 1);
        const int32_t id31 = __shfl_sync(full, idA, 31), sc31 = __shfl_sync(full, scA, 31);
        if (lane < K) {
          if (lane > pos) { idA = upIdA; scA = upScA; }
          else if (lane == pos) { idA = id; scA = dot; }
        }
        const int qb = 32 + lane;
        if (qb < K) {
          if (qb > pos) {
            idB = lane == 0 ? id31 : upIdB;
            scB = lane == 0 ? sc31 : upScB;
          } else if (qb == pos) {
            idB = id;
            scB = dot;
          }
        }
      }
      int changed = 0;
      if (lane < K) {
        const bool ch = idA != pool_id[lane];
        changed += ch;
        if (ch || !inplace) {
          ids_out[i * K + lane] = idA;
          scores_out[i * K + lane] = scA;
        }
      }
      if (32 + lane < K) {
        const bool ch = idB != pool_id[32 + lane];
        changed += ch;
        if (ch || !inplace) {
          ids_out[i * K + 32 + lane] = idB;
          scores_out[i * K + 32 + lane] = scB;
        }
      }
      for (int o = 16; o > 0; o >>= 1) changed += __shfl_xor_sync(full, changed, o);
      my_updates += unsigned(changed);
    }
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd(counters + 0, my_updates);
    atomicAdd(counters + 1, my_cands);
    atomicAdd(counters + 2, my_dots);
  }
}

}  // namespace

size_t join_smem_bytes(int K, int R, int d) { return join_smem(K, R, d).bytes; }

cudaError_t launch_join(const int8_t* codes, const uint64_t* sketch, int64_t n, int d, int K, int R,
                        const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out, int32_t* scores_out,
                        const int32_t* row_order, unsigned long long* counters, int num_sms, cudaStream_t s) {
  const size_t smem = join_smem(K, R, d).bytes;
  KNNG_CUDA_TRY(cudaFuncSetAttribute(join_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  int per_sm = 0;
  KNNG_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, join_kernel, kThreads, smem));
  if (per_sm < 1) per_sm = 1;
  const int64_t blocks = std::min<int64_t>(n, int64_t(num_sms) * per_sm);
  join_kernel<<<unsigned(blocks), kThreads, smem, s>>>(codes, sketch, n, d, K, R, ids_in, scores_in, ids_out,
                                                       scores_out, row_order, counters);
  note_launch();
  return cudaGetLastError();
}

}  // namespace knng
