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
// pool and keeps those above the starting threshold ("survivors"), whose
// insertion in visit order (h desc, j asc) is then resolved by rank counting.
//
// Duplicates: about half of the K*K two-hop candidates of a row repeat an id
// (1317 distinct of 2500 at 6.35M rows), so each row first inserts them into a
// shared-memory hash table (open addressing, keys = ids).  Every occurrence of
// an id has the same h, so h and the dot are computed once per distinct id.
// Among the occurrences of one id only the first in visit order can change
// the list (a later one finds the id in the list, or scores <= the threshold
// that evicted or rejected it), and when one occurrence is selected so is the
// first (ties at the cut are taken in j order), so the visit key of a
// distinct id is (h, first j).
//
// Across iterations a row's candidate set barely changes (over 80 % of the
// distinct ids recur from the third iteration on), and its pool threshold
// never falls, so with the candidate cache each row keeps its distinct ids
// with their h and a "dot <= threshold" flag for the next iteration.
//
// Sketches: W 64-bit words per row, d / 64 for the reference's coordinate-sign
// sketch or 2 for the optional 128-hyperplane sketch (hyperplane.cu); the
// score is 1024 - popcount over the W words either way.
//
// Stages per row (shared memory, K = 50, R = 400, d = 1024: ~54 KB):
//   A  own list, sketch, code row; clear table and histogram; start copying
//      the row's cache entries into shared memory (cp.async); insert the
//      starting list's ids with a real score, flagged (bit 31 of the key)
//   B  two-hop occurrences j = k*K + k2 spread over the block (thread t takes
//      j = t + 256r), insert each, record its slot per j and the first j per
//      slot (atomicMin); the first occurrence to touch a slot appends it to
//      the distinct list
//   B2 cached h / rejected flags of the distinct ids; the rest form the miss
//      list
//   C  Hamming of the misses, CB in flight per 8-lane group (the autotuned
//      candidate block): one 16-byte sketch chunk per lane (128-byte rows =
//      one line per candidate), group __popc
//   D  histogram of h over all occurrences, threshold h_t (warp scan)
//   E  selection: every occurrence with h > h_t plus the first
//      R - count(h > h_t) occurrences with h == h_t in j order; one block scan
//      of per-thread tie counts finds the cut position, then each distinct id
//      is selected from its h and first j
//   F  selected ids neither flagged as starting-list members nor known to be
//      rejected: dp4a dots, 8 lanes per candidate; keep those above the
//      starting pool[K-1].score, flag the others as rejected
//   F3 write the row's cache: this iteration's distinct ids, h and flags
//   G/H insertion by rank counting over 16-byte survivor records {visit key,
//      dot, id, flags} (or the reference's sequential loop for an unsorted or
//      unscored pool), write-back, update count
// Per row HBM/L2 bytes: K*8 (own list) + K*K*4 (two-hop ids) + d + d/8 (own
// row, sketch) + U*d/8 (U sketches scored) + r*d (r reranked rows) + 12 per
// distinct id (cache read and write).
#include "knng_internal.cuh"

#include <algorithm>
#include <map>
#include <mutex>
#include <cstdio>
#include <tuple>

namespace knng {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kGroups = kThreads / 8;  // 8-lane groups per CTA
constexpr int kHBins = 1025;
static_assert(kHBins * 4 >= kCacheCap * 2, "the histogram region stages the cached scores");
constexpr int32_t kEmpty = 0x7fffffff;     // never a valid id (num_trees * n < 2^31)
constexpr uint32_t kPoolFlag = 0x80000000u; // key bit: id is in the starting list with a real score
constexpr uint32_t kFirstMask = 0x1fffu;    // meta bits 0..12: first j (8191 = none); 16..26: Hamming score
constexpr uint32_t kKnown = 0x80000000u;    // meta bit 31: Hamming score taken from the row's candidate cache
constexpr uint32_t kRej = 0x40000000u;      // meta bit 30: dot known to be <= the row's pool threshold

struct JoinSmem {
  int K, R, KK, d, W, HT;
  size_t bytes;
  size_t o_code, o_sk, o_slot, o_key, o_meta, o_hist, o_ulist, o_surv, o_pool_id, o_pool_sc, o_miss;
};

__host__ __device__ inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline JoinSmem join_smem(int K, int R, int d) {
  JoinSmem s;
  s.K = K;
  s.R = R;
  s.KK = K * K;
  s.d = d;
  s.W = d / 64;  // room for the widest sketch (the sign sketch); a hyperplane sketch uses 2 words
  s.HT = 1024;
  while (s.HT < (3 * (s.KK + K)) / 2) s.HT <<= 1;  // load factor <= 2/3
  size_t o = 0;
  s.o_code = o;    o = align16(o + size_t(d));
  s.o_sk = o;      o = align16(o + size_t(s.W) * 8);
  s.o_slot = o;    o = align16(o + size_t(s.KK) * 2);
  s.o_key = o;     o = align16(o + size_t(s.HT) * 4);
  s.o_meta = o;    o = align16(o + size_t(s.HT) * 4);
  s.o_hist = o;    o = align16(o + size_t(kHBins) * 4);
  s.o_ulist = o;   o = align16(o + size_t(s.KK) * 2);
  const size_t u0 = o;  // stage C's miss list shares this region with stages F-H
  s.o_surv = o;    o = align16(o + size_t(R) * 16);  // survivors {visit key, dot, id, flags}
  s.o_miss = u0;  // also stages the row's cached ids (kCacheCap * 4 bytes) before stage B2
  if (o < align16(u0 + size_t(s.KK) * 2)) o = align16(u0 + size_t(s.KK) * 2);
  if (o < align16(u0 + size_t(kCacheCap) * 4)) o = align16(u0 + size_t(kCacheCap) * 4);
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

__device__ __forceinline__ uint32_t hash_slot(int32_t id, uint32_t mask) {
  return (uint32_t(id) * 2654435761u >> 7) & mask;
}

// Find or insert id (flagged keys match by their low 31 bits).  The table
// always has free slots (load <= 2/3), so the probe ends; the bound is a guard.
__device__ __forceinline__ int table_insert(int32_t* key, uint32_t mask, int32_t id, uint32_t flag) {
  uint32_t s = hash_slot(id, mask);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    int32_t k = key[s];
    if (k == kEmpty) {
      const int32_t prev = atomicCAS(&key[s], kEmpty, int32_t(uint32_t(id) | flag));
      if (prev == kEmpty) return int(s);
      k = prev;
    }
    if ((uint32_t(k) & 0x7fffffffu) == uint32_t(id)) return int(s);
    s = (s + 1) & mask;
  }
  return -1;
}

// 16-byte global -> shared copy that holds no registers (cp.async, L2 only).
__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Slot of id (flagged or not), or -1 when the table does not hold it.
__device__ __forceinline__ int table_find(const int32_t* key, uint32_t mask, int32_t id) {
  uint32_t s = hash_slot(id, mask);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    const int32_t k = key[s];
    if (k == kEmpty) return -1;
    if ((uint32_t(k) & 0x7fffffffu) == uint32_t(id)) return int(s);
    s = (s + 1) & mask;
  }
  return -1;
}

template <int CB, int MINB>
__global__ void __launch_bounds__(kThreads, MINB) join_kernel(
    const int8_t* __restrict__ codes, const uint64_t* __restrict__ sketch, int64_t n, int d, int K, int R, int W,
    const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out, int32_t* scores_out,
    const int32_t* __restrict__ row_order, unsigned long long* __restrict__ counters, JobTable jt, JoinCtl ctl) {
  extern __shared__ __align__(16) unsigned char smem[];
  if (ctl.all_done && *reinterpret_cast<volatile int*>(ctl.all_done)) return;
  const JoinSmem L = join_smem(K, R, d);
  uint4* my_code = reinterpret_cast<uint4*>(smem + L.o_code);
  uint4* my_sk = reinterpret_cast<uint4*>(smem + L.o_sk);
  int16_t* cand_slot = reinterpret_cast<int16_t*>(smem + L.o_slot);
  int32_t* key = reinterpret_cast<int32_t*>(smem + L.o_key);
  uint32_t* meta = reinterpret_cast<uint32_t*>(smem + L.o_meta);
  uint32_t* hist = reinterpret_cast<uint32_t*>(smem + L.o_hist);
  int16_t* ulist = reinterpret_cast<int16_t*>(smem + L.o_ulist);
  int16_t* need = cand_slot;  // stage F: the occurrence slots are dead after stage E
  int16_t* misslist = reinterpret_cast<int16_t*>(smem + L.o_miss);  // shares its region with need..order
  const int32_t* stage_id = reinterpret_cast<const int32_t*>(smem + L.o_miss);  // stage A..B2, same region
  const uint16_t* stage_hr = reinterpret_cast<const uint16_t*>(smem + L.o_hist);  // stage A..B2
  int4* surv = reinterpret_cast<int4*>(smem + L.o_surv);
  uint16_t* order = reinterpret_cast<uint16_t*>(cand_slot);  // serial insertion, after stage F
  int32_t* pool_id = reinterpret_cast<int32_t*>(smem + L.o_pool_id);
  int32_t* pool_sc = reinterpret_cast<int32_t*>(smem + L.o_pool_sc);
  __shared__ int s_cnt, s_ht, s_gt, s_jcut, s_nu, s_nneed, s_nprom, s_nmiss, s_ccnt;
  __shared__ int32_t s_wsum[kWarps], s_wsum2[kWarps];

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, sub = lane & 7, slot8 = lane >> 3;
  const int KK = L.KK, nchunk = d / 16, sk_chunks = W / 2;  // W: sketch words per row (<= L.W = d / 64)
  const uint32_t mask = uint32_t(L.HT - 1);
  const bool inplace = ids_out == ids_in;
  const bool cached = ctl.cache_ids != nullptr;
  // per-CTA statistics, kept by thread 0 in shared memory (no registers held
  // across the row loop): updates, sketches scored, rows reranked, distinct
  // candidates, rows skipped
  __shared__ unsigned long long s_stat[5];
  if (tid == 0)
    for (int q = 0; q < 5; ++q) s_stat[q] = 0;
  int run_job = -1;                 // per-job update count kept by warp 0 lane 0
  unsigned long long run_upd = 0;

  // job_done only changes between launches, so a CTA reads each job's flag
  // once; the next row's index is fetched one row ahead
  int flag_job = -1, flag_done = 0;
  const int64_t nrows = (ctl.row_limit > 0 && ctl.row_limit < n) ? ctl.row_limit : n;
  int64_t next_i = int64_t(blockIdx.x) < nrows ? (row_order ? int64_t(row_order[blockIdx.x]) : int64_t(blockIdx.x)) : 0;
  for (int64_t r = blockIdx.x; r < nrows; r += gridDim.x) {
    const int64_t i = next_i;
    if (r + gridDim.x < nrows) next_i = row_order ? int64_t(row_order[r + gridDim.x]) : r + gridDim.x;
    if (!KNNG_GUARD(ctl.check_err, i >= 0 && i < n)) continue;  // block-uniform
    int job = 0;
    if (ctl.job_done) {
      job = job_of(jt, i);
      if (job != flag_job) {
        flag_job = job;
        flag_done = ctl.job_done[job];
      }
      if (flag_done) {  // stopped job: its rows pass through unchanged
        if (!inplace)
          for (int k = tid; k < K; k += kThreads) {
            ids_out[i * K + k] = ids_in[i * K + k];
            scores_out[i * K + k] = scores_in[i * K + k];
          }
        continue;
      }
    }
    // ---- A
    // (unchanged-row skip, double-buffered iterations only) a row whose own
    // list and every neighbour's list came out of the previous iteration
    // unchanged sees exactly the inputs it saw then, so its result is its
    // current list: it is copied through without any work
    int moved = ctl.chg_in ? 0 : 1;
    for (int k = tid; k < K; k += kThreads) {
      const int32_t id = ids_in[i * K + k];
      pool_id[k] = id;
      pool_sc[k] = scores_in[i * K + k];
      KNNG_FLAG_IF(ctl.check_err, id < 0 || id >= n);
      if (ctl.chg_in) moved |= (id < 0 || id >= n) ? 1 : int(ctl.chg_in[id]);
    }
    if (ctl.chg_in && tid == 0) moved |= int(ctl.chg_in[i]);
    if (!cached)
      for (int h = tid; h < kHBins; h += kThreads) hist[h] = 0;
    for (int t = tid; t < L.HT / 4; t += kThreads) {
      reinterpret_cast<uint4*>(key)[t] = make_uint4(kEmpty, kEmpty, kEmpty, kEmpty);
      reinterpret_cast<uint4*>(meta)[t] = make_uint4(kFirstMask, kFirstMask, kFirstMask, kFirstMask);
    }
    if (tid == 0) {
      s_cnt = 0;
      s_nu = 0;
      s_nneed = 0;
      s_nprom = 0;
      s_ccnt = cached ? ctl.cache_cnt[i] : 0;
    }
    if (__syncthreads_or(moved) == 0) {  // block-uniform
      for (int k = tid; k < K; k += kThreads) {  // from global memory: the shared copies may be reused at once
        ids_out[i * K + k] = ids_in[i * K + k];
        scores_out[i * K + k] = scores_in[i * K + k];
      }
      if (tid == 0) {
        ctl.chg_out[i] = 0;
        ++s_stat[4];
      }
      continue;
    }
    for (int c = tid; c < nchunk; c += kThreads) my_code[c] = reinterpret_cast<const uint4*>(codes + i * d)[c];
    for (int c = tid; c < sk_chunks; c += kThreads) my_sk[c] = reinterpret_cast<const uint4*>(sketch + i * W)[c];
    if (cached) {
      // stage the row's cache entries into shared memory (ids over the region
      // of stages F-H, scores over the histogram) while stage B runs; the
      // rows' cache slices are 16-byte aligned and sized for cache_cap
      const int cc = min(s_ccnt, ctl.cache_cap);
      const int n_id = (cc * 4 + 15) / 16, n_hr = (cc * 2 + 15) / 16;
      const char* gid = reinterpret_cast<const char*>(ctl.cache_ids + i * ctl.cache_cap);
      const char* ghr = reinterpret_cast<const char*>(ctl.cache_hr + i * ctl.cache_cap);
      for (int t = tid; t < n_id + n_hr; t += kThreads) {
        if (t < n_id) cp_async16(smem + L.o_miss + 16 * t, gid + 16 * t);
        else cp_async16(smem + L.o_hist + 16 * (t - n_id), ghr + 16 * (t - n_id));
      }
      cp_async_commit();
    }
    int irregular = 0;
    for (int k = tid; k < K; k += kThreads) {
      const int32_t id = pool_id[k];
      if (pool_sc[k] != kScoreMinI && id >= 0 && id < n) table_insert(key, mask, id, kPoolFlag);
      irregular |= (pool_sc[k] == kScoreMinI) | (k + 1 < K && pool_sc[k] < pool_sc[k + 1]);
    }
    // An unscored entry (INT32_MIN, tiny inputs only) can share its id with a
    // survivor, and an unsorted pool (possible through the stage entry point)
    // breaks the rank formulas of stage G/H: both take the sequential loop.
    const bool serial_insert = __syncthreads_or(irregular) != 0;
    // ---- B  two-hop occurrences j = k*K + k2 spread over the block (thread t
    //         takes j = t + 256r), all loaded first; the first occurrence to
    //         touch a slot appends it to the distinct list
    {
      constexpr int kRounds = (kMaxK * kMaxK + kThreads - 1) / kThreads;
      const uint32_t kdiv = ((1u << 20) + uint32_t(K) - 1) / uint32_t(K);  // j / K = (j * kdiv) >> 20 for j < 4096
      int32_t v[kRounds];
#pragma unroll
      for (int t = 0; t < kRounds; ++t) {
        const int j = tid + kThreads * t;
        int32_t val = -1;
        if (j < KK) {
          const int k = int((uint32_t(j) * kdiv) >> 20);
          const int32_t n1 = pool_id[k];
          if (n1 >= 0 && n1 < n) {
            val = ids_in[int64_t(n1) * K + (j - k * K)];
            KNNG_FLAG_IF(ctl.check_err, val < 0 || val >= n);
          }
        }
        v[t] = val;
      }
      int local_cnt = 0;
#pragma unroll
      for (int t = 0; t < kRounds; ++t) {
        const int j = tid + kThreads * t;
        if (kThreads * t >= KK) break;  // block-uniform: no occurrence left for any thread
        const int32_t n2 = v[t];
        int sl = -1;
        bool first = false;
        if (j < KK) {
          if (n2 >= 0 && n2 < n && n2 != i) sl = table_insert(key, mask, n2, 0u);
          cand_slot[j] = int16_t(sl);
          if (sl >= 0) {
            // rounds visit j in increasing order, so once a slot records a
            // smaller first j (a plain read suffices) this occurrence is not
            // the first; otherwise the atomic decides, and exactly one of the
            // threads that saw the slot untouched gets kFirstMask back
            if (meta[sl] > uint32_t(j)) first = atomicMin(&meta[sl], uint32_t(j)) == kFirstMask;
            ++local_cnt;
          }
        }
        const unsigned bal = __ballot_sync(0xffffffffu, first);
        int base = 0;
        if (lane == 0 && bal) base = atomicAdd(&s_nu, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (first) ulist[base + __popc(bal & ((1u << lane) - 1u))] = int16_t(sl);
      }
      if (local_cnt) atomicAdd(&s_cnt, local_cnt);
    }
    if (cached) cp_async_wait_all();  // this thread's staging copies (stage A); the barrier publishes them
    __syncthreads();
    const int nu = s_nu;
    // ---- B2  candidate cache: the row's distinct candidates of the previous
    //          iteration with their Hamming scores and rejected flags.  Entries
    //          are only looked up (no slot is added), and a distinct id of this
    //          iteration without an entry goes to the miss list for stage C.
    const int16_t* clist = ulist;
    int ncl = nu;
    if (cached) {
      const int cc = min(s_ccnt, ctl.cache_cap);
      for (int q = tid; q < cc; q += kThreads) {
        const int sl = table_find(key, mask, stage_id[q]);
        if (sl >= 0) {
          const uint32_t hr = stage_hr[q];
          meta[sl] = kKnown | ((hr & 1u) ? kRej : 0u) | (uint32_t(hr >> 1) << 16) | (meta[sl] & kFirstMask);
        }
      }
      if (tid == 0) s_nmiss = 0;
      __syncthreads();
      for (int h = tid; h < kHBins; h += kThreads) hist[h] = 0;  // the staged scores are consumed
      for (int q0 = warp * 32; q0 < nu; q0 += kThreads) {
        const int q = q0 + lane;
        const int sl = q < nu ? int(ulist[q]) : -1;
        const bool miss = sl >= 0 && !(meta[sl] & kKnown);
        const unsigned bal = __ballot_sync(0xffffffffu, miss);
        int base = 0;
        if (lane == 0 && bal) base = atomicAdd(&s_nmiss, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (miss) misslist[base + __popc(bal & ((1u << lane) - 1u))] = int16_t(sl);
      }
      __syncthreads();
      clist = misslist;
      ncl = s_nmiss;
    }
    // ---- C  Hamming once per distinct id without a cached score (groups of 8
    //         lanes, CB candidates in flight per group)
    {
      const uint4 mine = sub < sk_chunks ? my_sk[sub] : make_uint4(0, 0, 0, 0);
      for (int wbase = warp * 4; wbase < ncl; wbase += CB * kGroups) {
        const int base = wbase + slot8;
        uint4 v[CB];
        int sl[CB];
#pragma unroll
        for (int u = 0; u < CB; ++u) {
          const int q = base + u * kGroups;
          sl[u] = q < ncl ? int(clist[q]) : -1;
          v[u] = make_uint4(0, 0, 0, 0);
          if (sl[u] >= 0 && sub < sk_chunks) {
            const int32_t id = int32_t(uint32_t(key[sl[u]]) & 0x7fffffffu);
            v[u] = __ldg(reinterpret_cast<const uint4*>(sketch + int64_t(id) * W) + sub);
          }
        }
#pragma unroll
        for (int u = 0; u < CB; ++u) {
          int pc = (sl[u] >= 0 && sub < sk_chunks) ? popc_u4(v[u], mine) : 0;
          pc += __shfl_xor_sync(0xffffffffu, pc, 1);
          pc += __shfl_xor_sync(0xffffffffu, pc, 2);
          pc += __shfl_xor_sync(0xffffffffu, pc, 4);
          if (sub == 0 && sl[u] >= 0) meta[sl[u]] = (uint32_t(1024 - pc) << 16) | (meta[sl[u]] & kFirstMask);
        }
      }
    }
    __syncthreads();
    // ---- D  histogram over occurrences, threshold
    for (int j = tid; j < KK; j += kThreads) {
      const int sl = cand_slot[j];
      if (sl >= 0) atomicAdd(&hist[(meta[sl] >> 16) & 0x7ffu], 1u);
    }
    __syncthreads();
    const int cnt = s_cnt;
    if (tid == 0) {
      s_stat[1] += unsigned(ncl);
      s_stat[3] += unsigned(nu);
    }
    if (cnt > R) {
      // bins from h = 1024 down: thread t sums bins 4t..4t+3 (index x = 1024 - h);
      // bin x = 1024 (h = 0) is handled last
      int sum = 0;
#pragma unroll
      for (int u = 0; u < 4; ++u) sum += int(hist[1024 - (4 * tid + u)]);
      int incl = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
      }
      if (lane == 31) s_wsum[warp] = incl;
      __syncthreads();
      int before = 0;
      for (int w = 0; w < warp; ++w) before += s_wsum[w];
      const int excl = before + incl - sum;
      if (excl < R && R <= excl + sum) {
        int run = excl;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int c = int(hist[1024 - (4 * tid + u)]);
          if (run + c >= R) {
            s_ht = 1024 - (4 * tid + u);
            s_gt = run;
            break;
          }
          run += c;
        }
      }
      if (tid == kThreads - 1 && excl + sum < R) {  // the cut falls in bin h = 0
        s_ht = 0;
        s_gt = excl + sum;
      }
    } else if (tid == 0) {
      s_ht = -1;  // every occurrence is selected
      s_gt = cnt;
    }
    __syncthreads();
    // ---- E  tie cut: the j of the (R - count(h > h_t))-th occurrence with h == h_t
    //         (thread-contiguous segments keep the j order); a distinct id with
    //         h == h_t is selected iff its first occurrence is at or before it
    {
      const int ht = s_ht, need_eq = R - s_gt;
      if (ht >= 0) {
        const int seg = (KK + kThreads - 1) / kThreads;
        const int j0 = tid * seg, j1 = min(KK, j0 + seg);
        int eq = 0;
        for (int j = j0; j < j1; ++j) {
          const int sl = cand_slot[j];
          eq += (sl >= 0 && int((meta[sl] >> 16) & 0x7ffu) == ht) ? 1 : 0;
        }
        int incl = eq;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int t = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += t;
        }
        if (lane == 31) s_wsum2[warp] = incl;
        __syncthreads();
        int rank = incl - eq;
        for (int w = 0; w < warp; ++w) rank += s_wsum2[w];
        if (rank < need_eq && need_eq <= rank + eq) {
          for (int j = j0; j < j1; ++j) {
            const int sl = cand_slot[j];
            if (sl >= 0 && int((meta[sl] >> 16) & 0x7ffu) == ht && ++rank == need_eq) {
              s_jcut = j;
              break;
            }
          }
        }
      }
    }
    __syncthreads();
    // ---- F1  selected distinct ids that are not starting-list members need a dot
    {
      const int ht = s_ht, jcut = ht >= 0 ? s_jcut : 0;
      for (int q0 = warp * 32; q0 < nu; q0 += kThreads) {  // warp-uniform trip count
        const int q = q0 + lane;
        bool want = false;
        int sl = -1;
        if (q < nu) {
          sl = ulist[q];
          const uint32_t m = meta[sl];
          const int h = int((m >> 16) & 0x7ffu);
          const bool sel = ht < 0 || h > ht || (h == ht && int(m & kFirstMask) <= jcut);
          // a cached rejection stands: the row's threshold never falls, so a
          // dot once <= it stays <= it
          want = sel && !(uint32_t(key[sl]) & kPoolFlag) && !(m & kRej);
        }
        const unsigned bal = __ballot_sync(0xffffffffu, want);
        int base = 0;
        if (lane == 0 && bal) base = atomicAdd(&s_nneed, __popc(bal));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (want) need[base + __popc(bal & ((1u << lane) - 1u))] = int16_t(sl);
      }
    }
    __syncthreads();
    // ---- F2  dots (8 lanes per candidate, up to eight 16-byte loads in flight per lane)
    {
      const int nneed = s_nneed;
      if (tid == 0) s_stat[2] += unsigned(nneed);
      const int32_t thr0 = pool_sc[K - 1];
      const int per_lane = d / 128;
      for (int wbase = warp * 4; wbase < nneed; wbase += kGroups) {
        const int q = wbase + slot8;
        const int sl = q < nneed ? int(need[q]) : -1;
        const int32_t id = sl >= 0 ? int32_t(uint32_t(key[sl]) & 0x7fffffffu) : 0;
        int acc = 0;
        if (sl >= 0) {
          const uint4* row = reinterpret_cast<const uint4*>(codes + int64_t(id) * d);
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
        if (sub == 0 && sl >= 0 && acc > thr0) {
          const uint32_t m = meta[sl];
          const int slot = atomicAdd(&s_nprom, 1);
          surv[slot] = make_int4(int((((m >> 16) & 0x7ffu) << 13) | (kFirstMask - (m & kFirstMask))), acc, id, 0);
        } else if (sub == 0 && sl >= 0 && cached) {
          meta[sl] |= kRej;
        }
      }
    }
    __syncthreads();
    // ---- F3  the row's cache for the next iteration: this iteration's distinct
    //          candidates (the first cache_cap of them) with score and flag
    if (cached) {
      const int cc = min(nu, ctl.cache_cap);
      int32_t* cid = ctl.cache_ids + i * ctl.cache_cap;
      uint16_t* chr = ctl.cache_hr + i * ctl.cache_cap;
      for (int q = tid; q < cc; q += kThreads) {
        const int sl = ulist[q];
        const uint32_t m = meta[sl];
        cid[q] = int32_t(uint32_t(key[sl]) & 0x7fffffffu);
        chr[q] = uint16_t((((m >> 16) & 0x7ffu) << 1) | ((m & kRej) ? 1u : 0u));
      }
      if (tid == 0) ctl.cache_cnt[i] = cc;
    }
    // ---- G/H  insertion of the survivors in visit order (pkey descending;
    //   keys are distinct).  The new pool goes to new_id/new_sc, laid over the
    //   hash table, which is dead after F2.
    const int P = s_nprom;
    int32_t* new_id = reinterpret_cast<int32_t*>(hist);  // dead after stage E; stage F3 may still read the table
    int32_t* new_sc = new_id + kMaxK;
    if (!serial_insert) {
      // The pool's last score only rises during the visits, and a rejected
      // survivor's dot is <= the last score at its visit, so the last score
      // before visit t is the K-th largest of {starting scores} and {dots of
      // all survivors visited before t}: survivor t is inserted iff fewer
      // than K of those values are >= its dot.  The final pool is the best K of
      // (starting entries, inserted survivors) ordered by score, ties to the
      // starting entries (in pool order) and then to earlier visits -- the
      // order the shift-insert loop leaves.  Needs a sorted starting pool
      // without unscored entries (else serial_insert is set).
      // A survivor record is {visit key, dot, id, flags}; flags bit 31 =
      // inserted, bits 0..30 = starting scores >= dot.  Stage G1 reads only
      // the first two words of the other records, so writing a record's
      // flags word does not race with it.
      for (int p = tid; p < P; p += kThreads) {
        const int2 me = *reinterpret_cast<const int2*>(surv + p);
        const uint32_t kp = uint32_t(me.x);
        const int32_t dp = me.y;
        int lo = 0, hi = K;  // first pool position with a score < dp (scores descend)
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (pool_sc[mid] >= dp) lo = mid + 1;
          else hi = mid;
        }
        int c = lo;
#pragma unroll 4
        for (int q = 0; q < P; ++q) {
          const int2 o = *reinterpret_cast<const int2*>(surv + q);
          c += (uint32_t(o.x) > kp && o.y >= dp) ? 1 : 0;
        }
        surv[p].w = int(uint32_t(lo) | (c < K ? 0x80000000u : 0u));
      }
      __syncthreads();
      // one unit per thread: starting entries 0..K-1, then survivors
      for (int u = tid; u < K + P; u += kThreads) {
        if (u < K) {
          const int32_t s = pool_sc[u];
          int rank = u;
#pragma unroll 4
          for (int q = 0; q < P; ++q) {
            const int4 o = surv[q];
            rank += (o.w < 0 && o.y > s) ? 1 : 0;
          }
          if (rank < K) {
            new_id[rank] = pool_id[u];
            new_sc[rank] = s;
          }
        } else {
          const int4 me = surv[u - K];
          if (me.w >= 0) continue;  // not inserted
          int rank = me.w & 0x7fffffff;
#pragma unroll 4
          for (int q = 0; q < P; ++q) {
            const int4 o = surv[q];
            rank += (o.w < 0 && (o.y > me.y || (o.y == me.y && uint32_t(o.x) > uint32_t(me.x)))) ? 1 : 0;
          }
          if (rank < K) {
            new_id[rank] = me.z;
            new_sc[rank] = me.y;
          }
        }
      }
    } else {
    // rank sort by (h desc, first j asc), then the reference's shift-insert
    // loop in warp 0 with the pool held two entries per lane
    for (int p = tid; p < P; p += kThreads) {
      const uint32_t kp = uint32_t(surv[p].x);
      int rank = 0;
      for (int q = 0; q < P; ++q) rank += uint32_t(surv[q].x) > kp ? 1 : 0;
      order[rank] = uint16_t(p);
    }
    __syncthreads();
    if (warp == 0) {
      int32_t idA = lane < K ? pool_id[lane] : -1, scA = lane < K ? pool_sc[lane] : kScoreMinI;
      int32_t idB = 32 + lane < K ? pool_id[32 + lane] : -1, scB = 32 + lane < K ? pool_sc[32 + lane] : kScoreMinI;
      const unsigned full = 0xffffffffu;
      for (int rr = 0; rr < P; ++rr) {
        const int p = order[rr];
        const int32_t id = surv[p].z, dot = surv[p].y;
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
      if (lane < K) {
        new_id[lane] = idA;
        new_sc[lane] = scA;
      }
      if (32 + lane < K) {
        new_id[32 + lane] = idB;
        new_sc[32 + lane] = scB;
      }
    }
    }
    __syncthreads();
    // ---- write-back of the positions whose id changed (every position when
    //      the output is the other buffer) and the update count
    if (warp == 0) {
      const unsigned full = 0xffffffffu;
      int changed = 0;
      for (int k = lane; k < K; k += 32) {
        const int32_t nid = new_id[k];
        const bool ch = nid != pool_id[k];
        changed += ch;
        if (ch || !inplace) {
          ids_out[i * K + k] = nid;
          scores_out[i * K + k] = new_sc[k];
        }
      }
      for (int o = 16; o > 0; o >>= 1) changed += __shfl_xor_sync(full, changed, o);
      if (lane == 0) s_stat[0] += unsigned(changed);
      if (ctl.chg_out && lane == 0) ctl.chg_out[i] = changed ? 1 : 0;
      if (ctl.job_upd && lane == 0) {
        if (job != run_job) {
          if (run_job >= 0 && run_upd) atomicAdd(ctl.job_upd + run_job, run_upd);
          run_job = job;
          run_upd = 0;
        }
        run_upd += unsigned(changed);
      }
    }
    __syncthreads();
  }
  if (tid == 0) {
    atomicAdd(counters + 0, s_stat[0]);
    atomicAdd(counters + 1, s_stat[1]);
    atomicAdd(counters + 2, s_stat[2]);
    atomicAdd(counters + 3, s_stat[3]);
    if (ctl.chg_in) atomicAdd(counters + 4, s_stat[4]);
    if (ctl.job_upd && run_job >= 0 && run_upd) atomicAdd(ctl.job_upd + run_job, run_upd);
  }
}

// Per-job early stop after an iteration, src/main.cpp:432-439 in float
// arithmetic: rate = float(updates) / float(n * K); a job stops when
// rate < stop or (iter > 0 and prev - rate < diff).  When every job has
// stopped, all_done is set and final_buf records the buffer that holds the
// final graphs; later iterations of the launch sequence then do nothing.
__global__ void stop_check_kernel(JobTable jt, JoinCtl ctl, int K, int iter, int out_buf, float stop_rate,
                                  float diff_tol) {
  if (*ctl.all_done) return;
  int all = 1;
  for (int b = threadIdx.x; b < jt.count; b += blockDim.x) {
    if (!ctl.job_done[b]) {
      const unsigned long long upd = ctl.job_upd[b];
      ctl.upd_log[int64_t(iter) * jt.count + b] = (long long)upd;
      const float rate = float(upd) / float((unsigned long long)jt.n[b] * (unsigned long long)K);
      const bool stop = rate < stop_rate || (iter > 0 && (ctl.job_prev[b] - rate) < diff_tol);
      ctl.job_prev[b] = rate;
      ctl.job_iters[b] = iter + 1;
      ctl.job_upd[b] = 0;
      if (stop) ctl.job_done[b] = 1;
      else all = 0;
    }
  }
  all = __syncthreads_and(all);
  if (threadIdx.x == 0) {
    *ctl.final_buf = out_buf;
    if (all) *ctl.all_done = 1;
  }
}

}  // namespace

size_t join_smem_bytes(int K, int R, int d) { return join_smem(K, R, d).bytes; }

// Resident CTAs per SM of a join variant at `smem` bytes of dynamic shared
// memory.  The attribute is set and the occupancy queried once per process and
// variant (under a mutex, so concurrent contexts and stream captures never
// issue these calls); a failure is returned as a CUDA error, not masked.
std::mutex g_variant_mu;
std::map<std::tuple<int, int, size_t>, int> g_variant_ctas;
char g_variant_err[256] = "";

template <int CB, int MINB>
cudaError_t max_ctas(size_t smem, int* per_sm_out) {
  std::lock_guard<std::mutex> lk(g_variant_mu);
  const auto key = std::make_tuple(CB, MINB, smem);
  auto it = g_variant_ctas.find(key);
  if (it != g_variant_ctas.end()) {
    *per_sm_out = it->second;
    return cudaSuccess;
  }
  cudaFuncAttributes fa{};
  cudaError_t e = cudaFuncGetAttributes(&fa, join_kernel<CB, MINB>);  // loads the function
  const char* what = "cudaFuncGetAttributes";
  if (e == cudaSuccess) {
    e = ensure_smem_attr(reinterpret_cast<const void*>(join_kernel<CB, MINB>), smem);
    what = "cudaFuncSetAttribute";
  }
  int per_sm = 0;
  if (e == cudaSuccess) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, join_kernel<CB, MINB>, kThreads, smem);
    what = "cudaOccupancyMaxActiveBlocksPerMultiprocessor";
  }
  if (e != cudaSuccess) {
    cudaGetLastError();  // reported through the return value
    std::snprintf(g_variant_err, sizeof(g_variant_err), "%s(join_kernel<%d,%d>, smem %zu, static smem %zu, regs %d): %s",
                  what, CB, MINB, smem, size_t(fa.sharedSizeBytes), fa.numRegs, cudaGetErrorString(e));
    return e;
  }
  per_sm = per_sm < 1 ? 1 : per_sm;
  g_variant_ctas.emplace(key, per_sm);
  *per_sm_out = per_sm;
  return cudaSuccess;
}

int join_max_ctas_per_sm(int K, int R, int d) {
  int per_sm = 1;
  return max_ctas<4, 4>(join_smem(K, R, d).bytes, &per_sm) == cudaSuccess ? per_sm : 1;
}

const char* join_variant_error() { return g_variant_err; }

cudaError_t join_prepare_all(int K, int R, int d) {
  for (int c : {3, 4})
    for (int b : {2, 4, 8}) {
      const cudaError_t e = join_prepare(K, R, d, c, b);
      if (e != cudaSuccess) return e;
    }
  return cudaSuccess;
}

cudaError_t join_prepare(int K, int R, int d, int ctas_per_sm, int cblock) {
  const size_t smem = join_smem(K, R, d).bytes;
  int per_sm = 0;
  if (ctas_per_sm == 3) {
    if (cblock == 2) return max_ctas<2, 3>(smem, &per_sm);
    if (cblock == 8) return max_ctas<8, 3>(smem, &per_sm);
    return max_ctas<4, 3>(smem, &per_sm);
  }
  if (cblock == 2) return max_ctas<2, 4>(smem, &per_sm);
  if (cblock == 8) return max_ctas<8, 4>(smem, &per_sm);
  return max_ctas<4, 4>(smem, &per_sm);
}

cudaError_t launch_stop_check(const JobTable& jt, const JoinCtl& ctl, int K, int iter, int out_buf, float stop_rate,
                              float diff_tol, cudaStream_t s) {
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  stop_check_kernel<<<1, 256, 0, s>>>(jt, ctl, K, iter, out_buf, stop_rate, diff_tol);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_join(const int8_t* codes, const uint64_t* sketch, int64_t n, int d, int K, int R,
                        const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out, int32_t* scores_out,
                        const int32_t* row_order, unsigned long long* counters, int num_sms, cudaStream_t s,
                        const JobTable* jt, const JoinCtl* ctl, int ctas_per_sm, int cblock, int sk_words) {
  const size_t smem = join_smem(K, R, d).bytes;
  const JobTable no_jobs{};
  const JoinCtl no_ctl{};
  cudaError_t e = cudaSuccess;
  auto go = [&](auto kern, cudaError_t qe, int max_per_sm) {
    if (qe != cudaSuccess) {
      e = qe;
      return;
    }
    const int64_t blocks = std::min<int64_t>(n, int64_t(num_sms) * max_per_sm);
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    kern<<<unsigned(blocks), kThreads, smem, s>>>(codes, sketch, n, d, K, R, sk_words > 0 ? sk_words : d / 64, ids_in,
                                                  scores_in, ids_out, scores_out, row_order, counters,
                                                  jt ? *jt : no_jobs, ctl ? *ctl : no_ctl);
    e = cudaGetLastError();
  };
  // ctas_per_sm 3: up to 85 registers per thread (no spills), 3 resident CTAs;
  // otherwise 64 registers, 4 resident CTAs
  int per_sm = 1;
  if (ctas_per_sm == 3) {
    if (cblock == 2) { cudaError_t q = max_ctas<2, 3>(smem, &per_sm); go(join_kernel<2, 3>, q, per_sm); }
    else if (cblock == 8) { cudaError_t q = max_ctas<8, 3>(smem, &per_sm); go(join_kernel<8, 3>, q, per_sm); }
    else { cudaError_t q = max_ctas<4, 3>(smem, &per_sm); go(join_kernel<4, 3>, q, per_sm); }
  } else {
    if (cblock == 2) { cudaError_t q = max_ctas<2, 4>(smem, &per_sm); go(join_kernel<2, 4>, q, per_sm); }
    else if (cblock == 8) { cudaError_t q = max_ctas<8, 4>(smem, &per_sm); go(join_kernel<8, 4>, q, per_sm); }
    else { cudaError_t q = max_ctas<4, 4>(smem, &per_sm); go(join_kernel<4, 4>, q, per_sm); }
  }
  note_launch();
  return e;
}

}  // namespace knng
