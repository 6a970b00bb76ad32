// init.cu -- K3 leaf Gram blocks, K4 top-K merge into the initial graph, K6 export.
//
// Reference: src/main.cpp:220-314.  For each row i the reference takes the
// union of the members of the T leaves that hold i (minus i), de-duplicates,
// scores each by exact int8 dot, fills with xorshift32 random ids while the
// pool holds fewer than K (state seed + i), keeps the top K by score and pads
// with random ids of score INT32_MIN.
//
// Here the dots come from one Gram block per leaf (K3: every member pair of a
// <= 64-member leaf, read once from HBM into shared memory), and a warp per
// row merges its T leaf rows into a sorted top-K list held two entries per
// lane (K4), one batched merge per 32 candidates (merge_batch).  The merge keeps the K best distinct (score desc, id asc) keys,
// which is the reference's pool order among equal scores (its pool is sorted
// by id before the unstable partial_sort; ties are unspecified there and fixed
// here).  Rows with fewer than K distinct candidates take the reference's
// random-fill path exactly, one thread per row (tiny inputs only).
#include "knng_internal.cuh"

#include <algorithm>

namespace knng {
namespace {

inline unsigned grid1(int64_t n, int t = 256) { return unsigned((n + t - 1) / t); }

__global__ void flags_to_i32(const uint8_t* __restrict__ f, int32_t* __restrict__ o, int64_t n) {
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += int64_t(gridDim.x) * blockDim.x)
    o[i] = f[i];
}

// leaf_start[idx[p]] = p for every flagged position p (idx = exclusive scan of flags)
__global__ void leaf_starts(const uint8_t* __restrict__ f, const int32_t* __restrict__ idx, int64_t n,
                            int32_t* __restrict__ leaf_start) {
  for (int64_t p = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; p < n; p += int64_t(gridDim.x) * blockDim.x)
    if (f[p]) leaf_start[idx[p]] = int32_t(p);
}

// per position: inverse permutation, leaf start and leaf size
__global__ void leaf_fill(const int32_t* __restrict__ leaf_start, int64_t nleaves, int64_t total, int64_t n,
                          const int32_t* __restrict__ perm, int32_t* __restrict__ pos, int32_t* __restrict__ leaf_lo,
                          uint8_t* __restrict__ leaf_sz, unsigned* err) {
  (void)err;
  for (int64_t l = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; l < nleaves; l += int64_t(gridDim.x) * blockDim.x) {
    const int64_t s = leaf_start[l];
    const int64_t e = l + 1 < nleaves ? leaf_start[l + 1] : total;
    const int64_t tb = (s / n) * n;
    // a leaf holds 1..kMaxLeaf positions of one tree
    KNNG_FLAG_IF(err, e - s < 1 || e - s > kMaxLeaf || e > tb + n);
    for (int64_t p = s; p < e; ++p) {
      leaf_lo[p] = int32_t(s);
      leaf_sz[p] = uint8_t(e - s);
      const int32_t v = perm[p];
      if (KNNG_GUARD(err, v >= 0 && v < n)) pos[tb + v] = int32_t(p);
    }
  }
}

// K3: one block per leaf.  The leaf's <= 64 code rows are staged in shared
// memory (row stride d + 16 bytes keeps the 8 column threads on distinct
// banks); thread (ty, tx) owns rows 4ty..4ty+3 x columns tx + 8j and runs 128
// dp4a per 12 shared-memory 16-byte loads.  Output: gram[p * 64 + j] = dot of
// the members at leaf offsets (p - start) and j, for j < size.
constexpr int kGramThreads = 128;

__global__ void __launch_bounds__(kGramThreads) leaf_gram(const int8_t* __restrict__ codes, int d,
                                                          const int32_t* __restrict__ perm,
                                                          const int32_t* __restrict__ leaf_start,
                                                          int64_t nleaves, int64_t total,
                                                          int32_t* __restrict__ gram, int64_t gram_pos0,
                                                          int64_t n_rows, unsigned* err) {
  (void)n_rows;
  (void)err;
  extern __shared__ uint4 rows_s[];
  const int stride16 = d / 16 + 1;  // in uint4
  for (int64_t l = blockIdx.x; l < nleaves; l += gridDim.x) {
    const int64_t s = leaf_start[l];
    const int64_t e = l + 1 < nleaves ? leaf_start[l + 1] : total;
    const int m = int(e - s);
    const int nchunk = d / 16;
    __syncthreads();
    for (int c = threadIdx.x; c < kMaxLeaf * nchunk; c += kGramThreads) {
      const int r = c / nchunk, cc = c % nchunk;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (r < m) {
        const int32_t id = perm[s + r];
        if (KNNG_GUARD(err, id >= 0 && id < n_rows)) v = __ldg(reinterpret_cast<const uint4*>(codes + int64_t(id) * d) + cc);
      }
      rows_s[r * stride16 + cc] = v;
    }
    __syncthreads();
    const int ty = threadIdx.x >> 3, tx = threadIdx.x & 7;
    if (ty * 4 >= m) continue;
    int acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) acc[a][b] = 0;
    const int jmax = (m + 7 - tx) / 8;  // columns tx + 8j < m
    for (int c = 0; c < nchunk; ++c) {
      uint4 A[4], B[8];
#pragma unroll
      for (int a = 0; a < 4; ++a) A[a] = rows_s[(ty * 4 + a) * stride16 + c];
#pragma unroll
      for (int b = 0; b < 8; ++b) B[b] = rows_s[(tx + 8 * b) * stride16 + c];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) {
          acc[a][b] = __dp4a(int(A[a].x), int(B[b].x), acc[a][b]);
          acc[a][b] = __dp4a(int(A[a].y), int(B[b].y), acc[a][b]);
          acc[a][b] = __dp4a(int(A[a].z), int(B[b].z), acc[a][b]);
          acc[a][b] = __dp4a(int(A[a].w), int(B[b].w), acc[a][b]);
        }
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      const int r = ty * 4 + a;
      if (r >= m) break;
      int32_t* out = gram + (s + r - gram_pos0) * int64_t(kMaxLeaf);
#pragma unroll
      for (int b = 0; b < 8; ++b)
        if (b < jmax) out[tx + 8 * b] = acc[a][b];
    }
  }
}

__device__ __forceinline__ uint64_t make_key(int32_t score, int32_t id) {
  return (uint64_t(uint32_t(score) ^ 0x80000000u) << 32) | uint64_t(~uint32_t(id));
}
__device__ __forceinline__ int32_t key_score(uint64_t k) { return int32_t(uint32_t(k >> 32) ^ 0x80000000u); }
__device__ __forceinline__ int32_t key_id(uint64_t k) { return int32_t(~uint32_t(k)); }

// Insert key ck into the descending list (kA = positions 0..31, kB = 32..63),
// length K, unless an equal key is present.  Returns the new threshold.
__device__ __forceinline__ uint64_t list_insert(uint64_t& kA, uint64_t& kB, uint64_t ck, int K, int lane) {
  const unsigned full = 0xffffffffu;
  const bool present = __any_sync(full, kA == ck || kB == ck);
  if (!present) {
    const int pos = __popc(__ballot_sync(full, kA > ck)) + __popc(__ballot_sync(full, kB > ck));
    const uint64_t upA = __shfl_up_sync(full, kA, 1);
    const uint64_t a31 = __shfl_sync(full, kA, 31);
    const uint64_t upB = __shfl_up_sync(full, kB, 1);
    if (lane > pos) kA = upA;
    else if (lane == pos) kA = ck;
    const int qb = 32 + lane;
    if (qb > pos) kB = lane == 0 ? a31 : upB;
    else if (qb == pos) kB = ck;
    if (lane >= K) kA = 0;
    if (qb >= K) kB = 0;
  }
  return (K - 1) < 32 ? __shfl_sync(full, kA, K - 1) : __shfl_sync(full, kB, K - 33);
}

// Merge one leaf half's candidate keys (one per lane, 0 = none) into the
// descending list kA/kB (positions lane and 32 + lane, length K; 0 = empty):
// afterwards it holds the K best distinct keys of both.  One pass for all the
// candidates above the threshold instead of one insertion each: the list goes
// to the warp's shared-memory row; such a candidate finds its rank in the list
// by binary search (an equal key is listed already) and its rank among the
// other candidates by counting; every list entry moves down by the number of
// candidates above it.  The ranks are a permutation of the merged order, so
// each entry and candidate is written once, and those at rank >= K drop out.
// Returns the new threshold (the K-th key, 0 while the list is not full).
__device__ __forceinline__ uint64_t merge_batch(uint64_t& kA, uint64_t& kB, uint64_t key, uint64_t thr, int K,
                                                int lane, uint64_t* sl) {
  const unsigned full = 0xffffffffu;
  bool want = key > thr;
  if (!__any_sync(full, want)) return thr;
  sl[lane] = kA;
  sl[32 + lane] = kB;
  __syncwarp();
  int lo = 0;
  if (want) {
    int hi = K;  // first list position whose key is <= key
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (sl[mid] > key) lo = mid + 1;
      else hi = mid;
    }
    if (lo < K && sl[lo] == key) want = false;
  }
  unsigned acc = __ballot_sync(full, want);
  int above = 0, cA = 0, cB = 0;
  while (acc) {
    const int src = __ffs(acc) - 1;
    acc &= acc - 1;
    const uint64_t ck = __shfl_sync(full, key, src);
    above += ck > key ? 1 : 0;
    cA += ck > kA ? 1 : 0;
    cB += ck > kB ? 1 : 0;
  }
  __syncwarp();
  if (lane < K && lane + cA < K) sl[lane + cA] = kA;
  if (32 + lane < K && 32 + lane + cB < K) sl[32 + lane + cB] = kB;
  if (want && lo + above < K) sl[lo + above] = key;
  __syncwarp();
  kA = lane < K ? sl[lane] : 0;
  kB = 32 + lane < K ? sl[32 + lane] : 0;
  __syncwarp();  // the row is rewritten by the next merge
  return (K - 1) < 32 ? __shfl_sync(full, kA, K - 1) : __shfl_sync(full, kB, K - 33);
}

// K4: one warp per row; merge the row's leaf Gram rows of trees [t0, t1) into
// its top-K list.  The first chunk of trees starts from an empty list, later
// chunks from the list the previous chunk wrote (keys round-trip exactly, and
// an empty entry, id -1 / INT32_MIN, is key 0), so the chunks give the list of
// all trees at once.  Gram rows are stored from position gram_pos0 on.
__global__ void __launch_bounds__(256) init_merge(int64_t n, int t0, int t1, int K, int first, int last,
                                                  const int32_t* __restrict__ perm,
                                                  const int32_t* __restrict__ pos,
                                                  const int32_t* __restrict__ leaf_lo,
                                                  const uint8_t* __restrict__ leaf_sz,
                                                  const int32_t* __restrict__ gram, int64_t gram_pos0,
                                                  int32_t* __restrict__ ids, int32_t* __restrict__ scores,
                                                  int32_t* __restrict__ fix_rows, int64_t* __restrict__ fix_count,
                                                  int64_t gram_rows, unsigned* err) {
  (void)gram_rows;
  (void)err;
  __shared__ uint64_t s_list[8][kMaxK];  // one list row per warp (merge_batch)
  const int lane = threadIdx.x & 31;
  const int64_t warps = int64_t(gridDim.x) * (blockDim.x >> 5);
  for (int64_t i = int64_t(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
    uint64_t kA = 0, kB = 0, thr = 0;
    if (!first) {
      if (lane < K) {
        const int32_t id = ids[i * K + lane];
        kA = id >= 0 ? make_key(scores[i * K + lane], id) : 0;
      }
      if (32 + lane < K) {
        const int32_t id = ids[i * K + 32 + lane];
        kB = id >= 0 ? make_key(scores[i * K + 32 + lane], id) : 0;
      }
      thr = (K - 1) < 32 ? __shfl_sync(0xffffffffu, kA, K - 1) : __shfl_sync(0xffffffffu, kB, K - 33);
    }
    for (int t = t0; t < t1; ++t) {
      const int64_t p = pos[int64_t(t) * n + i];
      // (bounds-checked build) the position lies in tree t, its leaf in the
      // same tree, and its Gram row in this chunk's rows
      if (!KNNG_GUARD(err, p >= int64_t(t) * n && p < int64_t(t + 1) * n && p - gram_pos0 < gram_rows)) continue;
      const int64_t s = leaf_lo[p];
      const int m = leaf_sz[p];
      if (!KNNG_GUARD(err, s >= int64_t(t) * n && s <= p && s + m <= int64_t(t + 1) * n && p < s + m)) continue;
      const int self = int(p - s);
      const int32_t* grow = gram + (p - gram_pos0) * int64_t(kMaxLeaf);
#pragma unroll
      for (int half = 0; half < 2; ++half) {
        const int j = lane + 32 * half;
        uint64_t key = 0;
        if (j < m && j != self) key = make_key(grow[j], perm[s + j]);
        thr = merge_batch(kA, kB, key, thr, K, lane, s_list[threadIdx.x >> 5]);
      }
    }
    const int real = __popc(__ballot_sync(0xffffffffu, kA != 0)) + __popc(__ballot_sync(0xffffffffu, kB != 0));
    int32_t* gi = ids + i * K;
    int32_t* gs = scores + i * K;
    if (lane < K) {
      gi[lane] = kA ? key_id(kA) : -1;
      gs[lane] = kA ? key_score(kA) : kScoreMinI;
    }
    if (32 + lane < K) {
      gi[32 + lane] = kB ? key_id(kB) : -1;
      gs[32 + lane] = kB ? key_score(kB) : kScoreMinI;
    }
    if (last && real < K && lane == 0) {
      const int64_t slot = atomicAdd(reinterpret_cast<unsigned long long*>(fix_count), 1ull);
      fix_rows[slot] = int32_t(i);
    }
  }
}

__device__ __forceinline__ uint32_t xorshift32(uint32_t s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

__device__ int32_t dot_rows(const int8_t* a, const int8_t* b, int d) {
  const int* pa = reinterpret_cast<const int*>(a);
  const int* pb = reinterpret_cast<const int*>(b);
  int s = 0;
  for (int k = 0; k < d / 4; ++k) s = __dp4a(pa[k], pb[k], s);
  return s;
}

// Rows whose leaves give fewer than K distinct candidates: the reference's
// pool is (candidates by id asc) + xorshift32 fills with exact dots; sorted by
// score (stable here), copied skipping adjacent equal ids, padded with random
// ids of score INT32_MIN.  src/main.cpp:271-312.  One thread per row.
__global__ void init_fixup(const int8_t* __restrict__ codes, int d, int64_t n_total, int K, uint32_t seed,
                           const int32_t* __restrict__ fix_rows, int64_t nfix, int32_t* __restrict__ ids,
                           int32_t* __restrict__ scores, JobTable jt) {
  const int64_t f = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (f >= nfix) return;
  (void)n_total;
  const int64_t gi = fix_rows[f];
  // random ids are drawn job-locally (state seed + local row, ids modulo the
  // job's n) exactly as a build of that job alone draws them
  const int b = job_of(jt, gi);
  const int64_t base = jt.off[b], n = jt.n[b], i = gi - base;
  ids += base * K;
  scores += base * K;
  codes += base * int64_t(d);
  int32_t pid[kMaxK], psc[kMaxK];
  int c = 0;
  for (int k = 0; k < K; ++k)
    if (ids[i * K + k] >= 0) {
      pid[c] = int32_t(ids[i * K + k] - base);  // job-local while the pool is built
      psc[c] = scores[i * K + k];
      ++c;
    }
  for (int a = 1; a < c; ++a) {  // candidates by id ascending
    const int32_t vi = pid[a], vs = psc[a];
    int b = a - 1;
    while (b >= 0 && pid[b] > vi) {
      pid[b + 1] = pid[b];
      psc[b + 1] = psc[b];
      --b;
    }
    pid[b + 1] = vi;
    psc[b + 1] = vs;
  }
  uint32_t rs = seed + uint32_t(i);
  const int8_t* vrow = codes + i * int64_t(d);
  // xorshift32 stays at 0 from a zero state; the reference would spin there
  // (seed + i == 0 with i == 0), so the draws are bounded.
  int budget = 1 << 20;
  while (c < K && --budget > 0) {
    rs = xorshift32(rs);
    const int64_t r = int64_t(uint64_t(rs) % uint64_t(n));
    if (r == i) continue;
    pid[c] = int32_t(r);
    psc[c] = dot_rows(vrow, codes + r * int64_t(d), d);
    ++c;
  }
  for (int a = 1; a < c; ++a) {  // stable by score descending
    const int32_t vi = pid[a], vs = psc[a];
    int b = a - 1;
    while (b >= 0 && psc[b] < vs) {
      pid[b + 1] = pid[b];
      psc[b + 1] = psc[b];
      --b;
    }
    pid[b + 1] = vi;
    psc[b + 1] = vs;
  }
  int added = 0, last = -1;
  for (int p = 0; p < c && added < K; ++p)
    if (pid[p] != last) {
      ids[i * K + added] = int32_t(pid[p] + base);
      scores[i * K + added] = psc[p];
      last = pid[p];
      ++added;
    }
  while (added < K) {
    rs = xorshift32(rs);
    const int64_t r = int64_t(uint64_t(rs) % uint64_t(n));
    if (r != i || --budget <= 0) {
      ids[i * K + added] = int32_t(base + (r != i ? r : (i + 1) % n));
      scores[i * K + added] = kScoreMinI;
      ++added;
    }
  }
}

// Random initial graph (archived variant archive/nndescent_optimized.cpp:97-118):
// row i draws K distinct ids from xorshift32 with state seed + (job-local) i,
// skipping itself, scores them by exact int8 dot and keeps them ordered by
// (score desc, id asc).  One warp per row: lane 0 draws, every lane scores
// candidates lane and lane + 32, the warp inserts them into its sorted list.
__global__ void __launch_bounds__(256) init_random_kernel(const int8_t* __restrict__ codes, int d, int64_t n_total,
                                                          int K, uint32_t seed, JobTable jt,
                                                          int32_t* __restrict__ ids, int32_t* __restrict__ scores) {
  __shared__ int32_t drawn[8][kMaxK];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t warps = int64_t(gridDim.x) * 8;
  for (int64_t gi = int64_t(blockIdx.x) * 8 + w; gi < n_total; gi += warps) {
    const int b = job_of(jt, gi);
    const int64_t base = jt.off[b], n = jt.n[b], i = gi - base;
    if (lane == 0) {
      uint32_t rs = seed + uint32_t(i);
      int c = 0;
      for (int budget = 1 << 22; c < K && budget > 0; --budget) {
        rs = xorshift32(rs);
        const int64_t r = int64_t(uint64_t(rs) % uint64_t(n));
        if (r == i) continue;
        bool dup = false;
        for (int q = 0; q < c; ++q) dup |= drawn[w][q] == int32_t(base + r);
        if (!dup) drawn[w][c++] = int32_t(base + r);
      }
      for (; c < K; ++c) drawn[w][c] = int32_t(base + (i + 1 + c) % n);  // budget guard only
    }
    __syncwarp();
    const int4* qi = reinterpret_cast<const int4*>(codes + gi * d);
    uint64_t key[2] = {0, 0};
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int c = lane + 32 * h;
      if (c < K) {
        const int4* qc = reinterpret_cast<const int4*>(codes + int64_t(drawn[w][c]) * d);
        int acc = 0;
        for (int u = 0; u < d / 16; ++u) {
          const int4 a = __ldg(qi + u), v = __ldg(qc + u);
          acc = __dp4a(a.x, v.x, acc);
          acc = __dp4a(a.y, v.y, acc);
          acc = __dp4a(a.z, v.z, acc);
          acc = __dp4a(a.w, v.w, acc);
        }
        key[h] = make_key(acc, drawn[w][c]);
      }
    }
    uint64_t kA = 0, kB = 0;
    for (int h = 0; h < 2; ++h)
      for (int src = 0; src < 32; ++src) {
        if (src + 32 * h >= K) break;
        const uint64_t ck = __shfl_sync(0xffffffffu, key[h], src);
        list_insert(kA, kB, ck, K, lane);
      }
    if (lane < K) {
      ids[gi * K + lane] = key_id(kA);
      scores[gi * K + lane] = key_score(kA);
    }
    if (32 + lane < K) {
      ids[gi * K + 32 + lane] = key_id(kB);
      scores[gi * K + 32 + lane] = key_score(kB);
    }
    __syncwarp();
  }
}

// Block-partitioned hybrid init (archive/nndescent_hybrid.cpp:98-144).  A job
// of n rows is split into nb = max(1, round(n / block_size)) consecutive
// blocks, block q = [q*n/nb, (q+1)*n/nb); row i keeps the K best rows of its
// block by exact int8 dot (ties to the lower id), its last `bridges` entries
// are replaced by random rows other than i with their dots (duplicates
// allowed, as in the archive), and the list is stably sorted by (score desc,
// id asc).  Bridges are xorshift32 draws from seed + (job-local) i, where the
// archive used a per-thread std::mt19937; the oracle restates this exactly.
// One warp per row: the row's code sits in shared memory, each lane scores
// one block member per step, and members above the current K-th key are
// inserted into the warp's list.  The host checks that every block holds
// K + 1 rows.
__global__ void __launch_bounds__(256) init_block_kernel(const int8_t* __restrict__ codes, int d, int64_t n_total,
                                                         int K, int bridges, int block_size, uint32_t seed,
                                                         JobTable jt, int32_t* __restrict__ ids,
                                                         int32_t* __restrict__ scores) {
  __shared__ __align__(16) int8_t row_code[8][kMaxDim];
  __shared__ uint64_t fin[8][kMaxK];
  __shared__ int64_t drawn[8][kMaxK];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t warps = int64_t(gridDim.x) * 8;
  const int chunks = d / 16;
  for (int64_t gi = int64_t(blockIdx.x) * 8 + w; gi < n_total; gi += warps) {
    const int b = job_of(jt, gi);
    const int64_t base = jt.off[b], n = jt.n[b], i = gi - base;
    int64_t nb = (n + block_size / 2) / block_size;
    if (nb < 1) nb = 1;
    int64_t q = i * nb / n;
    while ((q + 1) * n / nb <= i) ++q;
    while (q * n / nb > i) --q;
    const int64_t lo = q * n / nb, hi = (q + 1) * n / nb;
    int4* rc = reinterpret_cast<int4*>(row_code[w]);
    const int4* src = reinterpret_cast<const int4*>(codes + gi * d);
    for (int u = lane; u < chunks; u += 32) rc[u] = __ldg(src + u);
    __syncwarp();
    uint64_t kA = 0, kB = 0, thr = 0;
    for (int64_t j0 = lo; j0 < hi; j0 += 32) {
      const int64_t j = j0 + lane;
      uint64_t key = 0;
      if (j < hi && j != i) {
        const int4* cj = reinterpret_cast<const int4*>(codes + (base + j) * d);
        int acc = 0;
        for (int u = 0; u < chunks; ++u) {
          const int4 a = rc[u], v = __ldg(cj + u);
          acc = __dp4a(a.x, v.x, acc);
          acc = __dp4a(a.y, v.y, acc);
          acc = __dp4a(a.z, v.z, acc);
          acc = __dp4a(a.w, v.w, acc);
        }
        key = make_key(acc, int32_t(j));
      }
      unsigned m = __ballot_sync(full, key > thr);
      while (m) {
        const int s = __ffs(m) - 1;
        m &= m - 1;
        const uint64_t ck = __shfl_sync(full, key, s);
        if (ck > thr) thr = list_insert(kA, kB, ck, K, lane);
      }
    }
    if (lane < K) fin[w][lane] = kA;
    if (32 + lane < K) fin[w][32 + lane] = kB;
    if (lane == 0) {
      uint32_t rs = seed + uint32_t(i);
      for (int k = 0; k < bridges; ++k) {
        int64_t r = i;
        for (int budget = 1 << 20; r == i && budget > 0; --budget) {
          rs = xorshift32(rs);
          r = int64_t(uint64_t(rs) % uint64_t(n));
        }
        if (r == i) r = (i + 1) % n;  // xorshift32 from a zero state (seed + i == 0) stays at 0
        drawn[w][k] = r;
      }
    }
    __syncwarp();
    for (int k = 0; k < bridges; ++k) {
      const int64_t r = drawn[w][k];
      const int4* cr = reinterpret_cast<const int4*>(codes + (base + r) * d);
      int acc = 0;
      for (int u = lane; u < chunks; u += 32) {
        const int4 a = rc[u], v = __ldg(cr + u);
        acc = __dp4a(a.x, v.x, acc);
        acc = __dp4a(a.y, v.y, acc);
        acc = __dp4a(a.z, v.z, acc);
        acc = __dp4a(a.w, v.w, acc);
      }
      for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(full, acc, o);
      if (lane == 0) fin[w][K - 1 - k] = make_key(acc, int32_t(r));
    }
    __syncwarp();
    // stable rank sort, descending (a bridge can repeat an entry: equal keys
    // keep their position order)
    for (int e = lane; e < K; e += 32) {
      const uint64_t me = fin[w][e];
      int rank = 0;
      for (int f = 0; f < K; ++f) {
        const uint64_t o = fin[w][f];
        rank += (o > me || (o == me && f < e)) ? 1 : 0;
      }
      ids[gi * K + rank] = int32_t(base + key_id(me));
      scores[gi * K + rank] = key_score(me);
    }
    __syncwarp();
  }
}

__global__ void export_kernel(const int32_t* __restrict__ ids, const int32_t* __restrict__ scores, int64_t n,
                              int K, int k_eval, const int32_t* __restrict__ id_map, int32_t* __restrict__ knns,
                              float* __restrict__ dists, JobTable jt, unsigned* err) {
  (void)err;
  const int64_t tot = n * k_eval;
  for (int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; q < tot; q += int64_t(gridDim.x) * blockDim.x) {
    const int64_t i = q / k_eval;
    const int k = int(q % k_eval);
    int32_t id = ids[i * K + k];
    const int32_t sc = scores[i * K + k];
    if (id_map && KNNG_GUARD(err, id >= 0 && id < n)) id = id_map[id];
    else KNNG_FLAG_IF(err, id < 0 || id >= n);
    if (jt.count > 1) id -= jt.off[job_of(jt, i)];
    const int64_t o = i * k_eval + (k_eval - 1 - k);
    knns[o] = id + 1;
    dists[o] = float(sc);
  }
}

}  // namespace

size_t init_bytes(int64_t n, int T, int leaf) {
  (void)leaf;
  const size_t tn = size_t(T) * n;
  size_t b = tn * 4 * 3 + tn;           // pos, leaf_lo, leaf_idx, leaf_sz
  b += tn * 4;                          // leaf starts
  b += size_t(init_gram_trees(T)) * n * kMaxLeaf * 4;  // gram rows of one chunk of trees
  b += size_t(n) * 4;                   // fix rows
  b += scan_tmp_bytes(int64_t(tn)) + 4096;
  return b;
}

int run_init(const int8_t* codes, int64_t n, int d, int T, int leaf, int K, uint32_t seed, const int32_t* perm,
             const uint8_t* leaf_flag, int32_t* ids, int32_t* scores, const InitBufs& ib, cudaStream_t s,
             int64_t* leaves_out, std::string* err, const JobTable& jt, int gram_mode, int wait_limit) {
  (void)leaf;
  auto fail = [&](cudaError_t e, const char* what) {
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return int(KNNG_E_CUDA);
  };
  cudaError_t e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t tn = int64_t(T) * n;
  const unsigned g = unsigned(std::min<int64_t>(grid1(tn), int64_t(sms) * 32));
  int32_t* leaf_start = ib.leaf_idx + tn;  // second half of the leaf_idx allocation
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  flags_to_i32<<<g, 256, 0, s>>>(leaf_flag, ib.leaf_idx, tn);
  note_launch();
  if ((e = exclusive_scan_i32(ib.leaf_idx, ib.leaf_idx, tn, ib.dev_i64, ib.scan_tmp, s))) return fail(e, "leaf scan");
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  leaf_starts<<<g, 256, 0, s>>>(leaf_flag, ib.leaf_idx, tn, leaf_start);
  note_launch();
  int64_t nleaves = 0;
  // leaves before each tree's first position (the exclusive flag scan there):
  // tree t's leaves are [lt[t], lt[t + 1])
  int32_t lt[65] = {};  // num_trees <= 64; a fixed array: this stage allocates nothing on the host either
  if (T > 64) return fail(cudaErrorInvalidValue, "num_trees");
  if ((e = cudaMemcpyAsync(&nleaves, ib.dev_i64, 8, cudaMemcpyDeviceToHost, s))) return fail(e, "leaf count");
  if ((e = cudaMemcpy2DAsync(lt, sizeof(int32_t), ib.leaf_idx, size_t(n) * sizeof(int32_t), sizeof(int32_t),
                             size_t(T), cudaMemcpyDeviceToHost, s)))
    return fail(e, "tree leaf offsets");
  if ((e = cudaStreamSynchronize(s))) return fail(e, "leaf table");
  lt[T] = int32_t(nleaves);
  if (leaves_out) *leaves_out = nleaves;
  // error word of the tensor-core Gram's bounded waits and of the
  // bounds-checked build's checks
  unsigned* gerr = reinterpret_cast<unsigned*>(ib.dev_i64 + 3);
  const bool read_err = gram_mode == 1 || kChecked;
  if (read_err && (e = cudaMemsetAsync(gerr, 0, sizeof(unsigned), s))) return fail(e, "error word");
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  leaf_fill<<<unsigned(std::min<int64_t>(grid1(nleaves), int64_t(sms) * 32)), 256, 0, s>>>(
      leaf_start, nleaves, tn, n, perm, ib.pos, ib.leaf_lo, ib.leaf_sz, gerr);
  note_launch();
  if ((e = cudaMemsetAsync(ib.dev_i64 + 1, 0, 8, s))) return fail(e, "fix count");
  const size_t gram_smem = size_t(kMaxLeaf) * (d / 16 + 1) * 16;
  if (gram_mode != 1 && (e = ensure_smem_attr(reinterpret_cast<const void*>(leaf_gram), gram_smem)))
    return fail(e, "gram smem");
  // as many trees at a time as the Gram region holds (at least
  // init_gram_trees(T)): their leaf Gram rows, then the merge of those rows
  // into the lists
  const int chunk = ib.gram_rows > 0 ? int(std::max<int64_t>(1, std::min<int64_t>(T, ib.gram_rows / n)))
                                      : init_gram_trees(T);
  for (int t0 = 0; t0 < T; t0 += chunk) {
    const int t1 = std::min(T, t0 + chunk);
    const int64_t l0 = lt[t0], l1 = lt[t1];
    const int64_t pos0 = int64_t(t0) * n, pos1 = int64_t(t1) * n;
    if (l1 > l0) {
      if (gram_mode == 1) {
        if ((e = launch_leaf_gram_tc(codes, d, perm, leaf_start + l0, l1 - l0, pos1, ib.gram, pos0, gerr, sms, s,
                                     wait_limit, n)))
          return fail(e, "tensor-core gram");
      } else {
        cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
        leaf_gram<<<unsigned(std::min<int64_t>(l1 - l0, int64_t(sms) * 24)), kGramThreads, gram_smem, s>>>(
            codes, d, perm, leaf_start + l0, l1 - l0, pos1, ib.gram, pos0, n, gerr);
        note_launch();
      }
    }
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    init_merge<<<unsigned(std::min<int64_t>((n + 7) / 8, int64_t(sms) * 16)), 256, 0, s>>>(
        n, t0, t1, K, t0 == 0 ? 1 : 0, t1 == T ? 1 : 0, perm, ib.pos, ib.leaf_lo, ib.leaf_sz, ib.gram, pos0, ids,
        scores, ib.fix_rows, ib.dev_i64 + 1, int64_t(t1 - t0) * n, gerr);
    note_launch();
  }
  int64_t nfix = 0;
  unsigned gflag = 0;
  if ((e = cudaMemcpyAsync(&nfix, ib.dev_i64 + 1, 8, cudaMemcpyDeviceToHost, s))) return fail(e, "fix count");
  if (read_err && (e = cudaMemcpyAsync(&gflag, gerr, sizeof(unsigned), cudaMemcpyDeviceToHost, s)))
    return fail(e, "error word");
  if ((e = cudaStreamSynchronize(s))) return fail(e, "init merge");
  if (gflag & kErrTimeout) {
    if (err) *err = "tensor-core leaf Gram: an mbarrier wait timed out";
    return KNNG_E_TIMEOUT;
  }
  if (gflag & kErrBounds) {
    if (err) *err = "initial graph: a permutation entry or leaf position is outside its array (bounds check)";
    return KNNG_E_BOUNDS;
  }
  if (nfix > 0) {
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    init_fixup<<<grid1(nfix, 64), 64, 0, s>>>(codes, d, n, K, seed, ib.fix_rows, nfix, ids, scores, jt);
    note_launch();
    if ((e = cudaGetLastError())) return fail(e, "init fixup");
  }
  return 0;
}

cudaError_t launch_init_random(const int8_t* codes, int d, int64_t n_total, int K, uint32_t seed, const JobTable& jt,
                               int32_t* ids, int32_t* scores, int num_sms, cudaStream_t s) {
  const int64_t blocks = std::min<int64_t>((n_total + 7) / 8, int64_t(num_sms) * 16);
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  init_random_kernel<<<unsigned(blocks), 256, 0, s>>>(codes, d, n_total, K, seed, jt, ids, scores);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_init_block(const int8_t* codes, int d, int64_t n_total, int K, int bridges, int block_size,
                              uint32_t seed, const JobTable& jt, int32_t* ids, int32_t* scores, int num_sms,
                              cudaStream_t s) {
  const int64_t blocks = std::min<int64_t>((n_total + 7) / 8, int64_t(num_sms) * 16);
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  init_block_kernel<<<unsigned(blocks), 256, 0, s>>>(codes, d, n_total, K, bridges, block_size, seed, jt, ids, scores);
  note_launch();
  return cudaGetLastError();
}

cudaError_t launch_export(const int32_t* ids, const int32_t* scores, int64_t n, int K, int k_eval,
                          const int32_t* id_map, int32_t* knns, float* dists, cudaStream_t s, const JobTable* jt,
                          unsigned* err) {
  const int64_t tot = n * k_eval;
  if (tot <= 0) return cudaSuccess;
  const JobTable none{};
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  export_kernel<<<unsigned(std::min<int64_t>(grid1(tot), 4096)), 256, 0, s>>>(ids, scores, n, K, k_eval, id_map,
                                                                               knns, dists, jt ? *jt : none, err);
  note_launch();
  return cudaGetLastError();
}

// The bounds-checked build's error word for knng_export (a stage entry point
// without a context).  Host code reaches it only through its device address.
__device__ unsigned g_export_check;

cudaError_t export_check_word(unsigned** word) {
  return cudaGetSymbolAddress(reinterpret_cast<void**>(word), g_export_check);
}

}  // namespace knng
