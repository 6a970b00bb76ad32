// knng_oracle.cpp -- CPU restatement of the reference kNN-graph builder.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the parity tests, the
// smoke check and bench.py's CPU-baseline leg call it as the checker (or as the
// timed CPU port of the reference).  The product path (libknng, the CUDA
// kernels and the knng_main CLI) never links, loads or calls it.
//
// It restates Aftab5550/SISAP-2026-task1 src/main.cpp stage by stage, with the
// same libstdc++ primitives the reference uses (std::mt19937,
// std::uniform_int_distribution, std::sort/unique, std::partial_sort,
// std::nth_element), so that with one thread and tie_mode = TIE_REF it gives
// bit-identical results to the reference binary run with OMP_NUM_THREADS=1.
// tie_mode = TIE_STABLE replaces the reference's unspecified tie orders with a
// fixed rule that the GPU kernels implement exactly:
//   init : pool ordered by (score desc, pool position asc)  (std::stable_sort)
//   join : rerank set = first R of the candidates ordered by
//          (hamming desc, sequence position asc), processed in that order.
// jacobi = 1 reads every neighbour list from the graph as it was at the start
// of the iteration (double buffering); jacobi = 0 is the reference's in-place
// update, which with one thread is the row-order Gauss-Seidel schedule.
//
// Exported with C linkage for ctypes (tests/, bench.py).
#include <algorithm>
#include <chrono>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <random>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr int32_t kScoreMin = std::numeric_limits<int32_t>::min();

struct Neighbor {  // src/main.cpp:31-37 (ordered by score, descending)
  int id;
  int32_t score;
};
inline bool by_score_desc(const Neighbor& a, const Neighbor& b) { return a.score > b.score; }

inline int32_t dot_i8(const int8_t* __restrict a, const int8_t* __restrict b, int d) {
  int32_t s = 0;
  for (int k = 0; k < d; ++k) s += int32_t(a[k]) * int32_t(b[k]);
  return s;
}

inline int popc64(uint64_t v) { return __builtin_popcountll(v); }

void set_threads(int threads) {
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#else
  (void)threads;
#endif
}

}  // namespace

extern "C" {

enum { TIE_REF = 0, TIE_STABLE = 1 };
enum { QUANT_TRUNC = 0, QUANT_ROUND = 1 };

// Same field order as knng_params in include/knng.h (host structs are
// converted field by field in the Python harness, not shared).
struct oracle_params {
  int k_build;            // K_BUILD = 50            src/main.cpp:22
  int k_eval;             // K_EVAL = 15             src/main.cpp:21
  int num_trees;          // NUM_TREES = 16          src/main.cpp:23
  int rerank_mult;        // RERANK_MULTIPLIER = 8   src/main.cpp:24
  int leaf_size;          // LEAF_SIZE = 64          src/main.cpp:25
  int max_iterations;     // MAX_ITERATIONS = 30     src/main.cpp:27
  float early_stop_rate;  // EARLY_STOP_RATE = 0.04  src/main.cpp:28
  float rate_diff_tol;    // RATE_DIFF_TOLERANCE = 0.01 src/main.cpp:29
  int quant_mode;         // QUANT_TRUNC follows src/main.cpp:184-186
  int tie_mode;           // TIE_REF | TIE_STABLE
  int jacobi;             // 0 = in place (reference), 1 = double buffered
  int threads;            // OpenMP threads (<= 0: leave the runtime default)
  uint32_t seed;          // 1337, src/main.cpp:210 and :271
  int sketch_mode;        // 0: the reference's coordinate-sign sketch; 1: 128 seeded hyperplanes
};

void oracle_default_params(oracle_params* p) {
  p->k_build = 50;
  p->k_eval = 15;
  p->num_trees = 16;
  p->rerank_mult = 8;
  p->leaf_size = 64;
  p->max_iterations = 30;
  p->early_stop_rate = 0.04f;
  p->rate_diff_tol = 0.01f;
  p->quant_mode = QUANT_TRUNC;
  p->tie_mode = TIE_REF;
  p->jacobi = 0;
  p->threads = 1;
  p->seed = 1337;
  p->sketch_mode = 0;
}

// ---------------------------------------------------------------------------
// a1: quantize + sign sketch.  src/main.cpp:179-192.
//   scaled  = x * 127.0f
//   clamped = max(-128.0f, min(127.0f, scaled))   (std::min/std::max order)
//   code    = static_cast<int8_t>(clamped)        (truncation toward zero)
//   bit d of the sketch is set iff clamped > 0; word d/64, bit d%64.
// Subnormal inputs are read as zero: the reference is built with -ffast-math
// (CMakeLists.txt:6), whose start-up code enables denormals-are-zero, so a
// subnormal x gives code 0 and sign bit 0 in the reference binary.
// QUANT_ROUND is the optional mode that rounds half away from zero and clamps
// to [-127, 127]; the sign bit is taken from the same clamped float.
// sketch rows hold `words` u64; words past d/64 are written as zero.
void oracle_quantize(const float* x, int64_t n, int d, int quant_mode, int8_t* codes,
                     uint64_t* sketch, int words) {
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const float* row = x + i * d;
    int8_t* q = codes + i * d;
    uint64_t* b = sketch + i * words;
    for (int w = 0; w < words; ++w) b[w] = 0;
    for (int k = 0; k < d; ++k) {
      float v = row[k];
      if (std::fabs(v) < FLT_MIN) v = 0.0f;
      float scaled = v * 127.0f;
      float clamped;
      if (quant_mode == QUANT_ROUND) {
        float lo = -127.0f, hi = 127.0f;
        clamped = std::max(lo, std::min(hi, scaled));
        q[k] = static_cast<int8_t>(std::round(clamped));
      } else {
        float lo = -128.0f, hi = 127.0f;
        clamped = std::max(lo, std::min(hi, scaled));
        q[k] = static_cast<int8_t>(clamped);
      }
      if (clamped > 0) b[k / 64] |= (1ULL << (k % 64));
    }
  }
}

// ---------------------------------------------------------------------------
// Optional sketch: 128 seeded random hyperplanes (the README's "128-bit
// random-hyperplane sketches", README.md:33-34; src/main.cpp itself keeps the
// coordinate-sign sketch above, so this mode has no reference output and is
// pinned only by this restatement and a numpy one in the tests).
//   plane k, coordinate j:  h = SplitMix64((seed << 32) ^ (k << 10 | j)),
//     g = sum over the 4 low bytes b of h of (b >> 2) - 32  (in [-128, 124],
//     a sum of four uniforms: close to Gaussian);
//   bit k of row i = (sum_j q_ij * g_kj > 0), exact in int32; bit k % 64 of
//   word k / 64, two words per row.
// The Hamming score of two rows stays 1024 - popcount over their words.
static uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

int8_t oracle_plane_value(uint32_t seed, int k, int j) {
  const uint64_t h = splitmix64((uint64_t(seed) << 32) ^ uint64_t((uint32_t(k) << 10) | uint32_t(j)));
  int v = 0;
  for (int b = 0; b < 4; ++b) v += int((h >> (8 * b)) & 0xff) / 4 - 32;
  return int8_t(v);
}

void oracle_hyperplane_sketch(const int8_t* codes, int64_t n, int d, uint32_t seed, uint64_t* sketch) {
  std::vector<int8_t> g(size_t(128) * d);
  for (int k = 0; k < 128; ++k)
    for (int j = 0; j < d; ++j) g[size_t(k) * d + j] = oracle_plane_value(seed, k, j);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    const int8_t* q = codes + i * d;
    uint64_t w[2] = {0, 0};
    for (int k = 0; k < 128; ++k) {
      int32_t dot = 0;
      for (int j = 0; j < d; ++j) dot += int32_t(q[j]) * int32_t(g[size_t(k) * d + j]);
      if (dot > 0) w[k / 64] |= 1ull << (k % 64);
    }
    sketch[i * 2] = w[0];
    sketch[i * 2 + 1] = w[1];
  }
}

// ---------------------------------------------------------------------------
// a2/a3: RP forest.  build_tree src/main.cpp:47-99, forest loop :205-216.
// Tree t draws from std::mt19937(seed + t) in DFS pre-order, left subtree
// before right; a node of more than leaf_size members picks two member
// positions with std::uniform_int_distribution<int>(0, n - 1), redrawing the
// second while the ids are equal, and splits stably: p1 goes left, p2 right,
// any other member goes left iff dot(x, p1) > dot(x, p2).
//
// Output, per tree t (row-major [num_trees][n]):
//   perm[t*n + p]      id at position p of the tree's leaf order (DFS order;
//                      each node covers a contiguous range, left child first)
//   leaf_flag[t*n + p] 1 where a leaf starts, else 0
// If pivot_log is non-null, every internal node appends six int32
//   (tree, level, start, size, p1_id, p2_id); start is the position within
//   the tree.  *n_nodes receives the number of internal nodes (the log is
//   written only while it fits in pivot_cap nodes).
// Returns 0, or -1 on bad arguments.
int oracle_forest(const int8_t* codes, int64_t n, int d, const oracle_params* prm,
                  int32_t* perm, uint8_t* leaf_flag, int32_t* pivot_log, int64_t pivot_cap,
                  int64_t* n_nodes) {
  if (n <= 0 || n > INT32_MAX || d <= 0) return -1;
  const int T = prm->num_trees;
  const int64_t L = prm->leaf_size;
  set_threads(prm->threads);
  std::vector<std::vector<int32_t>> logs(T);
#pragma omp parallel for schedule(dynamic, 1)
  for (int t = 0; t < T; ++t) {
    std::mt19937 rng(prm->seed + uint32_t(t));
    int32_t* pm = perm + int64_t(t) * n;
    uint8_t* lf = leaf_flag + int64_t(t) * n;
    for (int64_t i = 0; i < n; ++i) {
      pm[i] = int32_t(i);
      lf[i] = 0;
    }
    std::vector<int32_t> right;
    right.reserve(size_t(n));
    struct Node { int64_t start, size; int level; };
    std::vector<Node> stack;
    stack.push_back({0, n, 0});
    while (!stack.empty()) {
      Node nd = stack.back();
      stack.pop_back();
      int32_t* seg = pm + nd.start;
      if (nd.size <= L) {
        lf[nd.start] = 1;
        continue;
      }
      std::uniform_int_distribution<int> dist(0, int(nd.size - 1));
      int32_t p1 = seg[dist(rng)];
      int32_t p2 = seg[dist(rng)];
      while (p1 == p2) p2 = seg[dist(rng)];
      logs[t].insert(logs[t].end(), {t, nd.level, int32_t(nd.start), int32_t(nd.size), p1, p2});
      const int8_t* v1 = codes + int64_t(p1) * d;
      const int8_t* v2 = codes + int64_t(p2) * d;
      int64_t nl = 0;
      right.clear();
      for (int64_t j = 0; j < nd.size; ++j) {
        int32_t idx = seg[j];
        bool left;
        if (idx == p1) {
          left = true;
        } else if (idx == p2) {
          left = false;
        } else {
          const int8_t* v = codes + int64_t(idx) * d;
          left = dot_i8(v, v1, d) > dot_i8(v, v2, d);
        }
        if (left) seg[nl++] = idx; else right.push_back(idx);
      }
      std::copy(right.begin(), right.end(), seg + nl);
      // push right first so the left subtree is consumed first (DFS pre-order)
      stack.push_back({nd.start + nl, nd.size - nl, nd.level + 1});
      stack.push_back({nd.start, nl, nd.level + 1});
    }
  }
  int64_t total = 0;
  for (int t = 0; t < T; ++t) total += int64_t(logs[t].size() / 6);
  if (n_nodes) *n_nodes = total;
  if (pivot_log) {
    int64_t w = 0;
    for (int t = 0; t < T; ++t)
      for (size_t k = 0; k + 6 <= logs[t].size() && w < pivot_cap; k += 6, ++w)
        std::memcpy(pivot_log + 6 * w, logs[t].data() + k, 6 * sizeof(int32_t));
  }
  return 0;
}

// xorshift32 step used for the random fill and pad ids, src/main.cpp:273-275.
static inline uint32_t xorshift32(uint32_t s) {
  s ^= s << 13;
  s ^= s >> 17;
  s ^= s << 5;
  return s;
}

// ---------------------------------------------------------------------------
// a4: graph initialisation from the leaves.  src/main.cpp:222-314.
// For each row i: the union of the members of the leaves that hold i (one per
// tree), minus i, sorted and de-duplicated; exact int8 dot to each; random
// xorshift32 fill (state seed + i) while the pool holds fewer than K; top-K by
// score descending; copy skipping adjacent equal ids; pad with random ids of
// score INT32_MIN.  Graph rows are [n][K] ids and scores.
int oracle_init(const int8_t* codes, int64_t n, int d, const oracle_params* prm,
                const int32_t* perm, const uint8_t* leaf_flag, int32_t* ids, int32_t* scores) {
  if (n <= 0 || n > INT32_MAX) return -1;
  const int T = prm->num_trees;
  const int K = prm->k_build;
  set_threads(prm->threads);
  // per tree: position of each id and the [lo, hi) range of its leaf
  std::vector<int32_t> pos(size_t(T) * n), lo(size_t(T) * n), hi(size_t(T) * n);
  for (int t = 0; t < T; ++t) {
    const int32_t* pm = perm + int64_t(t) * n;
    const uint8_t* lf = leaf_flag + int64_t(t) * n;
    int32_t* ps = pos.data() + int64_t(t) * n;
    int32_t* l = lo.data() + int64_t(t) * n;
    int32_t* h = hi.data() + int64_t(t) * n;
    for (int64_t p = 0; p < n; ++p) ps[pm[p]] = int32_t(p);
    int64_t start = 0;
    for (int64_t p = 1; p <= n; ++p) {
      if (p == n || lf[p]) {
        for (int64_t q = start; q < p; ++q) { l[q] = int32_t(start); h[q] = int32_t(p); }
        start = p;
      }
    }
  }
#pragma omp parallel
  {
    std::vector<int32_t> cands;
    std::vector<Neighbor> pool;
#pragma omp for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; ++i) {
      cands.clear();
      pool.clear();
      for (int t = 0; t < T; ++t) {
        int64_t p = pos[size_t(t) * n + i];
        const int32_t* pm = perm + int64_t(t) * n;
        for (int32_t q = lo[size_t(t) * n + p]; q < hi[size_t(t) * n + p]; ++q)
          if (pm[q] != i) cands.push_back(pm[q]);
      }
      std::sort(cands.begin(), cands.end());
      cands.erase(std::unique(cands.begin(), cands.end()), cands.end());
      const int8_t* v1 = codes + i * d;
      for (int32_t c : cands) pool.push_back({c, dot_i8(v1, codes + int64_t(c) * d, d)});
      uint32_t rs = prm->seed + uint32_t(i);
      while (pool.size() < size_t(K)) {
        rs = xorshift32(rs);
        int64_t r = int64_t(uint64_t(rs) % uint64_t(n));
        if (r == i) continue;
        pool.push_back({int(r), dot_i8(v1, codes + r * d, d)});
      }
      if (prm->tie_mode == TIE_STABLE) {
        std::stable_sort(pool.begin(), pool.end(), by_score_desc);
      } else if (size_t(K) < pool.size()) {
        std::partial_sort(pool.begin(), pool.begin() + K, pool.end(), by_score_desc);
      } else {
        std::sort(pool.begin(), pool.end(), by_score_desc);
      }
      int added = 0;
      int last = -1;
      int32_t* gi = ids + i * K;
      int32_t* gs = scores + i * K;
      for (size_t p = 0; p < pool.size() && added < K; ++p) {
        if (pool[p].id != last) {
          gi[added] = pool[p].id;
          gs[added] = pool[p].score;
          last = pool[p].id;
          ++added;
        }
      }
      while (added < K) {
        rs = xorshift32(rs);
        int64_t r = int64_t(uint64_t(rs) % uint64_t(n));
        if (r != i) {
          gi[added] = int32_t(r);
          gs[added] = kScoreMin;
          ++added;
        }
      }
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// Random initial graph, the archived variant archive/nndescent_optimized.cpp:
// 97-118 (K random neighbours per row scored by exact int8 dot, sorted by score
// descending).  The archive draws from one std::mt19937 per OpenMP thread, so
// its graph depends on the thread count; here row i draws from xorshift32 with
// state seed + i (the reference's fill stream, src/main.cpp:271-276), skipping
// i and ids already drawn, and ties are ordered by id ascending.
int oracle_init_random(const int8_t* codes, int64_t n, int d, const oracle_params* prm, int32_t* ids,
                       int32_t* scores) {
  const int K = prm->k_build;
  if (n <= K) return -1;
  set_threads(prm->threads);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    std::vector<Neighbor> pool;
    uint32_t rs = prm->seed + uint32_t(i);
    while (int(pool.size()) < K) {
      rs = xorshift32(rs);
      const int64_t r = int64_t(uint64_t(rs) % uint64_t(n));
      if (r == i) continue;
      bool dup = false;
      for (const Neighbor& q : pool) dup |= q.id == r;
      if (dup) continue;
      pool.push_back({int(r), dot_i8(codes + i * d, codes + r * d, d)});
    }
    std::sort(pool.begin(), pool.end(), [](const Neighbor& a, const Neighbor& b) {
      return a.score != b.score ? a.score > b.score : a.id < b.id;
    });
    for (int k = 0; k < K; ++k) {
      ids[i * K + k] = pool[k].id;
      scores[i * K + k] = pool[k].score;
    }
  }
  return 0;
}

// Block-partitioned hybrid init (archive/nndescent_hybrid.cpp:98-144): the
// rows are split into nb = max(1, round(n / block_size)) consecutive blocks,
// block q = [q*n/nb, (q+1)*n/nb) (for the archive's 200000 rows and blocks of
// 10000 these are its 20 blocks); row i keeps the K best rows of its block by
// exact int8 dot, its last `bridges` entries (positions K-1, K-2, ...) are
// replaced by random rows other than i with their dots (duplicates allowed, as
// in the archive), and the list is sorted by score.  The archive draws the
// bridges from a per-thread std::mt19937 under a dynamic schedule and breaks
// ties through partial_sort/sort; here the draws are xorshift32 from seed + i
// (the random fill of src/main.cpp:271-286) and ties go to the lower id, with
// duplicates kept in place, so the result is reproducible.  Every block must
// hold K rows besides i.
int oracle_init_block(const int8_t* codes, int64_t n, int d, const oracle_params* prm, int block_size, int bridges,
                      int32_t* ids, int32_t* scores) {
  const int K = prm->k_build;
  if (block_size < 1 || bridges < 0 || bridges > K) return -1;
  int64_t nb = (n + block_size / 2) / block_size;
  if (nb < 1) nb = 1;
  if (n / nb < K + 1) return -1;  // the smallest block has floor(n / nb) rows
  set_threads(prm->threads);
  auto better = [](const Neighbor& a, const Neighbor& b) {
    return a.score != b.score ? a.score > b.score : a.id < b.id;
  };
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) {
    int64_t q = i * nb / n;
    while ((q + 1) * n / nb <= i) ++q;
    while (q * n / nb > i) --q;
    const int64_t lo = q * n / nb, hi = (q + 1) * n / nb;
    std::vector<Neighbor> pool;
    pool.reserve(size_t(hi - lo));
    for (int64_t j = lo; j < hi; ++j)
      if (j != i) pool.push_back({int(j), dot_i8(codes + i * d, codes + j * d, d)});
    std::partial_sort(pool.begin(), pool.begin() + K, pool.end(), better);
    pool.resize(size_t(K));
    uint32_t rs = prm->seed + uint32_t(i);
    for (int k = 0; k < bridges; ++k) {
      int64_t r = i;
      for (int budget = 1 << 20; r == i && budget > 0; --budget) {
        rs = xorshift32(rs);
        r = int64_t(uint64_t(rs) % uint64_t(n));
      }
      if (r == i) r = (i + 1) % n;  // xorshift32 from a zero state (seed + i == 0) stays at 0
      pool[size_t(K - 1 - k)] = {int(r), dot_i8(codes + i * d, codes + r * d, d)};
    }
    std::stable_sort(pool.begin(), pool.end(), better);
    for (int k = 0; k < K; ++k) {
      ids[i * K + k] = pool[size_t(k)].id;
      scores[i * K + k] = pool[size_t(k)].score;
    }
  }
  return 0;
}

// ---------------------------------------------------------------------------
// a5: one NN-Descent iteration.  src/main.cpp:324-430.
// Row i: candidates are G[G[i][k]][k2] for k, k2 < K in that order, minus i,
// each scored h = 1024 - sum_w popcount(b_i[w] ^ b_c[w]); the best R = K *
// rerank_mult by h (std::nth_element under TIE_REF; the first R of a stable
// sort by h under TIE_STABLE) are visited in order: skipped if the id is in
// the row's current pool, else scored by exact int8 dot and shift-inserted
// when dot > pool[K-1].score (existing entries stay ahead of equal scores).
// Positions whose id changed are written back and counted.
// sketch rows have `words` u64.  jacobi = 1 reads neighbour lists from a copy
// of the ids taken before the iteration.  Returns the number of updates.
int64_t oracle_join_iter(const int8_t* codes, const uint64_t* sketch, int words, int64_t n, int d,
                         const oracle_params* prm, int32_t* ids, int32_t* scores) {
  const int K = prm->k_build;
  const int R = K * prm->rerank_mult;
  set_threads(prm->threads);
  std::vector<int32_t> snap;
  const int32_t* src = ids;
  if (prm->jacobi) {
    snap.assign(ids, ids + n * K);
    src = snap.data();
  }
  int64_t total = 0;
#pragma omp parallel
  {
    std::vector<Neighbor> pool(K);
    std::vector<std::pair<int, int32_t>> cand(size_t(K) * K);
#pragma omp for reduction(+ : total) schedule(dynamic, 128)
    for (int64_t i = 0; i < n; ++i) {
      for (int k = 0; k < K; ++k) pool[k] = {ids[i * K + k], scores[i * K + k]};
      int cnt = 0;
      const uint64_t* b1 = sketch + i * words;
      for (int k = 0; k < K; ++k) {
        int n1 = pool[k].id;
        for (int k2 = 0; k2 < K; ++k2) {
          int n2 = src[int64_t(n1) * K + k2];
          if (n2 == i) continue;
          const uint64_t* b2 = sketch + int64_t(n2) * words;
          int32_t h = 1024;
          for (int w = 0; w < words; ++w) h -= popc64(b1[w] ^ b2[w]);
          cand[cnt++] = {n2, h};
        }
      }
      int top = cnt < R ? cnt : R;
      auto by_h = [](const std::pair<int, int32_t>& a, const std::pair<int, int32_t>& b) {
        return a.second > b.second;
      };
      if (prm->tie_mode == TIE_STABLE) {
        std::stable_sort(cand.begin(), cand.begin() + cnt, by_h);
      } else if (top > 0 && top < cnt) {
        std::nth_element(cand.begin(), cand.begin() + top, cand.begin() + cnt, by_h);
      }
      const int8_t* v1 = codes + i * d;
      for (int m = 0; m < top; ++m) {
        int n2 = cand[m].first;
        bool exists = false;
        for (int p = 0; p < K; ++p)
          if (pool[p].id == n2) { exists = true; break; }
        if (exists) continue;
        int32_t dot = dot_i8(v1, codes + int64_t(n2) * d, d);
        if (dot > pool[K - 1].score) {
          int p = K - 1;
          while (p > 0 && pool[p - 1].score < dot) {
            pool[p] = pool[p - 1];
            --p;
          }
          pool[p] = {n2, dot};
        }
      }
      int64_t changes = 0;
      for (int k = 0; k < K; ++k) {
        if (ids[i * K + k] != pool[k].id) {
          ids[i * K + k] = pool[k].id;
          scores[i * K + k] = pool[k].score;
          ++changes;
        }
      }
      total += changes;
    }
  }
  return total;
}

// ---------------------------------------------------------------------------
// a6: export.  src/main.cpp:449-457.  knns = id + 1 and dists = float(score)
// of the first k_eval entries, each row reversed (worst first, best last).
void oracle_export(const int32_t* ids, const int32_t* scores, int64_t n, int K, int k_eval,
                   int32_t* knns, float* dists) {
  for (int64_t i = 0; i < n; ++i)
    for (int k = 0; k < k_eval; ++k) {
      knns[i * k_eval + (k_eval - 1 - k)] = ids[i * K + k] + 1;
      dists[i * k_eval + (k_eval - 1 - k)] = static_cast<float>(scores[i * K + k]);
    }
}

struct oracle_stats {
  double quantize_s, forest_s, init_s, join_s, build_s;
  int iterations;
  int64_t updates[64];
};

// Full pipeline, src/main.cpp:179-457.  build_s covers forest + init + join
// (src/main.cpp:203 to :442).  Early stop follows :432-439 in float
// arithmetic: rate = float(updates) / float(n * K); stop when rate < stop or
// (iter > 0 and prev - rate < diff).
int oracle_build(const float* x, int64_t n, int d, const oracle_params* prm, int32_t* knns,
                 float* dists, int32_t* ids_out, int32_t* scores_out, oracle_stats* st) {
  using clk = std::chrono::steady_clock;
  if (n <= 1 || d <= 0 || d % 64 != 0) return -1;
  const int K = prm->k_build;
  const int qwords = d / 64;
  const int words = prm->sketch_mode == 1 ? 2 : qwords;
  std::vector<int8_t> codes(size_t(n) * d);
  std::vector<uint64_t> qsk(size_t(n) * qwords);
  std::vector<uint64_t> sk(size_t(n) * words);
  oracle_stats local{};
  if (!st) st = &local;
  std::memset(st, 0, sizeof(*st));
  set_threads(prm->threads);
  auto t0 = clk::now();
  oracle_quantize(x, n, d, prm->quant_mode, codes.data(), qsk.data(), qwords);
  if (prm->sketch_mode == 1) oracle_hyperplane_sketch(codes.data(), n, d, prm->seed, sk.data());
  else sk.swap(qsk);
  auto t1 = clk::now();
  std::vector<int32_t> perm(size_t(prm->num_trees) * n);
  std::vector<uint8_t> lf(size_t(prm->num_trees) * n);
  int64_t nn = 0;
  if (oracle_forest(codes.data(), n, d, prm, perm.data(), lf.data(), nullptr, 0, &nn)) return -1;
  auto t2 = clk::now();
  std::vector<int32_t> ids(size_t(n) * K), sc(size_t(n) * K);
  if (oracle_init(codes.data(), n, d, prm, perm.data(), lf.data(), ids.data(), sc.data())) return -1;
  auto t3 = clk::now();
  float prev = 1.0f;
  int it = 0;
  for (; it < prm->max_iterations; ++it) {
    int64_t up = oracle_join_iter(codes.data(), sk.data(), words, n, d, prm, ids.data(), sc.data());
    if (it < 64) st->updates[it] = up;
    float rate = float(up) / float(uint64_t(n) * uint64_t(K));
    if (rate < prm->early_stop_rate || (it > 0 && (prev - rate) < prm->rate_diff_tol)) {
      ++it;
      break;
    }
    prev = rate;
  }
  auto t4 = clk::now();
  st->iterations = it;
  st->quantize_s = std::chrono::duration<double>(t1 - t0).count();
  st->forest_s = std::chrono::duration<double>(t2 - t1).count();
  st->init_s = std::chrono::duration<double>(t3 - t2).count();
  st->join_s = std::chrono::duration<double>(t4 - t3).count();
  st->build_s = std::chrono::duration<double>(t4 - t1).count();
  if (knns && dists) oracle_export(ids.data(), sc.data(), n, K, prm->k_eval, knns, dists);
  if (ids_out) std::memcpy(ids_out, ids.data(), ids.size() * sizeof(int32_t));
  if (scores_out) std::memcpy(scores_out, sc.data(), sc.size() * sizeof(int32_t));
  return 0;
}

}  // extern "C"
