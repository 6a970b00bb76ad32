// knng_internal.cuh -- shared declarations of the libknng translation units.
#pragma once
#include <cuda_runtime.h>

#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/knng.h"

namespace knng {

constexpr int kMaxK = 64;        // k_build upper bound (two pool entries per lane)
constexpr int kMaxDim = 1024;    // d upper bound (one 1 KB code row)
constexpr int kMaxLeaf = 64;     // leaf_size upper bound (64-wide Gram rows)
constexpr int kScoreMinI = INT32_MIN;

// Device-side error flag bits (written by kernels, read by the host).
enum : unsigned { kErrReplay = 1u, kErrBounds = 2u, kErrTimeout = 4u };

// Bounds-checked build (compiled with -DKNNG_CHECKS into libknng_checked.so).
// Every index a kernel derives from its inputs before it addresses memory
// (graph ids, permutation entries, leaf positions, id maps) is checked; a
// failed check ORs kErrBounds into the call's error word and the access is
// skipped or replaced by a harmless one, so a bad input ends in
// KNNG_E_BOUNDS, never in a fault or a trap.  In the default build
// KNNG_GUARD(err, ok) is `true` (no check is compiled) and KNNG_FLAG_IF
// compiles to nothing; guards that the default build needs for its own
// correctness are written out in full either way.
#ifdef KNNG_CHECKS
constexpr bool kChecked = true;
__device__ __forceinline__ bool check_note(unsigned* err, bool ok) {
  if (!ok && err) atomicOr(err, kErrBounds);
  return ok;
}
#define KNNG_GUARD(err, ok) (::knng::check_note((err), bool(ok)))
#define KNNG_FLAG_IF(err, bad) ((void)::knng::check_note((err), !(bad)))
#else
constexpr bool kChecked = false;
#define KNNG_GUARD(err, ok) true
#define KNNG_FLAG_IF(err, bad) ((void)0)
#endif

inline bool dim_ok(int d) { return d >= 128 && d <= kMaxDim && d % 128 == 0; }

// Runs an entry point's body and turns a C++ exception into a status, so none
// crosses the C ABI: std::bad_alloc -> KNNG_E_OOM, anything else ->
// KNNG_E_CUDA; `note` (may be null) receives a short message.
template <class F>
int abi_guard(std::string* note, F&& body) noexcept {
  try {
    return body();
  } catch (const std::bad_alloc&) {
    try {
      if (note) *note = "host memory allocation failed";
    } catch (...) {
    }
    return KNNG_E_OOM;
  } catch (...) {
    try {
      if (note) *note = "internal error (C++ exception)";
    } catch (...) {
    }
    return KNNG_E_CUDA;
  }
}

// Host-side count of kernels this library has launched (all contexts).
int64_t launches();
void note_launch(int k = 1);

// Raise a kernel's dynamic shared-memory limit to at least `bytes`.  The
// attribute belongs to the function (process-wide), not to a launch, so it is
// only ever raised, under one mutex: a concurrent launch that needs less can
// never find it lowered under it.
cudaError_t ensure_smem_attr(const void* func, size_t bytes);

// A batch of independent jobs laid out back to back: job b owns global rows
// [off[b], off[b] + n[b]) of an N-row problem (N = sum n).  Per-tree arrays are
// tree-major, [T][N], so tree t of job b is the range t*N + off[b] ... and a
// single build is the batch of one job (off = {0}, n = {N}).  Device copies of
// off/n are read by the kernels that need a row's job (pivot identity, random
// fills, per-job early stop, export of job-local ids).
struct JobTable {
  int count = 0;
  const int32_t* off = nullptr;  // device, [count], ascending
  const int32_t* n = nullptr;    // device, [count]
};

__device__ __forceinline__ int job_of(const JobTable& jt, int64_t row) {
  int lo = 0, hi = jt.count - 1;  // largest b with off[b] <= row
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (jt.off[mid] <= row) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// ---- hostcopy.cu ----
// Pinned host memory (cudaHostAlloc), grown on demand.
struct PinnedBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want);
  void release();
  template <class T>
  T* as(size_t byte_off = 0) const {
    return reinterpret_cast<T*>(static_cast<char*>(p) + byte_off);
  }
};
// Host threads that split one large memcpy between them (the caller takes a
// slice too); copy() returns when every slice is done.  One copy at a time.
class CopyPool {
 public:
  explicit CopyPool(int threads);
  ~CopyPool();
  void copy(void* dst, const void* src, size_t bytes);

 private:
  void run(int t);
  void slice(int t);
  int nthreads_;
  std::vector<std::thread> workers_;
  std::mutex mu_;
  std::condition_variable start_cv_, done_cv_;
  uint64_t gen_ = 0;
  int pending_ = 0;
  bool stop_ = false;
  char* dst_ = nullptr;
  const char* src_ = nullptr;
  size_t bytes_ = 0;
};
int host_copy_threads();            // CPUs this process may run on (1..32)
bool host_pageable(const void* p);  // host memory the device does not map

// ---- quantize.cu ----
cudaError_t launch_quantize(const float* x, int64_t n, int d, int quant_mode, int8_t* codes,
                            uint64_t* sketch, cudaStream_t s);

// ---- hyperplane.cu ----
// 128-bit sketches [n][2] of the int8 codes from 128 seeded integer hyperplanes.
cudaError_t launch_hyperplane_sketch(const int8_t* codes, int64_t n, int d, uint32_t seed, uint64_t* sketch,
                                     int num_sms, cudaStream_t s);

// ---- scan.cu ----
// Exclusive prefix sum of n int32 values into out (out may alias in); total
// (device int64, may be null) receives the sum.  tmp must hold
// scan_tmp_bytes(n) bytes.
size_t scan_tmp_bytes(int64_t n);
cudaError_t exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, int64_t* total,
                               void* tmp, cudaStream_t s);

// ---- forest.cu ----
struct ForestBufs {
  int32_t* perm_tmp;      // [T*n]
  uint8_t* side;          // [T*n]
  int32_t* node_a;        // node arrays, two generations: start,size,p1,p2
  int32_t* node_b;
  int32_t* node_c;        // nodes parked by the fused rounds for the per-level loop
  int32_t* tile_off;      // [max_nodes + 1]
  int32_t* tile_left;     // [max_tiles] (per-level path; shares tile_bins)
  int32_t* tile_left_off; // [max_tiles] (per-level path; shares tile_bins_off)
  int32_t* tile_bins;     // [8 * max_tiles] fused path: members per tile and path code
  int32_t* tile_bins_off; // [8 * max_tiles]
  int32_t* piv;           // [max_nodes * 14] fused path: pivot tables
  int32_t* child_cnt;     // [max_nodes + 1]
  int32_t* child_cnt2;    // [max_nodes + 1]
  int64_t* dev_i64;       // [4] device scalars
  unsigned* err;          // device error flags
  void* scan_tmp;
  int32_t* replay_dev;    // [n_replay * 6] or null
  int64_t max_nodes, max_tiles;
};
size_t forest_bytes(int64_t n, int T, int leaf, int64_t* max_nodes, int64_t* max_tiles);
int run_forest(const int8_t* codes, int64_t n, int d, int T, int leaf, uint32_t seed,
               const int32_t* replay_host, int64_t n_replay, int32_t* perm, uint8_t* leaf_flag,
               const ForestBufs& fb, cudaStream_t s, int64_t* levels_out, std::string* err,
               const JobTable& jt, int roots_with_split, int fuse);
// roots_with_split = number of jobs with n[b] > leaf (their T roots are split);
// fuse = 1: nodes of >= 512 members split three levels per pass (native
// pivots only; a replay table always takes the per-level path)

// ---- init.cu ----
// The initial-graph stage computes leaf Gram rows for kInitTreeChunk trees at
// a time (64 int32 per position: 512 B per row for two trees instead of
// 4 KB for sixteen), merging each chunk into the rows' lists.
constexpr int kInitTreeChunk = 2;
inline int init_gram_trees(int T) { return T < kInitTreeChunk ? T : kInitTreeChunk; }
struct InitBufs {
  int32_t* pos;       // [T*n] inverse permutation (absolute positions)
  int32_t* leaf_lo;   // [T*n] leaf start of each position
  uint8_t* leaf_sz;   // [T*n] leaf size of each position
  int32_t* leaf_idx;  // [T*n] scan scratch
  int32_t* gram;      // [gram_rows][64] int32 leaf Gram rows of one chunk of trees
  int64_t gram_rows = 0;  // rows the gram region holds (0: init_gram_trees(T) * n); a chunk is as
                          // many trees as fit
  int32_t* fix_rows;  // [n] rows whose candidate pool is smaller than K
  int64_t* dev_i64;   // [4]
  void* scan_tmp;
};
size_t init_bytes(int64_t n, int T, int leaf);
int run_init(const int8_t* codes, int64_t n, int d, int T, int leaf, int K, uint32_t seed,
             const int32_t* perm, const uint8_t* leaf_flag, int32_t* ids, int32_t* scores,
             const InitBufs& ib, cudaStream_t s, int64_t* leaves_out, std::string* err,
             const JobTable& jt, int gram_mode = 0, int wait_limit = 0);
// gram_mode 0: dp4a leaf Gram (leaf_gram); 1: tcgen05 f16 tensor-core Gram (leaf_gram_tc)
// wait_limit: knng_params::wait_limit (0 = default polls per bounded wait)
// Gram rows of the leaves [leaf_start, leaf_start + nleaves) (the last one ends
// at position `total`) go to gram[(position - gram_pos0) * 64 ...].
cudaError_t launch_leaf_gram_tc(const int8_t* codes, int d, const int32_t* perm, const int32_t* leaf_start,
                                int64_t nleaves, int64_t total, int32_t* gram, int64_t gram_pos0, unsigned* err,
                                int num_sms, cudaStream_t s, int wait_limit, int64_t n_rows);
// n_rows: rows of `codes` (the bounds-checked build checks every gathered id against it)

// Random initial graph (init_mode KNNG_INIT_RANDOM); every job needs n > K.
cudaError_t launch_init_random(const int8_t* codes, int d, int64_t n_total, int K, uint32_t seed, const JobTable& jt,
                               int32_t* ids, int32_t* scores, int num_sms, cudaStream_t s);
// Block-partitioned hybrid initial graph (init_mode KNNG_INIT_BLOCK); every
// block of every job needs k_build + 1 rows (checked by the caller).
cudaError_t launch_init_block(const int8_t* codes, int d, int64_t n_total, int K, int bridges, int block_size,
                              uint32_t seed, const JobTable& jt, int32_t* ids, int32_t* scores, int num_sms,
                              cudaStream_t s);

// ---- join.cu ----
// Per-batch NN-Descent control block in device memory.
struct JoinCtl {
  unsigned long long* counters;   // [5]: updates, sketches scored, reranked rows, distinct candidates,
                                  // rows skipped as unchanged
  unsigned long long* job_upd;    // [count]: updates of this iteration per job
  int* job_done;                  // [count]: job stopped (its rows pass through)
  float* job_prev;                // [count]: previous iteration's update rate
  int* job_iters;                 // [count]: iterations run per job
  int* all_done;                  // [1]
  int* final_buf;                 // [1]: buffer index holding every job's final graph
  long long* upd_log;             // [max_iter][count]: updates per iteration per job
  // Per-row candidate cache (all null: none).  Row i keeps its previous
  // iteration's distinct two-hop ids with their Hamming scores and whether the
  // dot is known to be <= the row's pool threshold (which never falls), so the
  // next iteration gathers sketches and code rows only for new candidates.
  int32_t* cache_ids;             // [n][cache_cap]
  uint16_t* cache_hr;             // [n][cache_cap]: score << 1 | rejected
  int* cache_cnt;                 // [n]: entries held (0 before the first iteration)
  int cache_cap;
  int64_t row_limit;              // rows processed (the first ones in visit order); 0: all
  // Unchanged-row skip of double-buffered iterations (both null: none).
  // chg_in[i] = 1 when row i's list changed in the previous iteration (all 1
  // before the first); the launch writes this iteration's flags to chg_out.
  const uint8_t* chg_in;
  uint8_t* chg_out;
  // error word of the bounds-checked build (null: none): an id outside [0, n)
  // in the input lists or the row order sets kErrBounds
  unsigned* check_err;
};
// Entries per row of the candidate cache (rows with more distinct candidates
// keep the first ones; the rest are scored again) and its bytes for n rows.
// The cache lives in the context's scratch buffer, over the forest and
// initial-graph scratch, which is dead once the initial graph exists.
constexpr int kCacheCap = 1536;
inline size_t cache_ids_bytes(int64_t n) { return (size_t(n) * kCacheCap * 4 + 255) & ~size_t(255); }
inline size_t cache_hr_bytes(int64_t n) { return (size_t(n) * kCacheCap * 2 + 255) & ~size_t(255); }
inline size_t cache_bytes(int64_t n) { return cache_ids_bytes(n) + cache_hr_bytes(n) + size_t(n) * 4; }
cudaError_t launch_join(const int8_t* codes, const uint64_t* sketch, int64_t n, int d, int K, int R,
                        const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out,
                        int32_t* scores_out, const int32_t* row_order, unsigned long long* counters,
                        int num_sms, cudaStream_t s, const JobTable* jt = nullptr,
                        const JoinCtl* ctl = nullptr, int ctas_per_sm = 0, int cblock = 4, int sk_words = 0);
// sk_words: 64-bit sketch words per row (0: d / 64, the sign sketch; 2: hyperplane sketch)
// ctas_per_sm: 4 (64 registers per thread) or 3 (up to 85, no spills);
// cblock: sketch candidates in flight per 8-lane group in the Hamming stage
// (2, 4 or 8).  Both are chosen by the autotuner.
// counters[0] += updates, counters[1] += sketches scored (distinct candidates
// without a cached score), counters[2] += reranked rows, counters[3] +=
// distinct candidates.
// With jt/ctl: rows of stopped jobs are copied through (when out != in) and
// per-job updates are added to ctl->job_upd; if ctl->all_done is set the launch
// does nothing.
cudaError_t launch_stop_check(const JobTable& jt, const JoinCtl& ctl, int K, int iter, int out_buf,
                              float stop_rate, float diff_tol, cudaStream_t s);
int join_max_ctas_per_sm(int K, int R, int d);
// Resolve a join variant's launch attributes before any stream capture.
cudaError_t join_prepare(int K, int R, int d, int ctas_per_sm, int cblock);
cudaError_t join_prepare_all(int K, int R, int d);  // every variant the autotuner may pick
const char* join_variant_error();                    // detail of the last failed resolution

// ---- export (init.cu) ----
cudaError_t launch_export(const int32_t* ids, const int32_t* scores, int64_t n, int K, int k_eval,
                          const int32_t* id_map, int32_t* knns, float* dists, cudaStream_t s,
                          const JobTable* jt = nullptr, unsigned* err = nullptr);
// With jt, ids are written job-local (id - off[job] + 1).  err: the
// bounds-checked build's error word (an id outside [0, n)), may be null.
// The bounds-checked build's error word of knng_export, which has no context:
// a file-scope device word of init.cu, resolved once per device.
cudaError_t export_check_word(unsigned** word);

}  // namespace knng

#define KNNG_CUDA_TRY(expr)                                  \
  do {                                                       \
    cudaError_t e_ = (expr);                                 \
    if (e_ != cudaSuccess) return e_;                        \
  } while (0)
