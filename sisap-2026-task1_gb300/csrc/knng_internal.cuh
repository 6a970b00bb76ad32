// knng_internal.cuh -- shared declarations of the libknng translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <string>

#include "../../include/knng.h"

namespace knng {

constexpr int kMaxK = 64;        // k_build upper bound (two pool entries per lane)
constexpr int kMaxDim = 1024;    // d upper bound (one 1 KB code row)
constexpr int kMaxLeaf = 64;     // leaf_size upper bound (64-wide Gram rows)
constexpr int kScoreMinI = INT32_MIN;

// Device-side error flag bits (written by kernels, read by the host).
enum : unsigned { kErrReplay = 1u, kErrBounds = 2u };

inline bool dim_ok(int d) { return d >= 128 && d <= kMaxDim && d % 128 == 0; }

// Host-side count of kernels this library has launched (all contexts).
int64_t launches();
void note_launch(int k = 1);

// ---- quantize.cu ----
cudaError_t launch_quantize(const float* x, int64_t n, int d, int quant_mode, int8_t* codes,
                            uint64_t* sketch, cudaStream_t s);

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
  int32_t* tile_off;      // [max_nodes + 1]
  int32_t* tile_left;     // [max_tiles]
  int32_t* tile_left_off; // [max_tiles]
  int32_t* child_cnt;     // [max_nodes + 1]
  int64_t* dev_i64;       // [4] device scalars
  unsigned* err;          // device error flags
  void* scan_tmp;
  int32_t* replay_dev;    // [n_replay * 6] or null
  int64_t max_nodes, max_tiles;
};
size_t forest_bytes(int64_t n, int T, int leaf, int64_t* max_nodes, int64_t* max_tiles);
int run_forest(const int8_t* codes, int64_t n, int d, int T, int leaf, uint32_t seed,
               const int32_t* replay_host, int64_t n_replay, int32_t* perm, uint8_t* leaf_flag,
               const ForestBufs& fb, cudaStream_t s, int64_t* levels_out, std::string* err);

// ---- init.cu ----
struct InitBufs {
  int32_t* pos;       // [T*n] inverse permutation (absolute positions)
  int32_t* leaf_lo;   // [T*n] leaf start of each position
  uint8_t* leaf_sz;   // [T*n] leaf size of each position
  int32_t* leaf_idx;  // [T*n] scan scratch
  int32_t* gram;      // [T*n][leaf] int32 leaf Gram rows
  int32_t* fix_rows;  // [n] rows whose candidate pool is smaller than K
  int64_t* dev_i64;   // [4]
  void* scan_tmp;
};
size_t init_bytes(int64_t n, int T, int leaf);
int run_init(const int8_t* codes, int64_t n, int d, int T, int leaf, int K, uint32_t seed,
             const int32_t* perm, const uint8_t* leaf_flag, int32_t* ids, int32_t* scores,
             const InitBufs& ib, cudaStream_t s, int64_t* leaves_out, std::string* err);

// ---- join.cu ----
cudaError_t launch_join(const int8_t* codes, const uint64_t* sketch, int64_t n, int d, int K, int R,
                        const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out,
                        int32_t* scores_out, const int32_t* row_order, unsigned long long* counters,
                        int num_sms, cudaStream_t s);
// counters[0] += updates, counters[1] += sketch candidates, counters[2] += reranked rows

// ---- export (init.cu) ----
cudaError_t launch_export(const int32_t* ids, const int32_t* scores, int64_t n, int K, int k_eval,
                          const int32_t* id_map, int32_t* knns, float* dists, cudaStream_t s);

}  // namespace knng

#define KNNG_CUDA_TRY(expr)                                  \
  do {                                                       \
    cudaError_t e_ = (expr);                                 \
    if (e_ != cudaSuccess) return e_;                        \
  } while (0)
