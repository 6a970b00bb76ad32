// forest.cu -- K2: random-projection forest, all trees level by level.
//
// Reference: build_tree, src/main.cpp:47-99, and the forest loop :205-216.  A
// node with more than leaf_size members picks two distinct members p1, p2 and
// splits stably: p1 goes left, p2 right, any other member x goes left iff
// dot(x, p1) > dot(x, p2) in exact int32 over the int8 codes.  The reference
// recurses depth first with one std::mt19937 per tree; here every tree's
// perm[t*n ...] array is split level-synchronously, one kernel sequence per
// level for all T trees at once.  A node always covers a contiguous range of
// its tree's perm, left child first, so the final perm of a tree is exactly
// the reference's DFS leaf order when the same pivots are used (replay mode),
// and node identity is (tree, start, size).
//
// Native pivots come from a counter-based hash of (seed, tree, start, size):
// the reference's pivot stream is a serial dependency through the whole DFS
// (the right subtree's draws wait for the left subtree's), so it is replayed
// only in tests, from the oracle's log.
//
// A batch of jobs is one problem of N rows (tree-major [T][N] arrays, job b at
// offset off[b] in every tree); every level serves all jobs' nodes at once.
//
// Per level: pick_pivots -> scan(tiles) -> side (8 lanes per row, dp4a,
// HBM-bound: d bytes read per active member) -> scan(left counts) -> scatter
// (stable partition into perm_tmp) -> copy back -> children (leaf flags,
// next node list).
#include "knng_internal.cuh"

#include <algorithm>
#include <vector>

namespace knng {
namespace {

constexpr int kTileElems = 256;

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

struct NodeArr {
  int32_t *start, *size, *p1, *p2;
};
__host__ __device__ inline NodeArr node_arr(int32_t* base, int64_t cap) {
  return NodeArr{base, base + cap, base + 2 * cap, base + 3 * cap};
}

__global__ void init_perm(int32_t* perm, int64_t n, int T) {
  const int64_t tot = n * T;
  for (int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < tot; i += int64_t(gridDim.x) * blockDim.x)
    perm[i] = int32_t(i % n);
}

// Roots: for tree t and job b the range t*N + off[b] of size n[b]; jobs with
// n[b] <= leaf are single leaves.  Node order is by start (tree, then job).
__global__ void root_nodes(NodeArr nd, int64_t N, int T, int leaf, uint8_t* leaf_flag, JobTable jt, int split_jobs) {
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    int k = t * split_jobs;
    for (int b = 0; b < jt.count; ++b) {
      const int64_t start = int64_t(t) * N + jt.off[b];
      if (jt.n[b] > leaf) {
        nd.start[k] = int32_t(start);
        nd.size[k] = jt.n[b];
        ++k;
      } else {
        leaf_flag[start] = 1;
      }
    }
  }
}

// Node identity is job-local -- (tree, start within the job's range, size) --
// so a job draws the same pivots alone and inside any batch.
__global__ void pick_pivots(NodeArr nd, int cnt, int64_t n, uint32_t seed, int level, const int32_t* perm,
                            const int32_t* replay, int32_t* tile_cnt, unsigned* err, JobTable jt) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t start = nd.start[k], size = nd.size[k];
  const int32_t tree = int32_t(int64_t(start) / n);
  const int32_t in_tree = int32_t(int64_t(start) - int64_t(tree) * n);
  const int32_t local = in_tree - jt.off[job_of(jt, in_tree)];
  int32_t p1, p2;
  if (replay) {
    const int32_t* r = replay + 6 * int64_t(k);
    if (r[0] != tree || r[1] != level || r[2] != local || r[3] != size) {
      atomicOr(err, kErrReplay);
      p1 = perm[start];
      p2 = perm[start + 1];
    } else {
      p1 = r[4];
      p2 = r[5];
    }
  } else {
    uint64_t h = splitmix64((uint64_t(seed) << 32) ^ uint64_t(uint32_t(tree)));
    h = splitmix64(h ^ uint64_t(uint32_t(local)));
    h = splitmix64(h ^ (uint64_t(uint32_t(size)) << 1));
    const uint64_t h2 = splitmix64(h ^ 0x5851F42D4C957F2Dull);
    int32_t a = int32_t(h % uint64_t(size));
    int32_t b = int32_t(h2 % uint64_t(size - 1));
    if (b >= a) ++b;
    p1 = perm[start + a];
    p2 = perm[start + b];
  }
  nd.p1[k] = p1;
  nd.p2[k] = p2;
  tile_cnt[k] = (size + kTileElems - 1) / kTileElems;
}

__device__ __forceinline__ int find_node(const int32_t* tile_off, int cnt, int b) {
  int lo = 0, hi = cnt - 1;  // largest k with tile_off[k] <= b
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (tile_off[mid] <= b) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// One block per tile of <= 256 members of one node.  8 lanes per member: lane
// sub reads 16-byte chunks sub, sub+8, ... of the member's code row and
// accumulates dp4a against both pivot rows staged in shared memory.
__global__ void __launch_bounds__(256) side_kernel(const int8_t* __restrict__ codes, int d,
                                                   const int32_t* __restrict__ perm, NodeArr nd, int cnt,
                                                   const int32_t* __restrict__ tile_off,
                                                   uint8_t* __restrict__ side, int32_t* __restrict__ tile_left) {
  __shared__ uint4 piv[2][kMaxDim / 16];
  __shared__ int node_s;
  __shared__ int32_t warp_cnt[8];
  const int b = blockIdx.x;
  if (threadIdx.x == 0) node_s = find_node(tile_off, cnt, b);
  __syncthreads();
  const int k = node_s;
  const int32_t start = nd.start[k], size = nd.size[k], p1 = nd.p1[k], p2 = nd.p2[k];
  const int64_t e0 = int64_t(start) + int64_t(b - tile_off[k]) * kTileElems;
  const int64_t e1 = min(int64_t(start) + size, e0 + kTileElems);
  const int nchunk = d / 16;
  for (int c = threadIdx.x; c < 2 * nchunk; c += blockDim.x) {
    const int which = c / nchunk, cc = c % nchunk;
    const int32_t pid = which ? p2 : p1;
    piv[which][cc] = reinterpret_cast<const uint4*>(codes + int64_t(pid) * d)[cc];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, sub = lane & 7, slot = lane >> 3;
  const int per_lane = d / 128;
  int my_left = 0;
  for (int step = 0; step < 8; ++step) {
    const int t = warp * 32 + step * 4 + slot;
    const int64_t e = e0 + t;
    const bool valid = e < e1;
    const int32_t id = valid ? perm[e] : 0;
    const uint4* row = reinterpret_cast<const uint4*>(codes + int64_t(id) * d);
    int d1 = 0, d2 = 0;
    if (valid) {
      uint4 v[8];
#pragma unroll
      for (int u = 0; u < 8; ++u)
        if (u < per_lane) v[u] = __ldg(row + sub + 8 * u);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        if (u < per_lane) {
          const uint4 a = piv[0][sub + 8 * u], c = piv[1][sub + 8 * u];
          d1 = __dp4a(int(v[u].x), int(a.x), d1);
          d1 = __dp4a(int(v[u].y), int(a.y), d1);
          d1 = __dp4a(int(v[u].z), int(a.z), d1);
          d1 = __dp4a(int(v[u].w), int(a.w), d1);
          d2 = __dp4a(int(v[u].x), int(c.x), d2);
          d2 = __dp4a(int(v[u].y), int(c.y), d2);
          d2 = __dp4a(int(v[u].z), int(c.z), d2);
          d2 = __dp4a(int(v[u].w), int(c.w), d2);
        }
      }
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
      d1 += __shfl_xor_sync(0xffffffffu, d1, o);
      d2 += __shfl_xor_sync(0xffffffffu, d2, o);
    }
    const bool left = (id == p1) || (id != p2 && d1 > d2);
    if (valid && sub == 0) {
      side[e] = left ? 1 : 0;
      my_left += left ? 1 : 0;
    }
  }
  for (int o = 16; o > 0; o >>= 1) my_left += __shfl_xor_sync(0xffffffffu, my_left, o);
  if (lane == 0) warp_cnt[warp] = my_left;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < 8; ++w) s += warp_cnt[w];
    tile_left[b] = s;
  }
}

__device__ __forceinline__ int32_t node_left(const NodeArr& nd, int k, const int32_t* tile_off,
                                             const int32_t* tile_left, const int32_t* tile_left_off) {
  const int f = tile_off[k];
  const int fl = f + (nd.size[k] + kTileElems - 1) / kTileElems - 1;
  return tile_left_off[fl] + tile_left[fl] - tile_left_off[f];
}

__global__ void __launch_bounds__(256) scatter_kernel(const int32_t* __restrict__ perm,
                                                      int32_t* __restrict__ perm_tmp, NodeArr nd, int cnt,
                                                      const int32_t* __restrict__ tile_off,
                                                      const uint8_t* __restrict__ side,
                                                      const int32_t* __restrict__ tile_left,
                                                      const int32_t* __restrict__ tile_left_off) {
  __shared__ int node_s;
  __shared__ int32_t warp_off[8];
  const int b = blockIdx.x;
  if (threadIdx.x == 0) node_s = find_node(tile_off, cnt, b);
  __syncthreads();
  const int k = node_s;
  const int32_t start = nd.start[k], size = nd.size[k];
  const int64_t e0 = int64_t(start) + int64_t(b - tile_off[k]) * kTileElems;
  const int64_t e1 = min(int64_t(start) + size, e0 + kTileElems);
  const int32_t nleft = node_left(nd, k, tile_off, tile_left, tile_left_off);
  const int32_t base = tile_left_off[b] - tile_left_off[tile_off[k]];
  const int64_t e = e0 + threadIdx.x;
  const bool valid = e < e1;
  const bool left = valid && side[e];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const unsigned bal = __ballot_sync(0xffffffffu, left);
  if (lane == 0) warp_off[warp] = __popc(bal);
  __syncthreads();
  int32_t pre = 0;
  for (int w = 0; w < warp; ++w) pre += warp_off[w];
  pre += __popc(bal & ((1u << lane) - 1u));
  if (valid) {
    const int32_t lrank = base + pre;
    const int32_t rrank = int32_t(e - start) - lrank;
    const int64_t np = int64_t(start) + (left ? lrank : nleft + rrank);
    perm_tmp[np] = perm[e];
  }
}

__global__ void __launch_bounds__(256) copyback_kernel(int32_t* __restrict__ perm,
                                                       const int32_t* __restrict__ perm_tmp, NodeArr nd,
                                                       int cnt, const int32_t* __restrict__ tile_off) {
  __shared__ int node_s;
  const int b = blockIdx.x;
  if (threadIdx.x == 0) node_s = find_node(tile_off, cnt, b);
  __syncthreads();
  const int k = node_s;
  const int64_t e0 = int64_t(nd.start[k]) + int64_t(b - tile_off[k]) * kTileElems;
  const int64_t e1 = min(int64_t(nd.start[k]) + nd.size[k], e0 + kTileElems);
  const int64_t e = e0 + threadIdx.x;
  if (e < e1) perm[e] = perm_tmp[e];
}

__global__ void children_count(NodeArr nd, int cnt, int leaf, const int32_t* tile_off, const int32_t* tile_left,
                               const int32_t* tile_left_off, uint8_t* leaf_flag, int32_t* child_cnt) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t nl = node_left(nd, k, tile_off, tile_left, tile_left_off);
  const int32_t nr = nd.size[k] - nl;
  const int64_t s = nd.start[k];
  if (nl <= leaf) leaf_flag[s] = 1;
  if (nr <= leaf) leaf_flag[s + nl] = 1;
  child_cnt[k] = (nl > leaf ? 1 : 0) + (nr > leaf ? 1 : 0);
}

__global__ void children_emit(NodeArr nd, int cnt, int leaf, const int32_t* tile_off, const int32_t* tile_left,
                              const int32_t* tile_left_off, const int32_t* child_off, NodeArr nx,
                              int64_t cap, unsigned* err) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t nl = node_left(nd, k, tile_off, tile_left, tile_left_off);
  const int32_t nr = nd.size[k] - nl;
  int32_t o = child_off[k];
  if (int64_t(o) + 2 > cap) {  // cannot happen: active nodes are disjoint and larger than leaf
    atomicOr(err, kErrBounds);
    return;
  }
  if (nl > leaf) {
    nx.start[o] = nd.start[k];
    nx.size[o] = nl;
    ++o;
  }
  if (nr > leaf) {
    nx.start[o] = nd.start[k] + nl;
    nx.size[o] = nr;
  }
}

inline unsigned grid1(int64_t n, int t = 256) { return unsigned((n + t - 1) / t); }

// Depth valve.  When pivots cannot separate a node (every member has the same
// code, so d1 == d2 sends all but p1 right) each level peels off one member and
// the depth grows with n; the reference recurses to that depth too.  Past
// kMaxLevels the remaining active nodes are cut into consecutive leaf_size
// leaves.  Real data stays far below (about 40 levels at 1M rows).
constexpr int kMaxLevels = 2048;

__global__ void chunk_leaves(NodeArr nd, int cnt, int leaf, uint8_t* leaf_flag) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int64_t s = nd.start[k], e = s + nd.size[k];
  for (int64_t p = s; p < e; p += leaf) leaf_flag[p] = 1;
}

}  // namespace

size_t forest_bytes(int64_t n, int T, int leaf, int64_t* max_nodes, int64_t* max_tiles) {
  const int64_t mn = int64_t(T) * (n / (leaf + 1) + 1) + 16;
  const int64_t mt = int64_t(T) * n / kTileElems + mn + 16;
  if (max_nodes) *max_nodes = mn;
  if (max_tiles) *max_tiles = mt;
  size_t b = 0;
  b += size_t(T) * n * 4;            // perm_tmp
  b += size_t(T) * n;                // side
  b += 2 * size_t(4 * mn) * 4;       // node generations
  b += size_t(mn + 1) * 4 * 2;       // tile_off, child_cnt
  b += size_t(mt) * 4 * 2;           // tile_left, tile_left_off
  b += scan_tmp_bytes(std::max(mn, mt)) + 4096;
  return b;
}

int run_forest(const int8_t* codes, int64_t n, int d, int T, int leaf, uint32_t seed, const int32_t* replay_host,
               int64_t n_replay, int32_t* perm, uint8_t* leaf_flag, const ForestBufs& fb, cudaStream_t s,
               int64_t* levels_out, std::string* err, const JobTable& jt, int roots_with_split) {
  auto fail = [&](cudaError_t e, const char* what) {
    if (err) *err = std::string(what) + ": " + cudaGetErrorString(e);
    return int(KNNG_E_CUDA);
  };
  cudaError_t e;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // replay table: sort by (level, tree, start) and index each level's slice
  std::vector<int32_t> rep;
  std::vector<int64_t> lvl_off;
  if (replay_host) {
    std::vector<int64_t> idx(n_replay);
    for (int64_t i = 0; i < n_replay; ++i) idx[i] = i;
    std::sort(idx.begin(), idx.end(), [&](int64_t a, int64_t b) {
      const int32_t* ra = replay_host + 6 * a;
      const int32_t* rb = replay_host + 6 * b;
      if (ra[1] != rb[1]) return ra[1] < rb[1];
      if (ra[0] != rb[0]) return ra[0] < rb[0];
      return ra[2] < rb[2];
    });
    rep.resize(6 * n_replay);
    for (int64_t i = 0; i < n_replay; ++i)
      std::copy(replay_host + 6 * idx[i], replay_host + 6 * idx[i] + 6, rep.begin() + 6 * i);
    int32_t maxl = n_replay ? rep[6 * (n_replay - 1) + 1] : -1;
    lvl_off.assign(size_t(maxl + 2), 0);
    for (int64_t i = 0; i < n_replay; ++i) lvl_off[size_t(rep[6 * i + 1]) + 1]++;
    for (size_t l = 1; l < lvl_off.size(); ++l) lvl_off[l] += lvl_off[l - 1];
    if (n_replay) {
      e = cudaMemcpyAsync(fb.replay_dev, rep.data(), rep.size() * 4, cudaMemcpyHostToDevice, s);
      if (e) return fail(e, "replay upload");
    }
  }
  e = cudaMemsetAsync(leaf_flag, 0, size_t(T) * n, s);
  if (e) return fail(e, "leaf_flag clear");
  e = cudaMemsetAsync(fb.err, 0, sizeof(unsigned), s);
  if (e) return fail(e, "err clear");
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  init_perm<<<std::min<int64_t>(grid1(n * T), int64_t(sms) * 16), 256, 0, s>>>(perm, n, T);
  note_launch();
  NodeArr cur = node_arr(fb.node_a, fb.max_nodes), nxt = node_arr(fb.node_b, fb.max_nodes);
  cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
  root_nodes<<<1, 64, 0, s>>>(cur, n, T, leaf, leaf_flag, jt, roots_with_split);
  note_launch();
  int64_t cnt = int64_t(T) * roots_with_split;
  int level = 0;
  int64_t host_i64[2];
  while (cnt > 0) {
    if (level >= kMaxLevels) {
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      chunk_leaves<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), leaf, leaf_flag);
      note_launch();
      break;
    }
    const int32_t* rep_dev = nullptr;
    if (replay_host) {
      if (size_t(level) + 1 >= lvl_off.size() || lvl_off[level + 1] - lvl_off[level] != cnt) {
        if (err) *err = "replay table does not match the forest at level " + std::to_string(level);
        return KNNG_E_REPLAY;
      }
      rep_dev = fb.replay_dev + 6 * lvl_off[level];
    }
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    pick_pivots<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), n, seed, level, perm, rep_dev, fb.child_cnt, fb.err, jt);
    note_launch();
    if ((e = exclusive_scan_i32(fb.child_cnt, fb.tile_off, cnt, fb.dev_i64, fb.scan_tmp, s))) return fail(e, "tile scan");
    if ((e = cudaMemcpyAsync(host_i64, fb.dev_i64, 8, cudaMemcpyDeviceToHost, s))) return fail(e, "tile count");
    if ((e = cudaStreamSynchronize(s))) return fail(e, "forest level");
    const int64_t tiles = host_i64[0];
    if (tiles > fb.max_tiles) {
      if (err) *err = "forest tile overflow";
      return KNNG_E_ARGS;
    }
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    side_kernel<<<unsigned(tiles), 256, 0, s>>>(codes, d, perm, cur, int(cnt), fb.tile_off, fb.side, fb.tile_left);
    note_launch();
    if ((e = exclusive_scan_i32(fb.tile_left, fb.tile_left_off, tiles, nullptr, fb.scan_tmp, s))) return fail(e, "left scan");
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    scatter_kernel<<<unsigned(tiles), 256, 0, s>>>(perm, fb.perm_tmp, cur, int(cnt), fb.tile_off, fb.side,
                                                   fb.tile_left, fb.tile_left_off);
    note_launch();
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    copyback_kernel<<<unsigned(tiles), 256, 0, s>>>(perm, fb.perm_tmp, cur, int(cnt), fb.tile_off);
    note_launch();
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    children_count<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), leaf, fb.tile_off, fb.tile_left, fb.tile_left_off,
                                              leaf_flag, fb.child_cnt);
    note_launch();
    if ((e = exclusive_scan_i32(fb.child_cnt, fb.child_cnt, cnt, fb.dev_i64 + 1, fb.scan_tmp, s))) return fail(e, "child scan");
    cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
    children_emit<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), leaf, fb.tile_off, fb.tile_left, fb.tile_left_off,
                                             fb.child_cnt, nxt, fb.max_nodes, fb.err);
    note_launch();
    if ((e = cudaMemcpyAsync(host_i64 + 1, fb.dev_i64 + 1, 8, cudaMemcpyDeviceToHost, s))) return fail(e, "child count");
    if ((e = cudaStreamSynchronize(s))) return fail(e, "forest level");
    cnt = host_i64[1];
    if (cnt > fb.max_nodes) {
      if (err) *err = "forest node overflow";
      return KNNG_E_ARGS;
    }
    std::swap(cur, nxt);
    ++level;
  }
  unsigned herr = 0;
  if ((e = cudaMemcpyAsync(&herr, fb.err, sizeof(unsigned), cudaMemcpyDeviceToHost, s))) return fail(e, "err read");
  if ((e = cudaStreamSynchronize(s))) return fail(e, "forest");
  if (herr & kErrBounds) {
    if (err) *err = "forest node list overflow";
    return KNNG_E_ARGS;
  }
  if (herr & kErrReplay) {
    if (err) *err = "replay pivot table does not match the forest nodes";
    return KNNG_E_REPLAY;
  }
  if (replay_host && size_t(level) + 1 != lvl_off.size()) {
    if (err) *err = "replay table has more levels than the forest";
    return KNNG_E_REPLAY;
  }
  if (levels_out) *levels_out = level;
  return 0;
}

}  // namespace knng
