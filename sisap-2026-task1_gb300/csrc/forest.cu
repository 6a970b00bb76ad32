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
//
// Fused levels (native pivots, the default): the side pass is HBM-bound on
// reading every active member's code row once per level, so large nodes are
// split kFuse levels at a time from one read of each row.  A node's pivots
// and those of its descendants down to kFuse - 1 levels below are fixed
// before the pass from a seeded sample of up to kCand distinct members (the
// node's "candidates", in a hashed order): the node's pivots are the first
// two candidates; a descendant's are the first two candidates, not already
// an ancestor's pivot, that the splits above it send into it -- each
// candidate's path is computed with the same exact dot products the member
// pass uses, so these pivots are members of the descendant.  Given the
// ancestors' splits, the candidates in a descendant are a uniform sample of
// its members, so a descendant's pivot pair is a uniformly drawn pair of its
// distinct members other than its ancestors' pivots, as in the per-level
// rule.  A descendant that receives fewer than two free candidates is not
// split in the pass and is queued as a node of its own.  The member pass
// then gives every member a kFuse-bit path code (first split in the high
// bit; bits below an unsplit descendant are 0), and one stable counting
// sort by code per node lays out all kFuse levels at once: each descendant
// is a contiguous range, left before right, as the per-level splits would
// leave it (inside a descendant that turns out to be a leaf the members
// are also ordered by the deeper bits, which no later stage depends on).
// Nodes smaller than kFuseMin take the per-level path after the fused
// rounds (the sample would be a large fraction of them).
#include "knng_internal.cuh"

#include <algorithm>
#include <vector>

namespace knng {
namespace {

constexpr int kTileElems = 256;
constexpr int kFuse = 3;                        // levels per fused pass
constexpr int kFuseNodes = (1 << kFuse) - 1;    // split nodes of one fused subtree (depth 0 .. kFuse-1)
constexpr int kFuseBins = 1 << kFuse;           // path codes
constexpr int kCand = 64;                       // pivot candidates per fused node
constexpr int32_t kFuseMin = 512;               // smaller nodes take the per-level path

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

// ---- fused levels ------------------------------------------------------------

__device__ __forceinline__ int64_t gcd64(int64_t a, int64_t b) {
  while (b) {
    const int64_t t = a % b;
    a = b;
    b = t;
  }
  return a;
}

// 8-lane partial dot of a member row (v: chunks sub, sub+8, ... in registers)
// with a row in shared memory.
__device__ __forceinline__ int dot_chunks(const uint4* v, const uint4* row, int sub, int per_lane) {
  int acc = 0;
#pragma unroll
  for (int u = 0; u < kMaxDim / 128; ++u) {
    if (u < per_lane) {
      const uint4 a = row[sub + 8 * u];
      acc = __dp4a(int(v[u].x), int(a.x), acc);
      acc = __dp4a(int(v[u].y), int(a.y), acc);
      acc = __dp4a(int(v[u].z), int(a.z), acc);
      acc = __dp4a(int(v[u].w), int(a.w), acc);
    }
  }
  return acc;
}

// Pivot table of fused node k, one warp per node: piv[k][2j], piv[k][2j+1]
// are the pivots of descendant j (j = 0 the node; 2j+1 and 2j+2 the left and
// right children of j), or -1 where j is not split in the pass.  The node's
// candidates are the members at positions a + q*b (mod size), q < S, with b
// coprime to size (distinct positions), in q order; node identity is
// job-local, as for pick_pivots.
__global__ void __launch_bounds__(256) fuse_pivots(NodeArr nd, int cnt, int64_t n, uint32_t seed,
                                                   const int32_t* __restrict__ perm,
                                                   const int8_t* __restrict__ codes, int d,
                                                   int32_t* __restrict__ piv, int32_t* __restrict__ tile_cnt,
                                                   JobTable jt) {
  __shared__ int32_t s_side[8][kCand];
  __shared__ int32_t s_pv[8][2 * kFuseNodes];
  const unsigned full = 0xffffffffu;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, sub = lane & 7, slot = lane >> 3;
  const int64_t k = (int64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  if (k >= cnt) return;  // whole warps
  const int32_t start = nd.start[k], size = nd.size[k];
  const int32_t tree = int32_t(int64_t(start) / n);
  const int32_t in_tree = int32_t(int64_t(start) - int64_t(tree) * n);
  const int32_t local = in_tree - jt.off[job_of(jt, in_tree)];
  uint64_t h = splitmix64((uint64_t(seed) << 32) ^ uint64_t(uint32_t(tree)));
  h = splitmix64(h ^ uint64_t(uint32_t(local)));
  h = splitmix64(h ^ (uint64_t(uint32_t(size)) << 1));
  const uint64_t h2 = splitmix64(h ^ 0x2545F4914F6CDD1Dull);
  const int64_t a = int64_t(h % uint64_t(size));
  int64_t b = 1 + int64_t(h2 % uint64_t(size - 1));  // size > leaf_size >= 2
  while (gcd64(b, size) != 1) b = b + 1 == size ? 1 : b + 1;
  const int S = size < kCand ? int(size) : kCand;
  int32_t cid[2];
  int cnode[2];
  bool cused[2];
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int q = lane + 32 * u;
    cused[u] = false;
    if (q < S) {
      cid[u] = perm[start + (a + int64_t(q) * b) % size];
      cnode[u] = 0;
    } else {
      cid[u] = -1;
      cnode[u] = -1;
    }
  }
  if (lane < 2 * kFuseNodes) s_pv[w][lane] = -1;
  __syncwarp();
  const int per_lane = d / 128;
  for (int dk = 0; dk < kFuse; ++dk) {
    const int j0 = (1 << dk) - 1;
    // pivots of the depth-dk nodes: the two lowest-q free candidates in each
    for (int j = j0; j < 2 * j0 + 1; ++j) {
      const unsigned m0 = __ballot_sync(full, cnode[0] == j && !cused[0]);
      const unsigned m1 = __ballot_sync(full, cnode[1] == j && !cused[1]);
      uint64_t m = uint64_t(m0) | (uint64_t(m1) << 32);
      if (__popcll(m) >= 2) {  // warp-uniform
        const int q1 = __ffsll(m) - 1;
        m &= m - 1;
        const int q2 = __ffsll(m) - 1;
        const int32_t p1 = __shfl_sync(full, (q1 >> 5) ? cid[1] : cid[0], q1 & 31);
        const int32_t p2 = __shfl_sync(full, (q2 >> 5) ? cid[1] : cid[0], q2 & 31);
        if (lane == (q1 & 31)) cused[q1 >> 5] = true;
        if (lane == (q2 & 31)) cused[q2 >> 5] = true;
        if (lane == 0) {
          s_pv[w][2 * j] = p1;
          s_pv[w][2 * j + 1] = p2;
        }
      }
    }
    __syncwarp();
    if (dk + 1 == kFuse) break;  // no pivots below the last fused level
    // every candidate in a split depth-dk node takes its side (8 lanes per candidate)
    for (int g = 0; g < S; g += 4) {
      const int q = g + slot, half = g >> 5;  // g % 4 == 0: the 4 candidates share a half
      const int32_t myid = __shfl_sync(full, half ? cid[1] : cid[0], q & 31);
      const int jn = __shfl_sync(full, half ? cnode[1] : cnode[0], q & 31);
      const int32_t p1 = (q < S && jn >= 0) ? s_pv[w][2 * jn] : -1;
      const int32_t p2 = (q < S && jn >= 0) ? s_pv[w][2 * jn + 1] : -1;
      const bool live = p1 >= 0;
      int d1 = 0, d2 = 0;
      if (live) {
        const uint4* x = reinterpret_cast<const uint4*>(codes + int64_t(myid) * d);
        const uint4* r1 = reinterpret_cast<const uint4*>(codes + int64_t(p1) * d);
        const uint4* r2 = reinterpret_cast<const uint4*>(codes + int64_t(p2) * d);
        for (int u = 0; u < per_lane; ++u) {
          const uint4 xv = __ldg(x + sub + 8 * u), av = __ldg(r1 + sub + 8 * u), cv = __ldg(r2 + sub + 8 * u);
          d1 = __dp4a(int(xv.x), int(av.x), d1);
          d1 = __dp4a(int(xv.y), int(av.y), d1);
          d1 = __dp4a(int(xv.z), int(av.z), d1);
          d1 = __dp4a(int(xv.w), int(av.w), d1);
          d2 = __dp4a(int(xv.x), int(cv.x), d2);
          d2 = __dp4a(int(xv.y), int(cv.y), d2);
          d2 = __dp4a(int(xv.z), int(cv.z), d2);
          d2 = __dp4a(int(xv.w), int(cv.w), d2);
        }
      }
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        d1 += __shfl_xor_sync(full, d1, o);
        d2 += __shfl_xor_sync(full, d2, o);
      }
      const int sd = myid == p1 ? 0 : myid == p2 ? 1 : (d1 > d2 ? 0 : 1);
      if (sub == 0 && q < S) s_side[w][q] = live ? sd : -1;
    }
    __syncwarp();
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int q = lane + 32 * u;
      if (q < S && cnode[u] >= 0) {
        const int sd = s_side[w][q];
        cnode[u] = sd < 0 ? -1 : 2 * cnode[u] + 1 + sd;
      }
    }
    __syncwarp();
  }
  if (lane < 2 * kFuseNodes) piv[k * (2 * kFuseNodes) + lane] = s_pv[w][lane];
  if (lane == 0) tile_cnt[k] = (size + kTileElems - 1) / kTileElems;
}

// Member pass of the fused levels: one block per tile of <= 256 members of one
// node, the node's (up to 14) pivot rows staged in shared memory; 8 lanes per
// member hold its code row in registers and walk its path down the fused
// levels.  side[e] = the member's path code; per tile and code the member
// count, at bins[8*f + code*nt + (tile - f)] (f: the node's first tile, nt:
// its tile count), so one exclusive scan of bins gives every member's place.
__global__ void __launch_bounds__(256) fuse_side(const int8_t* __restrict__ codes, int d,
                                                 const int32_t* __restrict__ perm, NodeArr nd, int cnt,
                                                 const int32_t* __restrict__ tile_off,
                                                 const int32_t* __restrict__ piv, uint8_t* __restrict__ side,
                                                 int32_t* __restrict__ bins) {
  __shared__ uint4 prow[2 * kFuseNodes][kMaxDim / 16];
  __shared__ int32_t spv[2 * kFuseNodes];
  __shared__ int32_t sbins[kFuseBins];
  __shared__ int node_s;
  const unsigned full = 0xffffffffu;
  const int b = blockIdx.x, tid = threadIdx.x;
  if (tid == 0) node_s = find_node(tile_off, cnt, b);
  if (tid < kFuseBins) sbins[tid] = 0;
  __syncthreads();
  const int k = node_s;
  if (tid < 2 * kFuseNodes) spv[tid] = piv[int64_t(k) * (2 * kFuseNodes) + tid];
  __syncthreads();
  const int nchunk = d / 16;
  for (int c = tid; c < 2 * kFuseNodes * nchunk; c += blockDim.x) {
    const int r = c / nchunk, cc = c % nchunk;
    const int32_t id = spv[r];
    if (id >= 0) prow[r][cc] = __ldg(reinterpret_cast<const uint4*>(codes + int64_t(id) * d) + cc);
  }
  __syncthreads();
  const int32_t start = nd.start[k], size = nd.size[k];
  const int f = tile_off[k], nt = (size + kTileElems - 1) / kTileElems;
  const int64_t e0 = int64_t(start) + int64_t(b - f) * kTileElems;
  const int64_t e1 = min(int64_t(start) + size, e0 + kTileElems);
  const int lane = tid & 31, warp = tid >> 5, sub = lane & 7, slot = lane >> 3;
  const int per_lane = d / 128;
  for (int step = 0; step < 8; ++step) {
    const int t = warp * 32 + step * 4 + slot;
    const int64_t e = e0 + t;
    const bool valid = e < e1;
    const int32_t id = valid ? perm[e] : -1;
    uint4 v[kMaxDim / 128];
    if (valid) {
      const uint4* row = reinterpret_cast<const uint4*>(codes + int64_t(id) * d);
#pragma unroll
      for (int u = 0; u < kMaxDim / 128; ++u)
        if (u < per_lane) v[u] = __ldg(row + sub + 8 * u);
    }
    int j = 0, code = 0;
    bool live = valid;
#pragma unroll
    for (int dk = 0; dk < kFuse; ++dk) {
      const int32_t p1 = live ? spv[2 * j] : -1, p2 = live ? spv[2 * j + 1] : -1;
      const bool act = p1 >= 0;
      int d1 = 0, d2 = 0;
      if (act) {
        d1 = dot_chunks(v, prow[2 * j], sub, per_lane);
        d2 = dot_chunks(v, prow[2 * j + 1], sub, per_lane);
      }
#pragma unroll
      for (int o = 1; o < 8; o <<= 1) {
        d1 += __shfl_xor_sync(full, d1, o);
        d2 += __shfl_xor_sync(full, d2, o);
      }
      if (act) {
        const int bit = id == p1 ? 0 : id == p2 ? 1 : (d1 > d2 ? 0 : 1);
        code |= bit << (kFuse - 1 - dk);
        j = 2 * j + 1 + bit;
      } else {
        live = false;
      }
    }
    if (valid && sub == 0) {
      side[e] = uint8_t(code);
      atomicAdd(&sbins[code], 1);
    }
  }
  __syncthreads();
  if (tid < kFuseBins) bins[8 * int64_t(f) + int64_t(tid) * nt + (b - f)] = sbins[tid];
}

// Stable counting sort of each node's members by path code into perm_tmp.
__global__ void __launch_bounds__(256) fuse_scatter(const int32_t* __restrict__ perm,
                                                    int32_t* __restrict__ perm_tmp, NodeArr nd, int cnt,
                                                    const int32_t* __restrict__ tile_off,
                                                    const uint8_t* __restrict__ side,
                                                    const int32_t* __restrict__ bins_off) {
  __shared__ int node_s;
  __shared__ int32_t wcnt[8][kFuseBins];
  const int b = blockIdx.x, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) node_s = find_node(tile_off, cnt, b);
  __syncthreads();
  const int k = node_s;
  const int32_t start = nd.start[k], size = nd.size[k];
  const int f = tile_off[k], nt = (size + kTileElems - 1) / kTileElems;
  const int64_t e0 = int64_t(start) + int64_t(b - f) * kTileElems;
  const int64_t e1 = min(int64_t(start) + size, e0 + kTileElems);
  const int64_t e = e0 + tid;
  const bool valid = e < e1;
  const int code = valid ? int(side[e]) : kFuseBins;
  int rank = 0;
#pragma unroll
  for (int v = 0; v < kFuseBins; ++v) {
    const unsigned bal = __ballot_sync(0xffffffffu, code == v);
    if (code == v) rank = __popc(bal & ((1u << lane) - 1u));
    if (lane == 0) wcnt[warp][v] = __popc(bal);
  }
  __syncthreads();
  if (valid) {
    int pre = 0;
    for (int w = 0; w < warp; ++w) pre += wcnt[w][code];
    const int64_t base = int64_t(8) * f;
    const int32_t before = bins_off[base + int64_t(code) * nt + (b - f)] - bins_off[base];
    perm_tmp[int64_t(start) + before + pre + rank] = perm[e];
  }
}

// After a fused pass: the sizes of node k's descendants from the scanned code
// counts; leaves are flagged, and every descendant that is neither a leaf nor
// split in the pass becomes a node: of the next fused round when it has at
// least kFuseMin members, else of the per-level phase.  emit = 0 counts them
// per node (and sets the leaf flags), emit = 1 writes them at the scanned
// offsets.
__global__ void fuse_children(NodeArr nd, int cnt, int leaf, const int32_t* __restrict__ tile_off,
                              const int32_t* __restrict__ bins_off, const int32_t* __restrict__ piv,
                              uint8_t* __restrict__ leaf_flag, int emit, int32_t* cnt_big, int32_t* cnt_small,
                              NodeArr big, NodeArr small, int64_t small_base, int64_t cap, unsigned* err) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= cnt) return;
  const int32_t start = nd.start[k], size = nd.size[k];
  const int f = tile_off[k], nt = (size + kTileElems - 1) / kTileElems;
  const int64_t base = int64_t(8) * f;
  int32_t pre[kFuseBins + 1];
  pre[0] = 0;
#pragma unroll
  for (int v = 0; v + 1 < kFuseBins; ++v) pre[v + 1] = bins_off[base + int64_t(v + 1) * nt] - bins_off[base];
  pre[kFuseBins] = size;
  bool split[kFuseNodes];
#pragma unroll
  for (int j = 0; j < kFuseNodes; ++j) split[j] = j == 0;
  int64_t ob = emit ? cnt_big[k] : 0, os = emit ? small_base + cnt_small[k] : 0;
  int nb = 0, ns = 0;
#pragma unroll
  for (int j = 0; j < kFuseNodes; ++j) {
    if (!split[j]) continue;
    const int dk = 31 - __clz(j + 1), cd = dk + 1;
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      const int ch = 2 * j + 1 + sd, p = ch - ((1 << cd) - 1);
      const int lo = p << (kFuse - cd), hi = (p + 1) << (kFuse - cd);
      const int32_t csize = pre[hi] - pre[lo];
      const int64_t cstart = int64_t(start) + pre[lo];
      if (csize <= 0) {  // cannot happen: a split sends its two pivots to different sides
        atomicOr(err, kErrBounds);
      } else if (csize <= leaf) {
        if (!emit) leaf_flag[cstart] = 1;
      } else if (cd < kFuse && piv[int64_t(k) * (2 * kFuseNodes) + 2 * ch] >= 0) {
        split[ch] = true;
      } else if (csize >= kFuseMin) {
        if (emit) {
          if (ob >= cap) {
            atomicOr(err, kErrBounds);
          } else {
            big.start[ob] = int32_t(cstart);
            big.size[ob] = csize;
          }
        }
        ++ob;
        ++nb;
      } else {
        if (emit) {
          if (os >= cap) {
            atomicOr(err, kErrBounds);
          } else {
            small.start[os] = int32_t(cstart);
            small.size[os] = csize;
          }
        }
        ++os;
        ++ns;
      }
    }
  }
  if (!emit) {
    cnt_big[k] = nb;
    cnt_small[k] = ns;
  }
}

}  // namespace

size_t forest_bytes(int64_t n, int T, int leaf, int64_t* max_nodes, int64_t* max_tiles) {
  const int64_t mn = int64_t(T) * (n / (leaf + 1) + 1) + 16;
  const int64_t mt = int64_t(T) * n / kTileElems + mn + 16;
  if (max_nodes) *max_nodes = mn;
  if (max_tiles) *max_tiles = mt;
  size_t b = 0;
  b += size_t(T) * n * 4;                      // perm_tmp
  b += size_t(T) * n;                          // side (path codes)
  b += 3 * size_t(4 * mn) * 4;                 // node generations, parked nodes
  b += size_t(mn + 1) * 4 * 3;                 // tile_off, child_cnt, child_cnt2
  b += size_t(mn) * (2 * kFuseNodes) * 4;      // pivot tables
  b += 2 * size_t(kFuseBins) * size_t(mt) * 4; // tile_bins, tile_bins_off (tile_left, tile_left_off)
  b += scan_tmp_bytes(std::max<int64_t>(mn, int64_t(kFuseBins) * mt)) + 4096;
  return b;
}

int run_forest(const int8_t* codes, int64_t n, int d, int T, int leaf, uint32_t seed, const int32_t* replay_host,
               int64_t n_replay, int32_t* perm, uint8_t* leaf_flag, const ForestBufs& fb, cudaStream_t s,
               int64_t* levels_out, std::string* err, const JobTable& jt, int roots_with_split, int fuse) {
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
  int64_t host_i64[3];
  if (fuse && !replay_host) {
    // fused rounds: kFuse levels per pass over nodes of >= kFuseMin members;
    // smaller nodes collect in `parked` for the per-level loop below
    NodeArr parked = node_arr(fb.node_c, fb.max_nodes);
    int64_t nparked = 0;
    while (cnt > 0 && level < kMaxLevels) {
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      fuse_pivots<<<grid1(cnt * 32), 256, 0, s>>>(cur, int(cnt), n, seed, perm, codes, d, fb.piv, fb.child_cnt,
                                                   jt);
      note_launch();
      if ((e = exclusive_scan_i32(fb.child_cnt, fb.tile_off, cnt, fb.dev_i64, fb.scan_tmp, s))) return fail(e, "tile scan");
      if ((e = cudaMemcpyAsync(host_i64, fb.dev_i64, 8, cudaMemcpyDeviceToHost, s))) return fail(e, "tile count");
      if ((e = cudaStreamSynchronize(s))) return fail(e, "fused forest round");
      const int64_t tiles = host_i64[0];
      if (tiles > fb.max_tiles) {
        if (err) *err = "forest tile overflow";
        return KNNG_E_ARGS;
      }
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      fuse_side<<<unsigned(tiles), 256, 0, s>>>(codes, d, perm, cur, int(cnt), fb.tile_off, fb.piv, fb.side,
                                                fb.tile_bins);
      note_launch();
      if ((e = exclusive_scan_i32(fb.tile_bins, fb.tile_bins_off, int64_t(kFuseBins) * tiles, nullptr, fb.scan_tmp, s)))
        return fail(e, "code scan");
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      fuse_scatter<<<unsigned(tiles), 256, 0, s>>>(perm, fb.perm_tmp, cur, int(cnt), fb.tile_off, fb.side,
                                                   fb.tile_bins_off);
      note_launch();
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      copyback_kernel<<<unsigned(tiles), 256, 0, s>>>(perm, fb.perm_tmp, cur, int(cnt), fb.tile_off);
      note_launch();
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      fuse_children<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), leaf, fb.tile_off, fb.tile_bins_off, fb.piv, leaf_flag,
                                               0, fb.child_cnt, fb.child_cnt2, nxt, parked, nparked, fb.max_nodes,
                                               fb.err);
      note_launch();
      if ((e = exclusive_scan_i32(fb.child_cnt, fb.child_cnt, cnt, fb.dev_i64 + 1, fb.scan_tmp, s)) ||
          (e = exclusive_scan_i32(fb.child_cnt2, fb.child_cnt2, cnt, fb.dev_i64 + 2, fb.scan_tmp, s)))
        return fail(e, "child scan");
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      fuse_children<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), leaf, fb.tile_off, fb.tile_bins_off, fb.piv, leaf_flag,
                                               1, fb.child_cnt, fb.child_cnt2, nxt, parked, nparked, fb.max_nodes,
                                               fb.err);
      note_launch();
      if ((e = cudaMemcpyAsync(host_i64 + 1, fb.dev_i64 + 1, 16, cudaMemcpyDeviceToHost, s))) return fail(e, "child count");
      if ((e = cudaStreamSynchronize(s))) return fail(e, "fused forest round");
      cnt = host_i64[1];
      nparked += host_i64[2];
      if (cnt > fb.max_nodes || nparked > fb.max_nodes) {
        if (err) *err = "forest node overflow";
        return KNNG_E_ARGS;
      }
      std::swap(cur, nxt);
      level += kFuse;
    }
    if (cnt > 0) {  // depth valve (see kMaxLevels): the rest become consecutive leaves
      cudaGetLastError();  // clear a stale, non-sticky error: the launch reports only its own
      chunk_leaves<<<grid1(cnt), 256, 0, s>>>(cur, int(cnt), leaf, leaf_flag);
      note_launch();
    }
    // the per-level loop takes the parked nodes
    cnt = nparked;
    nxt = cur.start == fb.node_a ? node_arr(fb.node_b, fb.max_nodes) : node_arr(fb.node_a, fb.max_nodes);
    cur = parked;
  }
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
