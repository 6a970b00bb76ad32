// api.cu -- C ABI of libknng: context, device arena and the build pipeline.
//
// knng_build runs the reference's stages (src/main.cpp:179-457) on one GPU,
// stream-ordered on the context's stream:
//   quantise+sketch (K1) -> forest (K2) -> leaf Gram + init merge (K3/K4)
//   -> NN-Descent iterations (K5, early stop on the host as :432-439)
//   -> export (K6).
// Host syncs happen only where the reference's control flow needs a device
// value: node/tile counts per forest level, the leaf count, and one update
// count per NN-Descent iteration.
#include "knng_internal.cuh"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <vector>

#include <atomic>
#include <mutex>
#include <thread>
#include <cmath>
#include <map>

namespace knng {
size_t join_smem_bytes(int K, int R, int d);
namespace {
std::atomic<int64_t> g_launches{0};
}
std::mutex g_capture_mu;
int64_t launches() { return g_launches.load(std::memory_order_relaxed); }

namespace {
std::mutex g_attr_mu;
std::map<const void*, size_t> g_attr_max;
}  // namespace

cudaError_t ensure_smem_attr(const void* func, size_t bytes) {
  std::lock_guard<std::mutex> lk(g_attr_mu);
  size_t& cur = g_attr_max[func];
  if (bytes <= cur) return cudaSuccess;
  const cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes));
  if (e != cudaSuccess) {
    cudaGetLastError();
    return e;
  }
  cur = bytes;
  return cudaSuccess;
}
void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
}  // namespace knng

using namespace knng;

constexpr int kMaxIterEvents = 2 * 64 + 2;

// A context-owned device buffer, allocated and freed in the order of the
// context's stream (the device's stream-ordered pool), so growing or trimming
// one context never synchronises the device under other contexts' work.
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaStream_t s = nullptr;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMallocAsync(&p, want, s);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFreeAsync(p, s);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as(size_t byte_off = 0) const {
    return reinterpret_cast<T*>(static_cast<char*>(p) + byte_off);
  }
};

// (ctas_per_sm, cblock) of the join for its first two iterations, where most
// candidates are new, and for the later ones, where the candidate cache serves
// most of them: the two favour different occupancy/in-flight trade-offs.
struct JoinCfg {
  std::pair<int, int> early{4, 4}, late{4, 4};
};

struct knng_ctx {
  knng_params prm{};
  int device = 0;
  int num_sms = 0;
  int pageable_access = 0;  // the device reads pageable host memory coherently (NVLink-C2C / ATS)
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  cudaEvent_t jev[2] = {};
  cudaEvent_t bev = nullptr;  // start of a batch (all dimension groups wait on it)
  cudaEvent_t freed[2] = {};  // pinned input slot s is free again once freed[s] completes
  // pageable caller memory goes through these pinned buffers, copied by host threads
  PinnedBuf pin_in, pin_out;
  std::unique_ptr<CopyPool> pool;
  void host_copy(void* dst, const void* src, size_t bytes) {
    if (!pool) pool.reset(new (std::nothrow) CopyPool(host_copy_threads()));
    if (pool) pool->copy(dst, src, bytes);
    else std::memcpy(dst, src, bytes);
  }
  cudaEvent_t itev[kMaxIterEvents] = {};
  std::string last_error;
  DevBuf codes, sketch, graph, perm, leaf_flag, scratch, outbuf, scalars, jobs, hsketch, rowflags;
  // join phase captured as a CUDA graph, reused while the launch key matches
  cudaGraphExec_t join_graph = nullptr;
  std::vector<uintptr_t> join_graph_key;
  // autotuned join configurations per (d, log2 rows): (ctas_per_sm, cblock) for
  // the first two iterations and for the later, cache-served ones
  std::map<std::pair<int, int>, JoinCfg> tuned;
  std::vector<knng_ctx*> subs;  // contexts of the second and later dimension groups of a batch
  std::vector<DevBuf*> buffers() {
    return {&codes, &sketch, &graph, &perm, &leaf_flag, &scratch, &outbuf, &scalars, &jobs, &hsketch, &rowflags};
  }
  // the sketches the join scores and their 64-bit words per row
  bool hyperplane() const { return prm.sketch_mode == KNNG_SKETCH_HYPERPLANE; }
  const uint64_t* join_sketch() const { return hyperplane() ? hsketch.as<uint64_t>() : sketch.as<uint64_t>(); }
  int sketch_words(int d) const { return hyperplane() ? 2 : d / 64; }
};

namespace {

constexpr int64_t kStageRows = 1 << 16;  // host-input rows per H2D chunk (256 MB at d = 1024)
// byte offset in the context's 4096-byte scalar block of the bounds-checked
// build's error word (the forest uses bytes 0..67, the initial graph 128..159,
// knng_join_iter's counters 256..319)
constexpr size_t kCheckWord = 768;

int set_error(knng_ctx* c, int status, const std::string& msg) {
  if (c) c->last_error = msg;
  return status;
}

int cuda_fail(knng_ctx* c, cudaError_t e, const char* what) {
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    return set_error(c, KNNG_E_OOM, std::string(what) + ": " + cudaGetErrorString(e));
  }
  return set_error(c, KNNG_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

int check_params(knng_ctx* c, const knng_params& p) {
  if (p.k_build < 1 || p.k_build > kMaxK) return set_error(c, KNNG_E_ARGS, "k_build must be in [1, 64]");
  if (p.k_eval < 1 || p.k_eval > p.k_build) return set_error(c, KNNG_E_ARGS, "k_eval must be in [1, k_build]");
  if (p.num_trees < 1 || p.num_trees > 64) return set_error(c, KNNG_E_ARGS, "num_trees must be in [1, 64]");
  if (p.leaf_size < 2 || p.leaf_size > kMaxLeaf) return set_error(c, KNNG_E_ARGS, "leaf_size must be in [2, 64]");
  if (p.rerank_mult < 1 || p.k_build * p.rerank_mult > 4096)
    return set_error(c, KNNG_E_ARGS, "rerank_mult must be >= 1 with k_build * rerank_mult <= 4096");
  if (p.max_iterations < 0 || p.max_iterations > 64) return set_error(c, KNNG_E_ARGS, "max_iterations must be in [0, 64]");
  if (p.quant_mode != KNNG_QUANT_TRUNC && p.quant_mode != KNNG_QUANT_ROUND) return set_error(c, KNNG_E_ARGS, "bad quant_mode");
  if (p.join_mode != KNNG_JOIN_JACOBI && p.join_mode != KNNG_JOIN_INPLACE) return set_error(c, KNNG_E_ARGS, "bad join_mode");
  if (p.row_order != KNNG_ORDER_NATURAL && p.row_order != KNNG_ORDER_LEAF) return set_error(c, KNNG_E_ARGS, "bad row_order");
  if (p.gram_mode != KNNG_GRAM_DP4A && p.gram_mode != KNNG_GRAM_TCGEN05) return set_error(c, KNNG_E_ARGS, "bad gram_mode");
  if (p.init_mode != KNNG_INIT_FOREST && p.init_mode != KNNG_INIT_RANDOM && p.init_mode != KNNG_INIT_BLOCK)
    return set_error(c, KNNG_E_ARGS, "bad init_mode");
  if (p.init_mode == KNNG_INIT_BLOCK && (p.block_size < 1 || p.bridges < 0 || p.bridges > p.k_build))
    return set_error(c, KNNG_E_ARGS, "block init needs block_size >= 1 and bridges in [0, k_build]");
  if (p.join_cache != 0 && p.join_cache != 1) return set_error(c, KNNG_E_ARGS, "join_cache must be 0 or 1");
  if (p.join_ctas_per_sm != 0 &&
      (p.join_ctas_per_sm < 3 || p.join_ctas_per_sm > 4 || (p.join_cblock != 2 && p.join_cblock != 4 && p.join_cblock != 8)))
    return set_error(c, KNNG_E_ARGS, "join_ctas_per_sm must be 0, or 3 or 4 with join_cblock 2, 4 or 8");
  if (p.sketch_mode != KNNG_SKETCH_SIGN && p.sketch_mode != KNNG_SKETCH_HYPERPLANE)
    return set_error(c, KNNG_E_ARGS, "bad sketch_mode");
  if (p.forest_fuse != 0 && p.forest_fuse != 1) return set_error(c, KNNG_E_ARGS, "forest_fuse must be 0 or 1");
  return KNNG_OK;
}

int check_shape(knng_ctx* c, int64_t n, int d) {
  if (n < 2) return set_error(c, KNNG_E_ARGS, "n must be >= 2");
  if (!dim_ok(d)) return set_error(c, KNNG_E_DIM, "d must be a multiple of 128 in [128, 1024]");
  if (c && int64_t(c->prm.num_trees) * n > INT32_MAX) return set_error(c, KNNG_E_ARGS, "num_trees * n must fit in int32");
  return KNNG_OK;
}

struct Scratch {
  ForestBufs fb{};
  InitBufs ib{};
};

size_t carve(char*& p, size_t bytes) {
  size_t b = (bytes + 255) & ~size_t(255);
  p += b;
  return b;
}

// Lays the forest or the init scratch over the ctx scratch region (the two are
// never live at the same time); the region is at least min_bytes long (the
// candidate cache, which a build lays over it after the initial graph).
int ensure_scratch(knng_ctx* c, int64_t n, Scratch* s, int64_t n_replay, size_t min_bytes = 0) {
  const int T = c->prm.num_trees, L = c->prm.leaf_size;
  int64_t mn = 0, mt = 0;
  const size_t fbytes = forest_bytes(n, T, L, &mn, &mt) + size_t(n_replay) * 24 + 8192;
  const size_t ibytes = init_bytes(n, T, L) + 8192;
  cudaError_t e = c->scratch.ensure(std::max(std::max(fbytes, ibytes), min_bytes));
  if (e) return cuda_fail(c, e, "scratch allocation");
  e = c->scalars.ensure(4096);
  if (e) return cuda_fail(c, e, "scalar allocation");
  const size_t tn = size_t(T) * n;
  {
    char* p = c->scratch.as<char>();
    ForestBufs& f = s->fb;
    f.max_nodes = mn;
    f.max_tiles = mt;
    f.perm_tmp = reinterpret_cast<int32_t*>(p); carve(p, tn * 4);
    f.side = reinterpret_cast<uint8_t*>(p); carve(p, tn);
    f.node_a = reinterpret_cast<int32_t*>(p); carve(p, size_t(4 * mn) * 4);
    f.node_b = reinterpret_cast<int32_t*>(p); carve(p, size_t(4 * mn) * 4);
    f.node_c = reinterpret_cast<int32_t*>(p); carve(p, size_t(4 * mn) * 4);
    f.tile_off = reinterpret_cast<int32_t*>(p); carve(p, size_t(mn + 1) * 4);
    f.child_cnt = reinterpret_cast<int32_t*>(p); carve(p, size_t(mn + 1) * 4);
    f.child_cnt2 = reinterpret_cast<int32_t*>(p); carve(p, size_t(mn + 1) * 4);
    f.piv = reinterpret_cast<int32_t*>(p); carve(p, size_t(mn) * 14 * 4);
    f.tile_bins = reinterpret_cast<int32_t*>(p); carve(p, size_t(8) * mt * 4);
    f.tile_bins_off = reinterpret_cast<int32_t*>(p); carve(p, size_t(8) * mt * 4);
    f.tile_left = f.tile_bins;  // the per-level path's tile counts (never live with the fused ones)
    f.tile_left_off = f.tile_bins_off;
    f.replay_dev = reinterpret_cast<int32_t*>(p); carve(p, size_t(n_replay) * 24 + 16);
    f.scan_tmp = p; carve(p, scan_tmp_bytes(std::max<int64_t>(mn, 8 * mt)));
    f.dev_i64 = c->scalars.as<int64_t>(0);
    f.err = c->scalars.as<unsigned>(64);
  }
  {
    char* p = c->scratch.as<char>();
    InitBufs& b = s->ib;
    b.pos = reinterpret_cast<int32_t*>(p); carve(p, tn * 4);
    b.leaf_lo = reinterpret_cast<int32_t*>(p); carve(p, tn * 4);
    b.leaf_idx = reinterpret_cast<int32_t*>(p); carve(p, tn * 8);
    b.leaf_sz = reinterpret_cast<uint8_t*>(p); carve(p, tn);
    b.fix_rows = reinterpret_cast<int32_t*>(p); carve(p, size_t(n) * 4);
    b.scan_tmp = p; carve(p, scan_tmp_bytes(int64_t(tn)));
    b.dev_i64 = c->scalars.as<int64_t>(128);
    // the leaf Gram rows take the rest of the region: at least one chunk of
    // init_gram_trees(T) trees (init_bytes), more when the region was sized
    // for the candidate cache
    b.gram = reinterpret_cast<int32_t*>(p);
    b.gram_rows = int64_t((c->scratch.bytes - size_t(p - c->scratch.as<char>())) / (kMaxLeaf * 4));
  }
  return KNNG_OK;
}

// Job table of one job covering all n rows (stage entry points).
int single_job(knng_ctx* c, int64_t n, JobTable* jt) {
  cudaError_t e = c->jobs.ensure(64);
  if (e) return cuda_fail(c, e, "job table allocation");
  const int32_t h[2] = {0, int32_t(n)};
  if ((e = cudaMemcpyAsync(c->jobs.p, h, sizeof(h), cudaMemcpyHostToDevice, c->stream)) ||
      (e = cudaStreamSynchronize(c->stream)))
    return cuda_fail(c, e, "job table upload");
  jt->count = 1;
  jt->off = c->jobs.as<int32_t>(0);
  jt->n = c->jobs.as<int32_t>(4);
  return KNNG_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

int quantize_input(knng_ctx* c, const void* rows, int64_t n, int d, int on_device, int64_t row0 = 0) {
  const int W = d / 64;
  cudaError_t e;
  int8_t* codes = c->codes.as<int8_t>() + row0 * d;
  uint64_t* sketch = c->sketch.as<uint64_t>() + row0 * W;
  if (on_device) {
    e = launch_quantize(static_cast<const float*>(rows), n, d, c->prm.quant_mode, codes, sketch, c->stream);
    return e ? cuda_fail(c, e, "quantize") : KNNG_OK;
  }
  // Host rows in memory the device maps (pinned or registered host memory,
  // managed memory) are quantised in place by one kernel over the host link.
  {
    cudaPointerAttributes at{};
    const float* direct = nullptr;
    if (cudaPointerGetAttributes(&at, rows) == cudaSuccess) {
      if ((at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged) && at.devicePointer)
        direct = static_cast<const float*>(at.devicePointer);
      else if (at.type == cudaMemoryTypeDevice)  // device rows passed as host rows: read them in place
        direct = static_cast<const float*>(rows);
    } else {
      cudaGetLastError();  // an unknown pointer is pageable memory
    }
    if (direct) {
      e = launch_quantize(direct, n, d, c->prm.quant_mode, codes, sketch, c->stream);
      return e ? cuda_fail(c, e, "quantize (host rows)") : KNNG_OK;
    }
  }
  // Pageable rows: host threads copy fixed-size chunks into two pinned slots
  // and the kernel quantises each slot in place while the threads fill the
  // other (hostcopy.cu says why the device never reads pageable memory).
  // Slot s is refilled once the kernel that read it (event freed[s]) is done.
  const int64_t chunk_rows = std::min<int64_t>(kStageRows, n);
  const size_t chunk_bytes = size_t(chunk_rows) * d * 4;
  if ((e = c->pin_in.ensure(2 * chunk_bytes))) return cuda_fail(c, e, "pinned input staging");
  float* slot_dev[2];
  for (int b = 0; b < 2; ++b)
    if ((e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&slot_dev[b]), c->pin_in.as<char>(b * chunk_bytes), 0)))
      return cuda_fail(c, e, "pinned input staging");
  const float* src = static_cast<const float*>(rows);
  for (int64_t off = 0, k = 0; off < n; off += chunk_rows, ++k) {
    const int64_t m = std::min<int64_t>(chunk_rows, n - off);
    const int b = int(k & 1);
    if ((e = cudaEventSynchronize(c->freed[b]))) return cuda_fail(c, e, "input staging");
    c->host_copy(c->pin_in.as<char>(b * chunk_bytes), src + off * d, size_t(m) * d * 4);
    if ((e = launch_quantize(slot_dev[b], m, d, c->prm.quant_mode, codes + off * d, sketch + off * W, c->stream)))
      return cuda_fail(c, e, "quantize");
    if ((e = cudaEventRecord(c->freed[b], c->stream))) return cuda_fail(c, e, "staging events");
  }
  return KNNG_OK;
}

struct BJob {
  const void* rows;
  int64_t n;
  int on_dev;
  int32_t* knns;
  float* dists;
  int out_dev;
  int iterations;  // out
};

// Times the join configurations on the batch's initial graph (output to the
// spare buffer, which iteration 0 overwrites) and keeps the fastest per
// (d, log2 rows), on the first 1/16 of the rows in visit order.  The early
// configuration is timed with no candidate cache;
// with a cache (cache_ctl), one more launch fills every row's cache from the
// same graph and the configurations are timed again with all candidates
// cached, which is what the later iterations look like.  The caller clears
// the cache before the NN-Descent phase.
JoinCfg autotune_join(knng_ctx* c, int64_t N, int d, int32_t* const ids[2], int32_t* const scs[2],
                      const int32_t* order, unsigned long long* scratch_counters, const JoinCtl* cache_ctl) {
  const knng_params& p = c->prm;
  JoinCfg best;
  if (p.join_ctas_per_sm) {  // a forced variant
    best.early = best.late = std::make_pair(p.join_ctas_per_sm, p.join_cblock);
    return best;
  }
  const auto key = std::make_pair(d, int(std::log2(double(N))));
  auto it = c->tuned.find(key);
  if (it != c->tuned.end()) return it->second;
  if (!p.autotune || p.join_mode != KNNG_JOIN_JACOBI) return best;
  if (join_prepare_all(p.k_build, p.k_build * p.rerank_mult, d) != cudaSuccess) {
    c->last_error = std::string("join variants: ") + join_variant_error();
    return best;
  }
  const std::pair<int, int> cand[] = {{4, 4}, {4, 8}, {3, 4}, {3, 8}, {4, 2}};
  const int K = p.k_build;
  // the sweeps process the first 1/16 of the rows (at least 64 per resident CTA),
  // so tuning costs about one join launch on the first build of a bucket
  JoinCtl plain{};
  plain.row_limit = std::min<int64_t>(N, std::max<int64_t>(N / 16, int64_t(c->num_sms) * 4 * 64));
  JoinCtl cached = cache_ctl ? *cache_ctl : plain;
  cached.row_limit = plain.row_limit;
  auto sweep = [&](const JoinCtl* ctl, std::pair<int, int>* out) {
    float best_ms = 1e30f;
    for (const auto& cf : cand) {
      cudaEventRecord(c->jev[0], c->stream);
      if (launch_join(c->codes.as<int8_t>(), c->join_sketch(), N, d, K, K * p.rerank_mult, ids[0], scs[0],
                      ids[1], scs[1], order, scratch_counters, c->num_sms, c->stream, nullptr, ctl, cf.first,
                      cf.second, c->sketch_words(d)) != cudaSuccess)
        return false;
      cudaEventRecord(c->jev[1], c->stream);
      cudaEventSynchronize(c->jev[1]);
      const float ms = elapsed(c->jev[0], c->jev[1]);
      if (ms < best_ms) {
        best_ms = ms;
        *out = cf;
      }
    }
    return true;
  };
  if (!sweep(&plain, &best.early)) return best;
  best.late = best.early;
  if (cache_ctl) {
    if (cudaMemsetAsync(cache_ctl->cache_cnt, 0, size_t(N) * 4, c->stream) != cudaSuccess ||
        launch_join(c->codes.as<int8_t>(), c->join_sketch(), N, d, K, K * p.rerank_mult, ids[0], scs[0],
                    ids[1], scs[1], order, scratch_counters, c->num_sms, c->stream, nullptr, &cached,
                    best.early.first, best.early.second, c->sketch_words(d)) != cudaSuccess ||
        !sweep(&cached, &best.late))
      return best;
  }
  c->tuned[key] = best;
  return best;
}

// The NN-Descent phase: max_iterations launches of the join, each followed by
// the per-job stop check; launches after every job has stopped do nothing.
cudaError_t join_phase(knng_ctx* c, int64_t N, int d, int32_t* const ids[2], int32_t* const scs[2],
                       const int32_t* order, const JobTable& jt, const JoinCtl& ctl, unsigned long long* counters,
                       const JoinCfg& cfg, bool capture, const char** step) {
  const knng_params& p = c->prm;
  const int K = p.k_build;
  const bool jac = p.join_mode == KNNG_JOIN_JACOBI;
  cudaError_t e;
  int cur = 0;
  for (int it = 0; it < p.max_iterations; ++it) {
    const int nxt = jac ? 1 - cur : cur;
    JoinCtl ci = ctl;  // this iteration's row-change flags: read the previous iteration's, write its own
    if (jac && c->rowflags.p) {
      ci.chg_in = c->rowflags.as<uint8_t>(size_t(it & 1) * size_t(N));
      ci.chg_out = c->rowflags.as<uint8_t>(size_t((it + 1) & 1) * size_t(N));
    }
    e = capture ? cudaEventRecordWithFlags(c->itev[2 * it], c->stream, cudaEventRecordExternal)
                : cudaEventRecord(c->itev[2 * it], c->stream);
    if (e) return (*step = "iteration start event", e);
    if ((e = launch_join(c->codes.as<int8_t>(), c->join_sketch(), N, d, K, K * p.rerank_mult, ids[cur],
                         scs[cur], ids[nxt], scs[nxt], order, counters + 8 * it, c->num_sms, c->stream, &jt, &ci,
                         (it < 2 ? cfg.early : cfg.late).first, (it < 2 ? cfg.early : cfg.late).second,
                         c->sketch_words(d))))
      return (*step = "join launch", e);
    e = capture ? cudaEventRecordWithFlags(c->itev[2 * it + 1], c->stream, cudaEventRecordExternal)
                : cudaEventRecord(c->itev[2 * it + 1], c->stream);
    if (e) return (*step = "iteration end event", e);
    if ((e = launch_stop_check(jt, ctl, K, it, nxt, p.early_stop_rate, p.rate_diff_tol, c->stream)))
      return (*step = "stop check", e);
    cur = nxt;
  }
  return cudaSuccess;
}

// One problem made of J jobs of the same dimension d (a single build is J = 1).
int run_batch(knng_ctx* c, BJob* jobs, int J, int d, knng_stats& S) {
  using clk = std::chrono::steady_clock;
  const auto t_start = clk::now();
  const int64_t launches0 = launches();
  const knng_params& p = c->prm;
  const int K = p.k_build, T = p.num_trees, W = d / 64, MI = p.max_iterations;
  std::memset(&S, 0, sizeof(S));
  std::vector<int32_t> hoff(J), hn(J);
  int64_t N = 0;
  int split = 0;
  for (int b = 0; b < J; ++b) {
    hoff[b] = int32_t(N);
    hn[b] = int32_t(jobs[b].n);
    N += jobs[b].n;
    if (jobs[b].n > p.leaf_size) ++split;
  }
  if (int64_t(T) * N > INT32_MAX) return set_error(c, KNNG_E_ARGS, "num_trees * total rows must fit in int32");
  cudaError_t e;
  const size_t nk = size_t(N) * K;
  if ((e = c->codes.ensure(size_t(N) * d)) || (e = c->sketch.ensure(size_t(N) * W * 8)) ||
      (e = c->graph.ensure(nk * 16)) || (e = c->perm.ensure(size_t(T) * N * 4)) ||
      (e = c->leaf_flag.ensure(size_t(T) * N)) || (c->hyperplane() && (e = c->hsketch.ensure(size_t(N) * 16))))
    return cuda_fail(c, e, "device allocation");
  Scratch s;
  int st = ensure_scratch(c, N, &s, 0, (p.join_cache && MI > 0) ? cache_bytes(N) : 0);
  if (st) return st;
  // job table + NN-Descent control block
  const size_t jb = size_t(J);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o += (bytes + 15) & ~size_t(15);
    return at;
  };
  const size_t o_off = take(jb * 4), o_n = take(jb * 4), o_upd = take(jb * 8), o_done = take(jb * 4),
               o_prev = take(jb * 4), o_iters = take(jb * 4), o_flags = take(16), o_log = take(size_t(MI + 1) * jb * 8),
               o_cnt = take(size_t(MI + 1) * 8 * 8);
  if ((e = c->jobs.ensure(o))) return cuda_fail(c, e, "job table allocation");
  cudaStream_t str = c->stream;
  if ((e = cudaMemsetAsync(c->jobs.p, 0, o, str)) ||
      (e = cudaMemcpyAsync(c->jobs.as<int32_t>(o_off), hoff.data(), jb * 4, cudaMemcpyHostToDevice, str)) ||
      (e = cudaMemcpyAsync(c->jobs.as<int32_t>(o_n), hn.data(), jb * 4, cudaMemcpyHostToDevice, str)))
    return cuda_fail(c, e, "job table upload");
  JobTable jt;
  jt.count = J;
  jt.off = c->jobs.as<int32_t>(o_off);
  jt.n = c->jobs.as<int32_t>(o_n);
  JoinCtl ctl;
  ctl.counters = c->jobs.as<unsigned long long>(o_cnt);
  ctl.job_upd = c->jobs.as<unsigned long long>(o_upd);
  ctl.job_done = c->jobs.as<int>(o_done);
  ctl.job_prev = c->jobs.as<float>(o_prev);
  ctl.job_iters = c->jobs.as<int>(o_iters);
  ctl.all_done = c->jobs.as<int>(o_flags);
  ctl.final_buf = c->jobs.as<int>(o_flags) + 1;
  ctl.upd_log = c->jobs.as<long long>(o_log);
  ctl.cache_ids = nullptr;
  ctl.cache_hr = nullptr;
  ctl.cache_cnt = nullptr;
  ctl.cache_cap = 0;
  ctl.row_limit = 0;  // every row
  ctl.chg_in = nullptr;  // set per iteration by join_phase
  ctl.chg_out = nullptr;
  // the bounds-checked build's error word of the join and the export
  ctl.check_err = kChecked ? c->scalars.as<unsigned>(kCheckWord) : nullptr;
  if (kChecked && (e = cudaMemsetAsync(ctl.check_err, 0, sizeof(unsigned), str)))
    return cuda_fail(c, e, "check word reset");
  const bool skip_rows = p.join_mode == KNNG_JOIN_JACOBI && MI > 0;
  if (skip_rows && (e = c->rowflags.ensure(size_t(2) * size_t(N)))) return cuda_fail(c, e, "row flag allocation");
  if (p.join_cache && MI > 0) {
    // over the forest and initial-graph scratch (sized for both by
    // ensure_scratch): that scratch is dead from the autotune on
    char* cp = c->scratch.as<char>();
    ctl.cache_ids = reinterpret_cast<int32_t*>(cp);
    cp += cache_ids_bytes(N);
    ctl.cache_hr = reinterpret_cast<uint16_t*>(cp);
    cp += cache_hr_bytes(N);
    ctl.cache_cnt = reinterpret_cast<int*>(cp);
    ctl.cache_cap = kCacheCap;
  }
  unsigned long long* tune_counters = ctl.counters + 8 * MI;
  int32_t* ids[2] = {c->graph.as<int32_t>(0), c->graph.as<int32_t>(nk * 8)};
  int32_t* scs[2] = {c->graph.as<int32_t>(nk * 4), c->graph.as<int32_t>(nk * 12)};

  cudaEventRecord(c->ev[0], str);
  for (int b = 0; b < J; ++b)
    if ((st = quantize_input(c, jobs[b].rows, jobs[b].n, d, jobs[b].on_dev, hoff[b]))) return st;
  // the optional hyperplane sketch, from the codes (like the sign sketch, before buildtime starts)
  if (c->hyperplane() &&
      (e = launch_hyperplane_sketch(c->codes.as<int8_t>(), N, d, p.seed, c->hsketch.as<uint64_t>(), c->num_sms, str)))
    return cuda_fail(c, e, "hyperplane sketch");
  cudaEventRecord(c->ev[1], str);
  int64_t levels = 0, leaves = 0;
  const bool forest_init = p.init_mode == KNNG_INIT_FOREST;
  if (p.init_mode == KNNG_INIT_RANDOM) {
    for (int b = 0; b < J; ++b)
      if (hn[b] <= K) return set_error(c, KNNG_E_ARGS, "random init needs n > k_build for every job");
  } else if (p.init_mode == KNNG_INIT_BLOCK) {
    for (int b = 0; b < J; ++b) {
      const int64_t nb = std::max<int64_t>(1, (hn[b] + p.block_size / 2) / p.block_size);
      if (hn[b] / nb < K + 1) return set_error(c, KNNG_E_ARGS, "block init needs k_build + 1 rows in every block");
    }
  } else if ((st = run_forest(c->codes.as<int8_t>(), N, d, T, p.leaf_size, p.seed, nullptr, 0, c->perm.as<int32_t>(),
                              c->leaf_flag.as<uint8_t>(), s.fb, str, &levels, &c->last_error, jt, split,
                              p.forest_fuse))) {
    return st;
  }
  cudaEventRecord(c->ev[2], str);
  if (p.init_mode == KNNG_INIT_RANDOM) {
    if ((e = launch_init_random(c->codes.as<int8_t>(), d, N, K, p.seed, jt, ids[0], scs[0], c->num_sms, str)))
      return cuda_fail(c, e, "random init");
  } else if (p.init_mode == KNNG_INIT_BLOCK) {
    if ((e = launch_init_block(c->codes.as<int8_t>(), d, N, K, p.bridges, p.block_size, p.seed, jt, ids[0], scs[0],
                               c->num_sms, str)))
      return cuda_fail(c, e, "block init");
  } else if ((st = run_init(c->codes.as<int8_t>(), N, d, T, p.leaf_size, K, p.seed, c->perm.as<int32_t>(),
                            c->leaf_flag.as<uint8_t>(), ids[0], scs[0], s.ib, str, &leaves, &c->last_error, jt,
                            p.gram_mode, p.wait_limit))) {
    return st;
  }
  // rows in tree-0 leaf order (no forest with the random or block init: natural order)
  const int32_t* order = (p.row_order == KNNG_ORDER_LEAF && forest_init) ? c->perm.as<int32_t>() : nullptr;
  JoinCtl tune_ctl{};  // the candidate cache alone, for the second autotune sweep
  tune_ctl.cache_ids = ctl.cache_ids;
  tune_ctl.cache_hr = ctl.cache_hr;
  tune_ctl.cache_cnt = ctl.cache_cnt;
  tune_ctl.cache_cap = ctl.cache_cap;
  const JoinCfg cfg = autotune_join(c, N, d, ids, scs, order, tune_counters, ctl.cache_ids ? &tune_ctl : nullptr);
  cudaEventRecord(c->ev[3], str);
  // every row starts the phase with an empty candidate cache, and counts as
  // changed before the first iteration
  if (ctl.cache_cnt && (e = cudaMemsetAsync(ctl.cache_cnt, 0, size_t(N) * 4, str)))
    return cuda_fail(c, e, "candidate cache reset");
  if (skip_rows && (e = cudaMemsetAsync(c->rowflags.p, 1, size_t(N), str))) return cuda_fail(c, e, "row flag reset");
  // NN-Descent, captured once per launch key and replayed
  bool graph_used = false;
  if ((e = join_prepare(K, K * p.rerank_mult, d, cfg.early.first, cfg.early.second)) ||
      (e = join_prepare(K, K * p.rerank_mult, d, cfg.late.first, cfg.late.second)))
    return cuda_fail(c, e, (std::string("join variant: ") + join_variant_error()).c_str());
  const char* step = "";
  if (p.use_graph) {
    const std::vector<uintptr_t> key = {uintptr_t(c->codes.p), uintptr_t(c->join_sketch()), uintptr_t(c->graph.p),
                                        uintptr_t(c->jobs.p), uintptr_t(c->perm.p), uintptr_t(ctl.cache_ids),
                                        uintptr_t(c->rowflags.p),
                                        uintptr_t(N), uintptr_t(d),
                                        uintptr_t(J), uintptr_t(o), uintptr_t(cfg.early.first), uintptr_t(cfg.early.second),
                                        uintptr_t(cfg.late.first), uintptr_t(cfg.late.second),
                                        uintptr_t(order != nullptr), uintptr_t(p.join_mode), uintptr_t(MI),
                                        uintptr_t(K), uintptr_t(p.rerank_mult)};
    if (!c->join_graph || c->join_graph_key != key) {
      if (c->join_graph) {
        cudaGraphExecDestroy(c->join_graph);
        c->join_graph = nullptr;
      }
      cudaGraph_t g = nullptr;
      std::lock_guard<std::mutex> capture_lock(g_capture_mu);  // one capture at a time per process
      if (cudaStreamBeginCapture(str, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const cudaError_t ce = join_phase(c, N, d, ids, scs, order, jt, ctl, ctl.counters, cfg, true, &step);
        const cudaError_t ee = cudaStreamEndCapture(str, &g);
        if (ce == cudaSuccess && ee == cudaSuccess && g &&
            cudaGraphInstantiate(&c->join_graph, g, 0) == cudaSuccess)
          c->join_graph_key = key;
        else
          c->join_graph = nullptr;
        if (g) cudaGraphDestroy(g);
      }
      cudaGetLastError();
    }
    if (c->join_graph) {
      if ((e = cudaGraphLaunch(c->join_graph, str))) return cuda_fail(c, e, "join graph launch");
      graph_used = true;
    }
  }
  if (!graph_used && (e = join_phase(c, N, d, ids, scs, order, jt, ctl, ctl.counters, cfg, false, &step)))
    return cuda_fail(c, e, (std::string("join phase (") + step + ")").c_str());
  cudaEventRecord(c->ev[4], str);
  // results of the control block
  std::vector<int> iters(jb);
  std::vector<long long> log(size_t(MI) * jb);
  std::vector<unsigned long long> cnt(size_t(MI) * 8);
  int flags[2] = {0, 0};
  if ((e = cudaMemcpyAsync(iters.data(), ctl.job_iters, jb * 4, cudaMemcpyDeviceToHost, str)) ||
      (MI && (e = cudaMemcpyAsync(log.data(), ctl.upd_log, log.size() * 8, cudaMemcpyDeviceToHost, str))) ||
      (MI && (e = cudaMemcpyAsync(cnt.data(), ctl.counters, cnt.size() * 8, cudaMemcpyDeviceToHost, str))) ||
      (e = cudaMemcpyAsync(flags, ctl.all_done, 8, cudaMemcpyDeviceToHost, str)) ||
      (e = cudaStreamSynchronize(str)))
    return cuda_fail(c, e, "join phase");
  const int fin = MI == 0 ? 0 : flags[1];
  // export (job-local 1-based ids) and hand out each job's rows
  const size_t outn = size_t(N) * p.k_eval;
  int32_t* kd;
  float* dd;
  const bool direct = J == 1 && jobs[0].out_dev;
  if (direct) {
    kd = jobs[0].knns;
    dd = jobs[0].dists;
  } else {
    if ((e = c->outbuf.ensure(outn * 8))) return cuda_fail(c, e, "output allocation");
    kd = c->outbuf.as<int32_t>(0);
    dd = c->outbuf.as<float>(outn * 4);
  }
  if ((e = launch_export(ids[fin], scs[fin], N, K, p.k_eval, nullptr, kd, dd, str, &jt, ctl.check_err)))
    return cuda_fail(c, e, "export");
  // pageable host outputs: copied into pinned memory here and by host threads
  // into the caller's buffers after the stream is done (hostcopy.cu)
  std::vector<char> via_pin(jb, 0);
  bool any_pin = false;
  for (int b = 0; b < J; ++b)
    if (!direct && !jobs[b].out_dev && (host_pageable(jobs[b].knns) || host_pageable(jobs[b].dists)))
      any_pin = (via_pin[b] = 1);
  if (any_pin && (e = c->pin_out.ensure(outn * 8))) return cuda_fail(c, e, "pinned output staging");
  if (!direct)
    for (int b = 0; b < J; ++b) {
      const size_t cnt_b = size_t(jobs[b].n) * p.k_eval, at = size_t(hoff[b]) * p.k_eval;
      const cudaMemcpyKind kind = jobs[b].out_dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
      int32_t* ko = via_pin[b] ? c->pin_out.as<int32_t>(at * 4) : jobs[b].knns;
      float* dso = via_pin[b] ? c->pin_out.as<float>((outn + at) * 4) : jobs[b].dists;
      if ((e = cudaMemcpyAsync(ko, kd + at, cnt_b * 4, kind, str)) ||
          (e = cudaMemcpyAsync(dso, dd + at, cnt_b * 4, kind, str)))
        return cuda_fail(c, e, "output copy");
    }
  cudaEventRecord(c->ev[5], str);
  unsigned check = 0;
  if (kChecked && (e = cudaMemcpyAsync(&check, ctl.check_err, sizeof(unsigned), cudaMemcpyDeviceToHost, str)))
    return cuda_fail(c, e, "check word");
  if ((e = cudaStreamSynchronize(str))) return cuda_fail(c, e, "build");
  if (check & kErrBounds)
    return set_error(c, KNNG_E_BOUNDS, "NN-Descent or export: an id outside [0, n) (bounds check)");
  for (int b = 0; b < J; ++b)
    if (via_pin[b]) {
      const size_t cnt_b = size_t(jobs[b].n) * p.k_eval, at = size_t(hoff[b]) * p.k_eval;
      c->host_copy(jobs[b].knns, c->pin_out.as<int32_t>(at * 4), cnt_b * 4);
      c->host_copy(jobs[b].dists, c->pin_out.as<float>((outn + at) * 4), cnt_b * 4);
    }
  int max_it = 0;
  for (int b = 0; b < J; ++b) {
    jobs[b].iterations = iters[b];
    max_it = std::max(max_it, iters[b]);
  }
  S.quantize_s = elapsed(c->ev[0], c->ev[1]) * 1e-3;
  S.forest_s = elapsed(c->ev[1], c->ev[2]) * 1e-3;
  S.init_s = elapsed(c->ev[2], c->ev[3]) * 1e-3;
  S.join_s = elapsed(c->ev[3], c->ev[4]) * 1e-3;
  S.export_s = elapsed(c->ev[4], c->ev[5]) * 1e-3;
  S.build_s = elapsed(c->ev[1], c->ev[4]) * 1e-3;
  S.device_s = elapsed(c->ev[0], c->ev[5]) * 1e-3;
  S.iterations = max_it;
  for (int it = 0; it < max_it && it < 64; ++it) {
    long long u = 0;
    for (int b = 0; b < J; ++b) u += log[size_t(it) * J + b];
    S.updates[it] = u;
    S.join_ms[it] = elapsed(c->itev[2 * it], c->itev[2 * it + 1]);
    S.join_candidates[it] = int64_t(cnt[8 * it + 1]);
    S.join_dots[it] = int64_t(cnt[8 * it + 2]);
    S.join_distinct[it] = int64_t(cnt[8 * it + 3]);
    S.join_skipped[it] = int64_t(cnt[8 * it + 4]);
  }
  S.forest_levels = levels;
  S.leaves = leaves;
  S.join_ctas_per_sm = cfg.late.first;  // the configuration of the later iterations
  S.join_cblock = cfg.late.second;
  S.graph_used = graph_used ? 1 : 0;
  S.kernel_launches = launches() - launches0;
  S.total_s = std::chrono::duration<double>(clk::now() - t_start).count();
  return KNNG_OK;
}

}  // namespace

extern "C" {

void knng_default_params(knng_params* p) {
  if (!p) return;
  p->k_build = 50;
  p->k_eval = 15;
  p->num_trees = 16;
  p->rerank_mult = 8;
  p->leaf_size = 64;
  p->max_iterations = 30;
  p->early_stop_rate = 0.04f;
  p->rate_diff_tol = 0.01f;
  p->quant_mode = KNNG_QUANT_TRUNC;
  p->join_mode = KNNG_JOIN_JACOBI;
  p->row_order = KNNG_ORDER_LEAF;
  p->seed = 1337;
  p->device = 0;
  p->autotune = 1;
  p->use_graph = 1;
  p->gram_mode = KNNG_GRAM_TCGEN05;
  p->init_mode = KNNG_INIT_FOREST;
  p->join_cache = 1;
  p->block_size = 10000;
  p->bridges = 2;
  p->wait_limit = 0;
  p->join_ctas_per_sm = 0;
  p->join_cblock = 0;
  p->sketch_mode = KNNG_SKETCH_SIGN;
  p->forest_fuse = 1;
}

const char* knng_status_string(int s) {
  switch (s) {
    case KNNG_OK: return "ok";
    case KNNG_E_ARGS: return "invalid argument";
    case KNNG_E_DIM: return "unsupported dimension";
    case KNNG_E_OOM: return "out of device memory";
    case KNNG_E_ADMIT: return "job not admitted";
    case KNNG_E_TIMEOUT: return "device wait timed out";
    case KNNG_E_CUDA: return "CUDA error";
    case KNNG_E_REPLAY: return "replay pivot table mismatch";
    case KNNG_E_BUSY: return "job not finished";
    case KNNG_E_NOTFOUND: return "unknown ticket";
    case KNNG_E_SCRATCH: return "input exceeds the fixed no-allocation scratch";
    case KNNG_E_BOUNDS: return "a device bounds check failed (bounds-checked build)";
    default: return "unknown status";
  }
}

const char* knng_last_error(const knng_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int knng_create(knng_ctx** out, const knng_params* p) {
  return abi_guard(nullptr, [&]() -> int {
    if (!out) return KNNG_E_ARGS;
    *out = nullptr;
    knng_ctx* c = new (std::nothrow) knng_ctx();
    if (!c) return KNNG_E_OOM;
    if (p) c->prm = *p; else knng_default_params(&c->prm);
    int st = check_params(c, c->prm);
    if (st) {
      delete c;
      return st;
    }
    cudaError_t e;
    c->device = c->prm.device;
    if ((e = cudaSetDevice(c->device)) ||
        (e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device)) ||
        (e = cudaDeviceGetAttribute(&c->pageable_access, cudaDevAttrPageableMemoryAccess, c->device)) ||
        (e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking))) {
      delete c;
      return KNNG_E_CUDA;
    }
    for (auto& ev : c->ev)
      if ((e = cudaEventCreate(&ev))) {
        knng_destroy(c);
        return KNNG_E_CUDA;
      }
    for (auto& ev : c->jev)
      if ((e = cudaEventCreate(&ev))) {
        knng_destroy(c);
        return KNNG_E_CUDA;
      }
    for (auto& ev : c->itev)
      if ((e = cudaEventCreate(&ev))) {
        knng_destroy(c);
        return KNNG_E_CUDA;
      }
    if ((e = cudaEventCreate(&c->bev))) {
      knng_destroy(c);
      return KNNG_E_CUDA;
    }
    for (int k = 0; k < 2; ++k)
      if ((e = cudaEventCreateWithFlags(&c->freed[k], cudaEventDisableTiming))) {
        knng_destroy(c);
        return KNNG_E_CUDA;
      }
    for (DevBuf* b : c->buffers()) b->s = c->stream;
    // resolve the join kernels' launch attributes now, outside any capture
    for (int d : {128, 256, 384, 512, 640, 768, 896, 1024})
      if ((e = join_prepare_all(c->prm.k_build, c->prm.k_build * c->prm.rerank_mult, d))) {
        c->last_error = std::string("join variants: ") + join_variant_error();
        break;
      }
    *out = c;
    return KNNG_OK;
  });
}

void knng_destroy(knng_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (knng_ctx* sub : c->subs) knng_destroy(sub);
  if (c->join_graph) cudaGraphExecDestroy(c->join_graph);
  for (DevBuf* b : c->buffers()) b->release();
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (auto& ev : c->itev)
    if (ev) cudaEventDestroy(ev);
  if (c->bev) cudaEventDestroy(c->bev);
  for (int k = 0; k < 2; ++k)
    if (c->freed[k]) cudaEventDestroy(c->freed[k]);
  c->pool.reset();
  c->pin_in.release();
  c->pin_out.release();
  for (auto& ev : c->ev)
    if (ev) cudaEventDestroy(ev);
  for (auto& ev : c->jev)
    if (ev) cudaEventDestroy(ev);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
}

int knng_quantize(const float* x_dev, int64_t n, int d, int quant_mode, int8_t* codes_dev, uint64_t* sketch_dev,
                  void* stream) {
  if (!x_dev || !codes_dev || !sketch_dev || n < 0) return KNNG_E_ARGS;
  if (!dim_ok(d) && !(d >= 64 && d % 64 == 0 && d <= kMaxDim)) return KNNG_E_DIM;
  if (quant_mode != KNNG_QUANT_TRUNC && quant_mode != KNNG_QUANT_ROUND) return KNNG_E_ARGS;
  cudaError_t e = launch_quantize(x_dev, n, d, quant_mode, codes_dev, sketch_dev, static_cast<cudaStream_t>(stream));
  return e ? KNNG_E_CUDA : KNNG_OK;
}

int knng_sketch_hyperplane(const int8_t* codes_dev, int64_t n, int d, uint32_t seed, uint64_t* sketch_dev,
                           void* stream) {
  if (!codes_dev || !sketch_dev || n < 0 || (reinterpret_cast<uintptr_t>(codes_dev) & 15)) return KNNG_E_ARGS;
  if (!dim_ok(d)) return KNNG_E_DIM;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
    return KNNG_E_CUDA;
  const cudaError_t e = launch_hyperplane_sketch(codes_dev, n, d, seed, sketch_dev, sms, static_cast<cudaStream_t>(stream));
  return e ? KNNG_E_CUDA : KNNG_OK;
}

int knng_forest(knng_ctx* c, const int8_t* codes_dev, int64_t n, int d, const int32_t* replay, int64_t n_replay,
                int32_t* perm_dev, uint8_t* leaf_flag_dev) {
  return abi_guard(c ? &c->last_error : nullptr, [&]() -> int {
    if (!c || !codes_dev || !perm_dev || !leaf_flag_dev || (n_replay > 0 && !replay)) return KNNG_E_ARGS;
    int st = check_shape(c, n, d);
    if (st) return st;
    cudaSetDevice(c->device);
    Scratch s;
    if ((st = ensure_scratch(c, n, &s, replay ? n_replay : 0))) return st;
    int64_t levels = 0;
    JobTable jt;
    if ((st = single_job(c, n, &jt))) return st;
    st = run_forest(codes_dev, n, d, c->prm.num_trees, c->prm.leaf_size, c->prm.seed, replay, replay ? n_replay : 0,
                    perm_dev, leaf_flag_dev, s.fb, c->stream, &levels, &c->last_error, jt,
                    n > c->prm.leaf_size ? 1 : 0, c->prm.forest_fuse);
    if (st) return st;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(c, e, "forest") : KNNG_OK;
  });
}

int knng_init_graph(knng_ctx* c, const int8_t* codes_dev, int64_t n, int d, const int32_t* perm_dev,
                    const uint8_t* leaf_flag_dev, int32_t* ids_dev, int32_t* scores_dev) {
  return abi_guard(c ? &c->last_error : nullptr, [&]() -> int {
    if (!c || !codes_dev || !perm_dev || !leaf_flag_dev || !ids_dev || !scores_dev) return KNNG_E_ARGS;
    int st = check_shape(c, n, d);
    if (st) return st;
    cudaSetDevice(c->device);
    Scratch s;
    if ((st = ensure_scratch(c, n, &s, 0))) return st;
    JobTable jt;
    if ((st = single_job(c, n, &jt))) return st;
    st = run_init(codes_dev, n, d, c->prm.num_trees, c->prm.leaf_size, c->prm.k_build, c->prm.seed, perm_dev,
                  leaf_flag_dev, ids_dev, scores_dev, s.ib, c->stream, nullptr, &c->last_error, jt, c->prm.gram_mode,
                  c->prm.wait_limit);
    if (st) return st;
    cudaError_t e = cudaStreamSynchronize(c->stream);
    return e ? cuda_fail(c, e, "init") : KNNG_OK;
  });
}

int knng_join_iter(knng_ctx* c, const int8_t* codes_dev, const uint64_t* sketch_dev, int64_t n, int d,
                   const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out, int32_t* scores_out,
                   int64_t* updates) {
  return abi_guard(c ? &c->last_error : nullptr, [&]() -> int {
    if (!c || !codes_dev || !sketch_dev || !ids_in || !scores_in || !ids_out || !scores_out) return KNNG_E_ARGS;
    if ((ids_out == ids_in) != (scores_out == scores_in)) return set_error(c, KNNG_E_ARGS, "mixed in-place buffers");
    int st = check_shape(c, n, d);
    if (st) return st;
    cudaSetDevice(c->device);
    cudaError_t e;
    if ((e = c->scalars.ensure(4096))) return cuda_fail(c, e, "scalar allocation");
    unsigned long long* up = c->scalars.as<unsigned long long>(256);
    if ((e = cudaMemsetAsync(up, 0, 64, c->stream))) return cuda_fail(c, e, "update counter");
    const int K = c->prm.k_build;
    const int cps = c->prm.join_ctas_per_sm ? c->prm.join_ctas_per_sm : 4;
    const int cb = c->prm.join_ctas_per_sm ? c->prm.join_cblock : 4;
    JoinCtl chk{};  // no jobs, no cache, no row flags: only the bounds-checked build's error word
    chk.check_err = kChecked ? c->scalars.as<unsigned>(kCheckWord) : nullptr;
    if (kChecked && (e = cudaMemsetAsync(chk.check_err, 0, sizeof(unsigned), c->stream)))
      return cuda_fail(c, e, "check word reset");
    if ((e = launch_join(codes_dev, sketch_dev, n, d, K, K * c->prm.rerank_mult, ids_in, scores_in, ids_out,
                         scores_out, nullptr, up, c->num_sms, c->stream, nullptr, kChecked ? &chk : nullptr, cps, cb,
                         c->sketch_words(d))))
      return cuda_fail(c, e, "join");
    unsigned long long h = 0;
    unsigned check = 0;
    if ((e = cudaMemcpyAsync(&h, up, 8, cudaMemcpyDeviceToHost, c->stream))) return cuda_fail(c, e, "update count");
    if (kChecked && (e = cudaMemcpyAsync(&check, chk.check_err, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream)))
      return cuda_fail(c, e, "check word");
    if ((e = cudaStreamSynchronize(c->stream))) return cuda_fail(c, e, "join");
    if (check & kErrBounds) return set_error(c, KNNG_E_BOUNDS, "join: an id outside [0, n) (bounds check)");
    if (updates) *updates = int64_t(h);
    return KNNG_OK;
  });
}

int knng_export(const int32_t* ids_dev, const int32_t* scores_dev, int64_t n, int k_build, int k_eval,
                const int32_t* id_map_dev, int32_t* knns_dev, float* dists_dev, void* stream) {
  if (!ids_dev || !scores_dev || !knns_dev || !dists_dev || n < 0 || k_eval < 1 || k_eval > k_build)
    return KNNG_E_ARGS;
  const cudaStream_t str = static_cast<cudaStream_t>(stream);
  unsigned* word = nullptr;
  if (kChecked && (export_check_word(&word) != cudaSuccess || cudaMemsetAsync(word, 0, sizeof(unsigned), str)))
    return KNNG_E_CUDA;
  cudaError_t e = launch_export(ids_dev, scores_dev, n, k_build, k_eval, id_map_dev, knns_dev, dists_dev, str,
                                nullptr, word);
  if (e) return KNNG_E_CUDA;
  if (kChecked) {  // the bounds-checked build waits for the stage to read its error word
    unsigned check = 0;
    if (cudaMemcpyAsync(&check, word, sizeof(unsigned), cudaMemcpyDeviceToHost, str) ||
        cudaStreamSynchronize(str))
      return KNNG_E_CUDA;
    if (check & kErrBounds) return KNNG_E_BOUNDS;
  }
  return KNNG_OK;
}

int knng_build(knng_ctx* c, const void* rows, int64_t n, int d, int rows_on_device, int32_t* knns, float* dists,
               int out_on_device, knng_stats* stats) {
  return abi_guard(c ? &c->last_error : nullptr, [&]() -> int {
    if (!c || !rows || !knns || !dists) return set_error(c, KNNG_E_ARGS, "null argument");
    int st = check_shape(c, n, d);
    if (st) return st;
    cudaSetDevice(c->device);
    BJob j{rows, n, rows_on_device, knns, dists, out_on_device, 0};
    knng_stats local{};
    return run_batch(c, &j, 1, d, stats ? *stats : local);
  });
}

int64_t knng_footprint_bytes(const knng_params* p, int64_t n, int d, int rows_on_device) {
  knng_params q;
  if (p) q = *p; else knng_default_params(&q);
  if (n < 1 || d < 1) return 0;
  const int T = q.num_trees, K = q.k_build;
  int64_t mn = 0, mt = 0;
  const size_t f = forest_bytes(n, T, q.leaf_size, &mn, &mt);
  const size_t in = init_bytes(n, T, q.leaf_size);
  size_t b = size_t(n) * d + size_t(n) * (d / 64) * 8 + size_t(n) * K * 16 + size_t(T) * n * 5;
  // the scratch region holds the forest, then the initial-graph scratch, then
  // the per-row candidate cache: the largest of the three
  const size_t cache = (q.join_cache && q.max_iterations > 0) ? cache_bytes(n) : 0;
  b += std::max(std::max(f, in), cache) + 64 * 1024;
  b += size_t(n) * q.k_eval * 8;                                   // export buffer
  b += size_t(q.max_iterations + 1) * 96 * 8 + 4096;               // control block (per job, bounded)
  if (q.join_mode == KNNG_JOIN_JACOBI) b += size_t(2) * n;          // row-change flags

  if (q.sketch_mode == KNNG_SKETCH_HYPERPLANE) b += size_t(n) * 16;  // hyperplane sketches
  (void)rows_on_device;  // host rows are staged through pinned host memory, not device memory
  return int64_t(b) + (int64_t(1) << 24);                          // pool rounding slack
}

int knng_trim(knng_ctx* c) {
  return abi_guard(c ? &c->last_error : nullptr, [&]() -> int {
    if (!c) return KNNG_E_ARGS;
    cudaSetDevice(c->device);
    if (c->join_graph) {
      cudaGraphExecDestroy(c->join_graph);
      c->join_graph = nullptr;
      c->join_graph_key.clear();
    }
    for (DevBuf* b : c->buffers()) b->release();
    cudaStreamSynchronize(c->stream);  // no copy still reads or writes the pinned buffers
    c->pin_in.release();
    c->pin_out.release();
    for (knng_ctx* sub : c->subs) knng_trim(sub);
    return KNNG_OK;
  });
}

int knng_build_batch(knng_ctx* c, knng_job* jobs, int count, knng_stats* stats) {
  return abi_guard(c ? &c->last_error : nullptr, [&]() -> int {
    if (!c || !jobs || count < 1) return set_error(c, KNNG_E_ARGS, "null argument or empty batch");
    for (int b = 0; b < count; ++b) {
      if (!jobs[b].rows || !jobs[b].knns || !jobs[b].dists) return set_error(c, KNNG_E_ARGS, "null job buffer");
      int st = check_shape(c, jobs[b].n, jobs[b].d);
      if (st) return st;
    }
    cudaSetDevice(c->device);
    knng_stats local{};
    knng_stats& S = stats ? *stats : local;
    std::memset(&S, 0, sizeof(S));
    // one problem per dimension: jobs of equal d are laid out back to back; the
    // groups run concurrently, each on its own context and stream
    std::vector<int> dims;
    for (int b = 0; b < count; ++b)
      if (std::find(dims.begin(), dims.end(), jobs[b].d) == dims.end()) dims.push_back(jobs[b].d);
    const int G = int(dims.size());
    while (int(c->subs.size()) < G - 1) {
      knng_ctx* sub = nullptr;
      const int st = knng_create(&sub, &c->prm);
      if (st) return set_error(c, st, "context for a dimension group");
      c->subs.push_back(sub);
    }
    std::vector<std::vector<BJob>> groups(G);
    std::vector<std::vector<int>> idx(G);
    for (int g = 0; g < G; ++g)
      for (int b = 0; b < count; ++b)
        if (jobs[b].d == dims[g]) {
          groups[g].push_back(BJob{jobs[b].rows, jobs[b].n, jobs[b].rows_on_device, jobs[b].knns, jobs[b].dists,
                                   jobs[b].out_on_device, 0});
          idx[g].push_back(b);
        }
    std::vector<knng_stats> gs(G);
    std::vector<int> gst(G, KNNG_OK);
    cudaEventRecord(c->bev, c->stream);  // batch start: every group's stream waits for it
    auto run_group = [&](int g) {
      knng_ctx* gc = g == 0 ? c : c->subs[size_t(g - 1)];
      cudaSetDevice(gc->device);
      cudaStreamWaitEvent(gc->stream, c->bev, 0);
      gst[g] = run_batch(gc, groups[g].data(), int(groups[g].size()), dims[g], gs[g]);
      if (gst[g] && gc != c) c->last_error = gc->last_error;
    };
    if (G == 1) {
      run_group(0);
    } else {
      std::vector<std::thread> th;
      for (int g = 1; g < G; ++g) th.emplace_back(run_group, g);
      run_group(0);
      for (auto& t : th) t.join();
    }
    float span_ms = 0.f;
    for (int g = 0; g < G; ++g) {
      knng_ctx* gc = g == 0 ? c : c->subs[size_t(g - 1)];
      for (size_t q = 0; q < groups[g].size(); ++q) {
        jobs[idx[g][q]].status = gst[g];
        jobs[idx[g][q]].iterations = groups[g][q].iterations;
      }
      if (gst[g] == KNNG_OK) span_ms = std::max(span_ms, elapsed(c->bev, gc->ev[5]));
    }
    for (int g = 0; g < G; ++g)
      if (gst[g]) return gst[g];
    for (int g = 0; g < G; ++g) {
      S.quantize_s += gs[g].quantize_s;
      S.forest_s += gs[g].forest_s;
      S.init_s += gs[g].init_s;
      S.join_s += gs[g].join_s;
      S.export_s += gs[g].export_s;
      S.build_s += gs[g].build_s;
      S.kernel_launches += gs[g].kernel_launches;
      S.forest_levels = std::max(S.forest_levels, gs[g].forest_levels);
      S.leaves += gs[g].leaves;
      S.iterations = std::max(S.iterations, gs[g].iterations);
      for (int it = 0; it < 64; ++it) {
        S.updates[it] += gs[g].updates[it];
        S.join_ms[it] += gs[g].join_ms[it];
        S.join_candidates[it] += gs[g].join_candidates[it];
        S.join_dots[it] += gs[g].join_dots[it];
        S.join_distinct[it] += gs[g].join_distinct[it];
        S.join_skipped[it] += gs[g].join_skipped[it];
      }
      S.join_ctas_per_sm = gs[g].join_ctas_per_sm;
      S.join_cblock = gs[g].join_cblock;
      S.graph_used = gs[g].graph_used;
    }
    // stage sums add up the groups' own times; device_s is the batch's span
    S.device_s = span_ms * 1e-3;
    return KNNG_OK;
  });
}

}  // extern "C"
