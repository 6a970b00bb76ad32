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
#include <new>
#include <string>
#include <vector>

#include <atomic>

namespace knng {
size_t join_smem_bytes(int K, int R, int d);
namespace {
std::atomic<int64_t> g_launches{0};
}
int64_t launches() { return g_launches.load(std::memory_order_relaxed); }
void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }
}  // namespace knng

using namespace knng;

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
  }
  template <class T>
  T* as(size_t byte_off = 0) const {
    return reinterpret_cast<T*>(static_cast<char*>(p) + byte_off);
  }
};

struct knng_ctx {
  knng_params prm{};
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev[8] = {};
  cudaEvent_t jev[2] = {};
  std::string last_error;
  DevBuf codes, sketch, graph, perm, leaf_flag, scratch, staging, outbuf, scalars;
};

namespace {

constexpr int64_t kStageRows = 1 << 16;  // host-input rows per H2D chunk

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
// never live at the same time).
int ensure_scratch(knng_ctx* c, int64_t n, Scratch* s, int64_t n_replay) {
  const int T = c->prm.num_trees, L = c->prm.leaf_size;
  int64_t mn = 0, mt = 0;
  const size_t fbytes = forest_bytes(n, T, L, &mn, &mt) + size_t(n_replay) * 24 + 8192;
  const size_t ibytes = init_bytes(n, T, L) + 8192;
  cudaError_t e = c->scratch.ensure(std::max(fbytes, ibytes));
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
    f.tile_off = reinterpret_cast<int32_t*>(p); carve(p, size_t(mn + 1) * 4);
    f.child_cnt = reinterpret_cast<int32_t*>(p); carve(p, size_t(mn + 1) * 4);
    f.tile_left = reinterpret_cast<int32_t*>(p); carve(p, size_t(mt) * 4);
    f.tile_left_off = reinterpret_cast<int32_t*>(p); carve(p, size_t(mt) * 4);
    f.replay_dev = reinterpret_cast<int32_t*>(p); carve(p, size_t(n_replay) * 24 + 16);
    f.scan_tmp = p; carve(p, scan_tmp_bytes(std::max(mn, mt)));
    f.dev_i64 = c->scalars.as<int64_t>(0);
    f.err = c->scalars.as<unsigned>(64);
  }
  {
    char* p = c->scratch.as<char>();
    InitBufs& b = s->ib;
    b.gram = reinterpret_cast<int32_t*>(p); carve(p, tn * kMaxLeaf * 4);
    b.pos = reinterpret_cast<int32_t*>(p); carve(p, tn * 4);
    b.leaf_lo = reinterpret_cast<int32_t*>(p); carve(p, tn * 4);
    b.leaf_idx = reinterpret_cast<int32_t*>(p); carve(p, tn * 8);
    b.leaf_sz = reinterpret_cast<uint8_t*>(p); carve(p, tn);
    b.fix_rows = reinterpret_cast<int32_t*>(p); carve(p, size_t(n) * 4);
    b.scan_tmp = p; carve(p, scan_tmp_bytes(int64_t(tn)));
    b.dev_i64 = c->scalars.as<int64_t>(128);
  }
  return KNNG_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b) {
  float ms = 0.f;
  cudaEventElapsedTime(&ms, a, b);
  return ms;
}

int quantize_input(knng_ctx* c, const void* rows, int64_t n, int d, int on_device) {
  const int W = d / 64;
  cudaError_t e;
  if (on_device) {
    e = launch_quantize(static_cast<const float*>(rows), n, d, c->prm.quant_mode, c->codes.as<int8_t>(),
                        c->sketch.as<uint64_t>(), c->stream);
    return e ? cuda_fail(c, e, "quantize") : KNNG_OK;
  }
  // Host rows: stream fixed-size chunks through two staging buffers so the
  // copy of chunk k+1 overlaps the quantisation of chunk k (the reference
  // streams 2.2M-row hyperslabs the same way, src/main.cpp:165-177).
  const size_t chunk_bytes = size_t(kStageRows) * d * 4;
  if ((e = c->staging.ensure(2 * chunk_bytes))) return cuda_fail(c, e, "staging allocation");
  const float* src = static_cast<const float*>(rows);
  for (int64_t off = 0, k = 0; off < n; off += kStageRows, ++k) {
    const int64_t m = std::min<int64_t>(kStageRows, n - off);
    float* stage = c->staging.as<float>((k & 1) * chunk_bytes);
    if ((e = cudaMemcpyAsync(stage, src + off * d, size_t(m) * d * 4, cudaMemcpyHostToDevice, c->stream)))
      return cuda_fail(c, e, "input copy");
    if ((e = launch_quantize(stage, m, d, c->prm.quant_mode, c->codes.as<int8_t>() + off * d,
                             c->sketch.as<uint64_t>() + off * W, c->stream)))
      return cuda_fail(c, e, "quantize");
  }
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
    default: return "unknown status";
  }
}

const char* knng_last_error(const knng_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int knng_create(knng_ctx** out, const knng_params* p) {
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
  *out = c;
  return KNNG_OK;
}

void knng_destroy(knng_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  for (DevBuf* b : {&c->codes, &c->sketch, &c->graph, &c->perm, &c->leaf_flag, &c->scratch, &c->staging,
                    &c->outbuf, &c->scalars})
    b->release();
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

int knng_forest(knng_ctx* c, const int8_t* codes_dev, int64_t n, int d, const int32_t* replay, int64_t n_replay,
                int32_t* perm_dev, uint8_t* leaf_flag_dev) {
  if (!c || !codes_dev || !perm_dev || !leaf_flag_dev || (n_replay > 0 && !replay)) return KNNG_E_ARGS;
  int st = check_shape(c, n, d);
  if (st) return st;
  cudaSetDevice(c->device);
  Scratch s;
  if ((st = ensure_scratch(c, n, &s, replay ? n_replay : 0))) return st;
  int64_t levels = 0;
  st = run_forest(codes_dev, n, d, c->prm.num_trees, c->prm.leaf_size, c->prm.seed, replay, replay ? n_replay : 0,
                  perm_dev, leaf_flag_dev, s.fb, c->stream, &levels, &c->last_error);
  if (st) return st;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  return e ? cuda_fail(c, e, "forest") : KNNG_OK;
}

int knng_init_graph(knng_ctx* c, const int8_t* codes_dev, int64_t n, int d, const int32_t* perm_dev,
                    const uint8_t* leaf_flag_dev, int32_t* ids_dev, int32_t* scores_dev) {
  if (!c || !codes_dev || !perm_dev || !leaf_flag_dev || !ids_dev || !scores_dev) return KNNG_E_ARGS;
  int st = check_shape(c, n, d);
  if (st) return st;
  cudaSetDevice(c->device);
  Scratch s;
  if ((st = ensure_scratch(c, n, &s, 0))) return st;
  st = run_init(codes_dev, n, d, c->prm.num_trees, c->prm.leaf_size, c->prm.k_build, c->prm.seed, perm_dev,
                leaf_flag_dev, ids_dev, scores_dev, s.ib, c->stream, nullptr, &c->last_error);
  if (st) return st;
  cudaError_t e = cudaStreamSynchronize(c->stream);
  return e ? cuda_fail(c, e, "init") : KNNG_OK;
}

int knng_join_iter(knng_ctx* c, const int8_t* codes_dev, const uint64_t* sketch_dev, int64_t n, int d,
                   const int32_t* ids_in, const int32_t* scores_in, int32_t* ids_out, int32_t* scores_out,
                   int64_t* updates) {
  if (!c || !codes_dev || !sketch_dev || !ids_in || !scores_in || !ids_out || !scores_out) return KNNG_E_ARGS;
  if ((ids_out == ids_in) != (scores_out == scores_in)) return set_error(c, KNNG_E_ARGS, "mixed in-place buffers");
  int st = check_shape(c, n, d);
  if (st) return st;
  cudaSetDevice(c->device);
  cudaError_t e;
  if ((e = c->scalars.ensure(4096))) return cuda_fail(c, e, "scalar allocation");
  unsigned long long* up = c->scalars.as<unsigned long long>(256);
  if ((e = cudaMemsetAsync(up, 0, 24, c->stream))) return cuda_fail(c, e, "update counter");
  const int K = c->prm.k_build;
  if ((e = launch_join(codes_dev, sketch_dev, n, d, K, K * c->prm.rerank_mult, ids_in, scores_in, ids_out,
                       scores_out, nullptr, up, c->num_sms, c->stream)))
    return cuda_fail(c, e, "join");
  unsigned long long h = 0;
  if ((e = cudaMemcpyAsync(&h, up, 8, cudaMemcpyDeviceToHost, c->stream))) return cuda_fail(c, e, "update count");
  if ((e = cudaStreamSynchronize(c->stream))) return cuda_fail(c, e, "join");
  if (updates) *updates = int64_t(h);
  return KNNG_OK;
}

int knng_export(const int32_t* ids_dev, const int32_t* scores_dev, int64_t n, int k_build, int k_eval,
                const int32_t* id_map_dev, int32_t* knns_dev, float* dists_dev, void* stream) {
  if (!ids_dev || !scores_dev || !knns_dev || !dists_dev || n < 0 || k_eval < 1 || k_eval > k_build)
    return KNNG_E_ARGS;
  cudaError_t e = launch_export(ids_dev, scores_dev, n, k_build, k_eval, id_map_dev, knns_dev, dists_dev,
                                static_cast<cudaStream_t>(stream));
  return e ? KNNG_E_CUDA : KNNG_OK;
}

int knng_build(knng_ctx* c, const void* rows, int64_t n, int d, int rows_on_device, int32_t* knns, float* dists,
               int out_on_device, knng_stats* stats) {
  using clk = std::chrono::steady_clock;
  const auto t_start = clk::now();
  const int64_t launches0 = launches();
  if (!c || !rows || !knns || !dists) return set_error(c, KNNG_E_ARGS, "null argument");
  int st = check_shape(c, n, d);
  if (st) return st;
  cudaSetDevice(c->device);
  const knng_params& p = c->prm;
  const int K = p.k_build, T = p.num_trees, W = d / 64;
  knng_stats local{};
  knng_stats& S = stats ? *stats : local;
  std::memset(&S, 0, sizeof(S));
  cudaError_t e;
  const size_t nk = size_t(n) * K;
  if ((e = c->codes.ensure(size_t(n) * d)) || (e = c->sketch.ensure(size_t(n) * W * 8)) ||
      (e = c->graph.ensure(nk * 16)) || (e = c->perm.ensure(size_t(T) * n * 4)) ||
      (e = c->leaf_flag.ensure(size_t(T) * n)))
    return cuda_fail(c, e, "device allocation");
  Scratch s;
  if ((st = ensure_scratch(c, n, &s, 0))) return st;
  cudaStream_t str = c->stream;
  int32_t* ids[2] = {c->graph.as<int32_t>(0), c->graph.as<int32_t>(nk * 8)};
  int32_t* scs[2] = {c->graph.as<int32_t>(nk * 4), c->graph.as<int32_t>(nk * 12)};
  cudaEventRecord(c->ev[0], str);
  if ((st = quantize_input(c, rows, n, d, rows_on_device))) return st;
  cudaEventRecord(c->ev[1], str);
  int64_t levels = 0, leaves = 0;
  if ((st = run_forest(c->codes.as<int8_t>(), n, d, T, p.leaf_size, p.seed, nullptr, 0, c->perm.as<int32_t>(),
                       c->leaf_flag.as<uint8_t>(), s.fb, str, &levels, &c->last_error)))
    return st;
  cudaEventRecord(c->ev[2], str);
  if ((st = run_init(c->codes.as<int8_t>(), n, d, T, p.leaf_size, K, p.seed, c->perm.as<int32_t>(),
                     c->leaf_flag.as<uint8_t>(), ids[0], scs[0], s.ib, str, &leaves, &c->last_error)))
    return st;
  cudaEventRecord(c->ev[3], str);
  unsigned long long* up = c->scalars.as<unsigned long long>(256);
  const int32_t* order = p.row_order == KNNG_ORDER_LEAF ? c->perm.as<int32_t>() : nullptr;
  int cur = 0, it = 0;
  float prev = 1.0f;
  for (; it < p.max_iterations; ++it) {
    const int nxt = p.join_mode == KNNG_JOIN_JACOBI ? 1 - cur : cur;
    unsigned long long h[3] = {0, 0, 0};
    if ((e = cudaMemsetAsync(up, 0, 24, str)) || (e = cudaEventRecord(c->jev[0], str)) ||
        (e = launch_join(c->codes.as<int8_t>(), c->sketch.as<uint64_t>(), n, d, K, K * p.rerank_mult, ids[cur],
                         scs[cur], ids[nxt], scs[nxt], order, up, c->num_sms, str)) ||
        (e = cudaEventRecord(c->jev[1], str)) ||
        (e = cudaMemcpyAsync(h, up, 24, cudaMemcpyDeviceToHost, str)) || (e = cudaStreamSynchronize(str)))
      return cuda_fail(c, e, "join iteration");
    cur = nxt;
    if (it < 64) {
      S.updates[it] = int64_t(h[0]);
      S.join_candidates[it] = int64_t(h[1]);
      S.join_dots[it] = int64_t(h[2]);
      S.join_ms[it] = elapsed(c->jev[0], c->jev[1]);
    }
    const float rate = float(h[0]) / float(uint64_t(n) * uint64_t(K));
    if (rate < p.early_stop_rate || (it > 0 && (prev - rate) < p.rate_diff_tol)) {
      ++it;
      break;
    }
    prev = rate;
  }

  cudaEventRecord(c->ev[4], str);
  int32_t* kd = knns;
  float* dd = dists;
  const size_t outn = size_t(n) * p.k_eval;
  if (!out_on_device) {
    if ((e = c->outbuf.ensure(outn * 8))) return cuda_fail(c, e, "output allocation");
    kd = c->outbuf.as<int32_t>(0);
    dd = c->outbuf.as<float>(outn * 4);
  }
  if ((e = launch_export(ids[cur], scs[cur], n, K, p.k_eval, nullptr, kd, dd, str))) return cuda_fail(c, e, "export");
  if (!out_on_device) {
    if ((e = cudaMemcpyAsync(knns, kd, outn * 4, cudaMemcpyDeviceToHost, str)) ||
        (e = cudaMemcpyAsync(dists, dd, outn * 4, cudaMemcpyDeviceToHost, str)))
      return cuda_fail(c, e, "output copy");
  }
  cudaEventRecord(c->ev[5], str);
  if ((e = cudaStreamSynchronize(str))) return cuda_fail(c, e, "build");
  S.quantize_s = elapsed(c->ev[0], c->ev[1]) * 1e-3;
  S.forest_s = elapsed(c->ev[1], c->ev[2]) * 1e-3;
  S.init_s = elapsed(c->ev[2], c->ev[3]) * 1e-3;
  S.join_s = elapsed(c->ev[3], c->ev[4]) * 1e-3;
  S.export_s = elapsed(c->ev[4], c->ev[5]) * 1e-3;
  S.build_s = elapsed(c->ev[1], c->ev[4]) * 1e-3;
  S.iterations = it;
  S.forest_levels = levels;
  S.leaves = leaves;
  S.device_s = elapsed(c->ev[0], c->ev[5]) * 1e-3;
  S.kernel_launches = launches() - launches0;
  S.total_s = std::chrono::duration<double>(clk::now() - t_start).count();
  return KNNG_OK;
}

}  // extern "C"
