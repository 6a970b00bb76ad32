// noalloc.cu -- knng_init_graph_noalloc: the initial-graph stage without any
// device allocation.
//
// Who needs it: callers that run inside a process whose GPU memory belongs to
// someone else's allocator -- a serving framework's caching pool, a database
// engine's device-memory manager, a plugin host -- and that may not call
// cudaMalloc/cudaFree themselves or let a library do it, because a raw
// allocation fragments or escapes that pool and cudaFree synchronises the whole
// device under the host's other streams.  Such a caller can still hand over
// its own input and output buffers; the stage's scratch (leaf Gram rows, the
// inverse permutation, leaf tables, scan space, counters) lives here instead,
// in one fixed file-scope device array.
//
// Limit: kNoAllocScratchBytes = 64 MiB, i.e. about 273 bytes per (tree, row)
// position plus 4 bytes per row: num_trees * n up to ~240,000 (n up to ~15,000
// rows with 16 trees).  Larger inputs are refused with KNNG_E_SCRATCH before
// any device work; use knng_init_graph (context-owned memory) for them.
//
// The array is part of the library's device image: every GPU that loads
// libknng.so holds these 64 MiB until the process exits.  Host code may not use
// the symbol g_init_scratch as a device address (on the host it names a
// host-side stand-in), so the first call on each device, with that device
// current, resolves the address with cudaGetSymbolAddress and caches it; make
// that first call before any stream capture.  All calls share the one array
// and it keeps the previous call's contents: the stage writes every scratch
// word it reads and clears its counter first.  Calls that overlap on the GPU
// (two streams or two host threads at once) race on the array and corrupt
// each other; serialise them.
#include "knng_internal.cuh"

#include <mutex>

namespace knng {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_init_scratch[kNoAllocScratchBytes];

std::mutex g_addr_mu;
void* g_addr[kMaxDevices] = {};

inline size_t round256(size_t b) { return (b + 255) & ~size_t(255); }

// The same carve as the context path's init scratch, from a caller-given base.
size_t carve_init(char* base, int64_t n, int T, InitBufs* ib) {
  const size_t tn = size_t(T) * size_t(n);
  size_t o = 0;
  auto take = [&](size_t bytes) {
    char* p = base ? base + o : nullptr;
    o += round256(bytes);
    return p;
  };
  char* gram = take(tn * kMaxLeaf * 4);
  char* pos = take(tn * 4);
  char* lo = take(tn * 4);
  char* idx = take(tn * 8);
  char* sz = take(tn);
  char* fix = take(size_t(n) * 4);
  char* scan = take(scan_tmp_bytes(int64_t(tn)));
  char* scal = take(4 * sizeof(int64_t));
  if (ib) {
    ib->gram = reinterpret_cast<int32_t*>(gram);
    ib->pos = reinterpret_cast<int32_t*>(pos);
    ib->leaf_lo = reinterpret_cast<int32_t*>(lo);
    ib->leaf_idx = reinterpret_cast<int32_t*>(idx);
    ib->leaf_sz = reinterpret_cast<uint8_t*>(sz);
    ib->fix_rows = reinterpret_cast<int32_t*>(fix);
    ib->scan_tmp = scan;
    ib->dev_i64 = reinterpret_cast<int64_t*>(scal);
  }
  return o;
}

// Device address of g_init_scratch on the current device (resolved once per device).
int scratch_address(int dev, void** out) {
  if (dev < 0 || dev >= kMaxDevices) return KNNG_E_ARGS;
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_init_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return KNNG_E_CUDA;
    }
    g_addr[dev] = p;
  }
  *out = g_addr[dev];
  return KNNG_OK;
}

}  // namespace
}  // namespace knng

extern "C" int knng_init_graph_noalloc(const int8_t* codes_dev, int64_t n, int d, int num_trees, int leaf_size,
                                       int k_build, uint32_t seed, const int32_t* perm_dev,
                                       const uint8_t* leaf_flag_dev, int32_t* ids_dev, int32_t* scores_dev,
                                       void* stream) {
  using namespace knng;
  if (!codes_dev || !perm_dev || !leaf_flag_dev || !ids_dev || !scores_dev) return KNNG_E_ARGS;
  if (n < 2 || num_trees < 1 || num_trees > 64 || leaf_size < 2 || leaf_size > kMaxLeaf || k_build < 1 ||
      k_build > kMaxK || int64_t(num_trees) * n > INT32_MAX)
    return KNNG_E_ARGS;
  if (!dim_ok(d)) return KNNG_E_DIM;
  if (carve_init(nullptr, n, num_trees, nullptr) > kNoAllocScratchBytes) return KNNG_E_SCRATCH;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return KNNG_E_CUDA;
  void* base = nullptr;
  int st = scratch_address(dev, &base);
  if (st) return st;
  InitBufs ib{};
  carve_init(static_cast<char*>(base), n, num_trees, &ib);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // one job covering all rows; its offset/size words live at the end of the scratch
  int32_t* jt_dev = reinterpret_cast<int32_t*>(ib.dev_i64 + 2);
  const int32_t jt_host[2] = {0, int32_t(n)};
  if (cudaMemcpyAsync(jt_dev, jt_host, sizeof(jt_host), cudaMemcpyHostToDevice, s) != cudaSuccess) return KNNG_E_CUDA;
  JobTable jt;
  jt.count = 1;
  jt.off = jt_dev;
  jt.n = jt_dev + 1;
  st = run_init(codes_dev, n, d, num_trees, leaf_size, k_build, seed, perm_dev, leaf_flag_dev, ids_dev, scores_dev,
                ib, s, nullptr, nullptr, jt);
  if (st) return st;
  return cudaStreamSynchronize(s) == cudaSuccess ? KNNG_OK : KNNG_E_CUDA;
}
