// hostcopy.cu -- transfers between the device and caller memory that the
// device does not map (pageable host memory: malloc, std::vector, numpy).
//
// The GPU and its copy engines never touch pageable caller memory.  On Grace +
// NVLink-C2C the GPU can read it through the CPU's page tables, but a large
// read there makes the driver start migrating the touched pages to GPU memory:
// on a GB300, after the quantise kernel had read 26 GB of pageable rows, every
// later build of the process took about 16.5 s of device time instead of
// 3.3 s, and a DMA from pageable memory ran at about 2 GB/s.  So host threads
// copy between the caller's memory and context-owned pinned buffers, which
// the GPU reads in place and the copy engines write at the link rate
// (pinned: about 210 GB/s device reads; 16 host threads: about 125 GB/s).
#include "knng_internal.cuh"

#include <sched.h>

#include <algorithm>
#include <cstring>

namespace knng {

cudaError_t PinnedBuf::ensure(size_t want) {
  if (want <= bytes) return cudaSuccess;
  release();
  void* q = nullptr;
  const cudaError_t e = cudaHostAlloc(&q, want, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return e;
  }
  p = q;
  bytes = want;
  return cudaSuccess;
}

void PinnedBuf::release() {
  if (p) cudaFreeHost(p);
  p = nullptr;
  bytes = 0;
}

int host_copy_threads() {
  cpu_set_t set;
  CPU_ZERO(&set);
  int n = 1;
  if (sched_getaffinity(0, sizeof(set), &set) == 0) n = CPU_COUNT(&set);
  return std::max(1, std::min(n, 32));
}

bool host_pageable(const void* ptr) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) {
    cudaGetLastError();
    return true;
  }
  return at.type == cudaMemoryTypeUnregistered;
}

CopyPool::CopyPool(int threads) : nthreads_(1) {
  // a thread that cannot be started leaves the pool smaller (no exception
  // leaves the library); the caller always copies slice 0 itself
  try {
    for (int t = 1; t < std::max(1, threads); ++t) {
      workers_.emplace_back([this, t] { run(t); });
      nthreads_ = t + 1;
    }
  } catch (...) {
  }
}

CopyPool::~CopyPool() {
  {
    std::lock_guard<std::mutex> lk(mu_);
    stop_ = true;
  }
  start_cv_.notify_all();
  for (auto& w : workers_) w.join();
}

// Slice t of the current job: 64-byte aligned boundaries, the last slice
// takes the remainder.
void CopyPool::slice(int t) {
  const size_t per = ((bytes_ / size_t(nthreads_)) + 63) & ~size_t(63);
  const size_t lo = std::min(bytes_, per * size_t(t)), hi = t + 1 == nthreads_ ? bytes_ : std::min(bytes_, lo + per);
  if (hi > lo) std::memcpy(dst_ + lo, src_ + lo, hi - lo);
}

void CopyPool::run(int t) {
  uint64_t seen = 0;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(mu_);
      start_cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
    }
    slice(t);
    {
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_cv_.notify_one();
    }
  }
}

void CopyPool::copy(void* dst, const void* src, size_t bytes) {
  if (bytes < (size_t(4) << 20) || nthreads_ == 1) {  // small: one thread
    std::memcpy(dst, src, bytes);
    return;
  }
  {
    std::lock_guard<std::mutex> lk(mu_);
    dst_ = static_cast<char*>(dst);
    src_ = static_cast<const char*>(src);
    bytes_ = bytes;
    pending_ = nthreads_ - 1;
    ++gen_;
  }
  start_cv_.notify_all();
  slice(0);  // the caller takes slice 0
  std::unique_lock<std::mutex> lk(mu_);
  done_cv_.wait(lk, [&] { return pending_ == 0; });
}

}  // namespace knng
