// serve.cu -- the serving loop: graph builds submitted as they arrive,
// admitted by device-memory footprint, batched continuously, overlapped on
// the device.
//
// No counterpart in the reference, which builds one graph per process
// (src/main.cpp:114-498).  A server owns `slots` worker threads, each with its
// own knng_ctx (CUDA stream + stream-ordered buffers).  Submitted jobs wait in
// one FIFO.  A worker that becomes free takes, in queue order, every job whose
// footprint (knng_footprint_bytes) still fits in the memory budget next to the
// batches already running -- a job that does not fit yet is passed over by
// later ones at most kMaxBypass times -- and builds them as one batch
// (knng_build_batch); jobs that arrive while other batches run are therefore
// admitted as soon as a slot and memory free up, and the batches of different
// slots run concurrently on their own streams.  A job larger than the whole
// budget is refused with KNNG_E_ADMIT.  After a batch the worker returns its
// buffers to the pool, so the memory charged to running batches bounds what
// the server holds.  Every job's knns/dists are bit-identical to knng_build
// of that job alone, whatever it was batched with.
#include "knng_internal.cuh"

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

namespace {

using clk = std::chrono::steady_clock;

struct Ticket {
  knng_job job{};
  int64_t footprint = 0;
  clk::time_point submitted, started, finished;
  bool done = false;
  int status = KNNG_E_BUSY;
  int batch_jobs = 0;
  int bypassed = 0;  // batches admitted ahead of this job while it did not fit
};

// How often a queued job that does not fit may be passed over by later,
// smaller jobs before admission waits for it (no starvation of large jobs).
constexpr int kMaxBypass = 4;

}  // namespace

struct knng_server {
  knng_server_params prm{};
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<uint64_t> queue;
  std::map<uint64_t, Ticket> tickets;
  uint64_t next_ticket = 1;
  int64_t in_use = 0;
  int running = 0;
  bool stop = false;
  std::vector<std::thread> workers;
  std::vector<knng_ctx*> ctxs;
  int64_t batches = 0, jobs_done = 0;
};

namespace {

void worker_loop(knng_server* sv, int slot) {
  knng_ctx* ctx = sv->ctxs[size_t(slot)];
  const int64_t budget = int64_t(sv->prm.mem_budget_gb * 1e9);
  // the only host allocations of the loop, made once: nothing below can throw
  std::vector<uint64_t> batch;
  std::vector<knng_job> jobs;
  try {
    batch.reserve(size_t(sv->prm.max_batch_jobs));
    jobs.reserve(size_t(sv->prm.max_batch_jobs));
  } catch (...) {
    return;  // this slot stays idle; the others serve the queue
  }
  for (;;) {
    batch.clear();
    jobs.clear();
    int64_t fp = 0;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      for (;;) {
        if (sv->stop) return;
        // refuse jobs that could never fit, wherever they are in the queue
        for (auto q = sv->queue.begin(); q != sv->queue.end();) {
          Ticket& t = sv->tickets[*q];
          if (t.footprint <= budget) {
            ++q;
            continue;
          }
          t.status = KNNG_E_ADMIT;
          t.done = true;
          t.started = t.finished = clk::now();
          q = sv->queue.erase(q);
          sv->cv_done.notify_all();
        }
        // FIFO with bounded backfill: a job that does not fit yet is passed
        // over by later jobs that do, until it has been passed over
        // kMaxBypass times; from then on nothing behind it is admitted, so the
        // memory that frees up goes to it.
        for (auto q = sv->queue.begin(); q != sv->queue.end() && int(batch.size()) < sv->prm.max_batch_jobs;) {
          Ticket& t = sv->tickets[*q];
          if (sv->in_use + fp + t.footprint <= budget) {
            fp += t.footprint;
            batch.push_back(*q);
            q = sv->queue.erase(q);
            continue;
          }
          if (t.bypassed >= kMaxBypass) break;
          ++q;
        }
        if (!batch.empty()) {
          // every job still queued that arrived before an admitted one was passed over
          clk::time_point latest = sv->tickets[batch.front()].submitted;
          for (uint64_t id : batch) latest = std::max(latest, sv->tickets[id].submitted);
          for (uint64_t id : sv->queue) {
            Ticket& t = sv->tickets[id];
            if (t.submitted >= latest) break;
            ++t.bypassed;
          }
        }
        if (!batch.empty()) break;
        sv->cv_work.wait(lk);
      }
      sv->in_use += fp;
      ++sv->running;
      const auto now = clk::now();
      for (uint64_t id : batch) sv->tickets[id].started = now;
    }
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      for (uint64_t id : batch) jobs.push_back(sv->tickets[id].job);
    }
    const int st = knng_build_batch(ctx, jobs.data(), int(jobs.size()), nullptr);
    knng_trim(ctx);
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      const auto now = clk::now();
      for (size_t b = 0; b < batch.size(); ++b) {
        Ticket& t = sv->tickets[batch[b]];
        t.job.status = st ? st : jobs[b].status;
        t.job.iterations = jobs[b].iterations;
        t.status = t.job.status;
        t.batch_jobs = int(batch.size());
        t.finished = now;
        t.done = true;
      }
      sv->in_use -= fp;
      --sv->running;
      ++sv->batches;
      sv->jobs_done += int64_t(batch.size());
    }
    sv->cv_done.notify_all();
    sv->cv_work.notify_all();  // memory freed: other idle slots may admit now
  }
}

void fill_result(const Ticket& t, knng_result* r) {
  if (!r) return;
  r->status = t.status;
  r->iterations = t.job.iterations;
  r->batch_jobs = t.batch_jobs;
  r->queued_s = std::chrono::duration<double>(t.started - t.submitted).count();
  r->run_s = std::chrono::duration<double>(t.finished - t.started).count();
  r->latency_s = std::chrono::duration<double>(t.finished - t.submitted).count();
}

}  // namespace

extern "C" {

void knng_server_default_params(knng_server_params* p) {
  if (!p) return;
  knng_default_params(&p->build);
  p->slots = 3;
  p->mem_budget_gb = 180.0;
  p->max_batch_jobs = 64;
}

int knng_server_create(knng_server** out, const knng_server_params* p) {
  if (!out) return KNNG_E_ARGS;
  *out = nullptr;
  knng_server* sv = new (std::nothrow) knng_server();
  if (!sv) return KNNG_E_OOM;
  if (p) sv->prm = *p; else knng_server_default_params(&sv->prm);
  if (sv->prm.slots < 1 || sv->prm.slots > 16 || sv->prm.max_batch_jobs < 1 || sv->prm.mem_budget_gb <= 0) {
    delete sv;
    return KNNG_E_ARGS;
  }
  try {
    sv->ctxs.reserve(size_t(sv->prm.slots));
    sv->workers.reserve(size_t(sv->prm.slots));
  } catch (...) {
    delete sv;
    return KNNG_E_OOM;
  }
  for (int s = 0; s < sv->prm.slots; ++s) {
    knng_ctx* c = nullptr;
    const int st = knng_create(&c, &sv->prm.build);
    if (st) {
      for (knng_ctx* x : sv->ctxs) knng_destroy(x);
      delete sv;
      return st;
    }
    sv->ctxs.push_back(c);
  }
  try {
    for (int s = 0; s < sv->prm.slots; ++s) sv->workers.emplace_back(worker_loop, sv, s);
  } catch (...) {  // a worker thread could not start: stop the ones that did
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      sv->stop = true;
    }
    sv->cv_work.notify_all();
    for (auto& t : sv->workers) t.join();
    for (knng_ctx* c : sv->ctxs) knng_destroy(c);
    delete sv;
    return KNNG_E_CUDA;
  }
  *out = sv;
  return KNNG_OK;
}

int knng_submit(knng_server* sv, const knng_job* job, uint64_t* ticket) {
  if (!sv || !job || !ticket || !job->rows || !job->knns || !job->dists || job->n < 2) return KNNG_E_ARGS;
  if (!knng::dim_ok(job->d)) return KNNG_E_DIM;
  Ticket t;
  t.job = *job;
  t.footprint = knng_footprint_bytes(&sv->prm.build, job->n, job->d, job->rows_on_device);
  t.submitted = clk::now();
  const int st = knng::abi_guard(nullptr, [&]() -> int {
    std::lock_guard<std::mutex> lk(sv->mu);
    const uint64_t id = sv->next_ticket;
    auto ins = sv->tickets.emplace(id, t);
    try {
      sv->queue.push_back(id);
    } catch (...) {
      sv->tickets.erase(ins.first);
      throw;
    }
    ++sv->next_ticket;
    *ticket = id;
    return KNNG_OK;
  });
  if (st == KNNG_OK) sv->cv_work.notify_one();
  return st;
}

int knng_poll(knng_server* sv, uint64_t ticket, knng_result* r) {
  if (!sv) return KNNG_E_ARGS;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->tickets.find(ticket);
  if (it == sv->tickets.end()) return KNNG_E_NOTFOUND;
  if (!it->second.done) return KNNG_E_BUSY;
  fill_result(it->second, r);
  return KNNG_OK;
}

int knng_wait(knng_server* sv, uint64_t ticket, double timeout_s, knng_result* r) {
  if (!sv) return KNNG_E_ARGS;
  std::unique_lock<std::mutex> lk(sv->mu);
  const auto until = clk::now() + std::chrono::duration_cast<clk::duration>(std::chrono::duration<double>(timeout_s));
  for (;;) {
    // looked up again after every wake-up: another thread may have released
    // the ticket while this one waited without the lock
    auto it = sv->tickets.find(ticket);
    if (it == sv->tickets.end()) return KNNG_E_NOTFOUND;
    if (it->second.done) {
      fill_result(it->second, r);
      return KNNG_OK;
    }
    if (sv->cv_done.wait_until(lk, until) == std::cv_status::timeout) {
      it = sv->tickets.find(ticket);
      if (it == sv->tickets.end()) return KNNG_E_NOTFOUND;
      if (!it->second.done) return KNNG_E_TIMEOUT;
    }
  }
}

int knng_release(knng_server* sv, uint64_t ticket) {
  if (!sv) return KNNG_E_ARGS;
  std::lock_guard<std::mutex> lk(sv->mu);
  auto it = sv->tickets.find(ticket);
  if (it == sv->tickets.end()) return KNNG_E_NOTFOUND;
  if (!it->second.done) return KNNG_E_BUSY;
  sv->tickets.erase(it);
  return KNNG_OK;
}

void knng_server_destroy(knng_server* sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto& t : sv->workers) t.join();
  for (knng_ctx* c : sv->ctxs) knng_destroy(c);
  delete sv;
}

}  // extern "C"
