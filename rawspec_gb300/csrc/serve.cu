// serve.cu -- the job server of rawspec_gb300_serve.h (host code).
//
// One request-loop thread owns every job's rawspec_context.  It admits
// pending jobs in submission order while a slot and the device-memory budget
// allow (the estimate of rawspec_gb300_device_bytes_estimate), and then, for
// each active job in turn: notices that its buffer in flight has completed
// (rawspec_check_for_completion: the context stream, dumps and callbacks
// included, is idle), hands it the next queued buffer
// (rawspec_copy_blocks_to_gpu_and_start_processing, which returns once the
// host blocks may be reused and leaves the kernels running on the job's
// streams), or, once the job is closed and drained, waits for it, frees it
// and returns its memory to the budget.  So the buffers of different jobs are
// copied and processed concurrently on the device, and a job submitted while
// others run starts as soon as it fits.
//
// Pushed buffers are copied by the pushing thread into the job's pool of
// pinned host slots (allocated when the job is admitted; a push to a pending
// job waits for them), which are the context's host blocks (caller-managed):
// the loop points the context's block pointers at the slot of the buffer for
// the call, so the request loop copies no data itself.  Slots return to a
// server-wide cache of pinned buffers when their job ends, so that jobs do
// not pay for page-locking memory.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "rawspec.h"
#include "rawspec_gb300.h"
#include "rawspec_gb300_serve.h"

namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Slot {
  char* data = nullptr;  // pinned, Nb host blocks
  double t_push = 0;
};

struct Job {
  int id = 0;
  rawspec_context ctx{};
  std::vector<float> aws;
  int fft_dir = 1;
  char expand4 = 0;
  size_t blk_bytes = 0;   // one host block
  rawspec_gb300_job_dump_fn fn = nullptr;
  void* user = nullptr;
  int state = RAWSPEC_GB300_JOB_PENDING;
  bool closed = false;
  int pushing = 0;               // pushes copying into a slot right now (the pool stays theirs)
  bool release_pending = false;  // the job ended while a push was copying: the last one frees the pool
  std::vector<std::pair<char*, size_t>> pool;  // pinned slots and their capacities
  std::vector<char*> free_slots;
  std::deque<Slot> queue;
  std::vector<char*> blocks;     // the context's host block pointers (caller-managed)
  bool inflight = false;
  Slot cur;                      // the buffer in flight
  std::atomic<double> t_inflight{0.0};
  size_t est = 0;
  long long buffers = 0;
  std::atomic<long long> dumps{0};
  std::vector<double> buf_lat;   // ms, loop thread
  std::mutex dump_mu;
  std::vector<double> dump_lat;  // ms, callback thread
  double t_submit = 0, t_admit = 0, t_done = 0;
};

double pct(std::vector<double> v, double q) {
  if (v.empty()) return 0.0;
  std::sort(v.begin(), v.end());
  const double pos = q * (double)(v.size() - 1);
  const size_t i = (size_t)pos;
  const double f = pos - (double)i;
  return i + 1 < v.size() ? v[i] * (1.0 - f) + v[i + 1] * f : v[i];
}

void job_dump_cb(rawspec_context* ctx, int product, int type) {
  Job* j = static_cast<Job*>(ctx->user_data);
  if (type == RAWSPEC_CALLBACK_POST_DUMP) {
    const double ms = 1e3 * (now_s() - j->t_inflight.load());
    {
      std::lock_guard<std::mutex> g(j->dump_mu);
      j->dump_lat.push_back(ms);
    }
    j->dumps++;
  }
  if (j->fn) j->fn(j->user, j->id, ctx, product, type);
}

}  // namespace

struct rawspec_gb300_server {
  int gpu = 0;
  std::mutex cache_mu;
  std::multimap<size_t, char*> cache;  // pinned buffers of finished jobs, by capacity
  size_t cache_bytes = 0;
  size_t budget = 0;
  int max_active = 1, max_queued = 2;
  std::mutex mu;
  std::condition_variable cv_loop;   // work for the request loop
  std::condition_variable cv_state;  // job state changes and queue space
  std::condition_variable cv_admit;  // pending jobs, or memory and slots freed
  std::map<int, std::unique_ptr<Job>> jobs;
  std::deque<int> pending;
  int next_id = 0;
  size_t used = 0, peak_used = 0;
  int active = 0, peak_active = 0;
  bool stop = false;
  // several ready jobs' buffers started together (RAWSPEC_GB300_SERVE_GROUP=0: never)
  bool group = true;
  long long group_calls = 0;
  std::thread loop;
  std::thread admitter;  // admission (pinned slots, context creation) off the request loop
};

namespace {

constexpr size_t kCacheCap = size_t(8) << 30;  // pinned bytes kept for later jobs
constexpr int kGroupMax = 16;                    // buffers started together at most
// Buffers from this size on keep the combined copy-and-process call, which
// overlaps the copy of each channel group with its processing; smaller ones
// are copied whole anyway and may share launches with other jobs' buffers.
constexpr size_t kGroupMaxBytes = size_t(16) << 20;

char* take_pinned(rawspec_gb300_server* s, size_t bytes, size_t* cap) {
  {
    std::lock_guard<std::mutex> g(s->cache_mu);
    auto it = s->cache.lower_bound(bytes);
    if (it != s->cache.end() && it->first <= 2 * bytes) {
      char* p = it->second;
      *cap = it->first;
      s->cache_bytes -= it->first;
      s->cache.erase(it);
      return p;
    }
  }
  char* p = nullptr;
  if (cudaHostAlloc((void**)&p, bytes, cudaHostAllocDefault) != cudaSuccess) return nullptr;
  *cap = bytes;
  return p;
}

void give_pinned(rawspec_gb300_server* s, char* p, size_t cap) {
  {
    std::lock_guard<std::mutex> g(s->cache_mu);
    if (s->cache_bytes + cap <= kCacheCap) {
      s->cache.emplace(cap, p);
      s->cache_bytes += cap;
      return;
    }
  }
  cudaFreeHost(p);
}

void free_pool(rawspec_gb300_server* s, Job* j) {
  if (j->pushing > 0) {  // a push is copying into one of the slots
    j->release_pending = true;
    return;
  }
  for (auto& pc : j->pool) give_pinned(s, pc.first, pc.second);
  j->pool.clear();
  j->free_slots.clear();
}

// Called with the lock held; the job leaves the active set.
void retire(rawspec_gb300_server* s, Job* j, int state) {
  j->state = state;
  j->t_done = now_s();
  s->active--;
  s->used -= j->est;
  s->cv_state.notify_all();
  s->cv_admit.notify_all();
}

// Admission in submission order, on a thread of its own: taking a job's
// pinned slots and creating its context take milliseconds (tens for a large
// job's first buffers of a size), during which the request loop keeps
// feeding the active jobs.
void admit_loop(rawspec_gb300_server* s) {
  cudaSetDevice(s->gpu);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    // admission in submission order
    while (!s->pending.empty()) {
      Job* j = s->jobs[s->pending.front()].get();
      if (s->active >= s->max_active || s->used + j->est > s->budget) break;
      s->pending.pop_front();
      s->active++;
      s->used += j->est;
      s->peak_active = std::max(s->peak_active, s->active);
      lk.unlock();
      // the job's pinned slots, which are also the context's host blocks
      // (already page-locked, so the library uses them as they are); the
      // loop points the block pointers at each buffer's slot
      int rc = 0;
      std::vector<std::pair<char*, size_t>> pool;
      for (int k = 0; k < s->max_queued && rc == 0; k++) {
        size_t cap = 0;
        char* p = take_pinned(s, j->blk_bytes * j->ctx.Nb, &cap);
        if (p) pool.emplace_back(p, cap);
        else rc = 1;
      }
      if (rc == 0) {
        j->blocks.resize(j->ctx.Nb);
        for (unsigned b = 0; b < j->ctx.Nb; b++) j->blocks[b] = pool[0].first + b * j->blk_bytes;
        j->ctx.h_blkbufs = j->blocks.data();
        j->ctx.Nb_host = j->ctx.Nb;
        rc = rawspec_initialize(&j->ctx);
      }
      lk.lock();
      j->pool = pool;
      for (auto& pc : pool) j->free_slots.push_back(pc.first);
      if (rc) {
        free_pool(s, j);
        retire(s, j, RAWSPEC_GB300_JOB_FAILED);
        continue;
      }
      const size_t actual = rawspec_gb300_device_bytes(&j->ctx);
      if (actual > j->est) {  // never expected: the estimate repeats the allocation plan
        s->used += actual - j->est;
        j->est = actual;
      }
      s->peak_used = std::max(s->peak_used, s->used);
      j->state = RAWSPEC_GB300_JOB_ACTIVE;
      j->t_admit = now_s();
      s->cv_state.notify_all();
      s->cv_loop.notify_all();
    }

    if (s->stop && s->pending.empty()) break;
    s->cv_admit.wait_for(lk, std::chrono::milliseconds(5));
  }
}

void request_loop(rawspec_gb300_server* s) {
  cudaSetDevice(s->gpu);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    bool progress = false, busy = false;
    // Jobs whose next buffer can start: with two or more, their buffers are
    // copied and then started together, so that launches of the same kernel
    // configuration share one grid (rawspec_gb300_start_processing_group).
    if (s->group) {
      std::vector<Job*> ready;
      for (auto& kv : s->jobs) {
        Job* j = kv.second.get();
        if (j->state != RAWSPEC_GB300_JOB_ACTIVE || j->queue.empty() || (int)ready.size() >= kGroupMax) continue;
        size_t in_bytes = 0;
        rawspec_gb300_device_input(&j->ctx, &in_bytes);
        if (in_bytes >= kGroupMaxBytes) continue;  // the pipelined single call serves it better
        if (j->inflight) {
          lk.unlock();
          const bool idle = rawspec_check_for_completion(&j->ctx) != 0;
          lk.lock();
          if (!idle) continue;
          j->inflight = false;
          j->buffers++;
          j->buf_lat.push_back(1e3 * (now_s() - j->cur.t_push));
          progress = true;
        }
        ready.push_back(j);
      }
      // only jobs that share a small-FFT kernel configuration with another
      // ready job gain from starting together; the others keep the single call
      {
        std::map<long long, int> count;
        std::vector<std::vector<long long>> keys(ready.size());
        for (size_t r = 0; r < ready.size(); r++) {
          const rawspec_context& c = ready[r]->ctx;
          for (unsigned i = 0; i < c.No; i++)
            if (rawspec_gb300_product_kernel(const_cast<rawspec_context*>(&c), (int)i) == RAWSPEC_GB300_K_SMALL)
              keys[r].push_back(((long long)c.Nts[i] << 16) | ((long long)c.Nbps << 8) | ((long long)c.Np << 4) |
                                (long long)(c.Npolout[i] + 4));
          std::sort(keys[r].begin(), keys[r].end());
          keys[r].erase(std::unique(keys[r].begin(), keys[r].end()), keys[r].end());
          for (long long k : keys[r]) count[k]++;
        }
        std::vector<Job*> shared;
        for (size_t r = 0; r < ready.size(); r++) {
          bool any = false;
          for (long long k : keys[r]) any = any || count[k] >= 2;
          if (any) shared.push_back(ready[r]);
        }
        ready.swap(shared);
      }
      if (ready.size() >= 2) {
        for (Job* j : ready) {
          j->cur = j->queue.front();
          j->queue.pop_front();
        }
        lk.unlock();
        std::vector<rawspec_context*> ctxs;
        std::vector<int> dirs;
        int rc = 0;
        for (Job* j : ready) {
          for (unsigned b = 0; b < j->ctx.Nb; b++) j->blocks[b] = j->cur.data + b * j->blk_bytes;
          j->t_inflight.store(j->cur.t_push);
          rc |= j->expand4 ? rawspec_copy_blocks_to_gpu_expanding_complex4(&j->ctx, 0, 0, j->ctx.Nb)
                           : rawspec_copy_blocks_to_gpu(&j->ctx, 0, 0, j->ctx.Nb);
          ctxs.push_back(&j->ctx);
          dirs.push_back(j->fft_dir);
        }
        if (rc == 0) rc = rawspec_gb300_start_processing_group(ctxs.data(), dirs.data(), (int)ctxs.size());
        if (rc == 0) s->group_calls++;
        lk.lock();
        for (Job* j : ready) {
          j->free_slots.push_back(j->cur.data);  // the copies have completed
          j->inflight = true;
        }
        s->cv_state.notify_all();
        progress = true;
        busy = true;
        if (rc) {
          for (Job* j : ready) {
            lk.unlock();
            rawspec_wait_for_completion(&j->ctx);
            rawspec_cleanup(&j->ctx);
            lk.lock();
            j->inflight = false;
            free_pool(s, j);
            retire(s, j, RAWSPEC_GB300_JOB_FAILED);
          }
        }
      }
    }
    for (auto& kv : s->jobs) {
      Job* j = kv.second.get();
      if (j->state != RAWSPEC_GB300_JOB_ACTIVE) continue;
      if (j->inflight) {
        lk.unlock();
        const bool idle = rawspec_check_for_completion(&j->ctx) != 0;
        lk.lock();
        if (!idle) {
          busy = true;
          continue;
        }
        j->inflight = false;
        j->buffers++;
        j->buf_lat.push_back(1e3 * (now_s() - j->cur.t_push));
        progress = true;
      }
      if (!j->queue.empty()) {
        j->cur = j->queue.front();
        j->queue.pop_front();
        lk.unlock();
        for (unsigned b = 0; b < j->ctx.Nb; b++) j->blocks[b] = j->cur.data + b * j->blk_bytes;
        j->t_inflight.store(j->cur.t_push);
        const int rc =
            rawspec_copy_blocks_to_gpu_and_start_processing(&j->ctx, j->ctx.Nb, j->expand4, j->fft_dir);
        lk.lock();
        j->free_slots.push_back(j->cur.data);  // the host blocks may be reused once the call returns
        s->cv_state.notify_all();
        progress = true;
        if (rc) {
          lk.unlock();
          rawspec_wait_for_completion(&j->ctx);
          rawspec_cleanup(&j->ctx);
          lk.lock();
          free_pool(s, j);
          retire(s, j, RAWSPEC_GB300_JOB_FAILED);
          continue;
        }
        j->inflight = true;
        busy = true;
      } else if (j->closed && j->pushing == 0) {
        lk.unlock();
        const int rc = rawspec_wait_for_completion(&j->ctx);
        rawspec_cleanup(&j->ctx);
        lk.lock();
        free_pool(s, j);
        retire(s, j, rc ? RAWSPEC_GB300_JOB_FAILED : RAWSPEC_GB300_JOB_DONE);
        progress = true;
      }
    }
    if (s->stop && s->pending.empty() && s->active == 0) break;
    if (!progress) s->cv_loop.wait_for(lk, busy ? std::chrono::microseconds(20) : std::chrono::milliseconds(5));
  }
}

Job* find(rawspec_gb300_server* s, int id) {
  auto it = s->jobs.find(id);
  return it == s->jobs.end() ? nullptr : it->second.get();
}

}  // namespace

#pragma GCC visibility push(default)
extern "C" {

rawspec_gb300_server* rawspec_gb300_server_create(int gpu_index, size_t hbm_budget, int max_active, int max_queued) {
  if (max_active < 1 || max_queued < 1 || hbm_budget == 0) return nullptr;
  if (cudaSetDevice(gpu_index) != cudaSuccess) return nullptr;
  auto* s = new (std::nothrow) rawspec_gb300_server();
  if (!s) return nullptr;
  s->gpu = gpu_index;
  s->budget = hbm_budget;
  s->max_active = max_active;
  s->max_queued = max_queued;
  if (const char* v = getenv("RAWSPEC_GB300_SERVE_GROUP")) s->group = v[0] != '0';
  try {
    s->loop = std::thread(request_loop, s);
  } catch (...) {
    delete s;
    return nullptr;
  }
  try {
    s->admitter = std::thread(admit_loop, s);
  } catch (...) {
    {
      std::lock_guard<std::mutex> g(s->mu);
      s->stop = true;
      s->cv_loop.notify_all();
    }
    s->loop.join();
    delete s;
    return nullptr;
  }
  return s;
}

int rawspec_gb300_server_submit(rawspec_gb300_server* s, const rawspec_context* job, int fft_dir,
                                rawspec_gb300_job_dump_fn fn, void* user) {
  if (!s || !job) return -1;
  auto j = std::make_unique<Job>();
  rawspec_context& c = j->ctx;
  // client fields only; the library's own fields start empty
  c.No = job->No;
  c.Np = job->Np;
  c.Nant = job->Nant;
  c.Nc = job->Nc;
  c.Ntpb = job->Ntpb;
  c.Nbc = job->Nbc;
  c.Nbps = job->Nbps;
  for (int i = 0; i < MAX_OUTPUTS; i++) {
    c.Npolout[i] = job->Npolout[i];
    c.Nts[i] = job->Nts[i];
    c.Nas[i] = job->Nas[i];
  }
  c.Nb = job->Nb;
  c.gpu_index = s->gpu;
  c.input_conjugated = job->input_conjugated;
  c.incoherently_sum = job->incoherently_sum;
  c.Naws = job->Naws;
  if (job->incoherently_sum && job->Naws > 0 && job->Aws) {
    j->aws.assign(job->Aws, job->Aws + job->Naws);
    c.Aws = j->aws.data();
  } else {
    c.Aws = nullptr;
  }
  j->expand4 = job->Nbps == 4 ? 1 : 0;
  rawspec_context v = c;
  size_t est = 0;
  if (rawspec_gb300_validate(&v) || rawspec_gb300_device_bytes_estimate(&c, &est) || est > s->budget) return -1;
  c.Nb = v.Nb;
  j->blk_bytes = j->expand4 ? (size_t)v.Nc * v.Ntpb * v.Np : (size_t)v.Nc * v.Ntpb * v.Np * 2 * (v.Nbps / 8);
  j->est = est;
  j->fft_dir = fft_dir;
  j->fn = fn;
  j->user = user;
  c.dump_callback = job_dump_cb;
  c.user_data = j.get();
  j->t_submit = now_s();
  std::lock_guard<std::mutex> g(s->mu);
  if (s->stop) return -1;
  const int id = s->next_id++;
  j->id = id;
  s->jobs[id] = std::move(j);
  s->pending.push_back(id);
  s->cv_admit.notify_all();
  return id;
}

int rawspec_gb300_server_push(rawspec_gb300_server* s, int job, const void* data, size_t bytes) {
  if (!s || !data) return 1;
  std::unique_lock<std::mutex> lk(s->mu);
  Job* j = find(s, job);
  if (!j || j->closed || j->state >= RAWSPEC_GB300_JOB_DONE || bytes != j->blk_bytes * j->ctx.Nb) return 1;
  if (!s->cv_state.wait_for(lk, std::chrono::seconds(60), [&] {
        return !j->free_slots.empty() || j->state >= RAWSPEC_GB300_JOB_DONE;
      }))
    return 1;
  if (j->state >= RAWSPEC_GB300_JOB_DONE) return 1;
  char* slot = j->free_slots.back();
  j->free_slots.pop_back();
  j->pushing++;
  lk.unlock();
  memcpy(slot, data, bytes);
  const double t = now_s();
  lk.lock();
  j->pushing--;
  if (j->state >= RAWSPEC_GB300_JOB_DONE) {  // the job failed meanwhile
    if (j->pushing == 0 && j->release_pending) {
      j->release_pending = false;
      free_pool(s, j);
    }
    return 1;
  }
  j->queue.push_back(Slot{slot, t});
  s->cv_loop.notify_all();
  return 0;
}

int rawspec_gb300_server_close_job(rawspec_gb300_server* s, int job) {
  if (!s) return 1;
  std::lock_guard<std::mutex> g(s->mu);
  Job* j = find(s, job);
  if (!j) return 1;
  j->closed = true;
  s->cv_loop.notify_all();
  return 0;
}

int rawspec_gb300_server_wait_job(rawspec_gb300_server* s, int job, double timeout_s) {
  if (!s) return -1;
  std::unique_lock<std::mutex> lk(s->mu);
  Job* j = find(s, job);
  if (!j) return -1;
  auto done = [&] { return j->state >= RAWSPEC_GB300_JOB_DONE; };
  if (timeout_s < 0) s->cv_state.wait(lk, done);
  else if (!s->cv_state.wait_for(lk, std::chrono::duration<double>(timeout_s), done)) return -1;
  return j->state;
}

int rawspec_gb300_server_job_stats(rawspec_gb300_server* s, int job, rawspec_gb300_job_stats* st) {
  if (!s || !st) return 1;
  std::lock_guard<std::mutex> g(s->mu);
  Job* j = find(s, job);
  if (!j) return 1;
  std::vector<double> dl;
  {
    std::lock_guard<std::mutex> g2(j->dump_mu);
    dl = j->dump_lat;
  }
  st->state = j->state;
  st->buffers = j->buffers;
  st->dumps = j->dumps.load();
  st->t_submit = j->t_submit;
  st->t_admit = j->t_admit;
  st->t_done = j->t_done;
  st->buffer_p50_ms = pct(j->buf_lat, 0.50);
  st->buffer_p99_ms = pct(j->buf_lat, 0.99);
  st->dump_p50_ms = pct(dl, 0.50);
  st->dump_p99_ms = pct(dl, 0.99);
  st->device_bytes = j->est;
  return 0;
}

int rawspec_gb300_server_get_stats(rawspec_gb300_server* s, rawspec_gb300_server_stats* st) {
  if (!s || !st) return 1;
  std::lock_guard<std::mutex> g(s->mu);
  memset(st, 0, sizeof(*st));
  std::vector<double> bl, dl;
  for (auto& kv : s->jobs) {
    Job* j = kv.second.get();
    switch (j->state) {
      case RAWSPEC_GB300_JOB_PENDING: st->pending++; break;
      case RAWSPEC_GB300_JOB_ACTIVE: st->active++; break;
      case RAWSPEC_GB300_JOB_DONE: st->done++; break;
      default: st->failed++; break;
    }
    st->buffers += j->buffers;
    st->dumps += j->dumps.load();
    bl.insert(bl.end(), j->buf_lat.begin(), j->buf_lat.end());
    std::lock_guard<std::mutex> g2(j->dump_mu);
    dl.insert(dl.end(), j->dump_lat.begin(), j->dump_lat.end());
  }
  st->budget = s->budget;
  st->used = s->used;
  st->peak_used = s->peak_used;
  st->peak_active = s->peak_active;
  st->group_calls = s->group_calls;
  st->buffer_p50_ms = pct(bl, 0.50);
  st->buffer_p99_ms = pct(bl, 0.99);
  st->dump_p50_ms = pct(dl, 0.50);
  st->dump_p99_ms = pct(dl, 0.99);
  return 0;
}

void rawspec_gb300_server_destroy(rawspec_gb300_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (auto& kv : s->jobs) kv.second->closed = true;
    s->stop = true;
    s->cv_loop.notify_all();
    s->cv_admit.notify_all();
  }
  s->admitter.join();  // admits the pending jobs (closed: they run their queued buffers and end)
  s->loop.join();
  for (auto& kv : s->jobs) free_pool(s, kv.second.get());
  for (auto& kv : s->cache) cudaFreeHost(kv.second);
  delete s;
}

}  // extern "C"
#pragma GCC visibility pop
