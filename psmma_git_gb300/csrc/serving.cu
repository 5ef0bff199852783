// Serving loop: continuous batching of structured multiplies on one device.
//
// Requests (any kind, any size, device-resident operands) are queued by psmma_server_submit.
// A dispatcher thread admits them in arrival order as soon as (a) one of `max_inflight`
// stream slots is free and (b) the request's workspace fits in the remaining part of an
// HBM budget that was allocated once at creation (first-fit arena, no allocation per
// request).  Each admitted request runs on its own stream, so requests that arrive while
// others are on the GPU overlap with them.  The stream's priority follows admission order: a
// request admitted while c others are in flight runs at the c-th highest priority (clamped
// to the device's range), so when SMs free up the GPU prefers the oldest request's kernels.
// Without it the requests share the SMs evenly and a large request is slowed by every request
// admitted after it, which sets the latency tail.  A host function enqueued after the request's
// kernels hands it to a completion thread, which frees its arena slice and slot, reads its
// CUDA-event GPU time and status, and wakes the waiters and the dispatcher.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "psmma_internal.h"

namespace psmma {
namespace {

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

constexpr size_t kArenaAlign = 4096;
size_t round_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// First-fit allocator over [0, size) with coalescing of free neighbours.
class Arena {
 public:
  void init(size_t size) { free_[0] = size; total_ = size; }
  bool alloc(size_t bytes, size_t* off) {
    bytes = round_up(std::max<size_t>(bytes, 1), kArenaAlign);
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        size_t rest = it->second - bytes, start = it->first + bytes;
        free_.erase(it);
        if (rest) free_[start] = rest;
        used_[*off] = bytes;
        return true;
      }
    }
    return false;
  }
  void release(size_t off) {
    auto u = used_.find(off);
    if (u == used_.end()) return;
    size_t sz = u->second;
    used_.erase(u);
    auto it = free_.emplace(off, sz).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }
  size_t total() const { return total_; }

 private:
  std::map<size_t, size_t> free_, used_;
  size_t total_ = 0;
};

struct Job {
  unsigned long long ticket = 0;
  psmma_request req;
  size_t work_bytes = 0;
  size_t work_off = 0;
  int slot = -1;
  double submit_s = 0, start_s = 0, end_s = 0;
  int status = PSMMA_OK;
  float gpu_ms = 0.0f;
  bool done = false;
};

}  // namespace
}  // namespace psmma

struct psmma_server {
  int device = 0;
  void* arena_base = nullptr;
  psmma::Arena arena;
  int max_inflight = 1;
  std::vector<std::vector<cudaStream_t>> streams;  // [slot][priority level], level 0 highest
  std::vector<cudaStream_t> slot_stream;           // the stream of the slot's current request
  int levels = 1;
  std::vector<cudaEvent_t> ev_start, ev_end;
  std::vector<bool> slot_busy;
  unsigned* dev_status = nullptr;   // one word per slot
  unsigned* host_status = nullptr;  // pinned, one word per slot

  std::mutex mu;
  std::condition_variable cv_dispatch, cv_done, cv_complete;
  std::deque<unsigned long long> pending;
  std::unordered_map<unsigned long long, psmma::Job> jobs;
  std::deque<int> completed_slots;
  std::vector<unsigned long long> slot_ticket;
  unsigned long long next_ticket = 1;
  bool stop = false;
  std::thread dispatcher, completer;
  unsigned long long n_done = 0;
};

namespace psmma {
namespace {

size_t request_workspace(const psmma_request& r) {
  psmma_opts o;
  memset(&o, 0, sizeof(o));
  o.precision = r.precision;
  o.n_moduli = r.n_moduli;
  if (r.kind == KIND_CAUCHY_EIG)
    return r.precision == PSMMA_PREC_SPLIT ? split_workspace_general(r.n, r.k, r.k, r.n_moduli) : 0;
  if (r.precision == PSMMA_PREC_SPLIT) return split_workspace_bytes(r.kind, r.n, r.k, r.n_moduli);
  if (r.kind == KIND_DFT) return dft_f64_workspace(r.n, r.k);
  return 0;
}

// Validates a request (the same rules as the direct entry points).
int check_request(const psmma_request& r) {
  if ((r.kind < KIND_CAUCHY || r.kind > KIND_DFT) && r.kind != KIND_CAUCHY_EIG) return PSMMA_EUNSUPPORTED;
  if (r.precision != PSMMA_PREC_FP64 && r.precision != PSMMA_PREC_SPLIT) return PSMMA_EUNSUPPORTED;
  if (r.n_moduli != 0 && (r.n_moduli < 8 || r.n_moduli > 16)) return PSMMA_EUNSUPPORTED;
  const bool dft = r.kind == KIND_DFT, eig = r.kind == KIND_CAUCHY_EIG;  // INFO numbers of PZMDFTL,
  if (r.n < 0) return dft || eig ? -1 : -2;                                   // PSCAUCHYEIG_COMPUTE
  if (r.k < 0) return dft || eig ? -2 : -3;
  if (r.lda < std::max(1, r.n)) return dft || eig ? -7 : -9;
  if (r.ldq < std::max(1, r.n)) return dft ? -10 : eig ? -17 : -14;
  if (r.n > 0 && r.k > 0) {
    if (!r.Q || !r.A) return PSMMA_ENULL;
    if (!dft) {
      long need = (r.kind == KIND_CAUCHY || eig) ? (long)r.k : 2L * r.k - 1;
      if (!r.gen || r.ldgen < need) return PSMMA_EGEN;
    }
  }
  return PSMMA_OK;
}

// Enqueues the request's kernels on the slot's stream (no synchronisation).
int launch_job(psmma_server* s, Job& j) {
  const psmma_request& r = j.req;
  cudaStream_t st = s->slot_stream[j.slot];
  void* work = j.work_bytes ? (char*)s->arena_base + j.work_off : nullptr;
  unsigned* status = s->dev_status + j.slot;
  if (cudaMemsetAsync(status, 0, sizeof(unsigned), st) != cudaSuccess) return PSMMA_EDEVICE;
  if (r.n == 0 || r.k == 0) return PSMMA_OK;
  if (r.kind == KIND_CAUCHY_EIG) {
    const GenSpec gs = eig_gens_packed(r.gen, r.ldgen, r.k);
    if (r.precision == PSMMA_PREC_SPLIT && r.alpha != 0.0)
      return launch_split_general(r.n, r.k, r.k, r.alpha, (const double*)r.A, r.lda, gs, r.beta, (double*)r.Q,
                                  r.ldq, r.n_moduli, work, j.work_bytes, st, status);
    return launch_struct_f64(r.n, r.k, r.k, r.alpha, (const double*)r.A, r.lda, gs, r.beta, (double*)r.Q, r.ldq, st);
  }
  if (r.precision == PSMMA_PREC_SPLIT && r.alpha != 0.0)
    return launch_split_any(r.kind, r.n, r.k, r.alpha, (const double*)r.A, r.lda, r.gen, r.ldgen, r.beta,
                            (double*)r.Q, r.ldq, r.n_moduli, work, j.work_bytes, st, status);
  if (r.kind == KIND_DFT) {
    if (r.alpha == 0.0) {
      GenSpec gs;
      gs.kind = KIND_DFT;
      return launch_struct_f64(2 * r.n, r.k, 2 * r.n, 0.0, nullptr, 2L * r.lda, gs, r.beta, (double*)r.Q, 2L * r.ldq,
                               st);
    }
    return launch_dft_f64(r.n, r.k, r.alpha, (const double*)r.A, r.lda, r.beta, (double*)r.Q, r.ldq, work,
                          j.work_bytes, st);
  }
  return launch_struct_f64(r.n, r.k, r.k, r.alpha, (const double*)r.A, r.lda,
                           reference_gens(r.kind, r.gen, r.ldgen, r.k), r.beta, (double*)r.Q, r.ldq, st);
}

struct HostCbCtx {
  psmma_server* s;
  int slot;
};

// Runs on a CUDA callback thread: no CUDA calls here, only hand-off to the completer.
void CUDART_CB on_stream_done(void* p) {
  HostCbCtx* c = (HostCbCtx*)p;
  psmma_server* s = c->s;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->completed_slots.push_back(c->slot);
  }
  s->cv_complete.notify_one();
  delete c;
}

void dispatcher_main(psmma_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    int slot = -1;
    size_t off = 0;
    s->cv_dispatch.wait(lk, [&] {
      if (s->stop) return true;
      if (s->pending.empty()) return false;
      slot = -1;
      for (int i = 0; i < s->max_inflight; ++i)
        if (!s->slot_busy[i]) { slot = i; break; }
      if (slot < 0) return false;
      Job& head = s->jobs[s->pending.front()];
      return head.work_bytes == 0 || s->arena.alloc(head.work_bytes, &off);
    });
    if (s->stop) return;
    int busy = 0;
    for (int i = 0; i < s->max_inflight; ++i) busy += s->slot_busy[i] ? 1 : 0;
    s->slot_stream[slot] = s->streams[slot][std::min(busy, s->levels - 1)];
    const unsigned long long t = s->pending.front();
    s->pending.pop_front();
    Job& j = s->jobs[t];
    j.slot = slot;
    j.work_off = off;
    j.start_s = now_s();
    s->slot_busy[slot] = true;
    s->slot_ticket[slot] = t;
    Job copy = j;
    lk.unlock();
    // enqueue outside the lock; only this thread launches work
    cudaStream_t st = s->slot_stream[slot];
    int e = (cudaEventRecord(s->ev_start[slot], st) == cudaSuccess) ? PSMMA_OK : PSMMA_EDEVICE;
    if (!e) e = launch_job(s, copy);
    if (cudaEventRecord(s->ev_end[slot], st) != cudaSuccess && !e) e = PSMMA_EDEVICE;
    cudaMemcpyAsync(s->host_status + slot, s->dev_status + slot, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    bool cb_ok = cudaLaunchHostFunc(st, on_stream_done, new HostCbCtx{s, slot}) == cudaSuccess;
    lk.lock();
    s->jobs[t].status = e;
    if (!cb_ok) {  // no callback will come: complete it here
      s->completed_slots.push_back(slot);
      s->cv_complete.notify_one();
    }
  }
}

void completer_main(psmma_server* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    s->cv_complete.wait(lk, [&] { return s->stop || !s->completed_slots.empty(); });
    if (s->completed_slots.empty() && s->stop) return;
    const int slot = s->completed_slots.front();
    s->completed_slots.pop_front();
    const unsigned long long t = s->slot_ticket[slot];
    lk.unlock();
    float ms = 0.0f;
    cudaEventSynchronize(s->ev_end[slot]);
    cudaEventElapsedTime(&ms, s->ev_start[slot], s->ev_end[slot]);
    const unsigned dev_st = s->host_status[slot];
    lk.lock();
    Job& j = s->jobs[t];
    j.end_s = now_s();
    j.gpu_ms = ms;
    if (!j.status && (dev_st & 1u)) j.status = PSMMA_ETIMEDOUT;
    j.done = true;
    if (j.work_bytes) s->arena.release(j.work_off);
    s->slot_busy[slot] = false;
    s->n_done++;
    s->cv_done.notify_all();
    s->cv_dispatch.notify_one();
  }
}

}  // namespace
}  // namespace psmma

using namespace psmma;

extern "C" {

int psmma_server_create(size_t hbm_budget_bytes, int max_inflight, psmma_server** out) {
  if (!out || max_inflight < 1 || max_inflight > 64) return PSMMA_EUNSUPPORTED;
  *out = nullptr;
  psmma_server* s = new psmma_server();
  if (cudaGetDevice(&s->device) != cudaSuccess) { delete s; return PSMMA_EDEVICE; }
  s->max_inflight = max_inflight;
  if (hbm_budget_bytes) {
    if (cudaMalloc(&s->arena_base, hbm_budget_bytes) != cudaSuccess) {
      cudaGetLastError();
      delete s;
      return PSMMA_ENOMEM;
    }
  }
  s->arena.init(hbm_budget_bytes);
  if (cudaMalloc((void**)&s->dev_status, sizeof(unsigned) * max_inflight) != cudaSuccess ||
      cudaMallocHost((void**)&s->host_status, sizeof(unsigned) * max_inflight) != cudaSuccess) {
    cudaFree(s->arena_base);
    cudaFree(s->dev_status);
    delete s;
    return PSMMA_ENOMEM;
  }
  int least = 0, greatest = 0;
  if (cudaDeviceGetStreamPriorityRange(&least, &greatest) != cudaSuccess) least = greatest = 0;
  s->levels = std::max(1, std::min(least - greatest + 1, max_inflight));
  s->streams.assign(max_inflight, std::vector<cudaStream_t>(s->levels, nullptr));
  s->slot_stream.assign(max_inflight, nullptr);
  s->ev_start.resize(max_inflight);
  s->ev_end.resize(max_inflight);
  s->slot_busy.assign(max_inflight, false);
  s->slot_ticket.assign(max_inflight, 0);
  for (int i = 0; i < max_inflight; ++i) {
    for (int l = 0; l < s->levels; ++l)
      cudaStreamCreateWithPriority(&s->streams[i][l], cudaStreamNonBlocking, greatest + l);
    s->slot_stream[i] = s->streams[i][0];
    cudaEventCreate(&s->ev_start[i]);
    cudaEventCreate(&s->ev_end[i]);
  }
  s->dispatcher = std::thread(dispatcher_main, s);
  s->completer = std::thread(completer_main, s);
  *out = s;
  return PSMMA_OK;
}

int psmma_server_submit(psmma_server* s, const psmma_request* r, unsigned long long* ticket) {
  if (!s || !r || !ticket) return PSMMA_ENULL;
  int st = check_request(*r);
  if (st) return st;
  const size_t need = request_workspace(*r);
  if (need > s->arena.total()) return PSMMA_ENOMEM;  // can never be admitted
  std::lock_guard<std::mutex> lk(s->mu);
  Job j;
  j.ticket = s->next_ticket++;
  j.req = *r;
  j.work_bytes = need;
  j.submit_s = now_s();
  s->jobs[j.ticket] = j;
  s->pending.push_back(j.ticket);
  *ticket = j.ticket;
  s->cv_dispatch.notify_one();
  return PSMMA_OK;
}

int psmma_server_wait(psmma_server* s, unsigned long long ticket, double timeout_s, psmma_completion* out) {
  if (!s) return PSMMA_ENULL;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->jobs.find(ticket);
  if (it == s->jobs.end()) return PSMMA_EUNSUPPORTED;
  bool ok = s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), [&] { return s->jobs[ticket].done; });
  if (!ok) return PSMMA_ETIMEDOUT;
  Job& j = s->jobs[ticket];
  if (out) {
    out->ticket = j.ticket;
    out->user_tag = j.req.user_tag;
    out->status = j.status;
    out->submit_s = j.submit_s;
    out->start_s = j.start_s;
    out->end_s = j.end_s;
    out->gpu_ms = j.gpu_ms;
  }
  const int st = j.status;
  s->jobs.erase(ticket);
  return st;
}

int psmma_server_pending(psmma_server* s, int* queued, int* inflight) {
  if (!s) return PSMMA_ENULL;
  std::lock_guard<std::mutex> lk(s->mu);
  if (queued) *queued = (int)s->pending.size();
  if (inflight) {
    int c = 0;
    for (bool b : s->slot_busy) c += b ? 1 : 0;
    *inflight = c;
  }
  return PSMMA_OK;
}

int psmma_server_destroy(psmma_server* s) {
  if (!s) return PSMMA_ENULL;
  {
    // finish what is in flight, drop what was never admitted
    std::unique_lock<std::mutex> lk(s->mu);
    s->pending.clear();
    s->cv_done.wait_for(lk, std::chrono::seconds(120), [&] {
      for (bool b : s->slot_busy)
        if (b) return false;
      return true;
    });
    s->stop = true;
  }
  s->cv_dispatch.notify_all();
  s->cv_complete.notify_all();
  s->dispatcher.join();
  s->completer.join();
  for (int i = 0; i < s->max_inflight; ++i) {
    for (int l = 0; l < s->levels; ++l) {
      cudaStreamSynchronize(s->streams[i][l]);
      cudaStreamDestroy(s->streams[i][l]);
    }
    cudaEventDestroy(s->ev_start[i]);
    cudaEventDestroy(s->ev_end[i]);
  }
  cudaFree(s->arena_base);
  cudaFree(s->dev_status);
  cudaFreeHost(s->host_status);
  delete s;
  return PSMMA_OK;
}

}  // extern "C"
