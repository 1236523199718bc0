// Request server: a device-resident search loop with continuous batching.
//
// Requests (one spectrum each, any length up to the configured maximum, the
// full template bank or a contiguous sub-range of it, 1..max_planes planes)
// are queued by fdas_server_submit and run by one dispatcher thread on a pool
// of "slots".  A slot is an FDAS handle sized for a power-of-two class of
// lengths; its template spectra are uploaded once and stay on the device, and
// fdas_reshape points it at each request's length, template range and plane
// count.  Every slot searches on its own CUDA stream, so requests admitted
// while others are running overlap on the device; a request is admitted as
// soon as a free slot of a large enough class exists, or a new slot's device
// bytes (dominated by the FOP, 4 x templates x bins per buffer set) fit into
// the HBM budget -- idle slots of other classes are released to make room.
// Results (the wide candidate list of the request) are kept per request until
// fdas_server_wait collects them.  Each request runs the same kernels on the
// same inputs as a plain fdas_launch on its own handle, so its result does not
// depend on what else is running.
//
// Latency: submit copies the spectrum straight into a pooled device buffer
// (the driver reads pageable host memory far faster than a host copy into
// pinned memory), the slot searches from there; a completer thread polls the
// in-flight searches' events and collects results; the dispatcher, the
// completer and fdas_server_wait spin (bounded, on the host) before they
// block, since a wake-up costs tens of microseconds.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "fdas_gb300.h"

namespace {

double now_ms() {
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  uint64_t id = 0;
  fdas_complex *spectrum = nullptr;  // device memory, from the server's pool (class_bins values)
  uint32_t class_bins = 0;
  uint32_t n_bins = 0, row_begin = 0, n_templates = 0, n_planes = 0;
  std::vector<float> thresholds;
  double t_submit = 0, t_start = 0, t_done = 0;
  std::atomic<bool> done{false};
  fdas_status status = FDAS_OK;
  std::string error;
  std::vector<fdas_candidate> candidates;
  uint32_t n_total = 0, n_dropped = 0;
};

struct Slot {
  fdas_handle *h = nullptr;
  uint32_t class_bins = 0;
  size_t bytes = 0;
  std::shared_ptr<Request> req;
  double t_idle = 0;
  cudaEvent_t done = nullptr;  // recorded after the search's last step on the slot's stream
  bool launched = false;       // a search is in flight (set and cleared under the server's lock)
};

}  // namespace

struct fdas_server {
  fdas_server_config cfg{};
  std::vector<fdas_complex> bank;
  uint32_t bank_rows = 0, bank_len = 0;
  fdas_template_layout layout = FDAS_TEMPLATES_TIME_DOMAIN;
  size_t budget = 0, used = 0;
  std::vector<std::unique_ptr<Slot>> slots;
  std::deque<std::shared_ptr<Request>> queue;
  std::map<uint64_t, std::shared_ptr<Request>> requests;
  uint64_t next_id = 1;
  std::map<uint32_t, std::vector<fdas_complex *>> pool;  // free device request buffers per length class
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_finished;
  // Bumped (under the lock) whenever the dispatcher may have work: a submit or
  // a freed slot; and whenever the completer has a new search to watch.
  std::atomic<uint64_t> work_seq{0}, launch_seq{0};
  std::atomic<bool> stop{false};
  std::thread worker, completer;
  std::string err;
  // statistics
  uint64_t n_completed = 0;
  uint32_t peak_busy = 0;
};

namespace {

constexpr int kPoolPerSlot = 2;  // request buffers a new slot adds to its class's pool

uint32_t class_of(uint32_t n, uint32_t min_class, uint32_t max_bins) {
  uint32_t c = min_class;
  while (c < n) c <<= 1;
  return std::min(c, max_bins);
}

// frees a slot's device memory; `s` given: also its byte count
void release_slot(fdas_server *s, Slot *sl) {
  if (sl->done) cudaEventDestroy(sl->done);
  fdas_destroy(sl->h);
  if (s) s->used -= sl->bytes;
}

// New slot for length class `cls`; the caller holds no lock (device calls).
std::unique_ptr<Slot> make_slot(fdas_server *s, uint32_t cls, std::string &err) {
  fdas_config c;
  fdas_default_config(&c, cls);
  c.device = s->cfg.device;
  c.n_templates = s->bank_rows;
  c.max_template_len = s->layout == FDAS_TEMPLATES_TIME_DOMAIN ? s->bank_len : c.max_template_len;
  c.n_planes = s->cfg.max_planes;
  c.candidate_capacity = s->cfg.candidate_capacity;
  auto sl = std::make_unique<Slot>();
  size_t free0 = 0, total = 0;
  cudaSetDevice(s->cfg.device);
  cudaMemGetInfo(&free0, &total);
  if (fdas_initialise_accelerator(&c, &sl->h) != FDAS_OK) {
    err = fdas_last_error(nullptr);
    return nullptr;
  }
  if (fdas_upload_templates(sl->h, s->bank.data(), s->layout, FDAS_SET_A) != FDAS_OK) {
    err = fdas_last_error(sl->h);
    fdas_destroy(sl->h);
    return nullptr;
  }
  if (cudaEventCreateWithFlags(&sl->done, cudaEventDisableTiming) != cudaSuccess) {
    err = "event creation failed";
    fdas_destroy(sl->h);
    return nullptr;
  }
  // request buffers of this class for the pool, allocated here on the
  // dispatcher thread: a device allocation inside submit can stall the caller
  // (tens of milliseconds were seen right after large frees)
  fdas_complex *bufs[kPoolPerSlot] = {};
  for (auto &b : bufs)
    if (cudaMalloc((void **)&b, sizeof(fdas_complex) * cls) != cudaSuccess) {
      cudaGetLastError();
      b = nullptr;
    }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto &pool = s->pool[cls];
    for (auto *b : bufs) {
      if (!b) continue;
      if (pool.size() < 2 * (size_t)s->cfg.max_slots) pool.push_back(b);  // slots come and go: keep it bounded
      else cudaFree(b);
    }
  }
  size_t free1 = 0;
  cudaMemGetInfo(&free1, &total);
  sl->bytes = free0 > free1 ? free0 - free1 : 0;
  sl->class_bins = cls;
  return sl;
}

// device bytes of a slot of class `cls`, estimated before it exists: both
// buffer sets' FOP, tiles, input and candidate records
size_t slot_bytes_estimate(const fdas_server *s, uint32_t cls) {
  const size_t stride = (cls + 255) / 256 * 256;
  const size_t tiles = (cls + 1627) / 1628 + 1;
  const size_t per_set = 4 * (size_t)s->bank_rows * stride + 8 * 2048 * tiles + 8 * (size_t)cls +
                         12 * (size_t)(s->cfg.candidate_capacity ? s->cfg.candidate_capacity : (1u << 22)) +
                         (8u << 20);
  return 2 * per_set;
}

// Collects the finished search of `sl` into `r` (no lock held; only the
// dispatcher thread touches a busy slot).
void finish(Slot *sl, Request *r) {
  fdas_status st = fdas_wait(sl->h, FDAS_SET_A);
  if (st == FDAS_OK) {
    uint32_t total = 0, dropped = 0;
    st = fdas_retrieve_candidate_list(sl->h, nullptr, 0, &total, &dropped, FDAS_SET_A);
    if (st == FDAS_OK) {
      r->candidates.resize(total);
      st = fdas_retrieve_candidate_list(sl->h, r->candidates.data(), total, &total, &dropped, FDAS_SET_A);
      r->n_total = total;
      r->n_dropped = dropped;
    }
  }
  if (st != FDAS_OK) r->error = fdas_last_error(sl->h);
  r->status = st;
  r->t_done = now_ms();
}

fdas_status start(fdas_server *s, Slot *sl, Request *r) {
  fdas_status st = fdas_reshape(sl->h, r->n_bins, r->row_begin, r->n_templates, 0, r->n_planes);
  if (st != FDAS_OK) return st;
  r->t_start = now_ms();
  // the spectrum is already in device memory (copied there by submit)
  st = fdas_enqueue_search_device(sl->h, r->spectrum, r->thresholds.data(), FDAS_ALL_ACCELERATIONS, FDAS_SET_A);
  if (st != FDAS_OK) return st;
  cudaStream_t stream = static_cast<cudaStream_t>(fdas_get_stream(sl->h, FDAS_SET_A));
  if (cudaEventRecord(sl->done, stream) != cudaSuccess) return FDAS_ERR_CUDA;
  return FDAS_OK;
}

void complete(fdas_server *s, const std::shared_ptr<Request> &r) {
  s->pool[r->class_bins].push_back(r->spectrum);
  r->spectrum = nullptr;
  r->done.store(true);
  ++s->n_completed;
  s->cv_done.notify_all();
}

// Spin (bounded, on the host) for up to `us` microseconds until `ready()`;
// a wake-up from a blocking wait costs tens of microseconds, a search of a
// short spectrum about a hundred.
template <typename F>
bool spin_until(F ready, double us) {
  const double t_end = now_ms() + us * 1e-3;
  while (!ready()) {
    if (now_ms() > t_end) return false;
    std::this_thread::yield();
  }
  return true;
}

// Completer thread: watches the searches in flight by polling their `done`
// events (a stream callback would add a driver-thread hop and a wake-up),
// collects each finished search's results and frees its slot.
void completer(fdas_server *s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->mu);
  std::vector<Slot *> flying;
  while (true) {
    flying.clear();
    for (auto &sl : s->slots)
      if (sl->req && sl->launched) flying.push_back(sl.get());
    if (flying.empty()) {
      if (s->stop) break;
      const uint64_t seq = s->launch_seq.load();
      lk.unlock();
      const bool more = spin_until([&] { return s->launch_seq.load() != seq; }, 200.0);
      lk.lock();
      if (!more) s->cv_finished.wait(lk, [&] { return s->stop || s->launch_seq.load() != seq; });
      continue;
    }
    const uint64_t seq = s->launch_seq.load();
    lk.unlock();
    Slot *ready = nullptr;
    // poll the flying searches until one is done or another is launched
    while (!ready) {
      for (Slot *sl : flying)
        if (cudaEventQuery(sl->done) != cudaErrorNotReady) {
          ready = sl;
          break;
        }
      if (ready || s->launch_seq.load() != seq) break;
      std::this_thread::yield();
    }
    if (!ready) {
      lk.lock();
      continue;
    }
    auto r = ready->req;
    finish(ready, r.get());
    lk.lock();
    ready->launched = false;
    ready->req.reset();
    ready->t_idle = r->t_done;
    complete(s, r);
    ++s->work_seq;
    s->cv_work.notify_one();
  }
}

// The first queued request that can be admitted (arrival order; a request
// waiting for memory does not hold back smaller ones behind it) is started.
// Called with the lock held; device work runs with it released.
bool admit_one(fdas_server *s, std::unique_lock<std::mutex> &lk) {
  std::vector<std::unique_ptr<Slot>> victims;
  for (auto it = s->queue.begin(); it != s->queue.end(); ++it) {
    auto r = *it;
    const uint32_t cls = r->class_bins;
    Slot *pick = nullptr;
    for (auto &sl : s->slots)
      if (!sl->req && sl->class_bins >= r->n_bins && sl->class_bins <= 2 * cls &&
          (!pick || sl->class_bins < pick->class_bins))
        pick = sl.get();
    bool create = false;
    if (!pick && s->slots.size() < s->cfg.max_slots) {
      const size_t need = slot_bytes_estimate(s, cls);
      // release idle slots (least recently used first) until the new one fits
      while (s->used + need > s->budget) {
        auto victim = s->slots.end();
        for (auto v = s->slots.begin(); v != s->slots.end(); ++v)
          if (!(*v)->req && (victim == s->slots.end() || (*v)->t_idle < (*victim)->t_idle)) victim = v;
        if (victim == s->slots.end()) break;
        s->used -= (*victim)->bytes;
        victims.push_back(std::move(*victim));
        s->slots.erase(victim);
      }
      create = s->used + need <= s->budget;
    }
    if (!pick && !create) continue;
    s->queue.erase(it);
    std::unique_ptr<Slot> fresh;
    if (pick) pick->req = r;  // reserved: the completer only sees it after the launch
    // device calls (which may wait for streams whose callbacks take the lock)
    // only with the lock released
    lk.unlock();
    for (auto &v : victims) release_slot(nullptr, v.get());
    victims.clear();
    std::string err;
    if (!pick) {
      fresh = make_slot(s, cls, err);
      pick = fresh.get();
      if (pick) pick->req = r;
    }
    fdas_status st = pick ? start(s, pick, r.get()) : FDAS_ERR_OUT_OF_MEMORY;
    if (st != FDAS_OK && pick) err = fdas_last_error(pick->h);
    lk.lock();
    if (fresh) {
      s->used += fresh->bytes;
      s->slots.push_back(std::move(fresh));
    }
    if (st == FDAS_OK) {
      pick->launched = true;  // the completer watches it from now on
      ++s->launch_seq;
      s->cv_finished.notify_one();
    }
    if (st != FDAS_OK) {
      if (pick) pick->req.reset();
      r->status = st;
      r->error = err;
      r->t_done = now_ms();
      complete(s, r);
    }
    uint32_t busy = 0;
    for (auto &sl : s->slots) busy += sl->req ? 1 : 0;
    s->peak_busy = std::max(s->peak_busy, busy);
    return true;
  }
  if (!victims.empty()) {  // released, but still nothing admissible
    lk.unlock();
    for (auto &v : victims) release_slot(nullptr, v.get());
    lk.lock();
  }
  return false;
}

void dispatcher(fdas_server *s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (!s->stop) {
    const uint64_t seq = s->work_seq.load();
    if (admit_one(s, lk)) continue;
    lk.unlock();
    const bool more = spin_until([&] { return s->work_seq.load() != seq || s->stop; }, 200.0);
    lk.lock();
    if (!more) s->cv_work.wait(lk, [&] { return s->work_seq.load() != seq || s->stop; });
  }
}

}  // namespace

extern "C" {

void fdas_server_default_config(fdas_server_config *c) {
  std::memset(c, 0, sizeof(*c));
  c->device = 0;
  c->max_bins = 1u << 21;
  c->min_class_bins = 1u << 15;
  c->max_planes = 16;
  c->max_slots = 8;
  c->hbm_budget_bytes = 0;
  c->candidate_capacity = 1u << 20;
}

fdas_status fdas_server_create(const fdas_server_config *cfg, const fdas_complex *bank, fdas_template_layout layout,
                               uint32_t bank_rows, uint32_t bank_len, fdas_server **out) {
  if (!cfg || !bank || !out || bank_rows == 0 || bank_rows % 2 == 0) return FDAS_ERR_INVALID_ARG;
  if (cfg->max_bins == 0 || cfg->max_slots == 0 || cfg->max_planes == 0 || cfg->max_planes > 16 ||
      cfg->min_class_bins == 0)
    return FDAS_ERR_INVALID_ARG;
  const uint32_t row_len = layout == FDAS_TEMPLATES_TIME_DOMAIN ? bank_len : 2048;
  if (row_len == 0) return FDAS_ERR_INVALID_ARG;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return FDAS_ERR_NO_DEVICE;
  }
  if (cfg->device < 0 || cfg->device >= ndev) return FDAS_ERR_INVALID_ARG;
  auto s = new fdas_server();
  s->cfg = *cfg;
  s->bank.assign(bank, bank + (size_t)bank_rows * row_len);
  s->bank_rows = bank_rows;
  s->bank_len = bank_len;
  s->layout = layout;
  size_t free_b = 0, total = 0;
  cudaSetDevice(cfg->device);
  if (cudaMemGetInfo(&free_b, &total) != cudaSuccess) {
    delete s;
    return FDAS_ERR_CUDA;
  }
  s->budget = cfg->hbm_budget_bytes ? (size_t)cfg->hbm_budget_bytes : free_b / 10 * 9;
  s->worker = std::thread(dispatcher, s);
  s->completer = std::thread(completer, s);
  *out = s;
  return FDAS_OK;
}

fdas_status fdas_server_submit(fdas_server *s, const fdas_complex *spectrum, uint32_t n_bins,
                               uint32_t template_row_begin, uint32_t n_templates, uint32_t n_planes,
                               const float *thresholds, uint64_t *request_id) {
  if (!s || !spectrum || !thresholds || !request_id) return FDAS_ERR_INVALID_ARG;
  if (n_bins == 0 || n_bins > s->cfg.max_bins) return FDAS_ERR_CAPACITY;
  if (n_templates == 0 || n_templates % 2 == 0 || template_row_begin + n_templates > s->bank_rows)
    return FDAS_ERR_INVALID_ARG;
  if (n_planes == 0 || n_planes > s->cfg.max_planes) return FDAS_ERR_INVALID_ARG;
  auto r = std::make_shared<Request>();
  r->t_submit = now_ms();  // the request's latency includes its copy into the server's buffer
  r->class_bins = class_of(n_bins, s->cfg.min_class_bins, s->cfg.max_bins);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto &freelist = s->pool[r->class_bins];
    if (!freelist.empty()) {
      r->spectrum = freelist.back();
      freelist.pop_back();
    }
  }
  int caller_dev = 0;  // the caller's current device is left as it was
  cudaGetDevice(&caller_dev);
  cudaSetDevice(s->cfg.device);
  fdas_status st = FDAS_OK;
  if (!r->spectrum && cudaMalloc((void **)&r->spectrum, sizeof(fdas_complex) * r->class_bins) != cudaSuccess) {
    cudaGetLastError();
    r->spectrum = nullptr;
    st = FDAS_ERR_OUT_OF_MEMORY;
  }
  // straight from the caller's memory into device memory, on this thread's
  // own stream, finished before submit returns (the caller may reuse its
  // buffer at once); the driver reads pageable memory at ~160 GB/s here, a
  // host copy into pinned memory would run at 15-30 GB/s
  if (st == FDAS_OK &&
      (cudaMemcpyAsync(r->spectrum, spectrum, sizeof(fdas_complex) * n_bins, cudaMemcpyDefault,
                       cudaStreamPerThread) != cudaSuccess ||
       cudaStreamSynchronize(cudaStreamPerThread) != cudaSuccess)) {
    cudaGetLastError();
    std::lock_guard<std::mutex> lk(s->mu);
    s->pool[r->class_bins].push_back(r->spectrum);
    st = FDAS_ERR_CUDA;
  }
  cudaSetDevice(caller_dev);
  if (st != FDAS_OK) return st;
  r->n_bins = n_bins;
  r->row_begin = template_row_begin;
  r->n_templates = n_templates;
  r->n_planes = n_planes;
  r->thresholds.assign(thresholds, thresholds + n_planes);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    s->requests[r->id] = r;
    s->queue.push_back(r);
    ++s->work_seq;
  }
  s->cv_work.notify_one();
  *request_id = r->id;
  return FDAS_OK;
}

fdas_status fdas_server_wait(fdas_server *s, uint64_t request_id, int32_t timeout_ms, fdas_candidate *out,
                             uint32_t capacity, uint32_t *n_total, uint32_t *n_dropped, double *latency_ms) {
  if (!s) return FDAS_ERR_INVALID_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->requests.find(request_id);
  if (it == s->requests.end()) return FDAS_ERR_INVALID_ARG;
  auto r = it->second;
  auto ready = [&] { return r->done.load(); };
  const double spin_us = timeout_ms < 0 ? 200.0 : std::min(200.0, 1e3 * timeout_ms);
  if (!ready() && spin_us > 0) {  // a short spin first: most searches end within it
    lk.unlock();
    spin_until(ready, spin_us);
    lk.lock();
  }
  if (timeout_ms < 0) s->cv_done.wait(lk, ready);
  else if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready)) return FDAS_ERR_TIMEOUT;
  if (!out && capacity == 0) {  // counts only: the request stays to be collected
    if (n_total) *n_total = r->n_total;
    if (n_dropped) *n_dropped = r->n_dropped;
    if (latency_ms) *latency_ms = r->t_done - r->t_submit;
    return r->status;
  }
  s->requests.erase(it);
  lk.unlock();
  if (out) std::memcpy(out, r->candidates.data(), sizeof(fdas_candidate) * std::min<size_t>(capacity, r->candidates.size()));
  if (n_total) *n_total = r->n_total;
  if (n_dropped) *n_dropped = r->n_dropped;
  if (latency_ms) *latency_ms = r->t_done - r->t_submit;
  if (r->status != FDAS_OK) {
    std::lock_guard<std::mutex> g(s->mu);
    s->err = r->error;
  }
  return r->status;
}

fdas_status fdas_server_stats(fdas_server *s, uint64_t *out, uint32_t n) {
  if (!s || !out) return FDAS_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  uint64_t busy = 0;
  for (auto &sl : s->slots) busy += sl->req ? 1 : 0;
  const uint64_t v[6] = {s->n_completed, (uint64_t)s->queue.size(), busy, (uint64_t)s->slots.size(), s->used,
                         s->peak_busy};
  for (uint32_t i = 0; i < n && i < 6; ++i) out[i] = v[i];
  return FDAS_OK;
}

const char *fdas_server_last_error(fdas_server *s) { return s ? s->err.c_str() : ""; }

void fdas_server_destroy(fdas_server *s) {
  if (!s) return;
  cudaSetDevice(s->cfg.device);
  // let searches in flight drain (their callbacks need the completer)
  for (;;) {
    std::unique_lock<std::mutex> lk(s->mu);
    bool busy = false;
    for (auto &sl : s->slots) busy |= (bool)sl->req;
    if (!busy) break;
    lk.unlock();
    std::this_thread::sleep_for(std::chrono::microseconds(200));
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    ++s->work_seq;
    ++s->launch_seq;
  }
  s->cv_work.notify_all();
  s->cv_finished.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->completer.joinable()) s->completer.join();
  for (auto &sl : s->slots) release_slot(s, sl.get());
  for (auto &r : s->queue) cudaFree(r->spectrum);
  for (auto &kv : s->pool)
    for (auto *p : kv.second) cudaFree(p);
  delete s;
}

}  // extern "C"
