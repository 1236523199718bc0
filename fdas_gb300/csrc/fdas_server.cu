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
#include <cuda_runtime.h>

#include <algorithm>
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
  fdas_complex *spectrum = nullptr;  // pinned, from the server's pool (class_bins values)
  uint32_t class_bins = 0;
  uint32_t n_bins = 0, row_begin = 0, n_templates = 0, n_planes = 0;
  std::vector<float> thresholds;
  double t_submit = 0, t_start = 0, t_done = 0;
  bool done = false;
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
  uint32_t *loc = nullptr;          // pinned fixed-size list of the launch
  float *pwr = nullptr;
  double t_idle = 0;
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
  std::map<uint32_t, std::vector<fdas_complex *>> pinned;  // free request buffers per length class
  std::deque<Slot *> finished;                            // searches whose stream has drained
  std::mutex mu;
  std::condition_variable cv_work, cv_done, cv_finished;
  bool stop = false;
  std::thread worker, completer;
  std::string err;
  // statistics
  uint64_t n_completed = 0;
  uint32_t peak_busy = 0;
};

namespace {

uint32_t class_of(uint32_t n, uint32_t min_class, uint32_t max_bins) {
  uint32_t c = min_class;
  while (c < n) c <<= 1;
  return std::min(c, max_bins);
}

// frees a slot's device and pinned memory; `s` given: also its byte count
void release_slot(fdas_server *s, Slot *sl) {
  fdas_destroy(sl->h);
  cudaFreeHost(sl->loc);
  cudaFreeHost(sl->pwr);
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
  const size_t list = (size_t)s->cfg.max_planes * 2048;
  if (cudaHostAlloc((void **)&sl->loc, sizeof(uint32_t) * list, cudaHostAllocDefault) != cudaSuccess ||
      cudaHostAlloc((void **)&sl->pwr, sizeof(float) * list, cudaHostAllocDefault) != cudaSuccess) {
    err = "pinned host allocation failed";
    fdas_destroy(sl->h);
    return nullptr;
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

struct Done {
  fdas_server *s;
  Slot *sl;
};

// stream callback after a slot's search: hand the slot to the completer
// (no CUDA call allowed here)
void CUDART_CB on_drained(void *arg) {
  Done *d = static_cast<Done *>(arg);
  {
    std::lock_guard<std::mutex> lk(d->s->mu);
    d->s->finished.push_back(d->sl);
  }
  d->s->cv_finished.notify_one();
  delete d;
}

fdas_status start(fdas_server *s, Slot *sl, Request *r) {
  fdas_status st = fdas_reshape(sl->h, r->n_bins, r->row_begin, r->n_templates, 0, r->n_planes);
  if (st != FDAS_OK) return st;
  r->t_start = now_ms();
  st = fdas_launch(sl->h, r->spectrum, r->thresholds.data(), sl->loc, sl->pwr, FDAS_ALL_ACCELERATIONS, FDAS_SET_A);
  if (st != FDAS_OK) return st;
  cudaStream_t stream = static_cast<cudaStream_t>(fdas_get_stream(sl->h, FDAS_SET_A));
  if (cudaLaunchHostFunc(stream, on_drained, new Done{s, sl}) != cudaSuccess) return FDAS_ERR_CUDA;
  return FDAS_OK;
}

void complete(fdas_server *s, const std::shared_ptr<Request> &r) {
  s->pinned[r->class_bins].push_back(r->spectrum);
  r->spectrum = nullptr;
  r->done = true;
  ++s->n_completed;
  s->cv_done.notify_all();
}

// Completer thread: collects drained slots' results, frees the slots.
void completer(fdas_server *s) {
  cudaSetDevice(s->cfg.device);
  std::unique_lock<std::mutex> lk(s->mu);
  while (true) {
    s->cv_finished.wait(lk, [&] { return s->stop || !s->finished.empty(); });
    if (s->finished.empty()) break;  // stop requested and nothing left
    Slot *sl = s->finished.front();
    s->finished.pop_front();
    auto r = sl->req;
    lk.unlock();
    finish(sl, r.get());
    lk.lock();
    sl->req.reset();
    sl->t_idle = r->t_done;
    complete(s, r);
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
    if (admit_one(s, lk)) continue;
    s->cv_work.wait(lk);  // woken by a submit or a freed slot
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
  r->class_bins = class_of(n_bins, s->cfg.min_class_bins, s->cfg.max_bins);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto &freelist = s->pinned[r->class_bins];
    if (!freelist.empty()) {
      r->spectrum = freelist.back();
      freelist.pop_back();
    }
  }
  if (!r->spectrum &&
      cudaHostAlloc((void **)&r->spectrum, sizeof(fdas_complex) * r->class_bins, cudaHostAllocDefault) != cudaSuccess) {
    cudaGetLastError();
    return FDAS_ERR_OUT_OF_MEMORY;
  }
  std::memcpy(r->spectrum, spectrum, sizeof(fdas_complex) * n_bins);
  r->n_bins = n_bins;
  r->row_begin = template_row_begin;
  r->n_templates = n_templates;
  r->n_planes = n_planes;
  r->thresholds.assign(thresholds, thresholds + n_planes);
  r->t_submit = now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    s->requests[r->id] = r;
    s->queue.push_back(r);
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
  auto ready = [&] { return r->done; };
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
  }
  s->cv_work.notify_all();
  s->cv_finished.notify_all();
  if (s->worker.joinable()) s->worker.join();
  if (s->completer.joinable()) s->completer.join();
  for (auto &sl : s->slots) release_slot(s, sl.get());
  for (auto &r : s->queue) cudaFreeHost(r->spectrum);
  for (auto &kv : s->pinned)
    for (auto *p : kv.second) cudaFreeHost(p);
  delete s;
}

}  // extern "C"
