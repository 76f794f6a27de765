// gme_serve.cpp -- the served path: requests one at a time, results as they finish.
//
// Host side only.  Callers queue requests (gme_submit) and collect results
// (gme_poll / gme_poll_many) from any thread; one dispatcher thread per server
// owns the GPU work.  It keeps `waves` launch slots, each a context of its own
// (stream, workspace, batch arena) plus pinned staging for symbols and mapped
// pinned memory for results and completion flags.  Whenever a slot is free and
// requests are queued, it admits queued requests in arrival order (up to the
// slot's share of the HBM budget and a cell cap), copies their symbols in one
// transfer, and launches the batched sequence on the slot's stream.  The batch
// kernel writes each result, then a completion flag, into host memory; the
// dispatcher polls the flags of every busy slot, so a request is complete as soon
// as its own pair is, and a slot is free again once its stream's event has fired.
// Slots on separate streams overlap: a new launch's CTAs take SMs over as the
// previous launch drains, so the GPU does not idle on a launch's tail.
//
// The reference has no served form: its host functions align one pair per call
// (EditDistance/GPU_Hyperlane_Share.cu:689-789, LCS/GPU_Hyperlane_Share.cu:696-793,
// SmithWaterman/GPU_Hyperlane_Share.cu:683-782).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <cuda_runtime.h>

#include "gme.h"
#include "gme_internal.h"

namespace {

int64_t now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

constexpr int32_t PENDING = -1;  // result status until the device writes the result

struct Request {
  uint64_t ticket = 0;
  int kind = 0, n1 = 0, n2 = 0;
  int64_t t_submit = 0;
  int64_t bytes = 0;          // device bytes the request adds to a launch
  std::vector<int32_t> sym;   // a then b
};

struct Finished {
  gme_result r;
  int64_t latency;
};

struct Slot {
  gme_context *ctx = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t ev = nullptr;
  int32_t *h_sym = nullptr;  // pinned staging of the launch's symbols
  int32_t *d_sym = nullptr;
  int64_t sym_cap = 0;
  gme_result *h_res = nullptr;  // mapped pinned: results and flags the kernel writes
  int *h_done = nullptr;
  gme_result *d_res = nullptr;  // their device addresses
  int *d_done = nullptr;
  int64_t res_cap = 0, done_cap = 0;
  std::vector<gme_pair> pairs;
  std::vector<Request> reqs;
  std::vector<int> open;  // requests of the launch not yet reported
  bool busy = false;
};

}  // namespace

struct gme_server {
  int device = 0;
  gme_scoring sc{};
  gme_server_config cfg{};
  int64_t wave_bytes = 0;  // device bytes one launch may add (a third of a slot's share)
  int NW = 0;              // batch kernel CTA shape (0: the tuned table's choice)
  long long grid4 = 0, grid8 = 0;  // the kernel's CTAs at 4 and 8 warps per CTA
  std::vector<Slot> slots;
  std::thread dispatcher;

  mutable std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;
  std::unordered_set<uint64_t> outstanding;           // queued or running
  std::unordered_map<uint64_t, Finished> finished;    // done, not yet taken
  std::deque<uint64_t> finished_order;                // completion order (may hold taken tickets)
  uint64_t next_ticket = 1;
  bool stop = false;
  gme_server_stats st{};
  std::string last_error;
};

namespace {

void set_error(gme_server *s, const std::string &m) {
  std::lock_guard<std::mutex> g(s->mu);
  s->last_error = m;
}

// Per-CTA rows of a launch whose widest pair is max_n1 wide, at the CTA shape the
// launch may take.
int64_t scratch_bytes(const gme_server *s, int max_n1) {
  if (s->NW) return gme::batch_scratch_bytes(s->NW == 8 ? s->grid8 : s->grid4, s->NW, max_n1);
  return std::max(gme::batch_scratch_bytes(s->grid4, 4, max_n1), gme::batch_scratch_bytes(s->grid8, 8, max_n1));
}

int64_t held_bytes(const gme_server *s) {
  int64_t n = 0;
  for (const Slot &sl : s->slots) n += gme::ctx_device_bytes(sl.ctx) + 4 * sl.sym_cap;
  return n;
}

// Records finished requests of a slot (indexes into sl.reqs) with their results.
void publish(gme_server *s, Slot &sl, const std::vector<int> &idx, const std::vector<gme_result> &res) {
  if (idx.empty()) return;
  const int64_t t = now_ns();
  {
    std::lock_guard<std::mutex> g(s->mu);
    for (size_t k = 0; k < idx.size(); ++k) {
      const Request &q = sl.reqs[idx[k]];
      s->outstanding.erase(q.ticket);
      s->finished[q.ticket] = Finished{res[k], t - q.t_submit};
      s->finished_order.push_back(q.ticket);
      s->st.completed += 1;
      s->st.running -= 1;
      s->st.cells_completed += (int64_t)q.n1 * q.n2;
    }
  }
  s->cv_done.notify_all();
}

// Collects what a busy slot has finished; frees the slot once its stream is done.
bool harvest(gme_server *s, Slot &sl) {
  std::vector<int> idx;
  std::vector<gme_result> res;
  for (size_t k = 0; k < sl.open.size();) {
    const int i = sl.open[k];
    if (__atomic_load_n(&sl.h_done[i], __ATOMIC_ACQUIRE)) {
      idx.push_back(i);
      res.push_back(sl.h_res[i]);
      sl.open[k] = sl.open.back();
      sl.open.pop_back();
    } else {
      ++k;
    }
  }
  const cudaError_t q = cudaEventQuery(sl.ev);
  if (q != cudaErrorNotReady) {
    // the launch is over: the pairs that went to the plain path (no flag) are
    // done too; a pair still PENDING was never computed (a wait gave up)
    int kstat = 0;
    if (q == cudaSuccess) {
      kstat = gme::ctx_batch_status(sl.ctx);
    } else {
      set_error(s, std::string("served launch failed: ") + cudaGetErrorString(q));
    }
    for (int i : sl.open) {
      gme_result r = sl.h_res[i];
      if (q != cudaSuccess) r.status = GME_ERR_CUDA;
      else if (r.status == PENDING) r.status = kstat ? kstat : GME_ERR_TIMEOUT;
      idx.push_back(i);
      res.push_back(r);
    }
    sl.open.clear();
    publish(s, sl, idx, res);
    sl.reqs.clear();
    sl.busy = false;
    return true;
  }
  publish(s, sl, idx, res);
  return !idx.empty();
}

template <class T>
int grow_pinned(T **h, int64_t *cap, int64_t need, unsigned flags) {
  if (*cap >= need && *h) return 0;
  if (*h) cudaFreeHost(*h);
  *h = nullptr;
  *cap = 0;
  const int64_t n = need + need / 4 + 256;
  if (cudaHostAlloc((void **)h, (size_t)n * sizeof(T), flags) != cudaSuccess) {
    *h = nullptr;
    return 1;
  }
  *cap = n;
  return 0;
}

// Fails a launch's requests at once with `status` (nothing of it is on the GPU).
void fail_launch(gme_server *s, Slot &sl, int status, const std::string &why) {
  set_error(s, why);
  std::vector<int> idx;
  std::vector<gme_result> res;
  for (size_t i = 0; i < sl.reqs.size(); ++i) {
    gme_result r{};
    r.status = status;
    r.kind = sl.reqs[i].kind;
    idx.push_back((int)i);
    res.push_back(r);
  }
  publish(s, sl, idx, res);
  sl.reqs.clear();
  sl.open.clear();
}

// Admits queued requests into a free slot and launches them.  Returns whether it
// launched anything.
bool launch(gme_server *s, Slot &sl) {
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop || s->queue.empty()) return false;
    int64_t cells = 0, bytes = 0;
    int max_n1 = 0;
    while (!s->queue.empty()) {
      const Request &q = s->queue.front();
      const int64_t c = (int64_t)q.n1 * q.n2;
      const int mn = std::max(max_n1, std::min(q.n1, gme::BATCH_MAX_N1));
      const int64_t b = bytes + q.bytes;
      const int64_t fixed = scratch_bytes(s, mn);
      if (!sl.reqs.empty() && (cells + c > s->cfg.wave_max_cells || b + fixed > s->wave_bytes)) break;
      cells += c;
      bytes = b;
      max_n1 = mn;
      sl.reqs.push_back(std::move(s->queue.front()));
      s->queue.pop_front();
    }
    s->st.queued = (int64_t)s->queue.size();
    s->st.running += (int64_t)sl.reqs.size();
  }
  const int64_t n = (int64_t)sl.reqs.size();
  int64_t nsym = 0;
  for (const Request &q : sl.reqs) nsym += q.n1 + q.n2;
  if (grow_pinned(&sl.h_res, &sl.res_cap, n, cudaHostAllocMapped) ||
      grow_pinned(&sl.h_done, &sl.done_cap, n, cudaHostAllocMapped)) {
    fail_launch(s, sl, GME_ERR_NOMEM, "served: pinned result buffers");
    return true;
  }
  if (cudaHostGetDevicePointer((void **)&sl.d_res, sl.h_res, 0) != cudaSuccess ||
      cudaHostGetDevicePointer((void **)&sl.d_done, sl.h_done, 0) != cudaSuccess) {
    fail_launch(s, sl, GME_ERR_CUDA, "served: cudaHostGetDevicePointer");
    return true;
  }
  if (sl.sym_cap < nsym + 1) {
    cudaFreeHost(sl.h_sym);
    cudaFree(sl.d_sym);
    sl.h_sym = nullptr;
    sl.d_sym = nullptr;
    sl.sym_cap = 0;
    const int64_t c = nsym + nsym / 4 + 1024;
    if (cudaHostAlloc((void **)&sl.h_sym, (size_t)c * 4, cudaHostAllocDefault) != cudaSuccess ||
        cudaMalloc((void **)&sl.d_sym, (size_t)c * 4) != cudaSuccess) {
      fail_launch(s, sl, GME_ERR_NOMEM, "served: symbol buffers");
      return true;
    }
    sl.sym_cap = c;
  }
  sl.pairs.resize(n);
  int64_t off = 0;
  for (int64_t i = 0; i < n; ++i) {
    const Request &q = sl.reqs[i];
    std::memcpy(sl.h_sym + off, q.sym.data(), (size_t)(q.n1 + q.n2) * 4);
    gme_pair &p = sl.pairs[i];
    p.a_off = off;
    p.b_off = off + q.n1;
    p.n1 = q.n1;
    p.n2 = q.n2;
    p.kind = q.kind;
    p.reserved = 0;
    off += q.n1 + q.n2;
    sl.h_done[i] = 0;
    sl.h_res[i] = gme_result{};
    sl.h_res[i].status = PENDING;
  }
  const int64_t k0 = gme_launch_count(sl.ctx);
  cudaError_t e = cudaSuccess;
  if (nsym > 0) e = cudaMemcpyAsync(sl.d_sym, sl.h_sym, (size_t)nsym * 4, cudaMemcpyHostToDevice, sl.st);
  if (e != cudaSuccess) {
    fail_launch(s, sl, GME_ERR_CUDA, std::string("served: symbol copy: ") + cudaGetErrorString(e));
    return true;
  }
  gme::ctx_set_served(sl.ctx, sl.d_done);
  const gme_status rc = gme_align_batch_device(sl.ctx, sl.d_sym, nsym, sl.pairs.data(), n, &s->sc,
                                               sl.d_res, sl.st);
  if (rc != GME_OK) {
    cudaStreamSynchronize(sl.st);
    fail_launch(s, sl, rc, std::string("served: launch: ") + gme_last_error(sl.ctx));
    return true;
  }
  if ((e = cudaEventRecord(sl.ev, sl.st)) != cudaSuccess) {
    cudaStreamSynchronize(sl.st);
    fail_launch(s, sl, GME_ERR_CUDA, "served: cudaEventRecord");
    return true;
  }
  sl.open.resize(n);
  for (int64_t i = 0; i < n; ++i) sl.open[i] = (int)i;
  sl.busy = true;
  const int64_t held = held_bytes(s);
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->st.waves_launched += 1;
    s->st.kernels_launched += gme_launch_count(sl.ctx) - k0;
    s->st.h2d_bytes += nsym * 4 + n * (int64_t)(sizeof(gme_pair) + 64);
    s->st.d2h_bytes += n * (int64_t)(sizeof(gme_result) + sizeof(int));
    s->st.hbm_bytes_held = held;
    s->st.hbm_bytes_peak = std::max(s->st.hbm_bytes_peak, held);
  }
  return true;
}

void dispatcher_main(gme_server *s) {
  cudaSetDevice(s->device);
  for (;;) {
    bool progressed = false, busy = false;
    for (Slot &sl : s->slots)
      if (sl.busy) progressed |= harvest(s, sl);
    for (Slot &sl : s->slots)
      if (!sl.busy && launch(s, sl)) progressed = true;
    for (Slot &sl : s->slots) busy |= sl.busy;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop && !busy) {
      // nothing on the GPU: what is still queued is closed
      const int64_t t = now_ns();
      while (!s->queue.empty()) {
        Request &q = s->queue.front();
        gme_result r{};
        r.status = GME_ERR_CLOSED;
        r.kind = q.kind;
        s->outstanding.erase(q.ticket);
        s->finished[q.ticket] = Finished{r, t - q.t_submit};
        s->finished_order.push_back(q.ticket);
        s->st.completed += 1;
        s->queue.pop_front();
      }
      s->st.queued = 0;
      lk.unlock();
      s->cv_done.notify_all();
      return;
    }
    if (!progressed) {
      if (!busy) {
        s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
      } else {
        // the GPU is working: poll again shortly (completion flags live in host memory)
        lk.unlock();
        std::this_thread::yield();
      }
    }
  }
}

}  // namespace

namespace {

// Validates one request and builds it (symbols copied); the ticket is set on queueing.
gme_status make_request(gme_server *s, int kind, const int32_t *a, int64_t n1, const int32_t *b, int64_t n2,
                        Request &q) {
  if (kind < GME_LCS || kind > GME_SW || n1 < 0 || n2 < 0 || (n1 && !a) || (n2 && !b)) return GME_ERR_INVALID;
  if (n1 > (1 << 30) - 4096 || n2 > (1 << 30) - 4096) return GME_ERR_OVERFLOW;
  if (kind == GME_SW) {
    const long long m = std::max<long long>(std::max<long long>(llabs(s->sc.match), llabs(s->sc.mismatch)),
                                            llabs(s->sc.gap));
    if (m * (n1 + n2 + 2) >= (1ll << 30)) return GME_ERR_OVERFLOW;
  }
  q.kind = kind;
  q.n1 = (int)n1;
  q.n2 = (int)n2;
  // pairs wider than the batch kernel's rows run on the plain path, whose
  // workspace holds both padded sequences and a boundary row per band
  q.bytes = gme::batch_pair_bytes(n1, n2) + (n1 > gme::BATCH_MAX_N1 ? 64 * (n1 + n2) + (1 << 20) : 0);
  // alone in a launch it brings the per-CTA rows for its width
  const int64_t fixed = scratch_bytes(s, (int)std::min<int64_t>(n1, gme::BATCH_MAX_N1));
  if (q.bytes + fixed > s->wave_bytes) return GME_ERR_BUDGET;
  q.sym.resize((size_t)(n1 + n2));
  if (n1) std::memcpy(q.sym.data(), a, (size_t)n1 * 4);
  if (n2) std::memcpy(q.sym.data() + n1, b, (size_t)n2 * 4);
  return GME_OK;
}

// Queues built requests (all or, when the queue fills, a prefix); returns how many.
int64_t enqueue(gme_server *s, std::vector<Request> &qs, uint64_t *tickets, gme_status *rc) {
  int64_t k = 0;
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) {
      *rc = GME_ERR_CLOSED;
      return 0;
    }
    const int64_t t = now_ns();
    for (; k < (int64_t)qs.size(); ++k) {
      if ((int64_t)s->queue.size() >= s->cfg.queue_max) {
        *rc = GME_ERR_NOT_READY;
        break;
      }
      Request &q = qs[k];
      q.ticket = s->next_ticket++;
      q.t_submit = t;
      tickets[k] = q.ticket;
      s->outstanding.insert(q.ticket);
      s->queue.push_back(std::move(q));
      s->st.submitted += 1;
    }
    s->st.queued = (int64_t)s->queue.size();
  }
  if (k) s->cv_work.notify_one();
  return k;
}

}  // namespace

extern "C" {

gme_status gme_server_create(int device, const gme_server_config *cfg, const gme_scoring *sc,
                             gme_server **out) {
  if (!out) return GME_ERR_INVALID;
  *out = nullptr;
  gme_server_config c = cfg ? *cfg : gme_server_config{};
  if (c.hbm_budget_bytes < 0 || c.wave_max_cells < 0 || c.waves < 0 || c.queue_max < 0 ||
      (c.warps_per_block && c.warps_per_block != 4 && c.warps_per_block != 8))
    return GME_ERR_INVALID;
  if (!c.hbm_budget_bytes) c.hbm_budget_bytes = 20ll << 30;
  if (!c.wave_max_cells) c.wave_max_cells = 1ll << 35;
  if (!c.waves) c.waves = 4;
  if (!c.queue_max) c.queue_max = 1 << 20;
  if (c.waves > 16) return GME_ERR_INVALID;
  gme_scoring s0 = gme_default_scoring();
  if (!sc) sc = &s0;
  if (sc->ed_boundary != GME_ED_REF_CPU && sc->ed_boundary != GME_ED_STANDARD) return GME_ERR_INVALID;
  gme_server *s = new (std::nothrow) gme_server();
  if (!s) return GME_ERR_NOMEM;
  s->device = device;
  s->sc = *sc;
  s->cfg = c;
  s->wave_bytes = c.hbm_budget_bytes / c.waves / 3;
  s->st.hbm_budget_bytes = c.hbm_budget_bytes;
  s->slots.resize(c.waves);
  gme_status rc = GME_OK;
  for (Slot &sl : s->slots) {
    if ((rc = gme_create(device, &sl.ctx)) != GME_OK) break;
    if (c.warps_per_block) {
      gme_batch_config bc{};
      bc.warps_per_block = c.warps_per_block;
      if ((rc = gme_set_batch_config(sl.ctx, &bc)) != GME_OK) break;
    }
    sl.st = gme::ctx_stream(sl.ctx);
    if (cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming) != cudaSuccess) {
      rc = GME_ERR_CUDA;
      break;
    }
  }
  if (rc == GME_OK) {
    s->NW = c.warps_per_block;
    s->grid4 = gme::batch_grid(gme::ctx_sms(s->slots[0].ctx), 4, 0);
    s->grid8 = gme::batch_grid(gme::ctx_sms(s->slots[0].ctx), 8, 0);
  }
  if (rc != GME_OK) {
    for (Slot &sl : s->slots) {
      if (sl.ev) cudaEventDestroy(sl.ev);
      if (sl.ctx) gme_destroy(sl.ctx);
    }
    delete s;
    return rc;
  }
  s->dispatcher = std::thread(dispatcher_main, s);
  *out = s;
  return GME_OK;
}

gme_status gme_server_destroy(gme_server *s) {
  if (!s) return GME_ERR_INVALID;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  if (s->dispatcher.joinable()) s->dispatcher.join();
  cudaSetDevice(s->device);
  for (Slot &sl : s->slots) {
    if (sl.ctx) cudaStreamSynchronize(sl.st);
    if (sl.ev) cudaEventDestroy(sl.ev);
    cudaFreeHost(sl.h_sym);
    cudaFree(sl.d_sym);
    cudaFreeHost(sl.h_res);
    cudaFreeHost(sl.h_done);
    if (sl.ctx) gme_destroy(sl.ctx);
  }
  delete s;
  return GME_OK;
}

gme_status gme_submit(gme_server *s, gme_kind kind, const int32_t *a, int64_t n1, const int32_t *b,
                      int64_t n2, uint64_t *ticket) {
  if (!s || !ticket) return GME_ERR_INVALID;
  std::vector<Request> qs(1);
  gme_status rc = make_request(s, kind, a, n1, b, n2, qs[0]);
  if (rc != GME_OK) return rc;
  enqueue(s, qs, ticket, &rc);
  return rc;
}

gme_status gme_submit_many(gme_server *s, const int32_t *symbols, const gme_pair *pairs, int64_t n,
                           uint64_t *tickets, int64_t *submitted) {
  if (!s || n < 0 || (n > 0 && (!pairs || !tickets || !symbols))) return GME_ERR_INVALID;
  if (submitted) *submitted = 0;
  std::vector<Request> qs;
  qs.reserve((size_t)n);
  gme_status rc = GME_OK;
  for (int64_t i = 0; i < n; ++i) {
    const gme_pair &p = pairs[i];
    if (p.a_off < 0 || p.b_off < 0) { rc = GME_ERR_INVALID; break; }
    qs.emplace_back();
    rc = make_request(s, p.kind, symbols + p.a_off, p.n1, symbols + p.b_off, p.n2, qs.back());
    if (rc != GME_OK) { qs.pop_back(); break; }
  }
  gme_status rq = GME_OK;
  const int64_t k = enqueue(s, qs, tickets, &rq);
  if (submitted) *submitted = k;
  return rc != GME_OK ? rc : rq;
}

gme_status gme_poll(gme_server *s, uint64_t ticket, gme_result *out, int64_t *latency_ns) {
  if (!s || !out) return GME_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  auto it = s->finished.find(ticket);
  if (it == s->finished.end()) return s->outstanding.count(ticket) ? GME_ERR_NOT_READY : GME_ERR_INVALID;
  *out = it->second.r;
  if (latency_ns) *latency_ns = it->second.latency;
  s->finished.erase(it);
  return GME_OK;
}

gme_status gme_poll_many(gme_server *s, uint64_t *tickets, gme_result *results, int64_t *latency_ns,
                         int64_t max, int64_t *count) {
  if (!s || !count || max < 0 || (max > 0 && !tickets)) return GME_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  int64_t k = 0;
  while (k < max && !s->finished_order.empty()) {
    const uint64_t t = s->finished_order.front();
    s->finished_order.pop_front();
    auto it = s->finished.find(t);
    if (it == s->finished.end()) continue;  // already taken by gme_poll
    tickets[k] = t;
    if (results) results[k] = it->second.r;
    if (latency_ns) latency_ns[k] = it->second.latency;
    s->finished.erase(it);
    ++k;
  }
  *count = k;
  return GME_OK;
}

gme_status gme_server_drain(gme_server *s, uint64_t timeout_ns) {
  if (!s) return GME_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->mu);
  const bool ok = s->cv_done.wait_for(lk, std::chrono::nanoseconds(timeout_ns),
                                      [&] { return s->st.completed >= s->st.submitted; });
  return ok ? GME_OK : GME_ERR_NOT_READY;
}

gme_status gme_server_get_stats(const gme_server *s, gme_server_stats *out) {
  if (!s || !out) return GME_ERR_INVALID;
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->st;
  return GME_OK;
}

const char *gme_server_last_error(const gme_server *s) {
  if (!s) return "no server";
  std::lock_guard<std::mutex> g(s->mu);
  return s->last_error.c_str();
}

}  // extern "C"
