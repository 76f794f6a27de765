// gme_serve.cpp -- the served path: requests one at a time, results as they finish.
//
// Host side only.  Callers queue requests (gme_submit) and collect results
// (gme_poll / gme_poll_many) from any thread; one dispatcher thread per server owns
// the GPU work, in one of two modes.
//
// Ring mode (the default).  One persistent kernel (serve_kernel, gme_batch.cu) stays
// on the GPU and takes jobs from rings of descriptors in device memory, two per kind:
// pairs of 2^22 cells and more run one per CTA, the rest one per warp.  A pair of SMs
// runs one kind at a time (the three kinds' loops do not fit its instruction cache).  The dispatcher admits
// queued requests in arrival order while the symbol arena and the rings have room,
// writes their padded symbols and descriptors into pinned staging, copies them to the
// device on a copy stream and, on the same stream after them, the rings' new tails;
// the kernel claims a job only below the tail it reads.  Each result, then its
// completion flag, goes to mapped pinned memory, and the dispatcher frees a job's ring
// slot and (in admission order) its arena space once the flag is up.  The kernel
// leaves as a whole once no CTA has found a job for a short time; the dispatcher
// launches it again whenever jobs are live and no launch is.  Pairs wider than the kernel's rows (16384) run as launches
// of the batched kernel on a launch slot, as in the other mode.
//
// Waves mode.  `waves` launch slots, each a context of its own (stream, workspace,
// batch arena) plus pinned staging for symbols and mapped pinned memory for results
// and completion flags.  Whenever a slot is free and requests are queued, the
// dispatcher admits queued requests in arrival order (up to the slot's share of the
// HBM budget and a cell cap), copies their symbols in one transfer, and launches the
// batched sequence on the slot's stream.  The batch kernel writes each result, then
// a completion flag, into host memory; the dispatcher polls the flags of every busy
// slot, so a request is complete as soon as its own pair is, and a slot is free
// again once its stream's event has fired.  Slots on separate streams overlap.
//
// The reference has no served form: its host functions align one pair per call
// (EditDistance/GPU_Hyperlane_Share.cu:689-789, LCS/GPU_Hyperlane_Share.cu:696-793,
// SmithWaterman/GPU_Hyperlane_Share.cu:683-782).
#include <algorithm>
#include <array>
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

// Ring mode: one job in flight (admitted, not yet reported).
struct RingJob {
  Request req;
  bool block = false;    // a CTA ring's job (else a warp ring's)
  int rslot = 0;         // its result slot: k * qb + ring slot in kind k's CTA ring,
                         // 3 * qb + k * qw + ring slot in its warp ring
  int64_t arena_end = 0; // the arena position (monotonic, ints) past its symbols
  int entries = 1;       // its CTA-ring slots (a team's entries: rslot and the ones after it)
  int team = -1;         // its team, or -1
  unsigned tag0 = 0;     // a team's tags: rows of its previous uses hold lower ones
  bool clear_rows = false;  // the team's tags start over: its rows are cleared first
  bool done = false;     // result reported
  bool released = false; // ring slots, team and arena space free again
};

// Ring mode: the persistent kernel's buffers and the dispatcher's view of them.
struct Ring {
  cudaStream_t kst = nullptr, cst = nullptr;  // the kernel's stream, the copy stream
  cudaEvent_t kev = nullptr;                  // the kernel's last launch has finished
  cudaEvent_t sev[2] = {nullptr, nullptr};    // copies out of staging buffer k are done
  bool launched = false;
  bool yielding = false;                      // the launch has been asked to leave
  int NW = 4, grid = 0, stride = 0;
  int qb = 0, qw = 0;
  int64_t arena_cap = 0;                      // ints
  int64_t fixed_bytes = 0;                    // everything but the arena's live part
  // device
  int *d_arena = nullptr;
  gme::BatchJob *d_jobs = nullptr;            // per result slot: the CTA rings, then the warp rings
  int *d_bad = nullptr;                       // 2 per result slot
  int *d_rows = nullptr;
  unsigned long long *d_wrap = nullptr;
  unsigned *d_gen = nullptr;
  int *d_ctrl = nullptr, *d_ring = nullptr;
  int4 *d_units = nullptr;                    // per CTA-ring slot
  unsigned char *d_team = nullptr;            // RING_TEAMS teams
  unsigned long long *d_twrap = nullptr;      // 2 rows of `stride` words per team
  // pinned host
  int4 *h_units = nullptr;
  int *h_tfree = nullptr, *d_tfree = nullptr; // mapped, one per team
  unsigned char *h_zero = nullptr;            // zeros: a team's state, or its two rows
  std::vector<int> teams_free;
  std::vector<unsigned> team_tag;             // per team: the next use's tag0
  gme::BatchJob *h_jobs = nullptr;
  int *h_bad = nullptr;
  int *h_tail = nullptr;                      // 8 per staging buffer: tails to copy; [16] stop
  int32_t *h_stage[2] = {nullptr, nullptr};
  int64_t stage_cap = 0;                      // ints per staging buffer
  int cur = 0;                                // staging buffer of the next round
  gme_result *h_res = nullptr, *d_res = nullptr;  // mapped, one per result slot
  int *h_done = nullptr, *d_done = nullptr;
  // admission state
  int tail[6] = {0, 0, 0, 0, 0, 0};           // tickets published so far, ring 2 * kind + (warp ring)
  std::vector<char> busy;                     // result slots holding a live job
  int64_t ahead = 0, atail = 0;               // arena: next free / oldest live position
  std::deque<RingJob> live;                   // admission order
  int64_t queued_cells = 0;                   // cells of the live jobs not yet done
  std::vector<RingJob *> by_slot;             // per result slot: its live job, or null
  std::vector<RingJob *> teams_done;          // teams reported, waiting for their last entry
  int *h_cq = nullptr, *d_cq = nullptr;       // completion queue (mapped): result slot + 1
  uint64_t cq_pos = 0;                        // the next entry to read
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
  Ring ring;               // ring mode (cfg.mode == GME_SERVE_RING)
  std::thread dispatcher;

  mutable std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request> queue;
  std::deque<Request> wide;  // ring mode: admitted requests too wide for the kernel's rows
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
  int64_t n = s->cfg.mode == GME_SERVE_RING ? s->ring.fixed_bytes + 4 * (s->ring.ahead - s->ring.atail) : 0;
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
    std::deque<Request> &queue = s->cfg.mode == GME_SERVE_RING ? s->wide : s->queue;
    if (s->stop || queue.empty()) return false;
    int64_t cells = 0, bytes = 0;
    int max_n1 = 0;
    while (!queue.empty()) {
      const Request &q = queue.front();
      const int64_t c = (int64_t)q.n1 * q.n2;
      const int mn = std::max(max_n1, std::min(q.n1, gme::BATCH_MAX_N1));
      const int64_t b = bytes + q.bytes;
      const int64_t fixed = scratch_bytes(s, mn);
      if (!sl.reqs.empty() && (cells + c > s->cfg.wave_max_cells || b + fixed > s->wave_bytes)) break;
      cells += c;
      bytes = b;
      max_n1 = mn;
      sl.reqs.push_back(std::move(queue.front()));
      queue.pop_front();
    }
    s->st.queued = (int64_t)(s->queue.size() + s->wide.size());
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


// ---------------------------------------------------------------------------
// Ring mode.
// ---------------------------------------------------------------------------
constexpr int RING_QB = 4096, RING_QW = 32768;  // slots of each kind's CTA ring and warp ring
constexpr unsigned long long RING_IDLE_NS = 20ull * 1000 * 1000;  // the kernel leaves after 20 ms idle
constexpr int64_t RING_STAGE_INTS = 16ll << 20;  // per staging buffer (64 MiB)
#ifndef GME_RING_BLOCK_CELLS
#define GME_RING_BLOCK_CELLS (1ll << 22)
#endif
#ifndef GME_RING_TEAM_CELLS
#define GME_RING_TEAM_CELLS (1ll << 26)
#endif
#ifndef GME_RING_TEAM_QUEUE
#define GME_RING_TEAM_QUEUE 4
#endif
constexpr int64_t RING_BLOCK_CELLS = GME_RING_BLOCK_CELLS;  // pairs this large run one per CTA
// pairs this large (and at least 2048 columns wide, 4 band groups high) are shared by a
// team of CTAs, one ring entry per group up to RING_TEAM_MAX, while the work queued
// ahead of them is short: below 1/RING_TEAM_QUEUE of the pair's own cells per CTA.  (A
// team shortens the pair's run by its size; with a longer queue the pair waits for it
// anyway, and CTAs that each run a pair of their own waste no time on hand-overs.)
constexpr int64_t RING_TEAM_CELLS = GME_RING_TEAM_CELLS;
constexpr int RING_TEAM_QUEUE = GME_RING_TEAM_QUEUE;
constexpr int RING_TEAMS = 64, RING_TEAM_MAX = 16;
constexpr int RING_CQ = 1 << 18;  // completion-queue entries (a power of 2 above the result slots)

// The entries a CTA-ring pair gets: 1, or its team's size.
int ring_entries(const gme_server *s, int n1, int n2) {
  const Ring &r = s->ring;
  const int groups = (n2 + 32 * 4 * r.NW - 1) / (32 * 4 * r.NW);
  const int64_t cells = (int64_t)n1 * n2;
  if (cells < RING_TEAM_CELLS || n1 < 2048 || groups < 4) return 1;
  if (r.queued_cells / r.grid * RING_TEAM_QUEUE > cells) return 1;
  return std::min(RING_TEAM_MAX, groups);
}

bool ring_block(const gme_server *s, int n1, int n2) {
  return (int64_t)n1 * n2 >= RING_BLOCK_CELLS && n2 > 32 * 4 * (s->ring.NW - 1);
}

// Ints a pair takes in the arena: a's padded segment, then b rounded up to whole bands.
int64_t ring_need(const gme_server *s, int n1, int n2) {
  const int mult = gme::serve_rows_mult(s->ring.NW, ring_block(s, n1, n2));
  return gme::serve_a_len(n1) + ((int64_t)n2 + mult - 1) / mult * mult;
}

template <class T>
int dev_alloc(T **p, int64_t n, int64_t *bytes) {
  *bytes += n * (int64_t)sizeof(T);
  return cudaMalloc((void **)p, (size_t)n * sizeof(T)) != cudaSuccess;
}

// The kernel's fixed buffers, the arena and the rings; false (and last_error) on failure.
bool ring_setup(gme_server *s, int sms) {
  Ring &r = s->ring;
  r.NW = s->cfg.warps_per_block ? s->cfg.warps_per_block : 4;
  r.grid = gme::serve_grid(sms, r.NW);
  r.stride = gme::serve_row_stride(gme::BATCH_MAX_N1);
  r.qb = RING_QB;
  r.qw = RING_QW;
  const int nres = 3 * (r.qb + r.qw);
  int64_t b = 0;
  if (cudaStreamCreateWithFlags(&r.kst, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&r.cst, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&r.kev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&r.sev[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&r.sev[1], cudaEventDisableTiming) != cudaSuccess) {
    s->last_error = "served: streams and events";
    return false;
  }
  if (dev_alloc(&r.d_rows, (int64_t)r.grid * r.NW * r.stride, &b) ||
      dev_alloc(&r.d_wrap, (int64_t)r.grid * 2 * r.stride, &b) || dev_alloc(&r.d_gen, 1, &b) ||
      dev_alloc(&r.d_ctrl, 16, &b) || dev_alloc(&r.d_ring, gme::RW_WORDS, &b) || dev_alloc(&r.d_jobs, nres, &b) ||
      dev_alloc(&r.d_bad, 2 * nres, &b) || dev_alloc(&r.d_units, 3 * r.qb, &b) ||
      dev_alloc(&r.d_team, RING_TEAMS * gme::serve_team_bytes(), &b) ||
      dev_alloc(&r.d_twrap, (int64_t)RING_TEAMS * 2 * r.stride, &b)) {
    s->last_error = "served: kernel buffers";
    return false;
  }
  // wrap rows start with tag 0, which no job is handed; the tag counter and the
  // control words start at 0; pairs of SMs start on the three kinds in turn
  int pairs[gme::RW_PAIRS];
  for (int p = 0; p < gme::RW_PAIRS; ++p) pairs[p] = p % 3;
  if (cudaMemset(r.d_wrap, 0, (size_t)r.grid * 2 * r.stride * 8) != cudaSuccess ||
      cudaMemset(r.d_gen, 0, 4) != cudaSuccess || cudaMemset(r.d_ctrl, 0, 64) != cudaSuccess ||
      cudaMemset(r.d_ring, 0, gme::RW_WORDS * 4) != cudaSuccess ||
      cudaMemset(r.d_twrap, 0, (size_t)RING_TEAMS * 2 * r.stride * 8) != cudaSuccess ||
      cudaMemcpy(r.d_ring + gme::RW_PAIR, pairs, sizeof(pairs), cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaDeviceSynchronize() != cudaSuccess) {
    s->last_error = "served: clearing kernel buffers";
    return false;
  }
  r.fixed_bytes = b;
  const int64_t rest = s->cfg.hbm_budget_bytes - b;
  if (rest < (64ll << 20)) {
    s->last_error = "served: the budget does not hold the kernel's rows";
    return false;
  }
  // half of the rest for the arena (at most 4 GiB), half for launches of wide pairs
  r.arena_cap = std::min<int64_t>(rest / 2, 4ll << 30) / 4;
  s->wave_bytes = rest / 2 / 3;
  // (slack past the end: a segment placed last ends at arena_cap)
  if (cudaMalloc((void **)&r.d_arena, (size_t)(r.arena_cap + 1024) * 4) != cudaSuccess) {
    s->last_error = "served: symbol arena";
    return false;
  }
  r.stage_cap = std::min<int64_t>(RING_STAGE_INTS, r.arena_cap);
  if (cudaHostAlloc((void **)&r.h_jobs, (size_t)nres * sizeof(gme::BatchJob), cudaHostAllocDefault) ||
      cudaHostAlloc((void **)&r.h_bad, (size_t)2 * nres * 4, cudaHostAllocDefault) ||
      cudaHostAlloc((void **)&r.h_tail, 32 * 4, cudaHostAllocDefault) ||
      cudaHostAlloc((void **)&r.h_stage[0], (size_t)r.stage_cap * 4, cudaHostAllocDefault) ||
      cudaHostAlloc((void **)&r.h_stage[1], (size_t)r.stage_cap * 4, cudaHostAllocDefault) ||
      cudaHostAlloc((void **)&r.h_res, (size_t)nres * sizeof(gme_result), cudaHostAllocMapped) ||
      cudaHostAlloc((void **)&r.h_done, (size_t)nres * 4, cudaHostAllocMapped) ||
      cudaHostAlloc((void **)&r.h_units, (size_t)3 * r.qb * sizeof(int4), cudaHostAllocDefault) ||
      cudaHostAlloc((void **)&r.h_tfree, RING_TEAMS * 4, cudaHostAllocMapped) ||
      cudaHostAlloc((void **)&r.h_cq, (size_t)RING_CQ * 4, cudaHostAllocMapped) ||
      cudaHostGetDevicePointer((void **)&r.d_cq, r.h_cq, 0) ||
      cudaHostAlloc((void **)&r.h_zero, (size_t)2 * r.stride * 8, cudaHostAllocDefault) ||
      cudaHostGetDevicePointer((void **)&r.d_res, r.h_res, 0) ||
      cudaHostGetDevicePointer((void **)&r.d_done, r.h_done, 0) ||
      cudaHostGetDevicePointer((void **)&r.d_tfree, r.h_tfree, 0)) {
    s->last_error = "served: pinned ring buffers";
    return false;
  }
  std::memset(r.h_done, 0, (size_t)nres * 4);
  std::memset(r.h_tfree, 0, RING_TEAMS * 4);
  std::memset(r.h_cq, 0, (size_t)RING_CQ * 4);
  r.cq_pos = 0;
  r.by_slot.assign(nres, nullptr);
  std::memset(r.h_zero, 0, (size_t)2 * r.stride * 8);
  r.team_tag.assign(RING_TEAMS, 0);
  r.busy.assign(nres, 0);
  r.teams_free.clear();
  for (int t = RING_TEAMS - 1; t >= 0; --t) r.teams_free.push_back(t);
  return true;
}

void ring_release(gme_server *s) {
  Ring &r = s->ring;
  if (r.kst) cudaStreamSynchronize(r.kst);
  if (r.cst) cudaStreamSynchronize(r.cst);
  cudaFree(r.d_rows); cudaFree(r.d_wrap); cudaFree(r.d_gen); cudaFree(r.d_ctrl); cudaFree(r.d_ring);
  cudaFree(r.d_jobs); cudaFree(r.d_bad); cudaFree(r.d_arena);
  cudaFree(r.d_units); cudaFree(r.d_team); cudaFree(r.d_twrap);
  cudaFreeHost(r.h_units); cudaFreeHost(r.h_tfree); cudaFreeHost(r.h_zero); cudaFreeHost(r.h_cq);
  cudaFreeHost(r.h_jobs); cudaFreeHost(r.h_bad); cudaFreeHost(r.h_tail);
  cudaFreeHost(r.h_stage[0]); cudaFreeHost(r.h_stage[1]); cudaFreeHost(r.h_res); cudaFreeHost(r.h_done);
  for (cudaEvent_t e : {r.kev, r.sev[0], r.sev[1]})
    if (e) cudaEventDestroy(e);
  if (r.kst) cudaStreamDestroy(r.kst);
  if (r.cst) cudaStreamDestroy(r.cst);
}

// Copies n symbols and returns the OR of them: above 0x7fff if any lies outside
// [0, 32767].  One pass, no early exit, so the compiler vectorizes it.
uint32_t copy_or(int32_t *__restrict__ dst, const int32_t *__restrict__ src, int64_t n) {
  uint32_t acc = 0;
  for (int64_t i = 0; i < n; ++i) {
    dst[i] = src[i];
    acc |= (uint32_t)src[i];
  }
  return acc;
}

// Admits queued requests into the rings (arrival order; requests too wide for the
// kernel's rows move to the launch slots' queue), stages them and publishes the
// tails.  Returns whether it admitted anything.
bool ring_admit(gme_server *s) {
  Ring &r = s->ring;
  std::vector<RingJob> adm;
  int64_t staged = 0;
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop) return false;
    int64_t ahead = r.ahead;
    int tails[6];
    std::copy(r.tail, r.tail + 6, tails);
    while (!s->queue.empty()) {
      Request &q = s->queue.front();
      if (q.n1 > gme::BATCH_MAX_N1) {
        s->wide.push_back(std::move(q));
        s->queue.pop_front();
        continue;
      }
      const bool blk = ring_block(s, q.n1, q.n2);
      const int ring = 2 * q.kind + (blk ? 0 : 1);
      int entries = blk ? ring_entries(s, q.n1, q.n2) : 1;
      if (entries > 1 && r.teams_free.empty()) entries = 1;  // no team free: the pair runs alone
      const int rslot = blk ? q.kind * r.qb + tails[ring] % r.qb : 3 * r.qb + q.kind * r.qw + tails[ring] % r.qw;
      bool full = false;
      for (int e = 0; e < entries; ++e)
        full |= r.busy[blk ? q.kind * r.qb + (tails[ring] + e) % r.qb : rslot] != 0;
      if (full) break;  // its ring is full
      const int64_t need = ring_need(s, q.n1, q.n2);
      const int64_t phys = ahead % r.arena_cap;
      const int64_t skip = phys + need > r.arena_cap ? r.arena_cap - phys : 0;
      if (ahead + skip + need - r.atail > r.arena_cap) break;  // the arena is full
      if (staged + need > r.stage_cap) break;                  // this round's staging is full
      RingJob j;
      j.block = blk;
      j.rslot = rslot;
      j.entries = entries;
      r.queued_cells += (int64_t)q.n1 * q.n2;
      if (entries > 1) {
        j.team = r.teams_free.back();
        r.teams_free.pop_back();
      }
      ahead += skip + need;
      j.arena_end = ahead;
      for (int e = 0; e < entries; ++e) r.busy[blk ? q.kind * r.qb + (tails[ring] + e) % r.qb : rslot] = 1;
      j.req = std::move(q);
      s->queue.pop_front();
      tails[ring] += entries;
      staged += need;
      adm.push_back(std::move(j));
    }
    s->st.queued = (int64_t)(s->queue.size() + s->wide.size());
    s->st.running += (int64_t)adm.size();
  }
  if (adm.empty()) return false;
  // this round's staging buffer: free once the copies of its last use are done
  const int k = r.cur;
  r.cur ^= 1;
  cudaEventSynchronize(r.sev[k]);
  int32_t *stage = r.h_stage[k];
  // runs of consecutive arena positions: {arena position, staging offset, ints}
  std::vector<std::array<int64_t, 3>> runs;
  int64_t soff = 0;
  const int padl = gme::serve_padl();
  for (RingJob &j : adm) {
    const Request &q = j.req;
    const int64_t need = ring_need(s, q.n1, q.n2);
    const int64_t start = (j.arena_end - need) % r.arena_cap;
    const int64_t alen = gme::serve_a_len(q.n1);
    int32_t *d = stage + soff;
    // pads zeroed, symbols copied and range-checked in one pass
    std::memset(d, 0, (size_t)padl * 4);
    const uint32_t or_a = copy_or(d + padl, q.sym.data(), q.n1);
    std::memset(d + padl + q.n1, 0, (size_t)(alen - padl - q.n1) * 4);
    const uint32_t or_b = copy_or(d + alen, q.sym.data() + q.n1, q.n2);
    std::memset(d + alen + q.n2, 0, (size_t)(need - alen - q.n2) * 4);
    if (!runs.empty() && runs.back()[0] + runs.back()[2] == start) runs.back()[2] += need;
    else runs.push_back({start, soff, need});
    soff += need;
    const int rslot = j.rslot;
    gme::BatchJob &jb = r.h_jobs[rslot];
    jb.a_off = start;
    jb.b_off = start + alen;
    jb.n1 = q.n1;
    jb.n2 = q.n2;
    jb.kind = q.kind;
    jb.index = rslot;
    jb.seg = 2 * rslot;
    jb.row_off = -1;
    jb.col_off = -1;
    if (j.block) {
      // every entry of a team carries the pair's descriptor (result slot: the first)
      const int k0 = rslot - q.kind * r.qb;
      if (j.team >= 0) {
        const unsigned groups = (unsigned)((q.n2 + 32 * 4 * r.NW - 1) / (32 * 4 * r.NW));
        unsigned &tag = r.team_tag[j.team];
        if (tag > 0xffffff00u - 2 * groups) {
          tag = 0;
          j.clear_rows = true;
        }
        j.tag0 = tag;
        tag += groups + 1;
      }
      for (int e = 0; e < j.entries; ++e) {
        const int sl = q.kind * r.qb + (k0 + e) % r.qb;
        r.h_jobs[sl] = jb;
        r.h_units[sl] = make_int4(j.team, (int)j.tag0, j.entries, 0);
      }
      if (j.team >= 0) r.h_tfree[j.team] = 0;
    }
    r.h_bad[2 * rslot] = or_a > 0x7fffu;
    r.h_bad[2 * rslot + 1] = or_b > 0x7fffu;
    r.h_done[rslot] = 0;
    r.h_res[rslot] = gme_result{};
    r.h_res[rslot].status = PENDING;
  }
  cudaError_t e = cudaSuccess;
  for (const auto &run : runs)
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(r.d_arena + run[0], stage + run[1], (size_t)run[2] * 4, cudaMemcpyHostToDevice, r.cst);
  // descriptors and symbol checks of the new tickets, as runs of ring slots
  auto copy_slots = [&](int base, int q, int t0, int t1) {
    for (int t = t0; t < t1 && e == cudaSuccess;) {
      const int sl = t % q, n = std::min(t1 - t, q - sl);
      e = cudaMemcpyAsync(r.d_jobs + base + sl, r.h_jobs + base + sl, (size_t)n * sizeof(gme::BatchJob),
                          cudaMemcpyHostToDevice, r.cst);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(r.d_bad + 2 * (base + sl), r.h_bad + 2 * (base + sl), (size_t)n * 8,
                            cudaMemcpyHostToDevice, r.cst);
      if (e == cudaSuccess && base < 3 * r.qb)
        e = cudaMemcpyAsync(r.d_units + base + sl, r.h_units + base + sl, (size_t)n * sizeof(int4),
                            cudaMemcpyHostToDevice, r.cst);
      t += n;
    }
  };
  // the new teams start cleared, by copies (a memset would be a kernel, which waits
  // for SMs the running kernel holds); their rows only when the tags run out
  const int64_t tbytes = gme::serve_team_bytes();
  for (const RingJob &j : adm)
    if (j.team >= 0 && e == cudaSuccess) {
      e = cudaMemcpyAsync(r.d_team + j.team * tbytes, r.h_zero, (size_t)tbytes, cudaMemcpyHostToDevice, r.cst);
      if (e == cudaSuccess && j.clear_rows)
        e = cudaMemcpyAsync(r.d_twrap + (int64_t)j.team * 2 * r.stride, r.h_zero, (size_t)2 * r.stride * 8,
                            cudaMemcpyHostToDevice, r.cst);
    }
  int tails[6];
  std::copy(r.tail, r.tail + 6, tails);
  for (const RingJob &j : adm) tails[2 * j.req.kind + (j.block ? 0 : 1)] += j.entries;
  for (int kd = 0; kd < 3; ++kd) {
    copy_slots(kd * r.qb, r.qb, r.tail[2 * kd], tails[2 * kd]);
    copy_slots(3 * r.qb + kd * r.qw, r.qw, r.tail[2 * kd + 1], tails[2 * kd + 1]);
  }
  // then, after them on the same stream, the tails the kernel claims below (the
  // host alone writes them: an unchanged one is written with its own value)
  std::copy(tails, tails + 6, r.h_tail + 8 * k);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(r.d_ring + gme::RW_TAIL, r.h_tail + 8 * k, 6 * 4, cudaMemcpyHostToDevice, r.cst);
  if (e == cudaSuccess) e = cudaEventRecord(r.sev[k], r.cst);
  std::copy(tails, tails + 6, r.tail);
  r.ahead = adm.back().arena_end;
  for (RingJob &j : adm) {
    r.live.push_back(std::move(j));
    r.by_slot[r.live.back().rslot] = &r.live.back();
  }
  const int64_t held = held_bytes(s);
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (e != cudaSuccess) s->last_error = std::string("served: ring copies: ") + cudaGetErrorString(e);
    s->st.h2d_bytes += soff * 4 + (int64_t)adm.size() * (int64_t)(sizeof(gme::BatchJob) + 8) + 24;
    s->st.d2h_bytes += (int64_t)adm.size() * (int64_t)(sizeof(gme_result) + sizeof(int));
    s->st.hbm_bytes_held = held;
    s->st.hbm_bytes_peak = std::max(s->st.hbm_bytes_peak, held);
  }
  return true;
}

// Reports the jobs the kernel has completed (its completion queue, in order) or, with
// fail_rest, every live job left with that status; frees ring slots, teams and (in
// admission order) arena space.  Returns whether anything completed.
bool ring_harvest(gme_server *s, bool fail_rest, int fail_status) {
  Ring &r = s->ring;
  std::vector<Finished> fin;
  std::vector<const Request *> who;
  auto release = [&](RingJob &j) {
    if (j.block) {
      const int k0 = j.rslot - j.req.kind * r.qb;
      for (int e = 0; e < j.entries; ++e) r.busy[j.req.kind * r.qb + (k0 + e) % r.qb] = 0;
    } else {
      r.busy[j.rslot] = 0;
    }
    r.by_slot[j.rslot] = nullptr;
    if (j.team >= 0) r.teams_free.push_back(j.team);
    j.released = true;
  };
  auto report = [&](RingJob &j, const gme_result &res) {
    j.done = true;
    r.queued_cells -= (int64_t)j.req.n1 * j.req.n2;
    fin.push_back(Finished{res, 0});
    who.push_back(&j.req);
    // a team's slots and its team are free once its last entry has left
    if (j.team >= 0 && !fail_rest) r.teams_done.push_back(&j);
    else release(j);
  };
  for (;;) {
    int *e = &r.h_cq[r.cq_pos & (RING_CQ - 1)];
    const int v = __atomic_load_n(e, __ATOMIC_ACQUIRE);
    if (v == 0) break;
    // the kernel writes this entry again only RING_CQ completions later, more than
    // there are live jobs
    __atomic_store_n(e, 0, __ATOMIC_RELAXED);
    ++r.cq_pos;
    RingJob *j = r.by_slot[v - 1];
    if (j && !j->done) report(*j, r.h_res[v - 1]);
  }
  if (fail_rest) {
    gme_result res{};
    res.status = fail_status;
    for (RingJob &j : r.live)
      if (!j.done) {
        res.kind = j.req.kind;
        report(j, res);
      }
    for (RingJob *j : r.teams_done) release(*j);
    r.teams_done.clear();
  }
  for (size_t k = 0; k < r.teams_done.size();) {
    RingJob &j = *r.teams_done[k];
    if (__atomic_load_n(&r.h_tfree[j.team], __ATOMIC_ACQUIRE)) {
      release(j);
      r.teams_done[k] = r.teams_done.back();
      r.teams_done.pop_back();
    } else {
      ++k;
    }
  }
  if (!fin.empty()) {
    const int64_t t = now_ns();
    {
      std::lock_guard<std::mutex> g(s->mu);
      for (size_t k = 0; k < fin.size(); ++k) {
        const Request &q = *who[k];
        fin[k].latency = t - q.t_submit;
        s->outstanding.erase(q.ticket);
        s->finished[q.ticket] = fin[k];
        s->finished_order.push_back(q.ticket);
        s->st.completed += 1;
        s->st.running -= 1;
        s->st.cells_completed += (int64_t)q.n1 * q.n2;
      }
    }
    s->cv_done.notify_all();
  }
  while (!r.live.empty() && r.live.front().released) {
    r.atail = r.live.front().arena_end;
    r.live.pop_front();
  }
  if (r.live.empty()) r.atail = r.ahead;
  {
    const int64_t held = held_bytes(s);
    std::lock_guard<std::mutex> g(s->mu);
    s->st.hbm_bytes_held = held;
  }
  return !fin.empty();
}

// Polls the kernel's last launch: once it has ended, reports what it finished and,
// if a bounded wait gave up, fails the live jobs and starts the rings over.
void ring_poll(gme_server *s) {
  Ring &r = s->ring;
  if (!r.launched || cudaEventQuery(r.kev) == cudaErrorNotReady) return;
  r.launched = false;
  r.yielding = false;
  int st = 0;
  if (cudaMemcpy(&st, r.d_ctrl + 8, 4, cudaMemcpyDeviceToHost) != cudaSuccess) st = GME_ERR_CUDA;
  // anything the launch finished is reported first
  ring_harvest(s, false, 0);
  if (st != 0) {
    set_error(s, "served: a device-side wait gave up; live requests fail");
    ring_harvest(s, true, st);
    cudaStreamSynchronize(r.cst);
    cudaMemset(r.d_ctrl, 0, 64);
    cudaMemset(r.d_ring, 0, gme::RW_PAIR * 4);
    cudaDeviceSynchronize();
    std::fill(r.tail, r.tail + 6, 0);
    r.ahead = r.atail = 0;
    std::fill(r.busy.begin(), r.busy.end(), 0);
    std::memset(r.h_cq, 0, (size_t)RING_CQ * 4);
    r.cq_pos = 0;
  }
}

// Asks the running kernel to leave (once per launch), so that a launch for pairs
// wider than its rows finds SMs; the dispatcher launches the kernel again after it.
void ring_yield(gme_server *s) {
  Ring &r = s->ring;
  if (!r.launched || r.yielding) return;
  r.h_tail[17] = 1;
  if (cudaMemcpyAsync(r.d_ring + gme::RW_EXIT, r.h_tail + 17, 4, cudaMemcpyHostToDevice, r.cst) == cudaSuccess)
    r.yielding = true;
}

// Launches the kernel when jobs are live and no launch is.
void ring_launch(gme_server *s) {
  Ring &r = s->ring;
  if (r.launched || r.live.empty()) return;
  gme::ServeArgs a;
  a.arena = r.d_arena;
  a.jobs_b = r.d_jobs;
  a.jobs_w = r.d_jobs + 3 * r.qb;
  a.qb = r.qb;
  a.qw = r.qw;
  a.symbad = r.d_bad;
  a.results = r.d_res;
  a.done = r.d_done;
  a.rows = r.d_rows;
  a.wrap = r.d_wrap;
  a.gen = r.d_gen;
  a.stride = r.stride;
  a.ctrl = r.d_ctrl;
  a.ring_ctl = r.d_ring;
  a.units = r.d_units;
  a.teams = r.d_team;
  a.twrap = r.d_twrap;
  a.tfree = r.d_tfree;
  a.cq = r.d_cq;
  a.cq_mask = RING_CQ - 1;
  a.sc = s->sc;
  a.timeout_ns = 10ull * 1000 * 1000 * 1000;
  a.idle_ns = RING_IDLE_NS;
  a.NW = r.NW;
  a.grid = r.grid;
  // the exit word of the last launch goes down first, on the kernel's stream (a copy:
  // a memset would be a kernel, waiting for SMs another launch may hold)
  cudaError_t e = cudaMemcpyAsync(r.d_ring + gme::RW_EXIT, r.h_zero, 4, cudaMemcpyHostToDevice, r.kst);
  if (e == cudaSuccess) e = gme::serve_launch(a, r.kst);
  if (e == cudaSuccess) e = cudaEventRecord(r.kev, r.kst);
  if (e != cudaSuccess) {
    set_error(s, std::string("served: kernel launch: ") + cudaGetErrorString(e));
    ring_harvest(s, true, GME_ERR_CUDA);
    return;
  }
  r.launched = true;
  std::lock_guard<std::mutex> g(s->mu);
  s->st.waves_launched += 1;
  s->st.kernels_launched += 1;
}

// Ring mode: asks the kernel to leave and waits for it (nothing is live).
void ring_stop(gme_server *s) {
  Ring &r = s->ring;
  if (!r.launched) return;
  r.h_tail[16] = 1;
  cudaMemcpyAsync(r.d_ring + gme::RW_STOP, r.h_tail + 16, 4, cudaMemcpyHostToDevice, r.cst);
  cudaStreamSynchronize(r.cst);
  cudaStreamSynchronize(r.kst);
  r.launched = false;
}

void ring_dispatcher(gme_server *s) {
  cudaSetDevice(s->device);
  for (;;) {
    bool progressed = false, busy = false;
    progressed |= ring_harvest(s, false, 0);
    for (Slot &sl : s->slots)
      if (sl.busy) progressed |= harvest(s, sl);
    progressed |= ring_admit(s);
    ring_poll(s);
    // pairs wider than the kernel's rows: the kernel steps aside for their launch
    bool wide;
    {
      std::lock_guard<std::mutex> g(s->mu);
      wide = !s->wide.empty();
    }
    bool slot_busy = false;
    for (Slot &sl : s->slots) slot_busy |= sl.busy;
    if (wide && !slot_busy) {
      if (s->ring.launched) ring_yield(s);
      else
        for (Slot &sl : s->slots)
          if (launch(s, sl)) slot_busy = progressed = true;
    }
    // and comes back once their launch has ended (each of its kernels fills the GPU)
    if (!slot_busy) ring_launch(s);
    busy = !s->ring.live.empty();
    for (Slot &sl : s->slots) busy |= sl.busy;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->stop && !busy) {
      lk.unlock();
      ring_stop(s);
      lk.lock();
      // nothing on the GPU: what is still queued is closed
      const int64_t t = now_ns();
      for (std::deque<Request> *qq : {&s->queue, &s->wide}) {
        while (!qq->empty()) {
          Request &q = qq->front();
          gme_result r{};
          r.status = GME_ERR_CLOSED;
          r.kind = q.kind;
          s->outstanding.erase(q.ticket);
          s->finished[q.ticket] = Finished{r, t - q.t_submit};
          s->finished_order.push_back(q.ticket);
          s->st.completed += 1;
          qq->pop_front();
        }
      }
      s->st.queued = 0;
      lk.unlock();
      s->cv_done.notify_all();
      return;
    }
    if (!progressed) {
      if (!busy && s->queue.empty() && s->wide.empty()) {
        s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty(); });
      } else {
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
  if (s->cfg.mode == GME_SERVE_RING && n1 <= gme::BATCH_MAX_N1) {
    // the ring kernel's pair: its staged symbols in the arena and a descriptor
    const int64_t need = ring_need(s, q.n1, q.n2);
    if (need > s->ring.arena_cap || need > s->ring.stage_cap) return GME_ERR_BUDGET;
    q.bytes = 4 * need + (int64_t)sizeof(gme::BatchJob);
    q.sym.resize((size_t)(n1 + n2));
    if (n1) std::memcpy(q.sym.data(), a, (size_t)n1 * 4);
    if (n2) std::memcpy(q.sym.data() + n1, b, (size_t)n2 * 4);
    return GME_OK;
  }
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
      (c.warps_per_block && c.warps_per_block != 4 && c.warps_per_block != 8) ||
      (c.mode != GME_SERVE_RING && c.mode != GME_SERVE_WAVES))
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
  // ring mode keeps one launch slot, for pairs wider than the kernel's rows
  s->slots.resize(c.mode == GME_SERVE_RING ? 1 : c.waves);
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
    if (c.mode == GME_SERVE_RING) {
      cudaSetDevice(device);
      if (!ring_setup(s, gme::ctx_sms(s->slots[0].ctx))) {
        rc = GME_ERR_NOMEM;
        ring_release(s);
      } else {
        const int64_t held = held_bytes(s);
        s->st.hbm_bytes_held = held;
        s->st.hbm_bytes_peak = held;
      }
    }
  }
  if (rc != GME_OK) {
    for (Slot &sl : s->slots) {
      if (sl.ev) cudaEventDestroy(sl.ev);
      if (sl.ctx) gme_destroy(sl.ctx);
    }
    delete s;
    return rc;
  }
  s->dispatcher = std::thread(c.mode == GME_SERVE_RING ? ring_dispatcher : dispatcher_main, s);
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
  if (s->cfg.mode == GME_SERVE_RING) ring_release(s);
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
