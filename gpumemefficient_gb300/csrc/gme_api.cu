// gme_api.cu -- the C ABI of include/gme.h: contexts, workspaces, the plain path.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "gme_common.cuh"
#include "gme_internal.h"

namespace gme {

int Workspace::fail(cudaError_t e, const char *what) {
  last_error = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
  return (e == cudaErrorMemoryAllocation) ? ST_NOMEM : ST_CUDA;
}

int Workspace::fail_msg(int status, const std::string &msg) {
  last_error = msg;
  return status;
}

static int grow(void **p, long long *cap, long long need, size_t elem, Workspace &ws, const char *what,
                bool zero) {
  if (*cap >= need && *p) return ST_OK;
  if (ws.sync_stream) cudaStreamSynchronize(ws.sync_stream);
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  long long n = need + need / 4 + 1024;
  cudaError_t e = cudaMalloc(p, (size_t)n * elem);
  if (e != cudaSuccess) {
    *p = nullptr;
    return ws.fail(e, what);
  }
  if (zero) {
    // the library's streams do not wait for the null stream: finish the clear here
    e = cudaMemset(*p, 0, (size_t)n * elem);
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) return ws.fail(e, what);
  }
  *cap = n;
  return ST_OK;
}

int Workspace::reserve(long long a_len, long long b_len, long long slot_words, int nbest) {
  int rc;
  if ((rc = grow((void **)&a_pad, &a_pad_cap, a_len, sizeof(int), *this, "cudaMalloc(a_pad)", false))) return rc;
  if ((rc = grow((void **)&b_pad, &b_pad_cap, b_len, sizeof(int), *this, "cudaMalloc(b_pad)", false))) return rc;
  if (slots_cap < slot_words || !slots) {
    if ((rc = grow((void **)&slots, &slots_cap, slot_words, 8, *this, "cudaMalloc(slots)", true))) return rc;
    slots_bytes = (size_t)slots_cap * 8;
    tag_next = 1;  // fresh zeroed memory: every tag is unused
  }
  long long bc = best_cap;
  if ((rc = grow(&best, &bc, nbest, 32, *this, "cudaMalloc(best)", false))) return rc;
  best_cap = (int)bc;
  if (!ctrl) {
    cudaError_t e = cudaMalloc(&ctrl, 16 * sizeof(int));
    if (e != cudaSuccess) return fail(e, "cudaMalloc(ctrl)");
    e = cudaMemset(ctrl, 0, 16 * sizeof(int));
    if (e == cudaSuccess) e = cudaStreamSynchronize(0);
    if (e != cudaSuccess) return fail(e, "cudaMemset(ctrl)");
  }
  return ST_OK;
}

void Workspace::release() {
  if (sync_stream) cudaStreamSynchronize(sync_stream);
  cudaFree(a_pad); cudaFree(b_pad); cudaFree(slots); cudaFree(best); cudaFree(ctrl);
  a_pad = b_pad = nullptr; slots = nullptr; best = nullptr; ctrl = nullptr;
  a_pad_cap = b_pad_cap = slots_cap = 0; best_cap = 0;
}

static int grow_ll(void **p, long long *cap, long long need, size_t elem, Workspace &ws, const char *what) {
  return grow(p, cap, need, elem, ws, what, false);
}

int BatchArena::reserve(long long staged, long long nseg, long long njobs, Workspace &ws) {
  int rc;
  if ((rc = grow_ll((void **)&d_staged, &staged_cap, staged, sizeof(int), ws, "cudaMalloc(batch staged)"))) return rc;
  if (seg_cap < nseg || !d_from) {
    long long c0 = seg_cap, c1 = seg_cap, c2 = seg_cap, c3 = seg_cap, c4 = seg_cap, c5 = seg_cap;
    if ((rc = grow_ll((void **)&d_from, &c0, nseg, 8, ws, "cudaMalloc(batch from)")) ||
        (rc = grow_ll((void **)&d_to, &c1, nseg, 8, ws, "cudaMalloc(batch to)")) ||
        (rc = grow_ll((void **)&d_len, &c2, nseg, 4, ws, "cudaMalloc(batch len)")) ||
        (rc = grow_ll((void **)&d_padl, &c3, nseg, 4, ws, "cudaMalloc(batch padl)")) ||
        (rc = grow_ll((void **)&d_total, &c4, nseg, 4, ws, "cudaMalloc(batch total)")) ||
        (rc = grow_ll((void **)&d_symbad, &c5, nseg, 4, ws, "cudaMalloc(batch symbol check)")))
      return rc;
    seg_cap = std::min(std::min(std::min(c0, c1), std::min(c2, c3)), std::min(c4, c5));
  }
  if ((rc = grow_ll((void **)&d_jobs, &jobs_cap, njobs, sizeof(BatchJob), ws, "cudaMalloc(batch jobs)"))) return rc;
  if (!d_ctrl) {
    cudaError_t e = cudaMalloc(&d_ctrl, 16 * sizeof(int));
    if (e != cudaSuccess) return ws.fail(e, "cudaMalloc(batch ctrl)");
  }
  return ST_OK;
}

int BatchArena::reserve_rows(long long ints, Workspace &ws) {
  return grow_ll((void **)&d_rows, &rows_cap, ints, sizeof(int), ws, "cudaMalloc(batch rows)");
}

// Wrap-row tags come from one counter that only grows, so a row never holds a tag
// that a later job is handed, whatever the layout of the rows (fresh rows are zero).
int BatchArena::reserve_wrap(long long words, Workspace &ws) {
  int rc;
  if ((rc = grow((void **)&d_wrap, &wrap_cap, words, 8, ws, "cudaMalloc(batch wrap rows)", true))) return rc;
  if (!d_gen) {
    long long gc = 0;
    if ((rc = grow((void **)&d_gen, &gc, 1, 4, ws, "cudaMalloc(batch wrap tags)", true))) return rc;
  }
  return ST_OK;
}

int BatchArena::reserve_team(long long units, long long bytes, Workspace &ws) {
  int rc;
  if ((rc = grow_ll((void **)&d_units, &units_cap, std::max(units, 1ll), sizeof(int4), ws, "cudaMalloc(batch team units)")))
    return rc;
  return grow_ll((void **)&d_team, &team_cap, std::max(bytes, 16ll), 1, ws, "cudaMalloc(batch teams)");
}

void BatchArena::release() {
  cudaFree(d_rows);
  d_rows = nullptr;
  rows_cap = 0;
  cudaFree(d_wrap); cudaFree(d_gen);
  d_wrap = nullptr; d_gen = nullptr; wrap_cap = 0;
  cudaFree(d_units); cudaFree(d_team);
  d_units = nullptr; d_team = nullptr; units_cap = team_cap = 0;
  cudaFree(d_staged); cudaFree(d_from); cudaFree(d_to); cudaFree(d_len); cudaFree(d_padl);
  cudaFree(d_total); cudaFree(d_jobs); cudaFree(d_ctrl); cudaFree(d_symbad);
  d_symbad = nullptr;
  d_staged = nullptr; d_from = d_to = nullptr; d_len = d_padl = d_total = nullptr; d_jobs = nullptr;
  d_ctrl = nullptr; staged_cap = seg_cap = jobs_cap = 0;
}

// A kernel that waits, with the library's bounded wait, on a word nothing sets.
__global__ void debug_wait_kernel(int *ctrl, const int *never, unsigned long long timeout_ns) {
  __shared__ int abort_flag;
  if (threadIdx.x == 0) abort_flag = 0;
  __syncthreads();
  Waiter W(timeout_ns, &ctrl[1], &abort_flag);
  W.wait([&] { return ld_relaxed_gpu_s32(never) != 0; });
}

int debug_wait_timeout(Workspace &ws, unsigned long long timeout_ns, int *kernel_status,
                       cudaStream_t st) {
  int rc = ws.reserve(16, 16, 16, 1);
  if (rc != ST_OK) return rc;
  cudaError_t e = cudaMemsetAsync(ws.ctrl, 0, 16 * sizeof(int), st);
  if (e != cudaSuccess) return ws.fail(e, "cudaMemsetAsync(ctrl)");
  // ctrl[8] is never written by anyone: the wait can only end by its deadline
  debug_wait_kernel<<<1, 32, 0, st>>>(ws.ctrl, ws.ctrl + 8, timeout_ns);
  ws.launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "debug_wait_kernel");
  int host[2] = {0, 0};
  if ((e = cudaMemcpyAsync(host, ws.ctrl, 2 * sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return ws.fail(e, "cudaMemcpyAsync(ctrl)");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return ws.fail(e, "cudaStreamSynchronize");
  *kernel_status = host[1];
  return ST_OK;
}

}  // namespace gme

struct gme_context {
  gme::Workspace ws;
  int device = 0;
  cudaStream_t stream = nullptr;
  unsigned long long timeout_ns = 10ull * 1000 * 1000 * 1000;
  gme_plain_config cfg{};
  // device staging for the host-buffer entry points
  int *d_a = nullptr; long long d_a_cap = 0;
  int *d_b = nullptr; long long d_b_cap = 0;
  int *d_row = nullptr; long long d_row_cap = 0;
  int *d_col = nullptr; long long d_col_cap = 0;
  gme_result *d_res = nullptr;
  gme_result *h_res = nullptr;  // pinned
  // batched path
  gme::BatchArena batch;
  gme::BatchTuning batch_tune;
  int *d_bsym = nullptr; long long d_bsym_cap = 0;
  gme_result *d_bres = nullptr; long long d_bres_cap = 0;
  // summed-area table staging for the host-buffer entry point
  int *d_sat = nullptr; long long d_sat_cap = 0;
};

using gme::ST_OK;

static gme_status to_status(int s) { return (gme_status)s; }

static gme_status check_sizes(gme_context *ctx, gme_kind kind, int64_t n1, int64_t n2,
                              const gme_scoring *sc) {
  const int64_t LIM = (1ll << 30) - 4096;
  if (kind < GME_LCS || kind > GME_SW) {
    ctx->ws.last_error = "invalid kind";
    return GME_ERR_INVALID;
  }
  if (n1 < 0 || n2 < 0) {
    ctx->ws.last_error = "negative length";
    return GME_ERR_INVALID;
  }
  if (n1 > LIM || n2 > LIM) {
    ctx->ws.last_error = "sequence longer than 2^30-4096";
    return GME_ERR_OVERFLOW;
  }
  if (kind == GME_SW) {
    if (!sc) {
      ctx->ws.last_error = "SW needs scoring constants";
      return GME_ERR_INVALID;
    }
    long long m = std::max<long long>(std::max<long long>(llabs(sc->match), llabs(sc->mismatch)),
                                      llabs(sc->gap));
    if (m * (long long)(n1 + n2 + 2) >= (1ll << 30)) {
      ctx->ws.last_error = "SW scores could overflow int32";
      return GME_ERR_OVERFLOW;
    }
  }
  if (kind == GME_ED && sc && sc->ed_boundary != GME_ED_REF_CPU && sc->ed_boundary != GME_ED_STANDARD) {
    ctx->ws.last_error = "invalid ed_boundary";
    return GME_ERR_INVALID;
  }
  return GME_OK;
}

static gme::Scoring to_scoring(const gme_scoring *sc) {
  gme::Scoring s;
  gme_scoring d = gme_default_scoring();
  if (!sc) sc = &d;
  s.match = sc->match;
  s.mismatch = sc->mismatch;
  s.gap = sc->gap;
  s.ed_rule = sc->ed_boundary;
  return s;
}

static int grow_dev(void **p, long long *cap, long long need, size_t elem, gme_context *ctx) {
  if (*cap >= need && *p) return ST_OK;
  cudaStreamSynchronize(ctx->stream);
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  long long n = need + need / 4 + 256;
  cudaError_t e = cudaMalloc(p, (size_t)n * elem);
  if (e != cudaSuccess) {
    *p = nullptr;
    return ctx->ws.fail(e, "cudaMalloc(staging)");
  }
  *cap = n;
  return ST_OK;
}

extern "C" {

const char *gme_status_string(gme_status s) {
  switch (s) {
    case GME_OK: return "ok";
    case GME_ERR_INVALID: return "invalid argument";
    case GME_ERR_CUDA: return "CUDA error";
    case GME_ERR_NOMEM: return "out of memory";
    case GME_ERR_TIMEOUT: return "device wait timed out";
    case GME_ERR_OVERFLOW: return "sizes could overflow int32 scores";
    case GME_ERR_BUDGET: return "request exceeds the HBM budget";
    case GME_ERR_NOT_READY: return "not ready";
    case GME_ERR_CLOSED: return "server closed";
  }
  return "unknown status";
}

gme_scoring gme_default_scoring(void) {
  gme_scoring s;
  s.match = 3;      // SmithWaterman/SW.cpp:45-47
  s.mismatch = -3;
  s.gap = -2;       // SmithWaterman/SW.cpp:63-64
  s.ed_boundary = GME_ED_REF_CPU;
  return s;
}

gme_status gme_create(int device, gme_context **out) {
  if (!out) return GME_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || device < 0 || device >= n) return e != cudaSuccess ? GME_ERR_CUDA : GME_ERR_INVALID;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return GME_ERR_CUDA;
  gme_context *ctx = new (std::nothrow) gme_context();
  if (!ctx) return GME_ERR_NOMEM;
  ctx->device = device;
  ctx->ws.device = device;
  cudaDeviceGetAttribute(&ctx->ws.sms, cudaDevAttrMultiProcessorCount, device);
  if ((e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)) != cudaSuccess) {
    delete ctx;
    return GME_ERR_CUDA;
  }
  ctx->ws.sync_stream = ctx->stream;
  if ((e = cudaMalloc(&ctx->d_res, sizeof(gme_result))) != cudaSuccess ||
      (e = cudaMallocHost(&ctx->h_res, sizeof(gme_result))) != cudaSuccess) {
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GME_ERR_NOMEM;
  }
  *out = ctx;
  return GME_OK;
}

gme_status gme_destroy(gme_context *ctx) {
  if (!ctx) return GME_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  ctx->ws.release();
  ctx->batch.release();
  cudaFree(ctx->d_bsym); cudaFree(ctx->d_bres); cudaFree(ctx->d_sat);
  cudaFree(ctx->d_a); cudaFree(ctx->d_b); cudaFree(ctx->d_row); cudaFree(ctx->d_col);
  cudaFree(ctx->d_res);
  cudaFreeHost(ctx->h_res);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return GME_OK;
}

const char *gme_last_error(const gme_context *ctx) {
  return ctx ? ctx->ws.last_error.c_str() : "no context";
}

gme_status gme_set_wait_timeout_ns(gme_context *ctx, uint64_t ns) {
  if (!ctx || ns == 0) return GME_ERR_INVALID;
  ctx->timeout_ns = ns;
  return GME_OK;
}

gme_status gme_set_plain_config(gme_context *ctx, const gme_plain_config *cfg) {
  if (!ctx) return GME_ERR_INVALID;
  if (!cfg) { ctx->cfg = gme_plain_config{}; return GME_OK; }
  if ((cfg->rows_per_lane || cfg->warps_per_band) &&
      !gme::plain_config_valid(cfg->rows_per_lane, cfg->warps_per_band)) {
    ctx->ws.last_error = "plain config: rows_per_lane must be 2 or 4, warps_per_band 4 or 8";
    return GME_ERR_INVALID;
  }
  if (cfg->grid < 0) return GME_ERR_INVALID;
  ctx->cfg = *cfg;
  return GME_OK;
}

gme_status gme_get_plain_config(const gme_context *ctx, int64_t n1, int64_t n2, gme_plain_config *r) {
  if (!ctx || !r) return GME_ERR_INVALID;
  int R, NW, grid;
  gme::plain_auto_config(ctx->ws.sms, n1, n2, &R, &NW, &grid);
  if (ctx->cfg.rows_per_lane) { R = ctx->cfg.rows_per_lane; NW = ctx->cfg.warps_per_band; }
  const long long H = (long long)NW * 32 * R;
  const long long nb = n2 > 0 ? (n2 + H - 1) / H : 0;
  grid = (int)std::min<long long>(nb, ctx->ws.sms);
  if (ctx->cfg.grid) grid = (int)std::min<long long>(nb, ctx->cfg.grid);
  r->rows_per_lane = R;
  r->warps_per_band = NW;
  r->grid = grid;
  r->reserved = 0;
  return GME_OK;
}

gme_status gme_align_device(gme_context *ctx, gme_kind kind, const int32_t *d_a, int64_t n1,
                            const int32_t *d_b, int64_t n2, const gme_scoring *sc,
                            gme_result *d_out, int32_t *d_last_row, int32_t *d_last_col,
                            void *stream) {
  if (!ctx || !d_out || (n1 > 0 && !d_a) || (n2 > 0 && !d_b)) return GME_ERR_INVALID;
  gme_status s = check_sizes(ctx, kind, n1, n2, sc);
  if (s != GME_OK) return s;
  cudaSetDevice(ctx->device);
  gme_plain_config c;
  gme_get_plain_config(ctx, n1, n2, &c);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  cudaStream_t prev = ctx->ws.sync_stream;
  ctx->ws.sync_stream = st;
  int rc = gme::plain_run(ctx->ws, (int)kind, d_a, n1, d_b, n2, to_scoring(sc), d_out, d_last_row,
                          d_last_col, st, c.rows_per_lane, c.warps_per_band, c.grid, ctx->timeout_ns);
  ctx->ws.sync_stream = prev;
  return to_status(rc);
}

gme_status gme_align(gme_context *ctx, gme_kind kind, const int32_t *a, int64_t n1,
                     const int32_t *b, int64_t n2, const gme_scoring *sc, gme_result *out,
                     int32_t *last_row, int32_t *last_col) {
  if (!ctx || !out || (n1 > 0 && !a) || (n2 > 0 && !b)) return GME_ERR_INVALID;
  gme_status s = check_sizes(ctx, kind, n1, n2, sc);
  if (s != GME_OK) return s;
  cudaSetDevice(ctx->device);
  int rc;
  if ((rc = grow_dev((void **)&ctx->d_a, &ctx->d_a_cap, std::max<int64_t>(n1, 1), 4, ctx)) ||
      (rc = grow_dev((void **)&ctx->d_b, &ctx->d_b_cap, std::max<int64_t>(n2, 1), 4, ctx)))
    return to_status(rc);
  if (last_row && (rc = grow_dev((void **)&ctx->d_row, &ctx->d_row_cap, n1 + 1, 4, ctx))) return to_status(rc);
  if (last_col && (rc = grow_dev((void **)&ctx->d_col, &ctx->d_col_cap, n2 + 1, 4, ctx))) return to_status(rc);
  cudaStream_t st = ctx->stream;
  cudaError_t e;
  if (n1 > 0 && (e = cudaMemcpyAsync(ctx->d_a, a, (size_t)n1 * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(a)"));
  if (n2 > 0 && (e = cudaMemcpyAsync(ctx->d_b, b, (size_t)n2 * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(b)"));
  s = gme_align_device(ctx, kind, ctx->d_a, n1, ctx->d_b, n2, sc, ctx->d_res,
                       last_row ? ctx->d_row : nullptr, last_col ? ctx->d_col : nullptr, st);
  if (s != GME_OK) return s;
  if ((e = cudaMemcpyAsync(ctx->h_res, ctx->d_res, sizeof(gme_result), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(result)"));
  if (last_row && (e = cudaMemcpyAsync(last_row, ctx->d_row, (size_t)(n1 + 1) * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(last_row)"));
  if (last_col && (e = cudaMemcpyAsync(last_col, ctx->d_col, (size_t)(n2 + 1) * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(last_col)"));
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return to_status(ctx->ws.fail(e, "cudaStreamSynchronize"));
  *out = *ctx->h_res;
  if (out->status != 0) {
    ctx->ws.last_error = "device-side wait timed out";
    return to_status(out->status);
  }
  return GME_OK;
}

gme_status gme_batch_tuned_config(const gme_pair *pairs, int64_t n, gme_batch_config *out) {
  if (!out || n < 0 || (n > 0 && !pairs)) return GME_ERR_INVALID;
  const gme::BatchTuning t = gme::batch_tuning_for(pairs, n, gme::BatchTuning{});
  out->warps_per_block = t.warps_per_block;
  out->blocks_per_sm = t.blocks_per_sm;
  out->block_min_cells = t.block_min_cells;
  out->long_min_cells = 0;
  out->team_min_cells = t.team_min_cells;
  out->packed16 = t.packed16 ? 0 : -1;
  out->team_split = t.team_split;
  out->rows_per_lane = t.rows_per_lane;
  return GME_OK;
}

gme_status gme_sat_device(gme_context *ctx, int32_t *d_table, int64_t n1, int64_t n2, int64_t ld,
                          int32_t *d_status, void *stream) {
  if (!ctx || (n1 > 0 && n2 > 0 && !d_table)) return GME_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  // a regrow of the tagged scratch must drain the stream this call runs on
  cudaStream_t prev = ctx->ws.sync_stream;
  ctx->ws.sync_stream = st;
  const int rc = gme::sat_run(ctx->ws, d_table, n1, n2, ld, d_status, st, ctx->timeout_ns);
  ctx->ws.sync_stream = prev;
  return to_status(rc);
}

gme_status gme_sat(gme_context *ctx, int32_t *table, int64_t n1, int64_t n2, int64_t ld) {
  if (!ctx || n1 < 0 || n2 < 0 || ld < n1 + 1 || (n1 > 0 && n2 > 0 && !table)) return GME_ERR_INVALID;
  if (n1 == 0 || n2 == 0) return GME_OK;
  cudaSetDevice(ctx->device);
  const long long cells = (n2 + 1) * ld;
  int rc;
  if ((rc = grow_dev((void **)&ctx->d_sat, &ctx->d_sat_cap, cells, 4, ctx))) return to_status(rc);
  cudaStream_t st = ctx->stream;
  cudaError_t e;
  if ((e = cudaMemcpyAsync(ctx->d_sat, table, (size_t)cells * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(sat table)"));
  gme_status s = to_status(gme::sat_run(ctx->ws, ctx->d_sat, n1, n2, ld, &ctx->d_res->status, st, ctx->timeout_ns));
  if (s != GME_OK) return s;
  if ((e = cudaMemcpyAsync(table + ld, ctx->d_sat + ld, (size_t)(cells - ld) * 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaMemcpyAsync(ctx->h_res, ctx->d_res, sizeof(gme_result), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(sat result)"));
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return to_status(ctx->ws.fail(e, "cudaStreamSynchronize"));
  if (ctx->h_res->status != 0) {
    ctx->ws.last_error = "sat: device-side wait timed out";
    return to_status(ctx->h_res->status);
  }
  return GME_OK;
}

// the plain path for the pairs a batch hands over (too wide for the batch kernel's rows,
// empty, or very large)
static int batch_plain_cb(void *p, int kind, const int *d_a, long long n1, const int *d_b, long long n2,
                          gme_result *d_out, int *d_last_row, int *d_last_col) {
  struct Arg { gme_context *ctx; const gme_scoring *sc; cudaStream_t st; };
  Arg *a = (Arg *)p;
  return (int)gme_align_device(a->ctx, (gme_kind)kind, d_a, n1, d_b, n2, a->sc, d_out, d_last_row,
                               d_last_col, a->st);
}

gme_status gme_set_batch_config(gme_context *ctx, const gme_batch_config *cfg) {
  if (!ctx) return GME_ERR_INVALID;
  gme::BatchTuning t;
  if (cfg) {
    if (cfg->warps_per_block) {
      if (!gme::batch_config_valid(cfg->warps_per_block)) {
        ctx->ws.last_error = "batch config: warps_per_block must be 4 or 8";
        return GME_ERR_INVALID;
      }
      t.warps_per_block = cfg->warps_per_block;
    }
    if (cfg->blocks_per_sm < 0 || cfg->block_min_cells < 0 || cfg->long_min_cells < -1 ||
        cfg->team_min_cells < -1 || cfg->team_split < 0)
      return GME_ERR_INVALID;
    t.blocks_per_sm = cfg->blocks_per_sm;
    if (cfg->block_min_cells) t.block_min_cells = cfg->block_min_cells;
    t.long_min_cells = cfg->long_min_cells;
    if (cfg->team_min_cells) t.team_min_cells = cfg->team_min_cells;
    if (cfg->team_split) t.team_split = cfg->team_split;
    if (cfg->packed16 < -1 || cfg->packed16 > 1) return GME_ERR_INVALID;
    t.packed16 = cfg->packed16 >= 0;
    if (cfg->rows_per_lane != 0 && cfg->rows_per_lane != 2 && cfg->rows_per_lane != 4) {
      ctx->ws.last_error = "batch config: rows_per_lane must be 2 or 4";
      return GME_ERR_INVALID;
    }
    if (cfg->rows_per_lane) t.rows_per_lane = cfg->rows_per_lane;
    // 2 rows per lane exists with 8 warps per CTA only
    if (t.rows_per_lane == 2) {
      if (cfg->warps_per_block == 4) {
        ctx->ws.last_error = "batch config: rows_per_lane 2 needs warps_per_block 8";
        return GME_ERR_INVALID;
      }
      t.warps_per_block = 8;
    }
  }
  // an all-zero configuration means "automatic" (the tuned table)
  t.user_set = cfg && (cfg->warps_per_block || cfg->blocks_per_sm || cfg->block_min_cells ||
                       cfg->long_min_cells || cfg->team_min_cells || cfg->team_split || cfg->rows_per_lane);
  if (!t.user_set && cfg) t.packed16 = cfg->packed16 >= 0;
  ctx->batch_tune = t;
  return GME_OK;
}

gme_status gme_align_batch_device(gme_context *ctx, const int32_t *d_symbols, int64_t nsym,
                                  const gme_pair *pairs, int64_t npairs, const gme_scoring *sc,
                                  gme_result *d_results, void *stream) {
  if (!ctx || npairs < 0 || (npairs > 0 && (!pairs || !d_results || !d_symbols)) || nsym < 0)
    return GME_ERR_INVALID;
  if (npairs == 0) return GME_OK;
  gme_scoring def = gme_default_scoring();
  if (!sc) sc = &def;
  for (int64_t i = 0; i < npairs; ++i) {
    gme_status s = check_sizes(ctx, (gme_kind)pairs[i].kind, pairs[i].n1, pairs[i].n2, sc);
    if (s != GME_OK) {
      ctx->ws.last_error = "pair " + std::to_string(i) + ": " + ctx->ws.last_error;
      return s;
    }
  }
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  struct { gme_context *ctx; const gme_scoring *sc; cudaStream_t st; } arg = {ctx, sc, st};
  int rc = gme::batch_run(ctx->ws, ctx->batch, d_symbols, nsym, pairs, npairs, to_scoring(sc),
                          d_results, st, ctx->batch_tune, ctx->timeout_ns, nullptr, nullptr, nullptr,
                          nullptr, batch_plain_cb, &arg);
  return to_status(rc);
}

gme_status gme_align_batch_device_rows(gme_context *ctx, const int32_t *d_symbols, int64_t nsym,
                                       const gme_pair *pairs, int64_t npairs, const gme_scoring *sc,
                                       gme_result *d_results, int32_t *d_last_rows,
                                       const int64_t *row_offsets, int32_t *d_last_cols,
                                       const int64_t *col_offsets, void *stream) {
  if (!ctx || npairs < 0 || (npairs > 0 && (!pairs || !d_results || !d_symbols)) || nsym < 0 ||
      (d_last_rows && !row_offsets) || (d_last_cols && !col_offsets))
    return GME_ERR_INVALID;
  if (npairs == 0) return GME_OK;
  gme_scoring def = gme_default_scoring();
  if (!sc) sc = &def;
  for (int64_t i = 0; i < npairs; ++i) {
    gme_status s = check_sizes(ctx, (gme_kind)pairs[i].kind, pairs[i].n1, pairs[i].n2, sc);
    if (s != GME_OK) {
      ctx->ws.last_error = "pair " + std::to_string(i) + ": " + ctx->ws.last_error;
      return s;
    }
  }
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  struct { gme_context *ctx; const gme_scoring *sc; cudaStream_t st; } arg = {ctx, sc, st};
  int rc = gme::batch_run(ctx->ws, ctx->batch, d_symbols, nsym, pairs, npairs, to_scoring(sc),
                          d_results, st, ctx->batch_tune, ctx->timeout_ns, d_last_rows,
                          (const long long *)row_offsets, d_last_cols, (const long long *)col_offsets,
                          batch_plain_cb, &arg);
  return to_status(rc);
}

gme_status gme_align_batch(gme_context *ctx, const int32_t *symbols, int64_t nsym,
                           const gme_pair *pairs, int64_t npairs, const gme_scoring *sc,
                           gme_result *results) {
  if (!ctx || npairs < 0 || nsym < 0 || (npairs > 0 && (!pairs || !results || !symbols)))
    return GME_ERR_INVALID;
  if (npairs == 0) return GME_OK;
  cudaSetDevice(ctx->device);
  int rc;
  if ((rc = grow_dev((void **)&ctx->d_bsym, &ctx->d_bsym_cap, std::max<int64_t>(nsym, 1), 4, ctx)) ||
      (rc = grow_dev((void **)&ctx->d_bres, &ctx->d_bres_cap, npairs, sizeof(gme_result), ctx)))
    return to_status(rc);
  cudaStream_t st = ctx->stream;
  cudaError_t e;
  if (nsym > 0 && (e = cudaMemcpyAsync(ctx->d_bsym, symbols, (size_t)nsym * 4, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(batch symbols)"));
  gme_status s = gme_align_batch_device(ctx, ctx->d_bsym, nsym, pairs, npairs, sc, ctx->d_bres, st);
  if (s != GME_OK) return s;
  if ((e = cudaMemcpyAsync(results, ctx->d_bres, (size_t)npairs * sizeof(gme_result), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
    return to_status(ctx->ws.fail(e, "cudaMemcpyAsync(batch results)"));
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return to_status(ctx->ws.fail(e, "cudaStreamSynchronize"));
  for (int64_t i = 0; i < npairs; ++i)
    if (results[i].status != 0) {
      ctx->ws.last_error = "device-side wait timed out";
      return to_status(results[i].status);
    }
  int bad = 0;
  if ((e = cudaMemcpy(&bad, ctx->batch.d_ctrl + 8, sizeof(int), cudaMemcpyDeviceToHost)) == cudaSuccess && bad)
    return to_status(bad);
  return GME_OK;
}

struct gme_batch_plan {
  gme_context *ctx = nullptr;
  gme::BatchArena ar;
  int64_t npairs = 0;
  int64_t max_len_sum = 0;
  cudaGraphExec_t exec = nullptr;  // captured launch sequence and what it was captured for
  const void *g_sym = nullptr;
  void *g_res = nullptr;
  cudaStream_t g_st = nullptr;
  gme_scoring g_sc{};
  int kernels = 0;
};

gme_status gme_batch_plan_create(gme_context *ctx, const gme_pair *pairs, int64_t npairs,
                                 int64_t nsym, gme_batch_plan **out) {
  if (!ctx || !out || npairs < 0 || nsym < 0 || (npairs > 0 && !pairs)) return GME_ERR_INVALID;
  *out = nullptr;
  gme_scoring def = gme_default_scoring();
  int64_t mx = 0;
  for (int64_t i = 0; i < npairs; ++i) {
    gme_status s = check_sizes(ctx, (gme_kind)pairs[i].kind, pairs[i].n1, pairs[i].n2, &def);
    if (s != GME_OK) {
      ctx->ws.last_error = "pair " + std::to_string(i) + ": " + ctx->ws.last_error;
      return s;
    }
    mx = std::max<int64_t>(mx, (int64_t)pairs[i].n1 + pairs[i].n2);
  }
  cudaSetDevice(ctx->device);
  gme_batch_plan *p = new (std::nothrow) gme_batch_plan();
  if (!p) return GME_ERR_NOMEM;
  p->ctx = ctx;
  p->npairs = npairs;
  p->max_len_sum = mx;
  int rc = gme::batch_plan(ctx->ws, p->ar, pairs, npairs, nsym, ctx->batch_tune, ctx->stream);
  // runs may come on other streams: the descriptors must have landed first
  if (rc == ST_OK) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = ctx->ws.fail(e, "cudaStreamSynchronize(batch plan)");
  }
  if (rc != ST_OK) {
    p->ar.release();
    delete p;
    return to_status(rc);
  }
  ctx->batch.last_block_jobs = p->ar.last_block_jobs;
  ctx->batch.last_warp_jobs = p->ar.last_warp_jobs;
  ctx->batch.last_long_jobs = p->ar.last_long_jobs;
  ctx->batch.last_team_jobs = p->ar.last_team_jobs;
  *out = p;
  return GME_OK;
}

gme_status gme_batch_plan_run(gme_batch_plan *p, const int32_t *d_symbols, const gme_scoring *sc,
                              gme_result *d_results, void *stream, int use_graph) {
  if (!p || (p->npairs > 0 && (!d_symbols || !d_results))) return GME_ERR_INVALID;
  gme_context *ctx = p->ctx;
  gme_scoring def = gme_default_scoring();
  if (!sc) sc = &def;
  if (sc->ed_boundary != GME_ED_REF_CPU && sc->ed_boundary != GME_ED_STANDARD) return GME_ERR_INVALID;
  const long long m = std::max<long long>(std::max<long long>(llabs(sc->match), llabs(sc->mismatch)), llabs(sc->gap));
  if (m * (p->max_len_sum + 2) >= (1ll << 30)) {
    ctx->ws.last_error = "SW scores could overflow int32";
    return GME_ERR_OVERFLOW;
  }
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  const gme::Scoring gs = to_scoring(sc);
  cudaError_t e;
  int rc;
  if (!use_graph) {
    int k = 0;
    rc = gme::batch_launch(ctx->ws, p->ar, d_symbols, gs, d_results, st, ctx->timeout_ns, &k);
    ctx->ws.launches += k;
    if (rc != ST_OK) return to_status(rc);
  } else {
    const bool same = p->exec && p->g_sym == d_symbols && p->g_res == d_results && p->g_st == st &&
                      memcmp(&p->g_sc, sc, sizeof(gme_scoring)) == 0;
    if (same) {
      if ((e = cudaGraphLaunch(p->exec, st)) != cudaSuccess) return to_status(ctx->ws.fail(e, "cudaGraphLaunch"));
      ctx->ws.launches += p->kernels;
    } else {
      if (p->exec) { cudaGraphExecDestroy(p->exec); p->exec = nullptr; }
      // this run executes uncaptured; the capture is for the next ones
      int k = 0;
      rc = gme::batch_launch(ctx->ws, p->ar, d_symbols, gs, d_results, st, ctx->timeout_ns, &k);
      ctx->ws.launches += k;
      if (rc != ST_OK) return to_status(rc);
      cudaGraph_t g = nullptr;
      if ((e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal)) != cudaSuccess)
        return to_status(ctx->ws.fail(e, "cudaStreamBeginCapture"));
      rc = gme::batch_launch(ctx->ws, p->ar, d_symbols, gs, d_results, st, ctx->timeout_ns, &k);
      e = cudaStreamEndCapture(st, &g);
      if (rc != ST_OK) { if (g) cudaGraphDestroy(g); return to_status(rc); }
      if (e != cudaSuccess) return to_status(ctx->ws.fail(e, "cudaStreamEndCapture"));
      e = cudaGraphInstantiate(&p->exec, g, 0);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) { p->exec = nullptr; return to_status(ctx->ws.fail(e, "cudaGraphInstantiate")); }
      p->kernels = k;
      p->g_sym = d_symbols; p->g_res = d_results; p->g_st = st; p->g_sc = *sc;
    }
  }
  struct { gme_context *ctx; const gme_scoring *sc; cudaStream_t st; } arg = {ctx, sc, st};
  return to_status(gme::batch_long(p->ar, d_symbols, d_results, nullptr, nullptr, batch_plain_cb, &arg));
}

gme_status gme_batch_plan_destroy(gme_batch_plan *p) {
  if (!p) return GME_ERR_INVALID;
  cudaSetDevice(p->ctx->device);
  cudaStreamSynchronize(p->ctx->stream);
  if (p->g_st) cudaStreamSynchronize(p->g_st);
  if (p->exec) cudaGraphExecDestroy(p->exec);
  p->ar.release();
  delete p;
  return GME_OK;
}

gme_status gme_batch_stats(const gme_context *ctx, int64_t *block_jobs, int64_t *warp_jobs,
                           int64_t *long_jobs, int64_t *team_jobs) {
  if (!ctx) return GME_ERR_INVALID;
  if (block_jobs) *block_jobs = ctx->batch.last_block_jobs;
  if (warp_jobs) *warp_jobs = ctx->batch.last_warp_jobs;
  if (long_jobs) *long_jobs = ctx->batch.last_long_jobs;
  if (team_jobs) *team_jobs = ctx->batch.last_team_jobs;
  return GME_OK;
}

gme_status gme_debug_wait_timeout(gme_context *ctx, uint64_t timeout_ns, int32_t *kernel_status) {
  if (!ctx || !kernel_status || timeout_ns == 0 || timeout_ns > 60ull * 1000 * 1000 * 1000)
    return GME_ERR_INVALID;
  cudaSetDevice(ctx->device);
  return to_status(gme::debug_wait_timeout(ctx->ws, timeout_ns, kernel_status, ctx->stream));
}

int64_t gme_launch_count(const gme_context *ctx) { return ctx ? ctx->ws.launches : -1; }

gme_status gme_baseline_align_device(gme_context *ctx, gme_baseline strategy, gme_kind kind, const int32_t *d_a,
                                     int64_t n1, const int32_t *d_b, int64_t n2, const gme_scoring *sc,
                                     int32_t *d_table, int32_t tile_x, int32_t tile_y, gme_result *d_out,
                                     void *stream) {
  if (!ctx || !d_a || !d_b || !d_table || !d_out || (strategy != GME_BASELINE_TILES && strategy != GME_BASELINE_CELLS))
    return GME_ERR_INVALID;
  gme_status s = check_sizes(ctx, kind, n1, n2, sc);
  if (s != GME_OK) return s;
  gme_scoring def = gme_default_scoring();
  if (!sc) sc = &def;
  cudaSetDevice(ctx->device);
  cudaStream_t st = stream ? (cudaStream_t)stream : ctx->stream;
  cudaStream_t prev = ctx->ws.sync_stream;
  ctx->ws.sync_stream = st;
  const int rc = gme::baseline_run(ctx->ws, (int)strategy, (int)kind, d_a, n1, d_b, n2, to_scoring(sc), d_table,
                                   tile_x, tile_y, d_out, st);
  ctx->ws.sync_stream = prev;
  return to_status(rc);
}

}  // extern "C"

namespace gme {

cudaStream_t ctx_stream(gme_context *ctx) { return ctx->stream; }

void ctx_set_served(gme_context *ctx, int *d_done) {
  ctx->batch.d_done = d_done;
  ctx->batch.sync_before_reuse = d_done == nullptr;
}

long long ctx_device_bytes(const gme_context *ctx) {
  const Workspace &w = ctx->ws;
  const BatchArena &b = ctx->batch;
  long long n = 4 * (w.a_pad_cap + w.b_pad_cap) + 8 * w.slots_cap + 32ll * w.best_cap + (w.ctrl ? 64 : 0);
  n += 4 * (b.staged_cap + b.rows_cap) + 32 * b.seg_cap + (long long)sizeof(BatchJob) * b.jobs_cap +
       8 * b.wrap_cap + (b.d_gen ? 4 * 1025 : 0) + (b.d_ctrl ? 64 : 0) + 16 * b.units_cap + b.team_cap;
  n += 4 * (ctx->d_a_cap + ctx->d_b_cap + ctx->d_row_cap + ctx->d_col_cap + ctx->d_bsym_cap) +
       (long long)sizeof(gme_result) * (ctx->d_bres_cap + 1);
  return n;
}

int ctx_sms(const gme_context *ctx) { return ctx->ws.sms; }
int ctx_device(const gme_context *ctx) { return ctx->device; }

int ctx_batch_status(gme_context *ctx) {
  int v = 0;
  if (!ctx->batch.d_ctrl) return 0;
  if (cudaMemcpy(&v, ctx->batch.d_ctrl + 8, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return ST_CUDA;
  return v;
}

}  // namespace gme
