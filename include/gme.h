/*
 * gme.h -- C ABI of the GB300 wavefront alignment library (libgme.so).
 *
 * Three integer dynamic programs over two integer-coded sequences, exactly as
 * the reference computes them:
 *   LCS  t = a==b ? diag+1 : max(left, up)                 LCS/LCS.cpp:59-63
 *   ED   t = a==b ? diag : min(up,left,diag)+1             EditDistance/ED.cpp:63-65
 *   SW   t = max(left+gap, up+gap, diag+(a==b?match:mismatch), 0)
 *                                                          SmithWaterman/SW.cpp:45-47,63-65
 * Table convention (the reference's GPU host functions, e.g.
 * EditDistance/GPU_Hyperlane_Share.cu:696-697): columns x = 0..n1 run over
 * `a` (arr1), rows y = 0..n2 run over `b` (arr2), cell (y,x) compares
 * a[x-1] with b[y-1].  The returned score is the bottom-right cell (y=n2,
 * x=n1), which is what every reference host function returns.
 *
 * Plain pointers and sizes only; no C++ or CUDA types appear in signatures
 * (streams are passed as void* holding a cudaStream_t).  Every function returns
 * a gme_status; nothing in this library calls exit() (the reference's
 * checkGPUError does, EditDistance/GPU_Hyperlane_Share.cu:682-687).
 *
 * The reference's own C++ signatures (int ED(int,int,int*,int*,int,int,int*,int,int)
 * and friends) are provided on top of this ABI by gme_reference.h.
 */
#ifndef GME_H
#define GME_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum gme_status {
  GME_OK = 0,
  GME_ERR_INVALID = 1,   /* bad argument (null pointer, negative size, bad kind) */
  GME_ERR_CUDA = 2,      /* a CUDA runtime call failed; see gme_last_error() */
  GME_ERR_NOMEM = 3,     /* device or pinned allocation failed */
  GME_ERR_TIMEOUT = 4,   /* a bounded device-side wait expired; results invalid */
  GME_ERR_OVERFLOW = 5,  /* sizes whose scores could overflow int32 */
  GME_ERR_BUDGET = 6,    /* served path: request larger than the HBM budget */
  GME_ERR_NOT_READY = 7, /* served path: ticket still in flight */
  GME_ERR_CLOSED = 8     /* served path: server shut down */
} gme_status;

typedef enum gme_kind { GME_LCS = 0, GME_ED = 1, GME_SW = 2 } gme_kind;

/* Edit-distance boundary (row 0 / column 0) convention. */
typedef enum gme_ed_boundary {
  /* EditDistance/ED.cpp:48-54 (the CPU oracle): row 0 = [0,0,1,2,...,n1-1],
   * column 0 = [0,1,...,n2]. */
  GME_ED_REF_CPU = 0,
  /* GPU_setInit, EditDistance/GPU_Hyperlane_Share.cu:16-22: row 0 = [0,1,...,n1],
   * column 0 = [0,1,...,n2] (textbook Levenshtein). */
  GME_ED_STANDARD = 1
} gme_ed_boundary;

/* Scoring constants.  A zeroed struct is NOT valid for SW; use gme_default_scoring(). */
typedef struct gme_scoring {
  int32_t match;       /* SW: added on a[x-1]==b[y-1]          (SW.cpp:46: +3) */
  int32_t mismatch;    /* SW: added otherwise                  (SW.cpp:46: -3) */
  int32_t gap;         /* SW: added to left and up             (SW.cpp:63-64: -2) */
  int32_t ed_boundary; /* ED: a gme_ed_boundary value */
} gme_scoring;

typedef struct gme_result {
  int32_t score;    /* bottom-right cell (all kinds) */
  int32_t sw_max;   /* SW: largest cell; 0 when no cell is positive */
  int64_t sw_max_y; /* SW: its row (1-based, over b); first maximum in row-major order; 0 if none */
  int64_t sw_max_x; /* SW: its column (1-based, over a) */
  int32_t status;   /* device-side status of the computation (a gme_status) */
  int32_t kind;     /* echo of the kind computed */
} gme_result;

/* Tuning of the plain (one pair per call) wavefront kernel. Zero fields = automatic. */
typedef struct gme_plain_config {
  int32_t rows_per_lane;   /* cells of one anti-diagonal held per thread: 2 or 4 */
  int32_t warps_per_band;  /* compute warps per CTA, 4 or 8; band height = warps*32*rows_per_lane */
  int32_t grid;            /* persistent CTAs (0 = one per band, capped by residency) */
  int32_t reserved;
} gme_plain_config;

typedef struct gme_context gme_context;

/* ---- context ---------------------------------------------------------------- */
/* A context owns a device, a workspace that grows on demand and is reused across
 * calls, and host staging buffers.  One context must not be used by two host
 * threads at once; separate contexts are independent. */
gme_status gme_create(int device, gme_context **ctx);
gme_status gme_destroy(gme_context *ctx);
const char *gme_status_string(gme_status s);
/* Text of the last error recorded on this context (never NULL). */
const char *gme_last_error(const gme_context *ctx);
gme_scoring gme_default_scoring(void);
/* Upper bound, in nanoseconds, of every device-side spin-wait (default 10 s). */
gme_status gme_set_wait_timeout_ns(gme_context *ctx, uint64_t ns);
gme_status gme_set_plain_config(gme_context *ctx, const gme_plain_config *cfg);
gme_status gme_get_plain_config(const gme_context *ctx, int64_t n1, int64_t n2,
                                gme_plain_config *resolved);

/* ---- plain path: one alignment per call ------------------------------------- */
/* Host buffers in and out (the reference host functions' contract: they take
 * host arrays and return the last cell, e.g. EditDistance/GPU_Hyperlane_Share.cu:689).
 * last_row (n1+1 values, row y=n2) and last_col (n2+1 values, column x=n1)
 * are optional (NULL).  Blocks until done. */
gme_status gme_align(gme_context *ctx, gme_kind kind, const int32_t *a, int64_t n1,
                     const int32_t *b, int64_t n2, const gme_scoring *sc, gme_result *out,
                     int32_t *last_row, int32_t *last_col);

/* Device buffers in and out, asynchronous on `stream`.  d_out is a device
 * gme_result; its `status` field reports a device-side timeout. */
gme_status gme_align_device(gme_context *ctx, gme_kind kind, const int32_t *d_a, int64_t n1,
                            const int32_t *d_b, int64_t n2, const gme_scoring *sc,
                            gme_result *d_out, int32_t *d_last_row, int32_t *d_last_col,
                            void *stream);

/* ---- batched path: many alignments in one launch --------------------------------
 * Pair i reads a = symbols[a_off .. a_off+n1), b = symbols[b_off .. b_off+n2) and
 * computes `kind` with the shared scoring; result i gets its score (and SW maximum).
 * One persistent work-queue kernel runs every pair whose n1 <= 16384, kinds one
 * after another and within a kind longest first: pairs of at least team_min_cells
 * cells on a team of 2..8 CTAs (each CTA takes every T-th group of row bands),
 * pairs of at least block_min_cells cells (and at least one band of 128 rows per
 * warp) one per CTA (the CTA's warps pipelined over the pair's bands), all others
 * one per warp.  Wider, empty or very large (see long_min_cells) pairs run on the
 * plain path, one launch each, on the same stream.  Replaces calling the
 * reference's one-pair host function (e.g. EditDistance/GPU_Hyperlane_Share.cu:689)
 * once per pair. */
typedef struct gme_pair {
  int64_t a_off, b_off; /* element offsets into the symbol buffer */
  int32_t n1, n2;       /* lengths of a (columns) and b (rows) */
  int32_t kind;         /* gme_kind */
  int32_t reserved;
} gme_pair;

typedef struct gme_batch_config {
  int32_t warps_per_block; /* 4 or 8 (0 = automatic) */
  int32_t blocks_per_sm;   /* CTAs per SM (0 = as many as fit) */
  int64_t block_min_cells; /* pairs with n1*n2 >= this run one per CTA (0 = 2^22) */
  int64_t long_min_cells;  /* pairs with n1*n2 >= this run on the plain path, many CTAs
                            * each (0 = automatic: max(2^27, 8 x the batch's cells / CTAs),
                            * so only a pair that even a team of 8 CTAs would take longer
                            * on than an even share of the batch; -1 = never) */
  int64_t team_min_cells;  /* pairs with n1*n2 >= this (and 4+ groups of bands) run on a
                            * team of CTAs (0 = 2^25; -1 = never) */
  int32_t packed16;        /* 0 or 1: pairs whose scores provably fit 16 bits (and whose
                            * symbols lie in [0, 32767]) run two cells per register on s16x2
                            * DPX (the default); -1: int32 for every pair */
  int32_t team_split;      /* groups of bands per team member: a team job of G groups runs
                            * on clamp(G / team_split, 2, 8) CTAs (0 = 2) */
  int32_t rows_per_lane;   /* rows of a band per lane: 4 (128-row bands; the default) or 2
                            * (64-row bands: more bands, shorter per-step chains; only
                            * with 8 warps per block); the packed 16-bit engine runs
                            * only at 4 */
} gme_batch_config;

gme_status gme_set_batch_config(gme_context *ctx, const gme_batch_config *cfg);
/* The settings a batch of these pairs is planned with when no configuration was set:
 * the entry of the autotuned table whose length range (2nd..98th percentile of
 * sqrt(n1*n2)) is nearest the batch's, in log scale.  Host only, needs no GPU.
 * long_min_cells is 0 (automatic); packed16 is 0 (on) or -1 (off), as the entry says. */
gme_status gme_batch_tuned_config(const gme_pair *pairs, int64_t n, gme_batch_config *out);
/* Host buffers; blocks until all results are in `results`. */
gme_status gme_align_batch(gme_context *ctx, const int32_t *symbols, int64_t nsym,
                           const gme_pair *pairs, int64_t npairs, const gme_scoring *sc,
                           gme_result *results);
/* Device symbols and results, host pair list (the plan is made on the host).
 * Returns once the work is queued on `stream`. */
gme_status gme_align_batch_device(gme_context *ctx, const int32_t *d_symbols, int64_t nsym,
                                  const gme_pair *pairs, int64_t npairs, const gme_scoring *sc,
                                  gme_result *d_results, void *stream);
/* As gme_align_batch_device, and each pair's boundary as well: pair i's last row
 * (row n2, n1+1 values) at d_last_rows + row_offsets[i] and its last column (column
 * n1, n2+1 values) at d_last_cols + col_offsets[i], as the plain path returns them.
 * An offset of -1 skips that pair; either buffer may be NULL (then its offsets are
 * not read).  Offsets are element offsets in host arrays of npairs entries. */
gme_status gme_align_batch_device_rows(gme_context *ctx, const int32_t *d_symbols, int64_t nsym,
                                       const gme_pair *pairs, int64_t npairs, const gme_scoring *sc,
                                       gme_result *d_results, int32_t *d_last_rows,
                                       const int64_t *row_offsets, int32_t *d_last_cols,
                                       const int64_t *col_offsets, void *stream);
/* A reusable plan for a fixed pair list: classification, ordering, staged layout
 * and descriptors are made once; each run only clears the tickets, stages the
 * symbols and launches the work-queue kernel.  With use_graph != 0 the first run
 * also captures that launch sequence into a CUDA graph, and later runs with the
 * same symbol/result pointers, stream and scoring replay the graph (one launch
 * from the host).  Pairs the batch hands to the plain path run outside the graph.
 * A plan belongs to its context's thread; runs of one plan must not overlap. */
typedef struct gme_batch_plan gme_batch_plan;
gme_status gme_batch_plan_create(gme_context *ctx, const gme_pair *pairs, int64_t npairs,
                                 int64_t nsym, gme_batch_plan **plan);
gme_status gme_batch_plan_run(gme_batch_plan *plan, const int32_t *d_symbols,
                              const gme_scoring *sc, gme_result *d_results, void *stream,
                              int use_graph);
gme_status gme_batch_plan_destroy(gme_batch_plan *plan);

/* How the last batch (or last plan made) was split: one-per-CTA, one-per-warp,
 * plain-path and team pairs (any pointer may be NULL). */
gme_status gme_batch_stats(const gme_context *ctx, int64_t *block_jobs, int64_t *warp_jobs,
                           int64_t *long_jobs, int64_t *team_jobs);

/* ---- served path: requests one at a time, each result as soon as it is done ----
 * A server owns a host request queue and a dispatcher thread.  gme_submit copies a
 * request into the queue and returns a ticket at once.  Two modes:
 *   GME_SERVE_RING (the default): one persistent kernel stays resident on the GPU and
 *     takes jobs from two device-resident rings (pairs of 2^22 cells and more, one per
 *     CTA; the rest, one per warp).  The dispatcher admits queued requests in arrival
 *     order while the symbol arena (the budget less the kernel's fixed rows) and the
 *     rings have room, copies their padded symbols and descriptors in, then publishes
 *     each ring's new tail; the kernel picks jobs up as they are published.  Each
 *     result and then its completion flag are written into pinned host memory, so a
 *     request completes when its own pair is done.  The kernel leaves after a short
 *     idle time and is launched again when work arrives.  Pairs wider than 16384 (the
 *     kernel's row width) run as launches of the batched kernel, as in the other mode.
 *   GME_SERVE_WAVES: admitted requests form waves; each wave is one launch of the
 *     batched work-queue kernel on one of `waves` launch slots (separate streams), up
 *     to wave_max_cells cells and the slot's share of the budget.
 * No counterpart in the reference, whose host functions align one pair per call
 * (EditDistance/GPU_Hyperlane_Share.cu:689-789). */
typedef enum gme_serve_mode { GME_SERVE_RING = 0, GME_SERVE_WAVES = 1 } gme_serve_mode;
typedef struct gme_server gme_server;
typedef struct gme_server_config {
  int64_t hbm_budget_bytes; /* device memory the server may hold in all (0 = 20 GiB) */
  int64_t wave_max_cells;   /* cells per launch at most (0 = 2^35) */
  int32_t waves;            /* launch slots = launches in flight at once (0 = 4) */
  int32_t queue_max;        /* requests the host queue holds (0 = 2^20) */
  int32_t warps_per_block;  /* kernel CTA shape, 4 or 8 (0 = automatic: 4 in ring mode) */
  int32_t mode;             /* a gme_serve_mode (0 = GME_SERVE_RING) */
} gme_server_config;

typedef struct gme_server_stats {
  int64_t submitted, completed; /* requests */
  int64_t queued, running;      /* waiting on the host; admitted to a launch */
  int64_t waves_launched;       /* waves mode: launches of the batched kernel sequence;
                                 * ring mode: launches of the persistent kernel */
  int64_t kernels_launched;     /* CUDA kernels, all slots */
  int64_t cells_completed;      /* sum of n1*n2 over completed requests */
  int64_t hbm_bytes_held;       /* device memory held by the server now */
  int64_t hbm_bytes_peak;       /* ... and at most so far */
  int64_t hbm_budget_bytes;
  int64_t h2d_bytes;            /* symbols and descriptors copied to the device */
  int64_t d2h_bytes;            /* results and flags the device wrote to host memory */
} gme_server_stats;

/* One scoring for every request of the server (as for a batch). */
gme_status gme_server_create(int device, const gme_server_config *cfg, const gme_scoring *sc,
                             gme_server **out);
/* Stops admitting, lets the launches in flight finish, completes what is still
 * queued with status GME_ERR_CLOSED, joins the dispatcher and frees everything. */
gme_status gme_server_destroy(gme_server *s);
/* Queues one alignment; a and b are copied, so they may be reused at once.  Never
 * waits for the GPU.  GME_ERR_BUDGET: the request alone needs more device memory
 * than one slot's share of the budget.  GME_ERR_NOT_READY: the queue is full. */
gme_status gme_submit(gme_server *s, gme_kind kind, const int32_t *a, int64_t n1, const int32_t *b,
                      int64_t n2, uint64_t *ticket);
/* Queues n alignments in one call: request i reads symbols as batch pair i does
 * (kind, a_off/n1, b_off/n2) and gets its own ticket tickets[i].  The same errors
 * as gme_submit; on one, the requests before it stay queued and *submitted says
 * how many there are. */
gme_status gme_submit_many(gme_server *s, const int32_t *symbols, const gme_pair *pairs, int64_t n,
                           uint64_t *tickets, int64_t *submitted);
/* GME_OK with *out (and *latency_ns, submission to completion; may be NULL) once
 * the request is done; the ticket is then forgotten.  GME_ERR_NOT_READY while it
 * is queued or running; GME_ERR_INVALID for a ticket never issued or already
 * taken.  out->status carries the request's own status. */
gme_status gme_poll(gme_server *s, uint64_t ticket, gme_result *out, int64_t *latency_ns);
/* Takes up to `max` finished requests in completion order.  results and
 * latency_ns may be NULL; *count gets the number taken. */
gme_status gme_poll_many(gme_server *s, uint64_t *tickets, gme_result *results,
                         int64_t *latency_ns, int64_t max, int64_t *count);
/* Blocks until every request submitted so far has completed; GME_ERR_NOT_READY
 * if timeout_ns passes first. */
gme_status gme_server_drain(gme_server *s, uint64_t timeout_ns);
gme_status gme_server_get_stats(const gme_server *s, gme_server_stats *out);
/* Text of the last error the server met (never NULL). */
const char *gme_server_last_error(const gme_server *s);

/* ---- alignment paths -------------------------------------------------------------
 * An optimal global alignment as an edit script, in memory linear in n1 + n2
 * (Hirschberg: the plain kernel's exported last rows of a forward and a backward
 * half-problem split it at the middle row; small subproblems are solved whole on
 * the GPU).  ops[k]: 'M' aligns a[i] with b[j] (LCS: only where equal), 'D' takes
 * a[i] against a gap, 'I' takes b[j] against a gap.  LCS maximises the number of
 * 'M'; ED uses the standard border (row 0 = 0, 1, 2, ...; sc may be NULL or must say
 * GME_ED_STANDARD) and minimises insertions, deletions and mismatches.  SW is not
 * supported (GME_ERR_INVALID).  *n_ops gets the script length (at most n1 + n2) and
 * *score the optimal score; with ops NULL only those are returned; GME_ERR_INVALID
 * if ops_cap is too small.  No counterpart in the reference, which returns scores
 * only (its boundary rows are what make the traceback possible). */
gme_status gme_align_path(gme_context *ctx, gme_kind kind, const int32_t *a, int64_t n1,
                          const int32_t *b, int64_t n2, const gme_scoring *sc, char *ops,
                          int64_t ops_cap, int64_t *n_ops, int32_t *score);

/* ---- summed-area table (SAT/GPU_Hyperlane_Share.cu) -----------------------------
 * In place on an int32 table of rows 0..n2 with row stride ld (>= n1 + 1; the
 * reference's layout has ld = n1 + 3): every cell of rows 1..n2 and columns 1..n1
 * becomes t[y][x-1] + t[y-1][x] + t[y][x] - t[y-1][x-1] (the reference's recurrence,
 * SAT/GPU_Hyperlane_Share.cu:169,196,231), evaluated row after row, left to right,
 * in wrapping 32-bit arithmetic; row 0 and column 0 keep their values, columns
 * beyond n1 are not touched.  One launch over column strips, rows handed from strip
 * to strip as tagged words with bounded waits.
 * gme_sat_device: device table, asynchronous on `stream`; d_status (may be NULL)
 * receives 0 or GME_ERR_TIMEOUT when the kernel has run.  gme_sat: host table (rows
 * 0..n2 copied in and rows 1..n2 back), blocking.  Replaces the reference's
 * SOR(n1, n2, table, tX, tY) (SAT/GPU_Hyperlane_Share.h:5), which computes the same
 * table on the device but never copies it back.
 * A context's SAT and plain-path calls share one tagged scratch buffer and one
 * control block: calls of one context queued on different streams must be
 * serialised by the caller (an event, or one stream for all of them). */
gme_status gme_sat_device(gme_context *ctx, int32_t *d_table, int64_t n1, int64_t n2, int64_t ld,
                          int32_t *d_status, void *stream);
gme_status gme_sat(gme_context *ctx, int32_t *table, int64_t n1, int64_t n2, int64_t ld);

/* ---- plain path without allocation --------------------------------------------
 * No counterpart in the reference.  For callers that cannot call cudaMalloc (code
 * running inside another runtime's memory pool, a plugin that must not allocate on
 * its hot path, a loop whose allocator is fenced off): the same computation as
 * gme_align_device, with every byte of scratch taken from one static device array
 * of about 4.4 MB that each GPU loading the library holds until exit.  Needs no
 * context and allocates nothing; runs on the calling thread's current device,
 * asynchronously on `stream`.
 *   - Sequences longer than GME_NOALLOC_MAX_LEN are rejected with GME_ERR_INVALID.
 *   - The first call on a device resolves the array's device address
 *     (cudaGetSymbolAddress); make that first call before any stream capture.
 *   - All calls on a device share the array: calls that overlap on the GPU (other
 *     streams, other host threads) race and must be serialised by the caller. */
#define GME_NOALLOC_MAX_LEN 8192
gme_status gme_align_device_noalloc(gme_kind kind, const int32_t *d_a, int64_t n1,
                                    const int32_t *d_b, int64_t n2, const gme_scoring *sc,
                                    gme_result *d_out, int32_t *d_last_row, int32_t *d_last_col,
                                    void *stream);

/* ---- diagnostics ------------------------------------------------------------- */
/* Runs the bounded device wait on a flag that nothing sets and reports what the
 * kernel returned (expected GME_ERR_TIMEOUT after `timeout_ns`).  Tests use it to
 * show a wait that runs out ends with a status, not a hang. */
gme_status gme_debug_wait_timeout(gme_context *ctx, uint64_t timeout_ns, int32_t *kernel_status);

/* ---- Comparison baselines (not the product path) ----
 * The reference's table-based strategies for the same recurrences, on this GPU, so
 * that the plain path can be timed beside them.  d_table is the caller's
 * (n2 + 1) x (n1 + 1) int32 table in device memory, written whole; d_out receives the
 * bottom-right cell and, for SW, the first maximum in row-major order.  Needs
 * 1 <= n1, n2 and (n1 + 1)(n2 + 1) < 2^32.
 *   GME_BASELINE_TILES: tiles of tile_y x tile_x cells, one launch per anti-diagonal of
 *     tiles, each swept in shared memory (LCS/GPU_TILE_SHARE.cu:12-207; the reference
 *     uses 128 x 64);
 *   GME_BASELINE_CELLS: one launch per anti-diagonal of cells, a thread per cell
 *     (EditDistance/GPU.cu:20-60); tile_x and tile_y are not read. */
typedef enum gme_baseline { GME_BASELINE_TILES = 0, GME_BASELINE_CELLS = 1 } gme_baseline;
gme_status gme_baseline_align_device(gme_context *ctx, gme_baseline strategy, gme_kind kind, const int32_t *d_a,
                                     int64_t n1, const int32_t *d_b, int64_t n2, const gme_scoring *sc,
                                     int32_t *d_table, int32_t tile_x, int32_t tile_y, gme_result *d_out,
                                     void *stream);
/* Number of kernels this context launched since creation (the bench counts them). */
int64_t gme_launch_count(const gme_context *ctx);

#ifdef __cplusplus
}
#endif

#endif /* GME_H */
