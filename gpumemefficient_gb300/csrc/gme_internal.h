// gme_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <vector>

#include "gme.h"

#ifndef GME_PLAIN_CHUNK
#define GME_PLAIN_CHUNK 32
#endif

namespace gme {

struct Scoring;

// Device workspace owned by one context.  Grows on demand, never shrinks, and is
// reused across calls so that a steady stream of calls allocates nothing.
struct Workspace {
  int device = 0;
  int sms = 0;
  int *a_pad = nullptr;
  long long a_pad_cap = 0;
  int *b_pad = nullptr;
  long long b_pad_cap = 0;
  unsigned long long *slots = nullptr;  // tagged band-boundary rows
  long long slots_cap = 0;              // words
  size_t slots_bytes = 0;
  void *best = nullptr;                 // per-CTA SW maxima (32 bytes each)
  int best_cap = 0;
  int *ctrl = nullptr;                  // ticket, status, spare
  unsigned tag_next = 1;                // next unused band tag since slots were cleared
  long long launches = 0;               // kernels launched (counted by the host)
  std::string last_error;
  cudaStream_t sync_stream = nullptr;   // stream drained before a workspace is regrown

  int reserve(long long a_len, long long b_len, long long slot_words, int nbest);
  int fail(cudaError_t e, const char *what);
  int fail_msg(int status, const std::string &msg);
  void release();
};

// One job of a batch as the batched kernel reads it.
struct BatchJob {
  long long a_off;  // staged a: symbols at a_off + PADL + i
  long long b_off;  // staged b: symbols at b_off + i, padded to whole bands
  int n1, n2;
  int kind;
  int index;  // result slot
  int seg;    // staged segment of a (b is seg + 1): its symbols' range check
  long long row_off = -1;  // last row (n1 + 1 values) at last_rows + row_off, or none
  long long col_off = -1;  // last column (n2 + 1 values) at last_cols + col_off, or none
};

struct BatchTuning {
  int warps_per_block = 4;  // compute warps of a CTA (block jobs pipeline them over bands)
  int blocks_per_sm = 0;    // 0 = as many as fit
  long long block_min_cells = 1ll << 22;  // pairs at least this large (and with a band per warp) run one per CTA
  // pairs at least this large run on the plain path (many CTAs each); 0 = automatic:
  // max(2^27, 8 x the batch's cells / CTAs), i.e. only a pair that even a team of 8
  // CTAs would take longer on than an even share of the batch; < 0 = never
  long long long_min_cells = 0;
  // pairs at least this large (with 4+ band groups) run on a team of CTAs; < 0 = never
  long long team_min_cells = 1ll << 25;
  // a team job of G band groups runs on clamp(G / team_split, 2, 8) CTAs
  int team_split = 2;
  // pairs whose values fit 16 bits run on the packed 16-bit engine (rows_per_lane 4 only)
  bool packed16 = true;
  // rows per lane of the kernel: 4 (128-row bands) or 2 (64-row bands)
  int rows_per_lane = 4;
  // false: the plan takes warps, CTAs per SM and cut-offs from the tuned table
  // (gme_tuned.h) for the batch's length bucket
  bool user_set = false;
};

// Device and host buffers of the batched path, owned by a context, grown on demand.
struct BatchArena {
  std::vector<long long> h_from, h_to;
  std::vector<int> h_len, h_padl, h_total;
  std::vector<BatchJob> h_jobs;
  int *d_staged = nullptr; long long staged_cap = 0;
  long long *d_from = nullptr, *d_to = nullptr;
  int *d_len = nullptr, *d_padl = nullptr, *d_total = nullptr; long long seg_cap = 0;
  int *d_symbad = nullptr;  // per segment: 1 if a symbol lies outside [0, 32767] (written by staging)
  int packed16 = 0;         // the plan's choice of engine for jobs that fit 16 bits
  BatchJob *d_jobs = nullptr; long long jobs_cap = 0;
  int *d_ctrl = nullptr;
  int *d_rows = nullptr; long long rows_cap = 0;  // warp jobs' rows
  unsigned long long *d_wrap = nullptr; long long wrap_cap = 0;  // block jobs' tagged wrap rows
  unsigned *d_gen = nullptr;                                     // the tags they have used
  int stride = 0;                                                // row stride of the plan
  int *d_done = nullptr;  // completion flags (served path), or null
  std::vector<int4> h_units;                          // team members {job, t, T, 0}
  int4 *d_units = nullptr; long long units_cap = 0;
  char *d_team = nullptr; long long team_cap = 0;      // team slots, then their wrap rows
  long long team_bytes = 0;                           // the part of it the plan uses
  int n_t = 0;
  int ku[4] = {0, 0, 0, 0};
  long long last_team_jobs = 0;
  long long last_block_jobs = 0, last_warp_jobs = 0, last_long_jobs = 0;
  // the plan
  long long nseg = 0;
  int n_b = 0, n_w = 0, NW = 4, R = 4, grid = 0;
  int kb[4] = {0, 0, 0, 0}, kw[4] = {0, 0, 0, 0};  // per-kind offsets into the two queues
  std::vector<int> longj;             // result slots of pairs for the plain path
  std::vector<gme_pair> long_pairs;   // their descriptors
  std::vector<long long> long_rows, long_cols;  // their last-row / last-column offsets (-1: none)
  bool sync_before_reuse = true;      // wait for the stream before overwriting the plan
  int reserve(long long staged, long long nseg, long long njobs, Workspace &ws);
  int reserve_rows(long long ints, Workspace &ws);
  int reserve_wrap(long long words, Workspace &ws);
  int reserve_team(long long units, long long bytes, Workspace &ws);
  void release();
};

// columns per ring transaction (and per band-slot group) of the plain kernel
constexpr int PLAIN_C = GME_PLAIN_CHUNK;

// batched path (gme_batch.cu)
bool batch_config_valid(int NW, int R = 4);
int batch_occupancy(int NW, int R = 4);
constexpr int BATCH_MAX_N1 = 16384;  // widest pair the batch kernel takes (wider: plain path)
long long batch_pair_bytes(long long n1, long long n2);
long long batch_grid(int sms, int NW, int blocks_per_sm, int R = 4);
long long batch_scratch_bytes(long long grid, int NW, int max_n1);
// the tuned table's entry for a batch of pairs (given.user_set: `given` itself)
BatchTuning batch_tuning_for(const gme_pair *pairs, long long npairs, const BatchTuning &given);
// the served path's persistent kernel (gme_batch.cu, serve_kernel)
// The served kernel's ring words (ints).  Six job rings, a CTA ring and a warp ring
// per kind: the head of kind k's CTA ring at [2k], of its warp ring at [2k + 1], their
// tails at [RW_TAIL + 2k] and [RW_TAIL + 2k + 1]; the stop word, CTAs that have left,
// the exit word (raised once the kernel has been idle), the time of the last claim
// (64 bits, nanoseconds), the completion queue's count and, per pair of SMs, the kind
// it runs.
constexpr int RW_TAIL = 8, RW_STOP = 16, RW_EXITS = 17, RW_EXIT = 18, RW_LAST = 20, RW_CQN = 22, RW_PAIR = 64,
              RW_PAIRS = 128, RW_WORDS = RW_PAIR + RW_PAIRS;
struct ServeArgs {
  int *arena;                 // staged symbols of the jobs (offsets in BatchJob are into it)
  BatchJob *jobs_b, *jobs_w;  // the CTA rings (kind k at k * qb) and the warp rings (k * qw)
  int qb, qw;                 // slots of each ring
  int *symbad;                // per job segment: 1 if a symbol lies outside [0, 32767]
  gme_result *results;        // results and completion flags (mapped host memory)
  int *done;
  int *rows;                  // grid * NW rows of `stride` ints (warp jobs)
  unsigned long long *wrap;   // grid * 2 tagged rows of `stride` words (CTA jobs)
  unsigned *gen;              // wrap-row tags handed out (kept across launches)
  int stride;
  int *ctrl;                  // [8] status
  int *ring_ctl;              // RW_WORDS ring words
  const int4 *units;          // per CTA-ring slot: {team, tag0, the pair's entries (1: alone), 0}
  void *teams;                // serve_team_bytes() per team, cleared before each use
  unsigned long long *twrap;  // 2 tagged rows of `stride` words per team (tags below tag0)
  int *tfree;                 // per team, mapped host memory: 1 once its last entry has left
  int *cq;                    // completion queue (mapped host memory): result slot + 1 per job done
  int cq_mask;                // its entries - 1 (a power of 2); the count is ring word RW_CQN
  gme_scoring sc;
  unsigned long long timeout_ns, idle_ns;
  int NW, grid;
};
int serve_grid(int sms, int NW);
int serve_row_stride(int max_n1);
int serve_padl();                 // symbols before a's first one in its staged segment
long long serve_a_len(int n1);    // ints of a's staged segment (pads included, 16-byte multiple)
int serve_rows_mult(int NW, bool block);
long long serve_team_bytes();
cudaError_t serve_launch(const ServeArgs &a, cudaStream_t st);
// summed-area table (gme_sat.cu)
// comparison baselines (gme_baselines.cu): strategy 0 = tiles, 1 = cells
int baseline_run(Workspace &ws, int strategy, int kind, const int *d_a, long long n1, const int *d_b, long long n2,
                 const Scoring &sc, int *d_table, int TX, int TY, gme_result *d_out, cudaStream_t st);
int sat_run(Workspace &ws, int *d_table, long long n1, long long n2, long long ld, int *d_status,
            cudaStream_t st, unsigned long long timeout_ns);
long long sat_scratch_words(long long n1, long long n2);
int batch_plan(Workspace &ws, BatchArena &ar, const gme_pair *pairs, long long npairs,
               long long nsym, const BatchTuning &tune, cudaStream_t st,
               const long long *row_offs = nullptr, const long long *col_offs = nullptr);
int batch_launch(Workspace &ws, BatchArena &ar, const int *d_sym, const Scoring &sc,
                 gme_result *d_results, cudaStream_t st, unsigned long long timeout_ns, int *kernels,
                 int *d_last_rows = nullptr, int *d_last_cols = nullptr);
int batch_long(BatchArena &ar, const int *d_sym, gme_result *d_results, int *d_last_rows, int *d_last_cols,
               int (*plain)(void *, int, const int *, long long, const int *, long long, gme_result *, int *, int *),
               void *plain_ctx);
int batch_run(Workspace &ws, BatchArena &ar, const int *d_sym, long long nsym, const gme_pair *pairs,
              long long npairs, const Scoring &sc, gme_result *d_results, cudaStream_t st,
              const BatchTuning &tune, unsigned long long timeout_ns,
              int *d_last_rows, const long long *row_offs, int *d_last_cols, const long long *col_offs,
              int (*plain)(void *, int, const int *, long long, const int *, long long, gme_result *, int *, int *),
              void *plain_ctx);

// plain path (gme_plain.cu)
bool plain_config_valid(int R, int NW);
void plain_auto_config(int sms, long long n1, long long n2, int *R, int *NW, int *grid);
int plain_run(Workspace &ws, int kind, const int *d_a, long long n1, const int *d_b, long long n2,
              const Scoring &sc, gme_result *d_out, int *d_last_row, int *d_last_col,
              cudaStream_t st, int R, int NW, int grid, unsigned long long timeout_ns);
int debug_wait_timeout(Workspace &ws, unsigned long long timeout_ns, int *kernel_status,
                       cudaStream_t st);

// internals of a context the served path drives (gme_api.cu)
cudaStream_t ctx_stream(gme_context *ctx);
// completion flags for the context's batches (null: none); its batches then trust
// the caller to reuse the arena only after the previous batch has finished
void ctx_set_served(gme_context *ctx, int *d_done);
long long ctx_device_bytes(const gme_context *ctx);
int ctx_sms(const gme_context *ctx);
int ctx_device(const gme_context *ctx);
// the status word of the context's last batch kernel (read after it has finished)
int ctx_batch_status(gme_context *ctx);

}  // namespace gme
