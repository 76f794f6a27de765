// gme_batch.cu -- many alignments of uneven lengths and mixed kinds in one launch.
//
// One persistent work-queue kernel.  Its CTAs first take "block jobs" (a whole
// pair per CTA: the CTA's NW warps are pipelined over the pair's row bands, band
// b on warp b % NW, handing rows through shared rings; the last warp's row wraps
// back to warp 0 for the next group of bands through a double-buffered row in
// shared memory).  When the block queue is empty every warp takes "warp jobs"
// on its own (a small pair swept band after band by one warp, its row kept in a
// per-warp shared buffer).  Jobs are ordered longest first.  Pairs too wide for
// the shared rows go to the plain path (one multi-CTA launch each, on the same
// stream).  The cell engine is the plain kernel's (gme_engine.cuh), so results
// are bit-exact with it and with the oracle.
//
// Replaces, for many pairs at once, the reference's one-pair-per-call host
// functions (EditDistance/GPU_Hyperlane_Share.cu:689-789 and its LCS/SW twins).
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "gme_batch_kernel.cuh"
#include "gme_tuned.h"

namespace gme {

// Claims the next job of a ring, if the host has published one: its ticket, or -1.
// The tail is read with acquire semantics, so the job's descriptor and symbols
// (copied in before the tail was published) are seen by the loads that follow.
__device__ __forceinline__ int ring_claim(int *ctl, int k, int c) {
  int *head = &ctl[2 * k + c];
  int h = ld_relaxed_gpu_s32(head);
  const int t = ld_acquire_gpu_s32(&ctl[RW_TAIL + 2 * k + c]);
  while (h < t) {
    const int got = atomicCAS(head, h, h + 1);
    if (got == h) return h;
    h = got;
  }
  return -1;
}

// Jobs waiting in kind k's CTA ring (c = 0) or warp ring (c = 1), as last seen.
__device__ __forceinline__ int ring_backlog(const int *ctl, int k, int c) {
  return ld_relaxed_gpu_s32(&ctl[RW_TAIL + 2 * k + c]) - ld_relaxed_gpu_s32(&ctl[2 * k + c]);
}

// The kind a pair of SMs runs (its word *pk): the current one while any job of it is
// waiting, else the kind with the most work waiting (a CTA job counted as 64 warp
// jobs), written back for the pair's other CTAs; -1 when every ring is empty.  One
// kind per pair of SMs at a time because the three kinds' loops do not fit the
// instruction cache the two SMs share (the batch kernel's measurement).
__device__ int pick_kind(const int *ctl, int *pk) {
  const int k0 = ld_relaxed_gpu_s32(pk);
  if (ring_backlog(ctl, k0, 0) > 0 || ring_backlog(ctl, k0, 1) > 0) return k0;
  int best = -1;
  long long bw = 0;
  for (int k = 0; k < 3; ++k) {
    const long long w = 64ll * ring_backlog(ctl, k, 0) + ring_backlog(ctl, k, 1);
    if (w > bw) { bw = w; best = k; }
  }
  if (best >= 0 && best != k0) atomicCAS(pk, k0, best);
  return best;
}

// One entry of a served team (ServeTeam): band groups of the pair, claimed one at a
// time, each swept by the CTA's warps as a block job's group is.  Group g's wrap row
// carries tag tag0 + g + 1; the host hands each use of a team a tag0 above every tag
// its rows hold, so they need no clearing between uses.
template <int KIND, int R, int NW>
__device__ void team_work(const BatchParams &P, BatchSmem<NW> &S, const BatchJob &jb, int warp, int lane,
                          Waiter &W, ServeTeam *tm, unsigned long long *wrap, unsigned tag0, int *freed,
                          int entries) {
  const int N = jb.n1, M = jb.n2;
  const int *a_sym = P.sym + jb.a_off;
  const int *b_sym = P.sym + jb.b_off;
  const int nb = (M + 32 * R - 1) / (32 * R);
  const int G = (nb + NW - 1) / NW;
  const bool p16 = R == 4 && job_p16(P, jb);
  for (;;) {
    if (threadIdx.x == 0) S.phase = *(volatile int *)&S.abort ? G : atomicAdd(&tm->next, 1);
    for (int i = threadIdx.x; i < NW * (RING / CB); i += blockDim.x) (&S.tag[0][0])[i] = 0;
    for (int i = threadIdx.x; i < NW; i += blockDim.x) S.cons[i] = 0;
    __syncthreads();
    const int g = S.phase;
    if (g >= G) break;
    const int band = g * NW + warp;
    SwBest tb = {0, 0, 0, 0};
    if (band < nb) {
      Src in;
      in.rule = P.sc.ed_rule;
      if (band == 0) {
        in.mode = IN_TOP;
      } else if (warp == 0) {
        in.mode = IN_ROW; in.row = wrap + ((g - 1) & 1) * P.stride; in.tag = tag0 + g;
      } else {
        in.mode = IN_RING; in.buf = S.ring[warp]; in.tags = S.tag[warp]; in.cons = &S.cons[warp]; in.base = 0;
      }
      Dst out;
      out.cons_seen = 0;
      if (band == nb - 1) {
        last_row_dst<KIND>(P, jb, out);
      } else if (warp == NW - 1) {
        out.mode = OUT_ROW; out.row = wrap + (g & 1) * P.stride; out.tag = tag0 + g + 1;
      } else {
        out.mode = OUT_RING; out.buf = S.ring[warp + 1]; out.tags = S.tag[warp + 1];
        out.cons = &S.cons[warp + 1]; out.base = 0;
      }
      int c = 0;
      sweep_job_band<KIND, R>(p16, P.sc, a_sym, b_sym, N, M, band * 32 * R, lane, in, out, W, c, tb,
                              col_dst<KIND>(P, jb, band, lane));
      if (band == nb - 1 && lane == 31) {
        *(volatile int *)&tm->corner = c;
        __threadfence();
      }
    }
    if (KIND == K_SW) {
      tb = warp_best(tb);
      if (lane == 0) S.best[warp] = tb;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      if (KIND == K_SW) {
        SwBest b = {0, 0, 0, 0};
        for (int k = 0; k < NW; ++k)
          if (better(S.best[k], b)) b = S.best[k];
        if (b.v > 0)
          atomicMax(&tm->best, ((unsigned long long)(unsigned)b.v << 32) |
                                   (0xffffffffu - (unsigned)(b.y * (N + 1) + b.x)));
      }
      __threadfence();
      if (atomicAdd(&tm->gdone, 1) == G - 1) {
        __threadfence();
        gme_result r;
        r.score = Rec<KIND>::to_v(*(volatile int *)&tm->corner, N, M);
        const unsigned long long k = KIND == K_SW ? atomicAdd(&tm->best, 0ull) : 0ull;
        r.sw_max = (int)(k >> 32);
        const long long lin = r.sw_max ? (long long)(0xffffffffu - (unsigned)k) : 0;
        r.sw_max_y = r.sw_max ? lin / (N + 1) : 0;
        r.sw_max_x = r.sw_max ? lin % (N + 1) : 0;
        r.status = job_status(P, S.abort);
        r.kind = KIND;
        put_result(P, jb.index, r);
      }
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&tm->left, 1) == entries - 1) {
      __threadfence_system();
      *(volatile int *)freed = 1;
    }
  }
}

// The served path's persistent kernel.  Launched once and left running while work
// arrives.  Jobs wait in six rings, a CTA ring (large pairs, the CTA's warps pipelined
// over the pair's bands, as block jobs of the batch kernel; the largest shared by a
// team of CTAs, ServeTeam) and a warp ring (small pairs, one per warp) per kind.  A CTA takes the next job of its SM pair's kind's CTA
// ring; when there is none, its warps take jobs of that kind's warp ring one after
// another, each on its own, and regroup once a CTA job of the kind is waiting and a
// slice of SLICE_NS has passed, or once no warp job is left.  The host appends jobs and
// publishes each ring's tail; results and completion flags go to mapped host memory as
// the batch kernel writes them.
// The kernel leaves as a whole: when the host sets the stop word, when a bounded wait
// anywhere has given up (the status word), or when no CTA has found a job for idle_ns
// (the time of the last claim; the first CTA to see it expire raises the exit word and
// no CTA claims a job after that).  The host launches the kernel again when it has
// work and the last launch has ended.
#ifndef GME_SERVE_SLICE_NS
#define GME_SERVE_SLICE_NS 4000000ull
#endif
constexpr unsigned long long SLICE_NS = GME_SERVE_SLICE_NS;

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32, NW == 4 ? GME_BATCH_MIN_BLOCKS : 1) serve_kernel(BatchParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BatchSmem<NW> &S = *reinterpret_cast<BatchSmem<NW> *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int *ctl = P.ring_ctl;
  unsigned long long *last = reinterpret_cast<unsigned long long *>(ctl + RW_LAST);
  unsigned smid;
  asm("mov.u32 %0, %%smid;" : "=r"(smid));
  int *pk = ctl + RW_PAIR + (int)((smid >> 1) % (unsigned)RW_PAIRS);
  if (threadIdx.x == 0) {
    S.abort = 0;
    atomicMax(last, globaltimer_ns());
  }
  __syncthreads();
  Waiter W(P.timeout_ns, &P.ctrl[8], &S.abort);
  auto stopping = [&]() {
    return *(volatile int *)&S.abort || ld_relaxed_gpu_s32(&ctl[RW_STOP]) != 0 ||
           ld_relaxed_gpu_s32(&ctl[RW_EXIT]) != 0 || ld_relaxed_gpu_s32(&P.ctrl[8]) != 0;
  };
  for (;;) {
    if (threadIdx.x == 0) {
      int job = -2;
      if (!stopping()) {
        const int k = pick_kind(ctl, pk);
        const int t = k >= 0 ? ring_claim(ctl, k, 0) : -1;
        const unsigned long long now = globaltimer_ns();
        if (t >= 0) {
          atomicMax(last, now);
          job = k * P.qb + t % P.qb;
          // a pair on this CTA alone: tags for its wrap rows, one per band group, never
          // used before
          if (P.units[job].z == 1) {
            const int n2 = P.jobs_b[job].n2;
            S.gen = atomicAdd(P.gen, (unsigned)((n2 + 32 * R * NW - 1) / (32 * R * NW)));
          }
        } else if (k < 0 && now > ld_relaxed_gpu_u64(last) + P.idle_ns) {
          atomicExch(&ctl[RW_EXIT], 1);
        } else {
          job = -1;
        }
      }
      S.job = job;
    }
    for (int i = threadIdx.x; i < NW * (RING / CB); i += blockDim.x) (&S.tag[0][0])[i] = 0;
    for (int i = threadIdx.x; i < NW; i += blockDim.x) S.cons[i] = 0;
    __syncthreads();
    const int job = S.job;
    if (job == -2) break;
    if (job >= 0) {
      const BatchJob jb = P.jobs_b[job];
      const int4 u = P.units[job];
      if (u.z > 1) {
        ServeTeam *tm = P.steam + u.x;
        unsigned long long *tw = P.twrap + (long long)u.x * 2 * P.stride;
        int *fr = P.tfree + u.x;
        switch (jb.kind) {
          case K_LCS: team_work<K_LCS, R, NW>(P, S, jb, warp, lane, W, tm, tw, (unsigned)u.y, fr, u.z); break;
          case K_ED: team_work<K_ED, R, NW>(P, S, jb, warp, lane, W, tm, tw, (unsigned)u.y, fr, u.z); break;
          default: team_work<K_SW, R, NW>(P, S, jb, warp, lane, W, tm, tw, (unsigned)u.y, fr, u.z); break;
        }
      } else {
        unsigned long long *wrap = P.wrap + (long long)blockIdx.x * 2 * P.stride;
        switch (jb.kind) {
          case K_LCS: block_job<K_LCS, R, NW>(P, S, jb, warp, lane, W, 0, 1, wrap, S.gen, nullptr); break;
          case K_ED: block_job<K_ED, R, NW>(P, S, jb, warp, lane, W, 0, 1, wrap, S.gen, nullptr); break;
          default: block_job<K_SW, R, NW>(P, S, jb, warp, lane, W, 0, 1, wrap, S.gen, nullptr); break;
        }
      }
      __syncthreads();
      continue;
    }
    // warp jobs, each warp on its own
    const unsigned long long t0 = globaltimer_ns();
    int ran = 0;
    for (;;) {
      int w = -1;
      if (lane == 0 && !stopping()) {
        int k = ld_relaxed_gpu_s32(pk);
        const bool cta_waiting = ring_backlog(ctl, k, 0) > 0;
        if (!(cta_waiting && globaltimer_ns() > t0 + SLICE_NS)) {
          int t = ring_claim(ctl, k, 1);
          if (t < 0 && !cta_waiting) {
            // nothing of this kind is left: the pair moves on
            k = pick_kind(ctl, pk);
            if (k >= 0) t = ring_claim(ctl, k, 1);
          }
          if (t >= 0) {
            atomicMax(last, globaltimer_ns());
            w = k * P.qw + t % P.qw;
          }
        }
      }
      w = __shfl_sync(FULL, w, 0);
      if (w < 0) break;
      const BatchJob jb = P.jobs_w[w];
      switch (jb.kind) {
        case K_LCS: warp_job<K_LCS, R, NW>(P, S, jb, warp, lane, W); break;
        case K_ED: warp_job<K_ED, R, NW>(P, S, jb, warp, lane, W); break;
        default: warp_job<K_SW, R, NW>(P, S, jb, warp, lane, W); break;
      }
      ++ran;
      if (*(volatile int *)&S.abort) break;
    }
    if (!__syncthreads_or(ran)) __nanosleep(2000);
  }
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(&ctl[RW_EXITS], 1);
}

// Copies every pair's sequences into the padded, aligned layout the engine reads,
// and records per segment whether a symbol lies outside [0, 32767] (then the pair
// cannot take the 16-bit engine, which compares symbols in 16-bit lanes).
__global__ void batch_stage_kernel(const int *__restrict__ src, const long long *__restrict__ from,
                                   const long long *__restrict__ to, const int *__restrict__ len,
                                   const int *__restrict__ padl, const int *__restrict__ total,
                                   int nseg, int *__restrict__ dst, int *__restrict__ bad) {
  for (int s = blockIdx.x; s < nseg; s += gridDim.x) {
    const long long f = from[s], t0 = to[s];
    const int n = len[s], pl = padl[s], tot = total[s];
    int b = 0;
    for (int i = threadIdx.x; i < tot; i += blockDim.x) {
      const int k = i - pl;
      int v = 0;
      if (k >= 0 && k < n) {
        v = src[f + k];
        b |= (unsigned)v > 0x7fffu;
      }
      dst[t0 + i] = v;
    }
    b = __syncthreads_or(b);
    if (threadIdx.x == 0) bad[s] = b;
  }
}

// ---------------------------------------------------------------------------
// Host side: plan (classify, order, lay out), stage, launch.
// ---------------------------------------------------------------------------
template <int R, int NW>
static cudaError_t launch_batch_t(const BatchParams &P, int grid, cudaStream_t st) {
  // the dynamic shared-memory limit is raised once, when the plan is made
  batch_kernel<R, NW><<<grid, NW * 32, sizeof(BatchSmem<NW>), st>>>(P);
  return cudaGetLastError();
}

cudaError_t batch_launch_r2(int NW, const BatchParams &P, int grid, cudaStream_t st);  // gme_batch_r2.cu
int batch_occupancy_r2(int NW);

static cudaError_t launch_batch(int R, int NW, const BatchParams &P, int grid, cudaStream_t st) {
  if (R == 2) return batch_launch_r2(NW, P, grid, st);
  switch (NW) {
    case 4: return launch_batch_t<4, 4>(P, grid, st);
    case 8: return launch_batch_t<4, 8>(P, grid, st);
  }
  return cudaErrorInvalidValue;
}

template <int R, int NW>
static int occupancy_t() {
  int n = 0;
  const size_t smem = sizeof(BatchSmem<NW>);
  cudaFuncSetAttribute(batch_kernel<R, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<R, NW>, NW * 32, smem);
  return n;
}

int batch_occupancy(int NW, int R) {
  if (R == 2) return batch_occupancy_r2(NW);
  switch (NW) {
    case 4: return occupancy_t<4, 4>();
    case 8: return occupancy_t<4, 8>();
  }
  return 0;
}

// (2 rows per lane only with 8 warps per CTA: gme_batch_r2.cu)
bool batch_config_valid(int NW, int R) { return (NW == 4 || NW == 8) && (R == 4 || (R == 2 && NW == 8)); }

// Device bytes one pair adds to a batch: its symbols as the caller holds them, the
// staged copy (pads, b rounded up to whole band groups) and its descriptors.
long long batch_pair_bytes(long long n1, long long n2) {
  const long long staged = (PADL + n1 + PADR + 3) / 4 * 4 + (n2 + 32 * 4 * 8 - 1) / (32 * 4 * 8) * (32 * 4 * 8);
  return 4 * (n1 + n2) + 4 * staged + 2 * 32 + (long long)sizeof(BatchJob);
}

// CTAs of the batch kernel's grid.
long long batch_grid(int sms, int NW, int blocks_per_sm, int R) {
  int occ = batch_occupancy(NW, R);
  if (occ < 1) occ = 1;
  return (long long)sms * std::min(occ, blocks_per_sm > 0 ? blocks_per_sm : occ);
}

// Device bytes of a batch's per-CTA rows (warp jobs' rows, block jobs' wrap rows).
long long batch_scratch_bytes(long long grid, int NW, int max_n1) {
  return grid * row_stride(max_n1) * (4ll * NW + 2 * 8);
}

// The plan: classify the pairs (per warp, per CTA, or plain path), order them
// longest first, lay the staged symbols out and upload the descriptors.  Waits
// for the arena's previous work on `st` before reusing its buffers.
// The settings a batch is planned with: the caller's, or the tuned entry whose
// length range is nearest (in log scale) to the batch's own, taken as the 2nd and
// 98th percentiles of sqrt(n1*n2) over its pairs.
BatchTuning batch_tuning_for(const gme_pair *pairs, long long npairs, const BatchTuning &given) {
  if (given.user_set || TUNED_BUCKETS == 0 || npairs == 0) return given;
  std::vector<float> len((size_t)npairs);
  for (long long i = 0; i < npairs; ++i)
    len[i] = std::sqrt((float)pairs[i].n1 * (float)pairs[i].n2) + 1.0f;
  const size_t i_lo = (size_t)(0.02 * (npairs - 1)), i_hi = (size_t)(0.98 * (npairs - 1));
  std::nth_element(len.begin(), len.begin() + i_lo, len.end());
  const float lo = len[i_lo];
  std::nth_element(len.begin(), len.begin() + i_hi, len.end());
  const float hi = len[i_hi];
  int best = 0;
  float best_d = 1e30f;
  for (int b = 0; b < TUNED_BUCKETS; ++b) {
    const float d = std::fabs(std::log(lo / (float)TUNED[b].lo)) + std::fabs(std::log(hi / (float)TUNED[b].hi));
    if (d < best_d) { best_d = d; best = b; }
  }
  BatchTuning t = given;
  t.warps_per_block = TUNED[best].warps_per_block;
  t.blocks_per_sm = TUNED[best].blocks_per_sm;
  t.block_min_cells = TUNED[best].block_min_cells;
  t.team_min_cells = TUNED[best].team_min_cells;
  t.team_split = TUNED[best].team_split;
  t.rows_per_lane = TUNED[best].rows_per_lane;
  t.packed16 = given.packed16 && TUNED[best].packed16;
  return t;
}

int batch_plan(Workspace &ws, BatchArena &ar, const gme_pair *pairs, long long npairs,
               long long nsym, const BatchTuning &tune_given, cudaStream_t st,
               const long long *row_offs, const long long *col_offs) {
  constexpr int R = 4;
  const BatchTuning tune = batch_tuning_for(pairs, npairs, tune_given);
  const int NW = tune.warps_per_block;
  const int RL = tune.rows_per_lane;  // the kernel's rows per lane (the layout is for 4)
  if (!batch_config_valid(NW, RL))
    return ws.fail_msg(ST_INVALID, "batch: warps_per_block must be 4 or 8, rows_per_lane 4 (or 2 with 8 warps)");
  std::vector<int> blockj, warpj, teamj;
  ar.longj.clear();
  int occ0 = batch_occupancy(NW, RL);
  if (occ0 < 1) occ0 = 1;
  const int grid0 = ws.sms * std::min(occ0, tune.blocks_per_sm > 0 ? tune.blocks_per_sm : occ0);
  long long total_cells = 0;
  for (long long i = 0; i < npairs; ++i) {
    const gme_pair &p = pairs[i];
    if (p.n1 < 0 || p.n2 < 0 || p.kind < 0 || p.kind > 2 || p.a_off < 0 || p.b_off < 0 ||
        p.a_off + p.n1 > nsym || p.b_off + p.n2 > nsym)
      return ws.fail_msg(ST_INVALID, "batch: pair " + std::to_string(i) + " out of range");
    total_cells += (long long)p.n1 * p.n2;
  }
  // the plain path takes a pair only when even a team of 8 CTAs would outlast an
  // even share of the batch (and always pairs too wide for the rows, or empty)
  long long long_min = tune.long_min_cells;
  if (long_min == 0) long_min = std::max(1ll << 27, 8 * (total_cells / grid0));
  if (long_min < 0) long_min = LLONG_MAX;
  const long long team_min = tune.team_min_cells > 0 ? tune.team_min_cells : LLONG_MAX;
  auto groups = [&](const gme_pair &p) { return ((p.n2 + 32 * R - 1) / (32 * R) + NW - 1) / NW; };
  for (long long i = 0; i < npairs; ++i) {
    const gme_pair &p = pairs[i];
    const long long cells = (long long)p.n1 * p.n2;
    if (p.n1 == 0 || p.n2 == 0 || p.n1 > BATCH_MAXN || cells >= long_min)
      ar.longj.push_back((int)i);
    else if (cells >= team_min && groups(p) >= 4 && (long long)(p.n1 + 1) * (p.n2 + 1) < (1ll << 32))
      teamj.push_back((int)i);
    else if (cells >= tune.block_min_cells && p.n2 > 32 * R * (NW - 1)) blockj.push_back((int)i);
    else warpj.push_back((int)i);
  }
  // Team sizes: the tuned rule, or, for a batch whose CTA pairs leave CTAs of the grid
  // idle (a few large pairs), teams sized by the pair's share of the grid: a pair of
  // c cells takes min(groups, 8, ceil(c / (cells of the CTA pairs / CTAs for them)))
  // CTAs.  Only for planned settings; a caller's own settings are kept as given.
  std::vector<int> fill_T;  // per pair: team size of the fill rule (0: the tuned rule)
  auto team_size = [&](int i) {
    if (!fill_T.empty() && fill_T[i] > 0) return fill_T[i];
    return std::max(2, std::min(8, (int)groups(pairs[i]) / std::max(1, tune.team_split)));
  };
  if (!tune.user_set && !blockj.empty()) {
    long long units = 0;
    for (int i : teamj) units += team_size(i);
    const long long other = units + ((long long)warpj.size() + NW - 1) / NW;
    const long long avail = grid0 - other;  // CTAs left for the CTA pairs
    if (avail > (long long)blockj.size()) {
      long long big = 0;
      for (int i : blockj) big += (long long)pairs[i].n1 * pairs[i].n2;
      const double per_cta = (double)big / (double)avail;
      fill_T.assign((size_t)npairs, 0);
      std::vector<int> keep;
      for (int i : blockj) {
        const gme_pair &p = pairs[i];
        const long long G = groups(p);
        const long long want = (long long)std::ceil((double)p.n1 * p.n2 / per_cta);
        const int T = (int)std::min(std::min(G, 8ll), want);
        if (T >= 2 && (long long)(p.n1 + 1) * (p.n2 + 1) < (1ll << 32)) {
          fill_T[i] = T;
          teamj.push_back(i);
        } else {
          keep.push_back(i);
        }
      }
      blockj.swap(keep);
    }
  }
  // one kind after another (an SM then runs one kind's code at a time), longest first
  auto by_cells = [&](int x, int y) {
    if (pairs[x].kind != pairs[y].kind) return pairs[x].kind < pairs[y].kind;
    const long long cx = (long long)pairs[x].n1 * pairs[x].n2, cy = (long long)pairs[y].n1 * pairs[y].n2;
    return cx != cy ? cx > cy : x < y;
  };
  std::sort(blockj.begin(), blockj.end(), by_cells);
  std::sort(warpj.begin(), warpj.end(), by_cells);
  // team jobs kind by kind as well: claiming every kind's teams first put the three
  // kinds' loops on one SM at once and halved the throughput of the [32, 16384] mix
  std::sort(teamj.begin(), teamj.end(), by_cells);
  ar.long_pairs.clear();
  ar.long_rows.clear();
  ar.long_cols.clear();
  for (int i : ar.longj) {
    ar.long_pairs.push_back(pairs[i]);
    ar.long_rows.push_back(row_offs ? row_offs[i] : -1);
    ar.long_cols.push_back(col_offs ? col_offs[i] : -1);
  }
  // staged layout: a padded with PADL/PADR at a 16-byte aligned start, b padded to whole bands
  const long long nseg = 2 * (long long)(blockj.size() + warpj.size() + teamj.size());
  ar.h_from.resize(nseg); ar.h_to.resize(nseg); ar.h_len.resize(nseg); ar.h_padl.resize(nseg); ar.h_total.resize(nseg);
  ar.h_jobs.resize(blockj.size() + warpj.size() + teamj.size());
  long long off = 0, seg = 0;
  auto place = [&](long long from, int len, int padl, int total) {
    ar.h_from[seg] = from; ar.h_to[seg] = off; ar.h_len[seg] = len; ar.h_padl[seg] = padl; ar.h_total[seg] = total;
    ++seg;
    const long long at = off;
    off += (total + 3) / 4 * 4;
    return at;
  };
  auto add = [&](int i, int rows_mult, size_t slot) {
    const gme_pair &p = pairs[i];
    BatchJob j;
    j.seg = (int)seg;
    j.a_off = place(p.a_off, p.n1, PADL, PADL + p.n1 + PADR);
    const int brows = (p.n2 + rows_mult - 1) / rows_mult * rows_mult;
    j.b_off = place(p.b_off, p.n2, 0, brows);
    j.n1 = p.n1; j.n2 = p.n2; j.kind = p.kind; j.index = (int)i;
    j.row_off = row_offs ? row_offs[i] : -1;
    j.col_off = col_offs ? col_offs[i] : -1;
    ar.h_jobs[slot] = j;
  };
  size_t slot = 0;
  for (int i : blockj) add(i, 32 * R * NW, slot++);
  for (int i : warpj) add(i, 32 * R, slot++);
  // a team of T CTAs per team job (team_size); members claimed in order
  ar.h_units.clear();
  for (size_t j = 0; j < teamj.size(); ++j) {
    add(teamj[j], 32 * R * NW, slot++);
    const int T = team_size(teamj[j]);
    for (int t = 0; t < T; ++t) ar.h_units.push_back(make_int4((int)j, t, T, 0));
  }
  cudaError_t e;
  if (ar.sync_before_reuse && (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return ws.fail(e, "cudaStreamSynchronize(batch arena)");
  int rc = ar.reserve(off + 64, nseg, (long long)ar.h_jobs.size(), ws);
  if (rc != ST_OK) return rc;
  int max_n1 = 0;
  for (const BatchJob &j : ar.h_jobs) max_n1 = std::max(max_n1, j.n1);
  ar.stride = row_stride(max_n1);
  ar.n_t = (int)teamj.size();
  ar.team_bytes = (long long)ar.n_t * (sizeof(TeamSlot) + 2ll * ar.stride * 8);
  if ((rc = ar.reserve_rows((long long)grid0 * NW * ar.stride, ws)) != ST_OK) return rc;
  if ((rc = ar.reserve_wrap((long long)grid0 * 2 * ar.stride, ws)) != ST_OK) return rc;
  if ((rc = ar.reserve_team((long long)ar.h_units.size(), ar.team_bytes, ws)) != ST_OK) return rc;
  if (!ar.h_units.empty() &&
      (e = cudaMemcpyAsync(ar.d_units, ar.h_units.data(), ar.h_units.size() * sizeof(int4), cudaMemcpyHostToDevice, st)))
    return ws.fail(e, "cudaMemcpyAsync(batch team units)");
  if (nseg > 0) {
    // pageable sources: each call has copied its bytes out before it returns, and
    // the copies are ordered before the launches that read them on `st`
    if ((e = cudaMemcpyAsync(ar.d_from, ar.h_from.data(), nseg * 8, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(ar.d_to, ar.h_to.data(), nseg * 8, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(ar.d_len, ar.h_len.data(), nseg * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(ar.d_padl, ar.h_padl.data(), nseg * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(ar.d_total, ar.h_total.data(), nseg * 4, cudaMemcpyHostToDevice, st)) ||
        (e = cudaMemcpyAsync(ar.d_jobs, ar.h_jobs.data(), ar.h_jobs.size() * sizeof(BatchJob), cudaMemcpyHostToDevice, st)))
      return ws.fail(e, "cudaMemcpyAsync(batch plan)");
  }
  ar.nseg = nseg;
  ar.n_b = (int)blockj.size();
  ar.n_w = (int)warpj.size();
  // kind boundaries of the queues (all sorted by kind first)
  for (int k = 0; k <= 3; ++k) {
    ar.kb[k] = (int)(std::lower_bound(blockj.begin(), blockj.end(), k, [&](int i, int kk) { return pairs[i].kind < kk; }) - blockj.begin());
    ar.kw[k] = (int)(std::lower_bound(warpj.begin(), warpj.end(), k, [&](int i, int kk) { return pairs[i].kind < kk; }) - warpj.begin());
    ar.ku[k] = (int)(std::lower_bound(ar.h_units.begin(), ar.h_units.end(), k, [&](const int4 &u, int kk) {
                       return pairs[teamj[u.x]].kind < kk; }) - ar.h_units.begin());
  }
  ar.NW = NW;
  ar.R = RL;
  ar.grid = grid0;
  ar.packed16 = tune.packed16 && RL == 4 ? 1 : 0;
  ar.last_block_jobs = ar.n_b;
  ar.last_warp_jobs = ar.n_w;
  ar.last_long_jobs = (long long)ar.longj.size();
  ar.last_team_jobs = ar.n_t;
  return ST_OK;
}

// The launches of a planned batch: clear the tickets, stage the symbols, run the
// work-queue kernel.  Stream operations only, so the sequence can be captured.
// Returns the number of kernels launched in *kernels.
int batch_launch(Workspace &ws, BatchArena &ar, const int *d_sym, const Scoring &sc,
                 gme_result *d_results, cudaStream_t st, unsigned long long timeout_ns, int *kernels,
                 int *d_last_rows, int *d_last_cols) {
  *kernels = 0;
  if (ar.nseg == 0) return ST_OK;
  cudaError_t e;
  if ((e = cudaMemsetAsync(ar.d_ctrl, 0, 16 * sizeof(int), st)) != cudaSuccess)
    return ws.fail(e, "cudaMemsetAsync(batch ctrl)");
  if (ar.team_bytes > 0 && (e = cudaMemsetAsync(ar.d_team, 0, (size_t)ar.team_bytes, st)) != cudaSuccess)
    return ws.fail(e, "cudaMemsetAsync(batch teams)");
  const int blocks = (int)std::min<long long>(ar.nseg, 65535);
  batch_stage_kernel<<<blocks, 256, 0, st>>>(d_sym, ar.d_from, ar.d_to, ar.d_len, ar.d_padl,
                                             ar.d_total, (int)ar.nseg, ar.d_staged, ar.d_symbad);
  if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "batch_stage_kernel");
  BatchParams P;
  std::memset(&P, 0, sizeof(P));  // the served kernel's fields stay null
  P.sym = ar.d_staged;
  P.jobs_b = ar.d_jobs;
  P.jobs_w = ar.d_jobs + ar.n_b;
  P.jobs_t = ar.d_jobs + ar.n_b + ar.n_w;
  P.units = ar.d_units;
  P.n_b = ar.n_b;
  P.n_w = ar.n_w;
  for (int k = 0; k < 4; ++k) { P.kb[k] = ar.kb[k]; P.kw[k] = ar.kw[k]; P.ku[k] = ar.ku[k]; }
  P.team = reinterpret_cast<TeamSlot *>(ar.d_team);
  P.twrap = reinterpret_cast<unsigned long long *>(ar.d_team + (long long)ar.n_t * sizeof(TeamSlot));
  P.results = d_results;
  P.done = ar.d_done;
  P.last_rows = d_last_rows;
  P.last_cols = d_last_cols;
  P.symbad = ar.d_symbad;
  P.packed16 = ar.packed16;
  P.rows = ar.d_rows;
  P.wrap = ar.d_wrap;
  P.gen = ar.d_gen;
  P.stride = ar.stride;
  P.ctrl = ar.d_ctrl;
  P.sc = sc;
  P.timeout_ns = timeout_ns;
  if ((e = launch_batch(ar.R, ar.NW, P, ar.grid, st)) != cudaSuccess) return ws.fail(e, "batch_kernel");
  *kernels = 2;
  return ST_OK;
}

// Pairs the shared-memory rows cannot hold (or empty ones): the plain path, one
// call each.  Never captured: the plain path hands out fresh band tags per call.
int batch_long(BatchArena &ar, const int *d_sym, gme_result *d_results, int *d_last_rows, int *d_last_cols,
               int (*plain)(void *, int, const int *, long long, const int *, long long, gme_result *, int *, int *),
               void *plain_ctx) {
  for (size_t k = 0; k < ar.longj.size(); ++k) {
    const gme_pair &p = ar.long_pairs[k];
    int *row = d_last_rows && ar.long_rows[k] >= 0 ? d_last_rows + ar.long_rows[k] : nullptr;
    int *col = d_last_cols && ar.long_cols[k] >= 0 ? d_last_cols + ar.long_cols[k] : nullptr;
    const int rc = plain(plain_ctx, p.kind, d_sym + p.a_off, p.n1, d_sym + p.b_off, p.n2,
                         d_results + ar.longj[k], row, col);
    if (rc != ST_OK) return rc;
  }
  return ST_OK;
}

int batch_run(Workspace &ws, BatchArena &ar, const int *d_sym, long long nsym, const gme_pair *pairs,
              long long npairs, const Scoring &sc, gme_result *d_results, cudaStream_t st,
              const BatchTuning &tune, unsigned long long timeout_ns,
              int *d_last_rows, const long long *row_offs, int *d_last_cols, const long long *col_offs,
              int (*plain)(void *, int, const int *, long long, const int *, long long, gme_result *, int *, int *),
              void *plain_ctx) {
  int rc = batch_plan(ws, ar, pairs, npairs, nsym, tune, st, d_last_rows ? row_offs : nullptr,
                      d_last_cols ? col_offs : nullptr);
  if (rc != ST_OK) return rc;
  int k = 0;
  rc = batch_launch(ws, ar, d_sym, sc, d_results, st, timeout_ns, &k, d_last_rows, d_last_cols);
  ws.launches += k;
  if (rc != ST_OK) return rc;
  return batch_long(ar, d_sym, d_results, d_last_rows, d_last_cols, plain, plain_ctx);
}


// ---------------------------------------------------------------------------
// The served kernel (serve_kernel): its shape, grid and launch.
// ---------------------------------------------------------------------------
template <int NW>
static cudaError_t serve_launch_t(const BatchParams &P, int grid, cudaStream_t st) {
  const size_t smem = sizeof(BatchSmem<NW>);
  cudaError_t e = cudaFuncSetAttribute(serve_kernel<4, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  serve_kernel<4, NW><<<grid, NW * 32, smem, st>>>(P);
  return cudaGetLastError();
}

int serve_grid(int sms, int NW) {
  int n = 0;
  if (NW == 8) {
    cudaFuncSetAttribute(serve_kernel<4, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BatchSmem<8>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, serve_kernel<4, 8>, 8 * 32, sizeof(BatchSmem<8>));
  } else {
    cudaFuncSetAttribute(serve_kernel<4, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(BatchSmem<4>));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, serve_kernel<4, 4>, 4 * 32, sizeof(BatchSmem<4>));
  }
  return sms * std::max(n, 1);
}

cudaError_t serve_launch(const ServeArgs &a, cudaStream_t st) {
  BatchParams P;
  std::memset(&P, 0, sizeof(P));
  P.sym = a.arena;
  P.jobs_b = a.jobs_b;
  P.jobs_w = a.jobs_w;
  P.results = a.results;
  P.done = a.done;
  P.symbad = a.symbad;
  P.packed16 = 1;
  P.rows = a.rows;
  P.wrap = a.wrap;
  P.gen = a.gen;
  P.stride = a.stride;
  P.ctrl = a.ctrl;
  P.sc.match = a.sc.match;
  P.sc.mismatch = a.sc.mismatch;
  P.sc.gap = a.sc.gap;
  P.sc.ed_rule = a.sc.ed_boundary;
  P.timeout_ns = a.timeout_ns;
  P.ring_ctl = a.ring_ctl;
  P.units = a.units;
  P.steam = reinterpret_cast<ServeTeam *>(a.teams);
  P.twrap = a.twrap;
  P.tfree = a.tfree;
  P.cq = a.cq;
  P.cq_n = reinterpret_cast<unsigned *>(a.ring_ctl + RW_CQN);
  P.cq_mask = a.cq_mask;
  P.qb = a.qb;
  P.qw = a.qw;
  P.idle_ns = a.idle_ns;
  return a.NW == 8 ? serve_launch_t<8>(P, a.grid, st) : serve_launch_t<4>(P, a.grid, st);
}

int serve_row_stride(int max_n1) { return row_stride(max_n1); }
int serve_padl() { return PADL; }
long long serve_a_len(int n1) { return (PADL + (long long)n1 + PADR + 3) / 4 * 4; }
int serve_rows_mult(int NW, bool block) { return block ? 32 * 4 * NW : 32 * 4; }
long long serve_team_bytes() { return sizeof(ServeTeam); }

}  // namespace gme
