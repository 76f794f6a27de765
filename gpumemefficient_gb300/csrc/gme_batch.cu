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

#include "gme_engine.cuh"
#include "gme_engine16.cuh"
#include "gme_internal.h"
#include "gme_tuned.h"

namespace gme {

// Wavefront steps per ring transaction in this kernel.  A dozen independent warps
// per SM each run their own pair at their own point in the loop, so the loop body
// must stay small for the instruction cache; with one chunk body per kind and engine
// 16 steps fit and halve the per-chunk ring and tag work against 8 (32 steps double the
// body again and lost 44% on the 16384-pair batch).
#ifndef GME_BATCH_CHUNK
#define GME_BATCH_CHUNK 16
#endif
constexpr int CB = GME_BATCH_CHUNK;
// Resident 4-warp CTAs per SM the register allocation is sized for (65536 registers
// / (128 threads x 3) caps a thread at 168).
#ifndef GME_BATCH_MIN_BLOCKS
#define GME_BATCH_MIN_BLOCKS 3
#endif


constexpr int BATCH_MAXN = BATCH_MAX_N1;
// a row is read up to one chunk past the last chunk (the read-ahead): j_end+1 with
// j_end = (n1 + 32R)/CB, so a row of n1 columns needs n1 + 32R + 2C entries (R <= 8);
// rows are laid out with the stride of the batch's widest pair
__host__ __device__ constexpr int row_stride(int max_n1) { return (max_n1 + 32 * 8 + 3 * CB + 7) / 8 * 8; }

// A pair shared by a team of T CTAs: member t sweeps band groups t, t+T, t+2T, ...
// handing each group's bottom row to the next member through the job's two tagged
// rows.  The members combine their results here; the last one to finish writes it.
struct __align__(16) TeamSlot {
  unsigned long long best;  // SW: (value << 32) | ~(y*(n1+1)+x), so the maximum is the first best cell
  int corner;               // stored value of the last band's bottom row at column n1
  int done;                 // members finished
};

// A large pair of the served kernel, shared by the CTAs that take its entries in the
// CTA ring: each claims the pair's next band group (next) and sweeps it with its warps,
// group g taking its incoming row from group g-1's CTA through two tagged rows.  A CTA
// waits only on groups claimed before its own, each on a running CTA, so a team never
// waits on an entry no CTA has taken.  The CTA that finishes the last group (gdone)
// writes the result; the last of the team's entries to leave (left) raises the team's
// release flag in mapped host memory, after which the host may reuse the team.
struct __align__(16) ServeTeam {
  unsigned long long best;  // SW: as TeamSlot::best
  int next, gdone, left, corner;
};

struct BatchParams {
  const int *sym;          // staged, padded symbols
  const BatchJob *jobs_b;  // block jobs, by kind, longest first
  const BatchJob *jobs_w;  // warp jobs, by kind, longest first
  const BatchJob *jobs_t;  // team jobs, by kind, longest first
  const int4 *units;       // team members {team job, member t, team size T, 0}, by kind
  int n_b, n_w;
  int kb[4], kw[4], ku[4]; // kind k: jobs_b[kb[k]..kb[k+1]), jobs_w[kw[k]..), units[ku[k]..)
  TeamSlot *team;          // one per team job (cleared by every launch)
  unsigned long long *twrap;  // two tagged rows of `stride` words per team job (cleared likewise)
  gme_result *results;
  int *done;               // optional: done[index] = 1 once results[index] is written (system scope)
  int *last_rows;          // optional: per job, its last row at jobs' row_off
  int *last_cols;          // optional: per job, its last column at jobs' col_off
  const int *symbad;       // per staged segment: 1 if a symbol lies outside [0, 32767]
  int packed16;            // jobs that qualify take the packed 16-bit engine
  int *rows;               // warp jobs: one row of `stride` ints per warp of the grid (L2-resident)
  unsigned long long *wrap;  // block jobs: two tagged rows of `stride` words per CTA
  unsigned *gen;           // tags handed out to wrap rows so far (kept across launches)
  int stride;
  int *ctrl;               // [2k] block ticket of kind k, [2k+1] warp ticket, [8] status, [10+k] team ticket
  Scoring sc;
  unsigned long long timeout_ns;
  // the served kernel's job rings (serve_kernel): the ring words (RW_*), the
  // rings' slots (jobs_b and jobs_w hold each kind's ring after the last's); per
  // CTA-ring slot, units[] holds {team, tag0, entries of the pair, 0} (entries 1: the
  // pair runs on the CTA alone); teams, their wrap rows and release flags
  ServeTeam *steam;
  int *tfree;
  int *cq;                 // optional: each job's result slot + 1, appended once it is done
  unsigned *cq_n;          //   (mapped host memory) at cq[(*cq_n)++ & cq_mask]
  int cq_mask;
  int *ring_ctl;
  int qb, qw;
  unsigned long long idle_ns;
};

template <int NW> struct __align__(16) BatchSmem {
  int ring[NW][RING];       // ring[w]: warp w-1 -> warp w (w >= 1)
  int tag[NW][RING / CB];
  int cons[NW];
  int job;
  int phase;
  int abort;
  unsigned gen;
  SwBest best[NW];
};

// ---------------------------------------------------------------------------
// Where a band's incoming row comes from and where its bottom row goes.  The mode
// is uniform across the warp and fixed for a band, so the switches cost a
// predictable branch per chunk and one sweep routine serves every combination.
// ---------------------------------------------------------------------------
enum : int { IN_TOP = 0, IN_RING = 1, IN_ROW = 2, IN_OWN = 3 };
enum : int { OUT_NONE = 0, OUT_RING = 1, OUT_ROW = 2, OUT_OWN = 3, OUT_USER = 4 };

struct Src {
  int mode;
  const int *buf;                  // ring values, or the warp's own row
  const int *tags;                 // ring chunk tags
  const unsigned long long *row;   // IN_ROW: tagged words {tag, value} in global memory
  int *cons;                       // ring: consumption counter (stream position)
  int base;                        // ring: stream position of column 0
  unsigned tag;                    // IN_ROW: the tag of the row wanted
  int rule;                        // top border: ED boundary rule
};

struct Dst {
  int mode;
  int *buf;          // ring or own row; OUT_USER: the caller's last row (table values)
  int *tags;
  unsigned long long *row;
  const int *cons;
  int base;
  unsigned tag;
  int cons_seen;
  int N, M;          // OUT_USER: columns 0..N are written, row M's values (ED adds x + y)
  int addxy;
};

__device__ __forceinline__ void ld_vol_u64x2(const unsigned long long *p, unsigned long long &a,
                                             unsigned long long &b) {
  asm volatile("ld.volatile.global.v2.u64 {%0,%1}, [%2];" : "=l"(a), "=l"(b) : "l"(p));
}
__device__ __forceinline__ void st_vol_u64x2(unsigned long long *p, unsigned long long a,
                                             unsigned long long b) {
  asm volatile("st.volatile.global.v2.u64 [%0], {%1,%2};" :: "l"(p), "l"(a), "l"(b) : "memory");
}

// Chunk j of the incoming row into d[]; returns whether it is ready (the same in
// every lane: all lanes read the same words).  A ring chunk's tag is acquired
// before its values; a global row's tag travels in the same 64-bit word as the
// value, so the row needs no fence on either side.
template <int KIND>
__device__ __forceinline__ bool src_fetch(const Src &s, int j, int (&d)[CB]) {
  if (s.mode == IN_TOP) {
#pragma unroll
    for (int k = 0; k < CB; ++k) d[k] = Rec<KIND>::top(CB * j + k, s.rule);
    return true;
  }
  if (s.mode == IN_ROW) {
    const unsigned long long *p = s.row + CB * j;
    bool ok = true;
#pragma unroll
    for (int k = 0; k < CB; k += 2) {
      unsigned long long w0, w1;
      ld_vol_u64x2(p + k, w0, w1);
      d[k] = (int)(unsigned)w0;
      d[k + 1] = (int)(unsigned)w1;
      ok &= (unsigned)(w0 >> 32) == s.tag && (unsigned)(w1 >> 32) == s.tag;
    }
    return ok;
  }
  if (s.mode == IN_OWN) {
    // the warp's own row in global memory, written by lane 31 one band earlier:
    // read at L2 (.cg) so that no lane sees a line its L1 kept from before the write
    const int *p = s.buf + CB * j;
#pragma unroll
    for (int k = 0; k < CB; k += 4) {
      const int4 q = __ldcg(reinterpret_cast<const int4 *>(p + k));
      d[k] = q.x; d[k + 1] = q.y; d[k + 2] = q.z; d[k + 3] = q.w;
    }
    return true;
  }
  const bool ok = ld_acquire_cta(&s.tags[(s.base / CB + j) & (RING / CB - 1)]) == s.base / CB + j + 1;
  const int *p = s.buf + ((s.base + CB * j) & (RING - 1));
#pragma unroll
  for (int k = 0; k < CB; k += 4) {
    const int4 q = *reinterpret_cast<const int4 *>(p + k);
    d[k] = q.x; d[k + 1] = q.y; d[k + 2] = q.z; d[k + 3] = q.w;
  }
  return ok;
}

__device__ __forceinline__ bool dst_put(Dst &o, int pos, const int (&q)[CB], int lane, Waiter &W) {
  if (o.mode == OUT_NONE) return true;
  if (o.mode == OUT_USER) {
    // the pair's last row, as table values, for the caller
    if (lane == 31) {
#pragma unroll
      for (int k = 0; k < CB; ++k)
        if (pos + k <= o.N) o.buf[pos + k] = q[k] + (o.addxy ? pos + k + o.M : 0);
    }
    return true;
  }
  if (o.mode == OUT_ROW) {
    if (lane == 31) {
      const unsigned long long t = (unsigned long long)o.tag << 32;
#pragma unroll
      for (int k = 0; k < CB; k += 2)
        st_vol_u64x2(o.row + pos + k, t | (unsigned)q[k], t | (unsigned)q[k + 1]);
    }
    return true;
  }
  int *p;
  if (o.mode == OUT_RING) {
    const int sp = o.base + pos;
    if (sp + CB - RING > o.cons_seen) {
      if (!W.wait([&] {
            o.cons_seen = __shfl_sync(FULL, lds_vol(o.cons), 0);
            return o.cons_seen >= sp + CB - RING;
          }))
        return false;
    }
    p = o.buf + (sp & (RING - 1));
  } else {
    p = o.buf + pos;
  }
  if (lane == 31) {
#pragma unroll
    for (int k = 0; k < CB; k += 4)
      *reinterpret_cast<int4 *>(p + k) = make_int4(q[k], q[k + 1], q[k + 2], q[k + 3]);
    if (o.mode == OUT_RING) st_release_cta(&o.tags[((o.base + pos) / CB) & (RING / CB - 1)], (o.base + pos) / CB + 1);
  }
  return true;
}

// ---------------------------------------------------------------------------
// One warp sweeps one band (32*R rows starting at row y0+1) of one pair.
// Returns false if a wait gave up.  On return `corner` (lane 31) holds the
// stored value of the band's bottom row at column n1 and `tb` the lane's SW best.
// ---------------------------------------------------------------------------
template <int KIND, int R>
__device__ __noinline__ bool sweep_band(const Scoring sc, const int *__restrict__ a_sym,
                                        const int *__restrict__ b_sym, int N, int M, int y0,
                                        int lane, Src in, Dst out, Waiter &W, int &corner,
                                        SwBest &tb, int *col_out) {
  const Rec<KIND> rec(sc);
  const int yl = y0 + lane * R + 1;  // first row of this lane
  int bs[R], cur[R], prv[R], smax[R], sstep[R];
#pragma unroll
  for (int r = 0; r < R; r += 4) {
    const int4 q = ldg4(b_sym + (yl - 1 + r));
    bs[r] = q.x; bs[r + 1] = q.y; bs[r + 2] = q.z; bs[r + 3] = q.w;
  }
  unsigned padmask = 0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    cur[r] = Rec<KIND>::left(yl + r);
    prv[r] = cur[r];
    smax[r] = 0;
    sstep[r] = 0;
    if (yl + r > M) padmask |= 1u << r;
  }
  const bool padwarp = __any_sync(FULL, padmask != 0);

  const int *sym = a_sym + (PADL - 1 - lane * R);
  int win[2 * CB];
#pragma unroll
  for (int k = 0; k < CB; k += 4) {
    const int4 q = ldg4(sym + k);
    win[k] = q.x; win[k + 1] = q.y; win[k + 2] = q.z; win[k + 3] = q.w;
  }
#pragma unroll
  for (int k = 0; k < R; k += 4) {
    const int4 q = ldg4(sym - R + k);
    win[2 * CB - R + k] = q.x; win[2 * CB - R + k + 1] = q.y;
    win[2 * CB - R + k + 2] = q.z; win[2 * CB - R + k + 3] = q.w;
  }
#pragma unroll
  for (int k = CB; k < 2 * CB - R; ++k) win[k] = 0;

  const int row_end = ((N + 1 + CB - 1) / CB) * CB;  // ring positions carrying this row
  int recv = 0, recv_prev = 0;
  int ib[2][CB];
  bool ok_next = src_fetch<KIND>(in, 0, ib[0]);

  // One chunk body per variant: the symbol window and the read-ahead buffer are
  // shifted by register moves after each chunk (about two moves per step), instead
  // of unrolling two window parities -- the loop then stays half as large in the
  // instruction cache, which a dozen warps per SM at different points of their own
  // pairs share.
  auto chunk = [&](int j, auto checked, auto padrows) -> bool {
    constexpr bool CK = decltype(checked)::value, PD = decltype(padrows)::value;
    const int s0 = CB * j;
    __syncwarp();
    if (s0 <= N && !__all_sync(FULL, ok_next)) {
      if (!W.wait([&] { return __all_sync(FULL, src_fetch<KIND>(in, j, ib[0])); })) return false;
    }
    // consumed: this chunk, but never past the end of this band's row -- the ring's
    // next positions already belong to the next band group of the same pair
    if (in.mode == IN_RING && lane == 31) sts_vol(in.cons, in.base + min(s0 + CB, row_end));
    if (lane == 0) recv = ib[0][0];
    ok_next = src_fetch<KIND>(in, j + 1, ib[1]);
    int outq[CB];
    steps_chunk<KIND, R, 0, CK, PD, CB>(rec, cur, prv, recv, recv_prev, win, sym + s0 + CB, bs, ib[0],
                                        outq, s0, lane, N, padmask, smax, sstep);
    // the next chunk's symbols (loaded into the upper half at step R) move down;
    // the last R-1 symbols of this chunk become the window's wrapped tail
    int tail[R - 1];
#pragma unroll
    for (int d = 0; d < R - 1; ++d) tail[d] = win[CB - R + 1 + d];
#pragma unroll
    for (int k = 0; k < CB; ++k) win[k] = win[k + CB];
#pragma unroll
    for (int d = 0; d < R - 1; ++d) win[2 * CB - R + 1 + d] = tail[d];
#pragma unroll
    for (int k = 0; k < CB; ++k) ib[0][k] = ib[1][k];
    const int pos = s0 - 32 * R;
    if (pos >= 0 && !dst_put(out, pos, outq, lane, W)) return false;
    return true;
  };

  // Two chunk bodies, each instantiated once: the steady one, and one that both
  // holds out-of-range cells and passes padding rows through (ramps, last band).
  using T = std::true_type;
  using F = std::false_type;
  const int j_end = (N + 32 * R) / CB;
  const int j_lo = padwarp ? j_end + 1 : min((32 * R) / CB, j_end + 1);
  const int j_hi = padwarp ? j_end : max(min((N - CB + 1) / CB, j_end), j_lo - 1);
  for (int j = 0; j <= j_end; ++j) {
    if (j >= j_lo && j <= j_hi) {
      if (!chunk(j, F{}, F{})) return false;
    } else {
      if (!chunk(j, T{}, T{})) return false;
    }
  }
  corner = cur[R - 1];
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const long long y = yl + r;
    if (col_out && y <= M) col_out[y] = Rec<KIND>::to_v(cur[r], N, y);  // column N, for the caller
    if (KIND == K_SW && y <= M && smax[r] > 0) {
      SwBest c = {smax[r], 0, y, (long long)(sstep[r] - lane * R - r)};
      if (better(c, tb)) tb = c;
    }
  }
  return true;
}

// The same band sweep on the packed 16-bit engine (gme_engine16.cuh): taken, when
// the batch asks for it, by a job whose values fit 16 bits and whose symbols lie in
// [0, 32767].  Rings, rows and
// results carry the same int32 values as the int32 sweep.
template <int KIND>
__device__ __noinline__ bool sweep_band16(const Scoring sc, const int *__restrict__ a_sym,
                                          const int *__restrict__ b_sym, int N, int M, int y0,
                                          int lane, Src in, Dst out, Waiter &W, int &corner,
                                          SwBest &tb, int *col_out) {
  constexpr int R = 4;
  const Rec16<KIND> rec(sc);
  const int yl = y0 + lane * R + 1;  // first row of this lane
  const int4 bq = ldg4(b_sym + (yl - 1));
  const unsigned bp[2] = {((unsigned)bq.x & 0xffffu) | ((unsigned)bq.z << 16),
                          ((unsigned)bq.y & 0xffffu) | ((unsigned)bq.w << 16)};
  // P0 holds rows 0 and 2, P1 rows 1 and 3; a padding row (beyond n2) copies the row above
  unsigned pm[2] = {0u, 0u};
  if (yl + 0 > M) pm[0] |= 0x0000ffffu;
  if (yl + 2 > M) pm[0] |= 0xffff0000u;
  if (yl + 1 > M) pm[1] |= 0x0000ffffu;
  if (yl + 3 > M) pm[1] |= 0xffff0000u;
  const bool padwarp = __any_sync(FULL, (pm[0] | pm[1]) != 0);
  unsigned cur[2] = {0u, 0u}, prv[2] = {0u, 0u};  // left border: stored value 0 for every kind
  unsigned smax[2] = {0u, 0u}, sstep[2] = {0u, 0u};
  const unsigned nn = (unsigned)N;

  const int *sym = a_sym + (PADL - 1 - lane * R);
  int win[2 * CB];
#pragma unroll
  for (int k = 0; k < CB; k += 4) {
    const int4 q = ldg4(sym + k);
    win[k] = q.x; win[k + 1] = q.y; win[k + 2] = q.z; win[k + 3] = q.w;
  }
  {
    const int4 q = ldg4(sym - R);
    win[2 * CB - R] = q.x; win[2 * CB - R + 1] = q.y; win[2 * CB - R + 2] = q.z; win[2 * CB - R + 3] = q.w;
  }
#pragma unroll
  for (int k = CB; k < 2 * CB - R; ++k) win[k] = 0;
  // the symbol pair of rows 0 and 2 at step -1 (symbol indices -1 and -3)
  unsigned pk_prev = __byte_perm((unsigned)win[2 * CB - 1], (unsigned)win[2 * CB - 3], 0x5410);

  const int row_end = ((N + 1 + CB - 1) / CB) * CB;  // ring positions carrying this row
  unsigned recv = 0u, recv_prev = 0u;
  int ib[2][CB];
  bool ok_next = src_fetch<KIND>(in, 0, ib[0]);

  auto chunk = [&](int j, auto checked, auto padrows) -> bool {
    constexpr bool CK = decltype(checked)::value, PD = decltype(padrows)::value;
    const int s0 = CB * j;
    __syncwarp();
    if (s0 <= N && !__all_sync(FULL, ok_next)) {
      if (!W.wait([&] { return __all_sync(FULL, src_fetch<KIND>(in, j, ib[0])); })) return false;
    }
    if (in.mode == IN_RING && lane == 31) sts_vol(in.cons, in.base + min(s0 + CB, row_end));
    if (lane == 0) recv = (unsigned)ib[0][0] << 16;
    ok_next = src_fetch<KIND>(in, j + 1, ib[1]);
    unsigned outq[CB];
    const unsigned x0 = (unsigned)(s0 - lane * R - 1);  // x-1 of row 0's cell at step s0
    const unsigned xm1[2] = {x0, x0};
    steps_chunk16<KIND, 0, CK, PD, CB>(rec, cur, prv, recv, recv_prev, pk_prev, win, sym + s0 + CB, bp,
                                       ib[0], outq, s0, lane, nn, xm1, pm, smax, sstep);
    int tail[R - 1];
#pragma unroll
    for (int d = 0; d < R - 1; ++d) tail[d] = win[CB - R + 1 + d];
#pragma unroll
    for (int k = 0; k < CB; ++k) win[k] = win[k + CB];
#pragma unroll
    for (int d = 0; d < R - 1; ++d) win[2 * CB - R + 1 + d] = tail[d];
#pragma unroll
    for (int k = 0; k < CB; ++k) ib[0][k] = ib[1][k];
    const int pos = s0 - 32 * R;
    if (pos >= 0) {
      int oq[CB];  // lane 31's row 3: the band's bottom row, as int32
#pragma unroll
      for (int k = 0; k < CB; ++k) oq[k] = (int)outq[k] >> 16;
      if (!dst_put(out, pos, oq, lane, W)) return false;
    }
    return true;
  };

  using T = std::true_type;
  using F = std::false_type;
  const int j_end = (N + 32 * R) / CB;
  const int j_lo = padwarp ? j_end + 1 : min((32 * R) / CB, j_end + 1);
  const int j_hi = padwarp ? j_end : max(min((N - CB + 1) / CB, j_end), j_lo - 1);
  for (int j = 0; j <= j_end; ++j) {
    if (j >= j_lo && j <= j_hi) {
      if (!chunk(j, F{}, F{})) return false;
    } else {
      if (!chunk(j, T{}, T{})) return false;
    }
  }
  corner = (int)cur[1] >> 16;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const long long y = yl + r;
    const int k = r & 1, sh = 16 * (r >> 1);
    if (col_out && y <= M) col_out[y] = Rec<KIND>::to_v((int)(short)(cur[k] >> sh), N, y);
    const int mx = (int)(short)(smax[k] >> sh);
    if (KIND == K_SW && y <= M && mx > 0) {
      const int st = (int)((sstep[k] >> sh) & 0xffffu);
      SwBest c = {mx, 0, y, (long long)(st - lane * R - r)};
      if (better(c, tb)) tb = c;
    }
  }
  return true;
}

// A band of a job on the engine the job qualifies for.
template <int KIND, int R>
__device__ __forceinline__ bool sweep_job_band(bool p16, const Scoring sc, const int *a_sym, const int *b_sym,
                                               int N, int M, int y0, int lane, Src in, Dst out, Waiter &W,
                                               int &corner, SwBest &tb, int *col_out) {
  if (R == 4 && p16) return sweep_band16<KIND>(sc, a_sym, b_sym, N, M, y0, lane, in, out, W, corner, tb, col_out);
  return sweep_band<KIND, R>(sc, a_sym, b_sym, N, M, y0, lane, in, out, W, corner, tb, col_out);
}

// Whether a job runs on the 16-bit engine: the batch asks for it, the job's values
// fit and the staging kernel found all of its symbols in [0, 32767].
__device__ __forceinline__ bool job_p16(const BatchParams &P, const BatchJob &jb) {
  return P.packed16 && fits16(jb.kind, jb.n1, jb.n2, P.sc) && P.symbad[jb.seg] == 0 &&
         P.symbad[jb.seg + 1] == 0;
}

__device__ __forceinline__ SwBest warp_best(SwBest b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    SwBest c;
    c.v = __shfl_down_sync(FULL, b.v, o);
    c.y = __shfl_down_sync(FULL, b.y, o);
    c.x = __shfl_down_sync(FULL, b.x, o);
    c.pad = 0;
    if (better(c, b)) b = c;
  }
  return b;
}

// Where the band that ends a job sends its bottom row: the caller's last row if asked
// for (row n2 as table values), else nowhere.
template <int KIND>
__device__ __forceinline__ void last_row_dst(const BatchParams &P, const BatchJob &jb, Dst &out) {
  if (P.last_rows && jb.row_off >= 0) {
    out.mode = OUT_USER;
    out.buf = P.last_rows + jb.row_off;
    out.N = jb.n1;
    out.M = jb.n2;
    out.addxy = KIND == K_ED;
  } else {
    out.mode = OUT_NONE;
  }
}

// Where a band writes its rows' values at column n1 (the job's last column), or
// null; the first band's lane 0 also writes row 0 (the top border at column n1).
template <int KIND>
__device__ __forceinline__ int *col_dst(const BatchParams &P, const BatchJob &jb, int band, int lane) {
  if (!P.last_cols || jb.col_off < 0) return nullptr;
  int *c = P.last_cols + jb.col_off;
  if (band == 0 && lane == 0) c[0] = Rec<KIND>::to_v(Rec<KIND>::top(jb.n1, P.sc.ed_rule), jb.n1, 0);
  return c;
}

// A job's status: a timeout if any wait of this CTA or of the launch gave up (a
// team member's result may then be incomplete).
__device__ __forceinline__ int job_status(const BatchParams &P, const int &abort) {
  return (*(const volatile int *)&abort || ld_relaxed_gpu_s32(&P.ctrl[8])) ? ST_TIMEOUT : 0;
}

// A job's result, then (if asked for) its completion flag, ordered at system
// scope so that a host thread polling the flag in mapped memory sees the result.
__device__ __forceinline__ void put_result(const BatchParams &P, int index, const gme_result &r) {
  P.results[index] = r;
  if (P.done || P.cq) __threadfence_system();
  if (P.done) *(volatile int *)&P.done[index] = 1;
  if (P.cq) {
    const unsigned pos = atomicAdd(P.cq_n, 1u);
    *(volatile int *)&P.cq[pos & (unsigned)P.cq_mask] = index + 1;
  }
}

// A pair on a CTA, or on member t of a team of T CTAs: warp w sweeps bands
// g*NW + w of the groups g = t, t+T, t+2T, ...; band b takes its incoming row from
// warp b-1 (ring[w]) or, for w = 0, from the wrap row that warp NW-1 wrote for
// group g-1 (on this CTA, or on the previous member).  The wrap rows are two
// tagged rows in global memory, alternating by group; group g's row carries tag
// tag0 + g + 1.  A CTA's own rows (T = 1) take tag0 from a counter that only grows,
// so no row holds a tag handed out later; a team's rows are cleared at launch.
template <int KIND, int R, int NW>
__device__ void block_job(const BatchParams &P, BatchSmem<NW> &S, const BatchJob &jb, int warp,
                          int lane, Waiter &W, int t, int T, unsigned long long *wrap, unsigned tag0,
                          TeamSlot *team) {
  const int N = jb.n1, M = jb.n2;
  const int *a_sym = P.sym + jb.a_off;
  const int *b_sym = P.sym + jb.b_off;
  const int nb = (M + 32 * R - 1) / (32 * R);
  const int L = ((N + 1 + CB - 1) / CB) * CB + 2 * CB;  // stream positions per band row
  const bool p16 = R == 4 && job_p16(P, jb);
  SwBest tb = {0, 0, 0, 0};
  int corner = 0, corner_band = -1;
  bool ok = true;
  // ring stream positions count this CTA's groups (i), so that every ring starts
  // at position 0 with its consumption counter; the wrap rows go by the group (g)
  for (int g = t, i = 0; ok && g * NW + warp < nb; g += T, ++i) {
    const int band = g * NW + warp;
    Src in;
    in.rule = P.sc.ed_rule;
    if (band == 0) {
      in.mode = IN_TOP;
    } else if (warp == 0) {
      in.mode = IN_ROW; in.row = wrap + ((g - 1) & 1) * P.stride; in.tag = tag0 + g;
    } else {
      in.mode = IN_RING; in.buf = S.ring[warp]; in.tags = S.tag[warp]; in.cons = &S.cons[warp];
      in.base = i * L;
    }
    Dst out;
    out.cons_seen = 0;
    if (band == nb - 1) {
      last_row_dst<KIND>(P, jb, out);
    } else if (warp == NW - 1) {
      out.mode = OUT_ROW; out.row = wrap + (g & 1) * P.stride; out.tag = tag0 + g + 1;
    } else {
      out.mode = OUT_RING; out.buf = S.ring[warp + 1]; out.tags = S.tag[warp + 1];
      out.cons = &S.cons[warp + 1]; out.base = i * L;
    }
    int c = 0;
    ok = sweep_job_band<KIND, R>(p16, P.sc, a_sym, b_sym, N, M, band * 32 * R, lane, in, out, W, c, tb,
                                 col_dst<KIND>(P, jb, band, lane));
    if (band == nb - 1) { corner = c; corner_band = band; }
  }
  // results: the corner from the warp that swept the last band, SW best over the CTA
  if (KIND == K_SW) {
    tb = warp_best(tb);
    if (lane == 0) S.best[warp] = tb;
  }
  __syncthreads();
  SwBest b = {0, 0, 0, 0};
  if (KIND == K_SW)
    for (int k = 0; k < NW; ++k)
      if (better(S.best[k], b)) b = S.best[k];
  if (T == 1) {
    if (corner_band >= 0 && lane == 31) {
      gme_result r;
      r.score = Rec<KIND>::to_v(corner, N, M);
      r.sw_max = b.v;
      r.sw_max_y = b.y;
      r.sw_max_x = b.x;
      r.status = job_status(P, S.abort);
      r.kind = KIND;
      put_result(P, jb.index, r);
    }
    return;
  }
  // a team: publish this member's part, the last member to finish writes the result
  if (corner_band >= 0 && lane == 31) {
    *(volatile int *)&team->corner = corner;
    __threadfence();
  }
  if (KIND == K_SW && threadIdx.x == 0 && b.v > 0)
    atomicMax(&team->best, ((unsigned long long)(unsigned)b.v << 32) |
                               (0xffffffffu - (unsigned)(b.y * (N + 1) + b.x)));
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&team->done, 1) == T - 1) {
      __threadfence();
      gme_result r;
      r.score = Rec<KIND>::to_v(*(volatile int *)&team->corner, N, M);
      const unsigned long long k = KIND == K_SW ? atomicAdd(&team->best, 0ull) : 0ull;
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

// A small pair on one warp: bands one after another through the warp's own row.
template <int KIND, int R, int NW>
__device__ void warp_job(const BatchParams &P, BatchSmem<NW> &S, const BatchJob &jb, int warp,
                         int lane, Waiter &W) {
  const int N = jb.n1, M = jb.n2;
  const int *a_sym = P.sym + jb.a_off;
  const int *b_sym = P.sym + jb.b_off;
  const int nb = (M + 32 * R - 1) / (32 * R);
  if (N == 0 || M == 0) {
    // an empty sequence: the table is its borders (the served kernel takes such pairs)
    if (lane == 31) {
      gme_result r;
      r.score = (M == 0) ? Rec<KIND>::to_v(Rec<KIND>::top(N, P.sc.ed_rule), N, 0)
                         : Rec<KIND>::to_v(Rec<KIND>::left(M), 0, M);
      r.sw_max = 0; r.sw_max_y = 0; r.sw_max_x = 0;
      r.status = job_status(P, S.abort);
      r.kind = KIND;
      put_result(P, jb.index, r);
    }
    return;
  }
  int *row = P.rows + ((long long)blockIdx.x * NW + warp) * P.stride;
  const bool p16 = R == 4 && job_p16(P, jb);
  SwBest tb = {0, 0, 0, 0};
  int corner = 0;
  for (int band = 0; band < nb; ++band) {
    Src in;
    in.rule = P.sc.ed_rule;
    in.mode = band == 0 ? IN_TOP : IN_OWN;
    in.buf = row;
    Dst out;
    out.cons_seen = 0;
    out.mode = OUT_OWN;
    out.buf = row;
    if (band == nb - 1) last_row_dst<KIND>(P, jb, out);
    if (!sweep_job_band<KIND, R>(p16, P.sc, a_sym, b_sym, N, M, band * 32 * R, lane, in, out, W, corner, tb,
                                 col_dst<KIND>(P, jb, band, lane)))
      return;
  }
  if (KIND == K_SW) tb = warp_best(tb);
  SwBest b0;
  b0.v = __shfl_sync(FULL, tb.v, 0);
  b0.y = __shfl_sync(FULL, tb.y, 0);
  b0.x = __shfl_sync(FULL, tb.x, 0);
  if (lane == 31) {
    gme_result r;
    r.score = Rec<KIND>::to_v(corner, N, M);
    r.sw_max = KIND == K_SW ? b0.v : 0;
    r.sw_max_y = KIND == K_SW ? b0.y : 0;
    r.sw_max_x = KIND == K_SW ? b0.x : 0;
    r.status = job_status(P, S.abort);
    r.kind = KIND;
    put_result(P, jb.index, r);
  }
}

template <int R, int NW>
__global__ void __launch_bounds__(NW * 32, NW == 4 ? GME_BATCH_MIN_BLOCKS : 1) batch_kernel(BatchParams P) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  BatchSmem<NW> &S = *reinterpret_cast<BatchSmem<NW> *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) S.abort = 0;
  __syncthreads();
  Waiter W(P.timeout_ns, &P.ctrl[8], &S.abort);
  // One kind after another, so that an SM runs one kind's code at a time (the
  // three kinds' loops do not fit the instruction cache together); within a kind
  // first the large pairs one per CTA, then the rest one per warp.  Each pair of
  // SMs starts at kind (smid / 2) % 3, so that the largest pairs of every kind start
  // at once instead of the last kind's at the end of the batch.  Measured: the two
  // SMs of a pair behave as sharing an instruction cache (starting each single SM at
  // its own kind lost 40%, each pair +10% on the 16384-pair batch, +17% on the
  // [32, 16384] mix).
  unsigned smid;
  asm("mov.u32 %0, %%smid;" : "=r"(smid));
  const int kfirst = (int)((smid >> 1) % 3u);
  for (int kk = 0; kk < 3; ++kk) {
    const int k = kfirst + kk < 3 ? kfirst + kk : kfirst + kk - 3;
    const int b0 = P.kb[k], nb = P.kb[k + 1] - b0, w0 = P.kw[k], nw = P.kw[k + 1] - w0;
    const int u0 = P.ku[k], nu = P.ku[k + 1] - u0;
    // phase 1: members of team jobs (claimed in order, so a member waits only on
    // members claimed before it, all of them running), then block jobs, one pair
    // per CTA; one call site per kind keeps the loop's code small
    if (threadIdx.x == 0) S.phase = 0;
    for (;;) {
      if (threadIdx.x == 0) {
        int job = -1;
        if (!S.abort && S.phase == 0) {
          const int t = nu ? atomicAdd(&P.ctrl[10 + k], 1) : nu;
          if (t < nu) job = t;
          else S.phase = 1;
        }
        if (!S.abort && S.phase == 1) {
          const int t = nb ? atomicAdd(&P.ctrl[2 * k], 1) : nb;
          if (t < nb) {
            job = t;
            // tags for the job's wrap rows, one per band group, never used before
            const int n2 = P.jobs_b[b0 + t].n2;
            S.gen = atomicAdd(P.gen, (unsigned)((n2 + 32 * R * NW - 1) / (32 * R * NW)));
          }
        }
        S.job = job;
      }
      for (int i = threadIdx.x; i < NW * (RING / CB); i += blockDim.x) (&S.tag[0][0])[i] = 0;
      for (int i = threadIdx.x; i < NW; i += blockDim.x) S.cons[i] = 0;
      __syncthreads();
      const int t = S.job;
      if (t < 0) break;
      BatchJob jb;
      int mt = 0, mT = 1;
      unsigned long long *wrap;
      unsigned tag0 = 0;
      TeamSlot *team = nullptr;
      if (S.phase == 0) {
        const int4 u = P.units[u0 + t];
        jb = P.jobs_t[u.x];
        mt = u.y;
        mT = u.z;
        wrap = P.twrap + (long long)u.x * 2 * P.stride;
        team = &P.team[u.x];
      } else {
        jb = P.jobs_b[b0 + t];
        wrap = P.wrap + (long long)blockIdx.x * 2 * P.stride;
        tag0 = S.gen;
      }
      switch (k) {
        case K_LCS: block_job<K_LCS, R, NW>(P, S, jb, warp, lane, W, mt, mT, wrap, tag0, team); break;
        case K_ED: block_job<K_ED, R, NW>(P, S, jb, warp, lane, W, mt, mT, wrap, tag0, team); break;
        default: block_job<K_SW, R, NW>(P, S, jb, warp, lane, W, mt, mT, wrap, tag0, team); break;
      }
      __syncthreads();
    }
    // phase 2: warp jobs, one pair per warp
    for (;;) {
      int t = 0;
      if (lane == 0) t = (S.abort || nw == 0) ? nw : atomicAdd(&P.ctrl[2 * k + 1], 1);
      t = __shfl_sync(FULL, t, 0);
      if (t >= nw) break;
      const BatchJob jb = P.jobs_w[w0 + t];
      switch (k) {
        case K_LCS: warp_job<K_LCS, R, NW>(P, S, jb, warp, lane, W); break;
        case K_ED: warp_job<K_ED, R, NW>(P, S, jb, warp, lane, W); break;
        default: warp_job<K_SW, R, NW>(P, S, jb, warp, lane, W); break;
      }
      if (*(volatile int *)&S.abort) break;
    }
    __syncthreads();
  }
}

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

static cudaError_t launch_batch(int NW, const BatchParams &P, int grid, cudaStream_t st) {
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

int batch_occupancy(int NW) {
  switch (NW) {
    case 4: return occupancy_t<4, 4>();
    case 8: return occupancy_t<4, 8>();
  }
  return 0;
}

bool batch_config_valid(int NW) { return NW == 4 || NW == 8; }

// Device bytes one pair adds to a batch: its symbols as the caller holds them, the
// staged copy (pads, b rounded up to whole band groups) and its descriptors.
long long batch_pair_bytes(long long n1, long long n2) {
  const long long staged = (PADL + n1 + PADR + 3) / 4 * 4 + (n2 + 32 * 4 * 8 - 1) / (32 * 4 * 8) * (32 * 4 * 8);
  return 4 * (n1 + n2) + 4 * staged + 2 * 32 + (long long)sizeof(BatchJob);
}

// CTAs of the batch kernel's grid.
long long batch_grid(int sms, int NW, int blocks_per_sm) {
  int occ = batch_occupancy(NW);
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
  return t;
}

int batch_plan(Workspace &ws, BatchArena &ar, const gme_pair *pairs, long long npairs,
               long long nsym, const BatchTuning &tune_given, cudaStream_t st,
               const long long *row_offs, const long long *col_offs) {
  constexpr int R = 4;
  const BatchTuning tune = batch_tuning_for(pairs, npairs, tune_given);
  const int NW = tune.warps_per_block;
  if (!batch_config_valid(NW)) return ws.fail_msg(ST_INVALID, "batch: warps_per_block must be 4 or 8");
  std::vector<int> blockj, warpj, teamj;
  ar.longj.clear();
  int occ0 = batch_occupancy(NW);
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
  // a team of T = groups / team_split (2..8) CTAs per team job; members claimed in order
  ar.h_units.clear();
  for (size_t j = 0; j < teamj.size(); ++j) {
    add(teamj[j], 32 * R * NW, slot++);
    const int G = (int)groups(pairs[teamj[j]]);
    const int T = std::max(2, std::min(8, G / std::max(1, tune.team_split)));
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
  ar.grid = grid0;
  ar.packed16 = tune.packed16 ? 1 : 0;
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
  if ((e = launch_batch(ar.NW, P, ar.grid, st)) != cudaSuccess) return ws.fail(e, "batch_kernel");
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
