// gme_batch_kernel.cuh -- device code of the batched work-queue kernel: the job
// routines (warp jobs, block jobs, team members) and batch_kernel itself, templated on
// rows per lane R and warps per CTA NW.  Each translation unit instantiates its own
// shapes: gme_batch.cu the R = 4 kernels (and the served kernel, which shares the job
// routines), gme_batch_r2.cu the R = 2 ones, so that they compile in parallel.
#pragma once
#include <algorithm>
#include <climits>
#include <cstring>

#include "gme_engine.cuh"
#include "gme_engine16.cuh"
#include "gme_internal.h"

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
  // (b's staged segment starts 16-byte aligned and lane rows start at multiples of R,
  // so the lane's symbols are 16-byte aligned at R = 4 and 8-byte aligned at R = 2)
  ld_syms<R, R>(b_sym + (yl - 1), bs);
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

  // (PADL - 1 is a multiple of 4: the same alignment as b's)
  static_assert((PADL - 1) % 4 == 0, "a's window must share b's alignment");
  const int *sym = a_sym + (PADL - 1 - lane * R);
  int win[2 * CB];
  ld_syms<R, CB>(sym, win);
  ld_syms<R, R>(sym - R, &win[2 * CB - R]);
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
  if constexpr (R == 4) {
    if (p16) return sweep_band16<KIND>(sc, a_sym, b_sym, N, M, y0, lane, in, out, W, corner, tb, col_out);
  }
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


}  // namespace gme
