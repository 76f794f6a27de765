// gme_plain_kernel.cuh -- one alignment per call: the single persistent wavefront kernel.
//
// Included once per kind by gme_plain_lcs.cu, gme_plain_ed.cu and gme_plain_sw.cu
// (three translation units compiled in parallel); the host side is gme_plain.cu.
//
// Replaces the reference's per-tile-row launch loop (EditDistance/
// GPU_Hyperlane_Share.cu:752-764, one <<<1,1024>>> GPU() launch per tile row on
// SM-count streams, rows chained by the dev_lock spin counters at :110-129) and
// the full (n+pad)^2 int table it keeps in device memory (:698-713).
//
// Decomposition
//   * The table's rows are cut into BANDS of H = NW*32*R rows (the reference's
//     "tile row" / curBatch).  A band is owned by one CTA; CTAs claim bands in
//     order from an atomic ticket, so the CTA that waits on band b-1 always
//     waits on a CTA that is already running (no residency assumption).
//   * Inside a band each compute warp owns 32*R rows and each lane R of them
//     (a vertical strip).  At warp step s, lane t, row r computes column
//     x = s - t*R - r: the whole warp sweeps one anti-diagonal per step, so the
//     R cells of a lane are independent (instruction-level parallelism) and the
//     only value crossing lanes each step is the bottom cell of the lane above,
//     carried with one __shfl_sync (the LCS-SHFL idea, LCS-SHFL/
//     GPU_Hyperlane_Share.cu:339-361).  Over a run of steps a warp's cells form a
//     parallelogram: the reference's "hyperlane" tile (GPU_Hyperlane_Share.cu
//     :320-496), here kept in registers instead of a skewed shared tile.
//   * Warps of a band hand their bottom row to the next warp through a
//     shared-memory ring with release/acquire progress counters (replacing
//     moveToShare/moveToGlobal, :24-79).  Lane 31 feeds the incoming row to
//     lane 0 through the same shuffle.
//   * Bands hand their bottom row to the next band through a global buffer of
//     64-bit words {tag, value}.  The tag names the producing band, so a
//     consumer polls the data itself (one L2 round trip, no separate flag) and
//     the reference's non-atomic dev_lock += 1 / unbounded volatile spin becomes
//     a tagged, bounded wait.  One extra warp per CTA (the I/O warp) moves rows
//     between global memory and the first/last rings.
//   * Nothing of the table is kept: memory is O(n1) per band in flight, the
//     last row/column are produced on the fly.
#pragma once

#include <type_traits>

#include "gme_engine.cuh"
#include "gme_internal.h"

namespace gme {

// Column symbols are staged in one of two forms, chosen on the device for each call
// from the range of the pair's symbols (plain_range_kernel, plain_stage_kernel):
//   COST_CMP    the symbols themselves: a cell's cost is a compare and a select;
//   COST_TABLE  when every symbol of both sequences lies within 7 consecutive values
//               and the scoring constants fit 8 bits: each column holds a PRMT
//               selector of its code (symbol - min), each row a table of 8 signed
//               bytes (the cost of each code against the row's code, and 0 for code
//               7, the sentinel that fills the pads), and a cell's cost is one PRMT.
//               Cells left of column 1 then compute the border value (0) by
//               themselves, so the warps' ramp-in runs without range checks.
enum : int { COST_CMP = 0, COST_TABLE = 1 };
constexpr int SENTINEL = 7;
// PRMT selector of a table code: byte `code` of the 8-byte table, sign-extended
__host__ __device__ constexpr int cost_selector(int code) { return code * 0x1111 + 0x8880; }

struct PlainParams {
  const int *a_pad;   // a_pad[PADL + i] = a[i] (or its selector); pads: 0 (or the sentinel's)
  const int *a_pad2;  // a_pad shifted right by two (16-byte loads for lanes whose base is 8 mod 16)
  const int *b_pad;   // b_pad[i] = b[i] (or its code), length nbands*H
  int N, M;           // n1 (columns, over a), n2 (rows, over b)
  int H, nbands;
  int nslot;
  long long slot_stride;          // u64 words per slot
  unsigned long long *slots;      // nslot * slot_stride tagged words
  unsigned tag0;                  // tag of band b = tag0 + b
  int *ctrl;                      // [0] ticket, [1] status, [2]/[3] symbol range, [4] cost form
  int *last_col;                  // optional, device, n2+1 values
  SwBest *best;                   // one per CTA
  Scoring sc;
  unsigned long long timeout_ns;
};

// Columns per ring transaction: a chunk of PC = pc_of<KIND> wavefront steps between
// ring checks.  PLAIN_C (32) for LCS and ED; 16 for SW, whose per-row maxima leave
// too few registers for 32-step chunks.  Measured on GB300 at 4 rows per lane: SW
// 32768^2 3.84 ms at 16 against 5.25 ms at 32, ED 65536^2 3.99 ms at 32 against
// 4.33 ms at 16; at 2 rows per lane: SW 2.77 against 2.89 ms, ED 3.74 against 4.24 ms.
// The band slots' stride is a multiple of PLAIN_C, hence of every kind's chunk.
#ifndef GME_PLAIN_CHUNK_SW
#define GME_PLAIN_CHUNK_SW 16
#endif
template <int KIND> constexpr int pc_of = (KIND == K_SW && PLAIN_C > GME_PLAIN_CHUNK_SW) ? GME_PLAIN_CHUNK_SW : PLAIN_C;

// I/O warps per CTA: 2 = one for the incoming row (global slot -> ring 0), one for
// the outgoing row (last ring -> global slot); 1 = one warp doing both in turn.
#ifndef GME_PLAIN_IO_WARPS
#define GME_PLAIN_IO_WARPS 2
#endif
constexpr int PLAIN_IO = GME_PLAIN_IO_WARPS;
static_assert(PLAIN_IO == 1 || PLAIN_IO == 2, "one or two I/O warps");
static_assert(PLAIN_C % 16 == 0 && RING % PLAIN_C == 0, "chunks of 16-byte groups that tile the ring");

template <int NW, int PC> struct __align__(16) PlainSmem {
  int ring[NW + 1][RING];
  int tag[NW + 1][RING / PC];
  int cons[NW + 1];
  // where lanes other than 31 put their stores of the outgoing row (16-byte groups)
  alignas(16) int sink[NW][PC];
  int band;
  int abort;
  SwBest best[NW + PLAIN_IO];
};

__device__ __forceinline__ void st_release_cta_if(bool p, int *a, int v) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n @q st.release.cta.shared.b32 [%1], %2;\n}" ::"r"((unsigned)p),
               "r"(smem_addr(a)), "r"(v) : "memory");
}
__device__ __forceinline__ void sts_vol_if(bool p, int *a, int v) {
  asm volatile("{\n .reg .pred q;\n setp.ne.u32 q, %0, 0;\n @q st.volatile.shared.b32 [%1], %2;\n}" ::"r"((unsigned)p),
               "r"(smem_addr(a)), "r"(v) : "memory");
}
__device__ __forceinline__ int prmt(unsigned lo, unsigned hi, int sel) {
  int d;
  asm("prmt.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(lo), "r"(hi), "r"(sel));
  return d;
}

// n consecutive symbols from a 16-byte aligned p into d[0..n)
template <int n>
__device__ __forceinline__ void ld_syms16(const int *p, int *d) {
#pragma unroll
  for (int k = 0; k < n; k += 4) {
    const int4 q = ldg4(p + k);
    d[k] = q.x; d[k + 1] = q.y; d[k + 2] = q.z; d[k + 3] = q.w;
  }
}

// 16-byte store of the outgoing row: lane 31 writes into the ring, the other lanes
// into the warp's sink.  No "memory" clobber, so that the compiler may place the
// incoming-row loads across it; the chunk's release (which has one) orders these
// stores before the tag.
__device__ __forceinline__ void sts4(unsigned addr, int a, int b, int c, int d) {
  asm volatile("st.shared.v4.b32 [%0], {%1,%2,%3,%4};" ::"r"(addr), "r"(a), "r"(b), "r"(c), "r"(d));
}
__device__ __forceinline__ void lds4(const int *p, int *d) {
  const int4 q = *reinterpret_cast<const int4 *>(p);
  d[0] = q.x; d[1] = q.y; d[2] = q.z; d[3] = q.w;
}

// ---------------------------------------------------------------------------
// PC wavefront steps of one lane (R rows), the plain kernel's form of the engine in
// gme_engine.cuh (same state, same order: the bottom row first and shuffled at once).
// COST_TABLE: rt0/rt1 are the row's cost table, win holds selectors; COST_CMP: rt0 is
// the row's symbol, win holds symbols.  The window refill (the next chunk's PC
// symbols at step R) uses 16-byte loads from sym_next; the incoming row's tag for
// the next chunk is read one step later (tag_ahead -> tag_next).
//
// The incoming row (inc: this chunk's PC columns in the ring, already validated;
// head: its first 4) is read in 16-byte groups four steps ahead of lane 31's
// shuffles to lane 0, and the next chunk's first group is read into head at step
// PC-4, after its tag (valid if that tag matches).  The outgoing row (lane 31's
// bottom cell, one column per step) is stored in 16-byte groups every 4 steps at
// out (OUT).  No lane holds a whole chunk of either row in registers.
// ---------------------------------------------------------------------------
template <int KIND, int R, int COST, int PAR, bool CHECKED, bool PADROWS, bool OUT>
__device__ __forceinline__ void plain_steps(const Rec<KIND> &rec, int (&cur)[R], int (&prv)[R], int &recv,
                                            int &recv_prev, int (&win)[2 * pc_of<KIND>], const int *sym_next,
                                            const unsigned (&rt0)[R], const unsigned (&rt1)[R],
                                            const int *inc, int (&head)[4], const int *inc_next,
                                            const int *tag_ahead, int &tag_next, unsigned out, int s0, int lane,
                                            int N, unsigned padmask, int (&smax)[R], int (&sstep)[R]) {
  constexpr int PC = pc_of<KIND>;
  static_assert(R + 1 < PC - 4 && PC % 4 == 0, "the tag read precedes the next chunk's first group");
  int iv[PC];  // the incoming row of this chunk (registers: only the groups in flight)
#pragma unroll
  for (int k = 0; k < 4; ++k) iv[k] = head[k];
  int oq[PC];  // the outgoing row of this chunk, stored every 4 steps
#pragma unroll
  for (int q = 0; q < PC; ++q) {
    if (q % 4 == 0) {
      if (q + 4 < PC) lds4(inc + q + 4, &iv[q + 4]);
      else lds4(inc_next, head);
    }
    if (q == R) ld_syms16<PC>(sym_next, &win[(PAR ^ 1) * PC]);
    if (q == R + 1) tag_next = ld_acquire_cta(tag_ahead);
    const int s = s0 + q;
    const int rcv = recv;
    oq[q] = cur[R - 1];  // lane 31: bottom cell after step s-1 (column s-32R)
    if (OUT && q % 4 == 3) sts4(out + 4 * (q - 3), oq[q - 3], oq[q - 2], oq[q - 1], oq[q]);
    // the incoming row at column s+1, which lane 31 passes to lane 0 for the next step;
    // the chunk's last step sends nothing useful: lane 0 re-latches the next chunk's
    // first column from the validated ring
    const int nxt = (q + 1 < PC) ? iv[q + 1] : 0;
    int D[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int sym = win[(PAR * PC + q - r + 2 * PC) % (2 * PC)];
      const int c = (COST == COST_TABLE) ? prmt(rt0[r], rt1[r], sym)
                                         : (sym == (int)rt0[r] ? rec.ceq : rec.cne);
      D[r] = (r ? prv[r - 1] : recv_prev) + c;
    }
    int nv[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
      const int r = (k == 0) ? R - 1 : k - 1;  // bottom row first
      const int up = r ? cur[r - 1] : rcv;
      int v = rec.cell(up, cur[r], D[r]);
      if (CHECKED) {
        const int x = s - lane * R - r;
        if ((unsigned)(x - 1) >= (unsigned)N) v = cur[r];
      }
      if (PADROWS) {
        if (padmask & (1u << r)) v = up;
      }
      if (KIND == K_SW) {
        if (v > smax[r]) { smax[r] = v; sstep[r] = s; }
      }
      nv[r] = v;
      if (k == 0) {
        const int send = (lane == 31) ? nxt : v;
        recv = __shfl_sync(FULL, send, (lane + 31) & 31);  // for step s+1
        recv_prev = rcv;
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) { prv[r] = cur[r]; cur[r] = nv[r]; }
  }
}

// One compute warp sweeping its 32*R rows of a band across all N columns.  Every
// warp hands its bottom row to the next ring (the last active warp's ring is
// drained to global memory by the band's I/O warp).
//
// The incoming row's tag runs one chunk ahead: during chunk j the warp already reads
// the tag of chunk j+1, so at the start of chunk j+1 the check is a register
// compare.  In steady state this makes each warp trail the one above by one extra
// chunk (PC steps).  The values are read from the ring 16 bytes at a time, ahead of use.
//
// Chunk boundaries carry no divergent branch: every lane stores the outgoing row
// every 4 steps (lane 31 into the ring, the others into a per-warp sink) and the
// release of its tag and the consumption count are predicated stores of lane 31.
template <int KIND, int R, int NW, int COST>
__device__ void compute_band(const PlainParams &P, PlainSmem<NW, pc_of<KIND>> &S, int band, int warp, int lane,
                             Waiter &W, SwBest &tb) {
  constexpr int PC = pc_of<KIND>;
  const Rec<KIND> rec(P.sc);
  const int N = P.N, M = P.M;
  const int yl = band * P.H + warp * 32 * R + lane * R + 1;  // first row of this lane
  int cur[R], prv[R], smax[R], sstep[R];
  unsigned rt0[R], rt1[R];
  {
    int bs[R];
    ld_syms<R, R>(P.b_pad + (yl - 1), bs);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      if (COST == COST_TABLE) {
        // the row's cost table: byte k = cost of code k against the row's code,
        // byte 7 (the sentinel) = 0
        const unsigned ne = (unsigned)(rec.cne & 0xff) * 0x01010101u;
        const unsigned eq = (unsigned)(rec.ceq & 0xff);
        const int cb = bs[r] & 7;  // pad rows hold code 0
        unsigned lo = ne, hi = ne & 0x00ffffffu;
        if (cb < 4) lo = (lo & ~(0xffu << (8 * cb))) | (eq << (8 * cb));
        else hi = (hi & ~(0xffu << (8 * (cb - 4)))) | (eq << (8 * (cb - 4)));
        rt0[r] = lo;
        rt1[r] = hi;
      } else {
        rt0[r] = (unsigned)bs[r];
        rt1[r] = 0;
      }
    }
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

  // Symbol window for chunk 0: i in [0, PC) at win[0..PC), i in [-R, 0) at
  // win[2PC-R..2PC).  sym[i] is this lane's symbol index i (column i - r + 1 for row
  // r); its base is 16-byte aligned: PADL - 1 is a multiple of 4, and lanes whose
  // offset R*lane is 2 mod 4 read the copy shifted by two.
  const int base = PADL - 1 - lane * R;
  const int *sym = ((base & 3) == 0) ? P.a_pad + base : P.a_pad2 + base + 2;
  int win[2 * PC];
  ld_syms16<PC>(sym, win);
  ld_syms<R, R>(sym - R, &win[2 * PC - R]);
#pragma unroll
  for (int k = PC; k < 2 * PC - R; ++k) win[k] = 0;

  const int *ring_in = S.ring[warp];
  int *ring_out = S.ring[warp + 1];
  int *tag_in = S.tag[warp], *tag_out = S.tag[warp + 1];
  int *cons_in = &S.cons[warp], *cons_out = &S.cons[warp + 1];
  const unsigned sink = smem_addr(S.sink[warp]);
  int cons_seen = 0;
  int recv = 0, recv_prev = 0;
  int tag_next = ld_acquire_cta(&tag_in[0]);
  int head[4];  // the incoming row's first 4 columns of the next chunk
  lds4(ring_in, head);

  // OUT: 1 = the chunk's outgoing columns start at or after 0, 0 = before (no output),
  // 2 = decided per chunk (pad warps)
  auto chunk = [&](int j, auto par, auto checked, auto padrows, auto out) -> bool {
    constexpr int PAR = decltype(par)::value;
    constexpr bool CK = decltype(checked)::value, PD = decltype(padrows)::value;
    constexpr int OUT = decltype(out)::value;
    const int s0 = PC * j;
    if (s0 <= N && !__all_sync(FULL, tag_next == j + 1)) {
      // the read-ahead found the chunk not yet written: wait for it.  Lanes may read
      // the tag at different moments; the decision is warp-uniform so that no lane
      // leaves the wait alone.
      auto ready = [&] { return __all_sync(FULL, ld_acquire_cta(&tag_in[j & (RING / PC - 1)]) == j + 1); };
      if (!W.wait(ready)) return false;
      lds4(&ring_in[s0 & (RING - 1)], head);
    }
    // columns before s0 are consumed: their slots may be refilled
    sts_vol_if(lane == 31, cons_in, s0);
    const int *inc = &ring_in[s0 & (RING - 1)];
    if (lane == 0) recv = head[0];  // the incoming row's column s0 (see plain_steps)
    // outgoing row: columns pos..pos+PC-1, pos = s0 - 32R, stored 4 columns at a time
    const int pos = s0 - 32 * R;
    const bool out_on = OUT == 1 || (OUT == 2 && pos >= 0);
    if (OUT != 0 && out_on && pos + PC - RING > cons_seen) {
      if (!W.wait([&] {
            cons_seen = __shfl_sync(FULL, lds_vol(cons_out), 0);
            return cons_seen >= pos + PC - RING;
          }))
        return false;
    }
    const unsigned outp = (lane == 31 && out_on) ? smem_addr(&ring_out[pos & (RING - 1)]) : sink;
    plain_steps<KIND, R, COST, PAR, CK, PD, OUT != 0>(rec, cur, prv, recv, recv_prev, win, sym + s0 + PC, rt0,
                                                      rt1, inc, head, &ring_in[(s0 + PC) & (RING - 1)],
                                                      &tag_in[(j + 1) & (RING / PC - 1)], tag_next, outp, s0,
                                                      lane, N, padmask, smax, sstep);
    if (out_on) st_release_cta_if(lane == 31, &tag_out[(pos / PC) & (RING / PC - 1)], pos / PC + 1);
    return true;
  };

  using T = std::true_type;
  using F = std::false_type;
  using P0 = std::integral_constant<int, 0>;
  using P1 = std::integral_constant<int, 1>;
  // chunks ja..jb (inclusive) in parity order
  auto range = [&](int ja, int jb, auto ck, auto pd, auto out) -> bool {
    int j = ja;
    if (j <= jb && (j & 1)) {
      if (!chunk(j, P1{}, ck, pd, out)) return false;
      ++j;
    }
    for (; j + 1 <= jb; j += 2) {
      if (!chunk(j, P0{}, ck, pd, out)) return false;
      if (!chunk(j + 1, P1{}, ck, pd, out)) return false;
    }
    if (j <= jb && !chunk(j, P0{}, ck, pd, out)) return false;
    return true;
  };
  using O0 = std::integral_constant<int, 0>;
  using O1 = std::integral_constant<int, 1>;
  using O2 = std::integral_constant<int, 2>;
  // last chunk: its output covers column N (outputs lag the inputs by 32R columns)
  const int j_end = (N + 32 * R) / PC;
  // chunks 0 .. j_out-1 produce no output (their columns are left of column 0)
  const int j_out = min((32 * R) / PC, j_end + 1);
  // chunks 0 .. j_full have every cell of the warp at x <= N (none when N < PC - 1)
  const int j_full = (N >= PC - 1) ? min((N - PC + 1) / PC, j_end) : -1;
  if (padwarp) {
    if (!range(0, j_end, T{}, T{}, O2{})) return;
  } else {
    // ramp-in: cells left of column 1 hold the border value.  In the table form they
    // compute it by themselves, so only chunks that also reach past column N need the
    // range check; the compare form checks them all
    const int j_in = (COST == COST_TABLE) ? min(j_out - 1, j_full) : -1;
    if (!range(0, j_in, F{}, F{}, O0{})) return;
    if (!range(j_in + 1, j_out - 1, T{}, F{}, O0{})) return;
    // steady chunks: every cell of the warp has 1 <= x <= N for all PC steps
    const int j_hi = max(j_full, j_out - 1);
    if (!range(j_out, j_hi, F{}, F{}, O1{})) return;
    // ramp-out: cells beyond column N hold their value at column N
    if (!range(j_hi + 1, j_end, T{}, F{}, O1{})) return;
  }

  // every row now holds its value at column N (cells beyond N were held)
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const long long y = yl + r;
    if (y <= M) {
      if (P.last_col) P.last_col[y] = Rec<KIND>::to_v(cur[r], N, y);
      if (KIND == K_SW && smax[r] > 0) {
        SwBest c = {smax[r], 0, y, (long long)(sstep[r] - lane * R - r)};
        if (better(c, tb)) tb = c;
      }
    }
  }
}

// The I/O warps of a band.  Incoming row: forwards the band above's tagged global
// words (or, for band 0, the table's top border) into ring 0 and releases each
// completed chunk.  Outgoing row: copies the chunks the last compute warp has
// released from ring `active` to the band's global slot as tagged words.  Role 0
// does both in one loop (the global poll issued first and consumed last, so its L2
// round trip overlaps the drain); role 1 only the incoming row, role 2 only the
// outgoing one, so that a released chunk leaves within a shared-memory poll rather
// than within a global one.
template <int KIND, int NW>
__device__ void io_band(const PlainParams &P, PlainSmem<NW, pc_of<KIND>> &S, int band, int active, int lane,
                        int role) {
  constexpr int PC = pc_of<KIND>;
  const int N1 = P.N + 1;
  const unsigned long long *src =
      band > 0 ? P.slots + (long long)((band - 1) % P.nslot) * P.slot_stride : nullptr;
  unsigned long long *dst = P.slots + (long long)(band % P.nslot) * P.slot_stride;
  const unsigned src_tag = P.tag0 + (unsigned)(band - 1);
  const unsigned long long dst_tag = (unsigned long long)(P.tag0 + (unsigned)band) << 32;
  int *ring0 = S.ring[0];
  const int *ringo = S.ring[active];
  const int *tago = S.tag[active];
  int in_pos = role == 2 ? N1 : 0, out_pos = role == 1 ? N1 : 0;
  unsigned idle = 0;
  unsigned long long deadline = 0;

  while (in_pos < N1 || out_pos < N1) {
    bool moved = false;
    // (a) incoming: issue the poll of up to 128 columns (consumed in (c))
    const int space = RING - (in_pos - __shfl_sync(FULL, lds_vol(&S.cons[0]), 0));
    const int want = in_pos < N1 ? min(N1 - in_pos, space) : 0;
    const int p = in_pos + 4 * lane;
    unsigned long long w[4] = {0, 0, 0, 0};
    if (want > 0 && band > 0 && 4 * lane < want) {
      const volatile unsigned long long *sp = src + p;
      asm volatile("ld.volatile.global.v2.u64 {%0,%1}, [%2];" : "=l"(w[0]), "=l"(w[1]) : "l"(sp));
      asm volatile("ld.volatile.global.v2.u64 {%0,%1}, [%2+16];" : "=l"(w[2]), "=l"(w[3]) : "l"(sp));
    }
    // (b) outgoing: lane k looks at chunk out_pos/PC + k
    if (out_pos < N1) {
      const int c = out_pos / PC + lane;
      bool ready = false;
      if (lane < 8 && c * PC < N1) ready = ld_acquire_cta(&tago[c & (RING / PC - 1)]) == c + 1;
      const unsigned rm = __ballot_sync(FULL, ready);
      const int nch = (rm == FULL) ? 32 : (__ffs(~rm) - 1);
      if (nch > 0) {
        if (lane < nch) {
#pragma unroll
          for (int k = 0; k < PC; k += 4) {
            const int4 q = *reinterpret_cast<const int4 *>(&ringo[(c * PC + k) & (RING - 1)]);
            volatile unsigned long long *dp = dst + c * PC + k;
            const unsigned long long w0 = dst_tag | (unsigned)q.x, w1 = dst_tag | (unsigned)q.y;
            const unsigned long long w2 = dst_tag | (unsigned)q.z, w3 = dst_tag | (unsigned)q.w;
            asm volatile("st.volatile.global.v2.u64 [%0], {%1,%2};" :: "l"(dp), "l"(w0), "l"(w1) : "memory");
            asm volatile("st.volatile.global.v2.u64 [%0+16], {%1,%2};" :: "l"(dp), "l"(w2), "l"(w3) : "memory");
          }
        }
        out_pos = min(out_pos + nch * PC, N1);
        __syncwarp();
        if (lane == 0) sts_vol(&S.cons[active], out_pos);
        moved = true;
      }
    }
    // (c) incoming: take the valid prefix of the poll and release completed chunks
    if (want > 0) {
      int v[4];
      bool ok = 4 * lane < want;
      if (band == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) v[k] = Rec<KIND>::top(p + k, P.sc.ed_rule);
      } else {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          v[k] = (int)(unsigned)w[k];
          if (p + k < N1 && (unsigned)(w[k] >> 32) != src_tag) ok = false;
        }
      }
      const unsigned okm = __ballot_sync(FULL, ok);
      const int lanes_ok = (okm == FULL) ? 32 : (__ffs(~okm) - 1);
      const int n = min(4 * lanes_ok, want);
      if (n > 0) {
        if (4 * lane < n)
          *reinterpret_cast<int4 *>(&ring0[p & (RING - 1)]) = make_int4(v[0], v[1], v[2], v[3]);
        __syncwarp();
        // release the chunks this round completed (the last one may be partial)
        const int c0 = in_pos / PC;
        const int c1 = (in_pos + n >= N1) ? (N1 + PC - 1) / PC : (in_pos + n) / PC;
        if (lane < c1 - c0) st_release_cta(&S.tag[0][(c0 + lane) & (RING / PC - 1)], c0 + lane + 1);
        in_pos += n;
        moved = true;
      }
    }
    if (moved) {
      idle = 0;
    } else {
      // bounded wait: nothing could move this round
      if (idle == 0) deadline = globaltimer_ns() + P.timeout_ns;
      if ((++idle & 15u) == 0) {
        int give = 0;
        if (*(volatile int *)&S.abort) give = 1;
        else if (ld_relaxed_gpu_s32(&P.ctrl[1]) != 0) give = 2;
        else if (globaltimer_ns() > deadline) give = 3;
        give = __shfl_sync(FULL, give, 0);
        if (give) {
          if (give == 3) atomicCAS(&P.ctrl[1], 0, ST_TIMEOUT);
          S.abort = 1;
          return;
        }
      }
      if (role == 2) __nanosleep(32);
      else if (band == 0 || in_pos >= N1) __nanosleep(128);
    }
  }
}

template <int KIND, int R, int NW>
__global__ void __launch_bounds__((NW + PLAIN_IO) * 32, 1) plain_kernel(PlainParams P) {
  constexpr int PC = pc_of<KIND>;
  __shared__ PlainSmem<NW, PC> S;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) S.abort = 0;
  __syncthreads();
  Waiter W(P.timeout_ns, &P.ctrl[1], &S.abort);
  SwBest tb = {0, 0, 0, 0};
  const bool table = P.ctrl[4] != 0;  // the staging kernel's choice of cost form
  for (;;) {
    if (threadIdx.x == 0) {
      S.band = S.abort ? P.nbands : atomicAdd(&P.ctrl[0], 1);
#pragma unroll
      for (int k = 0; k <= NW; ++k) S.cons[k] = 0;
    }
    for (int i = threadIdx.x; i < (NW + 1) * (RING / PC); i += blockDim.x) (&S.tag[0][0])[i] = 0;
    __syncthreads();
    const int band = S.band;
    if (band >= P.nbands) break;
    const int rows_left = P.M - band * P.H;
    const int active = min(NW, (rows_left + 32 * R - 1) / (32 * R));
    if (warp < NW) {
      if (warp < active) {
        if (table) compute_band<KIND, R, NW, COST_TABLE>(P, S, band, warp, lane, W, tb);
        else compute_band<KIND, R, NW, COST_CMP>(P, S, band, warp, lane, W, tb);
      }
    } else {
      io_band<KIND, NW>(P, S, band, active, lane, PLAIN_IO == 1 ? 0 : warp - NW + 1);
    }
    __syncthreads();
  }
  if (KIND == K_SW) {
    // block reduction of the per-thread first maxima
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      SwBest c;
      c.v = __shfl_down_sync(FULL, tb.v, o);
      c.y = __shfl_down_sync(FULL, tb.y, o);
      c.x = __shfl_down_sync(FULL, tb.x, o);
      c.pad = 0;
      if (better(c, tb)) tb = c;
    }
    if (lane == 0) S.best[warp] = tb;
    __syncthreads();
    if (threadIdx.x == 0) {
      SwBest b = S.best[0];
      for (int k = 1; k < NW + PLAIN_IO; ++k)
        if (better(S.best[k], b)) b = S.best[k];
      P.best[blockIdx.x] = b;
    }
  }
}

template <int KIND, int R, int NW>
inline cudaError_t launch_plain_t(const PlainParams &P, int grid, cudaStream_t st) {
  plain_kernel<KIND, R, NW><<<grid, (NW + PLAIN_IO) * 32, 0, st>>>(P);
  return cudaGetLastError();
}

// the plain kernel of one kind at one of the supported shapes (plain_config_valid)
template <int KIND>
cudaError_t launch_plain_k(int R, int NW, const PlainParams &P, int grid, cudaStream_t st) {
  if (R == 2 && NW == 4) return launch_plain_t<KIND, 2, 4>(P, grid, st);
  if (R == 2 && NW == 8) return launch_plain_t<KIND, 2, 8>(P, grid, st);
  if (R == 4 && NW == 4) return launch_plain_t<KIND, 4, 4>(P, grid, st);
  if (R == 4 && NW == 8) return launch_plain_t<KIND, 4, 8>(P, grid, st);
  return cudaErrorInvalidValue;
}

}  // namespace gme
