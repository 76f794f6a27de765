// gme_engine16.cuh -- the wavefront step with two cells per 32-bit register.
//
// For pairs whose scores provably fit 16 bits (and whose symbols fit 16 bits), a
// lane's four rows live in two registers: P0 = rows 0 and 2 (low, high half), P1 =
// rows 1 and 3.  One s16x2 DPX instruction (__vimax3_s16x2 / __vimin3_s16x2 /
// __viaddmax_s16x2[_relu]) updates two cells and another forms both diagonal terms.
//
// The neighbours line up by construction: the cell above rows 1 and 3 is rows 0 and
// 2 (P0 of the previous step), the cell above rows 0 and 2 is (the lane above's
// row 3, row 1) -- one __byte_perm splices the shuffled value into P1's low half.
// The diagonal works the same way one step further back.  The same recurrences as
// the int32 engine (gme_common.cuh), evaluated in 16-bit lanes: bit-exact whenever
// no value leaves [-32768, 32767], which the caller's bound guarantees, and the
// symbols lie in [0, 32767].
#pragma once

#include "gme_engine.cuh"

namespace gme {

__device__ __forceinline__ unsigned pack2(int v) {
  const unsigned h = (unsigned)v & 0xffffu;
  return h | (h << 16);
}

// Per-half arithmetic in native instructions.  The packed helpers of the CUDA SIMD
// family (__vadd2, __vcmpeq2, ...) are emulated with several integer instructions on
// this GPU; only the DPX s16x2 forms are single instructions.  So:
//   * a per-half add is __viaddmax_s16x2(a, b, 0x8000'8000) (max with -32768 = a + b);
//   * per-half symbol equality comes from x = a ^ b (halves < 0x8000): x + 0x7fff'7fff
//     sets bit 15 of a half exactly when that half of x is non-zero, and no carry
//     crosses into the other half.
constexpr unsigned MIN16 = 0x80008000u;
__device__ __forceinline__ unsigned ne01(unsigned pk, unsigned bp) {
  return ((((pk ^ bp) + 0x7fff7fffu) >> 15) & 0x00010001u);  // 1 in each half that differs
}

template <int KIND> struct Rec16;

template <> struct Rec16<K_LCS> {
  __device__ __forceinline__ explicit Rec16(const Scoring &) {}
  // D = diag + (eq ? 1 : 0)
  __device__ __forceinline__ unsigned dterm(unsigned diag, unsigned ne) const {
    return __viaddmax_s16x2(diag, ne ^ 0x00010001u, MIN16);
  }
  __device__ __forceinline__ unsigned cell(unsigned up, unsigned left, unsigned D) const {
    return __vimax3_s16x2(up, left, D);
  }
};

template <> struct Rec16<K_ED> {
  __device__ __forceinline__ explicit Rec16(const Scoring &) {}
  // stored form w = v - (x + y): D = diag + (eq ? -2 : -1) = diag + (0xfffe | ne) per half
  __device__ __forceinline__ unsigned dterm(unsigned diag, unsigned ne) const {
    return __viaddmax_s16x2(diag, ne | 0xfffefffeu, MIN16);
  }
  __device__ __forceinline__ unsigned cell(unsigned up, unsigned left, unsigned D) const {
    return __vimin3_s16x2(up, left, D);
  }
};

template <> struct Rec16<K_SW> {
  unsigned ma, mm, gap;  // match, mismatch, gap in both halves
  __device__ __forceinline__ explicit Rec16(const Scoring &s)
      : ma(pack2(s.match)), mm(pack2(s.mismatch)), gap(pack2(s.gap)) {}
  __device__ __forceinline__ unsigned dterm(unsigned diag, unsigned ne) const {
    const unsigned m = ne * 0xffffu;  // 0xffff in each half that differs
    return __viaddmax_s16x2(diag, (ma & ~m) | (mm & m), MIN16);
  }
  __device__ __forceinline__ unsigned cell(unsigned up, unsigned left, unsigned D) const {
    return __viaddmax_s16x2_relu(up, gap, __viaddmax_s16x2(left, gap, D));
  }
};

// Whether a pair's values stay inside 16 bits (with margin): LCS scores are at most
// min(n1, n2); ED's stored values lie in [-(n1 + n2) - 2, 0]; SW's in [-|m|, |m| *
// min(n1, n2)] with m the largest scoring constant.
__device__ __forceinline__ bool fits16(int kind, int n1, int n2, const Scoring &sc) {
  const int mn = min(n1, n2);
  if (kind == K_LCS) return mn <= 32000;
  if (kind == K_ED) return n1 + n2 <= 32000;
  const int m = max(max(abs(sc.match), abs(sc.mismatch)), abs(sc.gap));
  return (long long)m * (mn + 2) <= 32000;
}

// C steps of one lane, four rows, packed.  State entering step s: cur = cells after
// step s-1, prv = after s-2 (P0, P1); recv/recv_prev carry the cell above row 0 in
// their HIGH half (the lane above sends its P1, whose high half is its row 3; lane
// 31 sends the incoming row's value shifted up).  pk_prev is the packed symbol pair
// of rows 0 and 2 one step earlier, which is this step's pair for rows 1 and 3.
// xm1: x-1 of row 0's cell at step s0, in both entries (rows 1, 2, 3 are 1, 2, 3
// columns behind); a cell is inside the table when x-1 < nn = n1 as unsigned.  outq
// receives P1 after each step; lane 31's high halves are the band's bottom row.
template <int KIND, int PAR, bool CHECKED, bool PADROWS, int CH>
__device__ __forceinline__ void steps_chunk16(const Rec16<KIND> &rec, unsigned (&cur)[2], unsigned (&prv)[2],
                                              unsigned &recv, unsigned &recv_prev, unsigned &pk_prev,
                                              int (&win)[2 * CH], const int *sym_next,
                                              const unsigned (&bp)[2], const int (&inv)[CH],
                                              unsigned (&outq)[CH], int s0, int lane, unsigned nn,
                                              const unsigned (&xm1_0)[2], const unsigned (&pm)[2],
                                              unsigned (&smax)[2], unsigned (&sstep)[2]) {
  constexpr int R = 4;
  static_assert(R < CH, "the window refill at step R needs R < CH");
  const unsigned xm1[2] = {xm1_0[0], xm1_0[1]};
#pragma unroll
  for (int q = 0; q < CH; ++q) {
    if (q == R) {
#pragma unroll
      for (int i = 0; i < CH / 4; ++i) {
        const int4 v = ldg4(sym_next + 4 * i);
        const int h = (PAR ^ 1) * CH + 4 * i;
        win[h] = v.x; win[h + 1] = v.y; win[h + 2] = v.z; win[h + 3] = v.w;
      }
    }
    const int s = s0 + q;
    const unsigned rcv = recv;
    outq[q] = cur[1];
    // symbols of rows 0 and 2 at this step (columns x and x-2); rows 1 and 3 reuse
    // the pair of the previous step
    const unsigned pk0 = __byte_perm((unsigned)win[(PAR * CH + q + 2 * CH) % (2 * CH)],
                                     (unsigned)win[(PAR * CH + q - 2 + 2 * CH) % (2 * CH)], 0x5410);
    const unsigned pk1 = pk_prev;
    const unsigned D0 = rec.dterm(__byte_perm(recv_prev, prv[1], 0x5432), ne01(pk0, bp[0]));
    const unsigned D1 = rec.dterm(prv[0], ne01(pk1, bp[1]));
    const unsigned S = (unsigned)s * 0x10001u;
    // rows 1 and 3 first: row 3 goes to the lane below at once
    unsigned v1 = rec.cell(cur[0], cur[1], D1);
    if (CHECKED) {
      // rows 1 and 3 hold cells x = s - tR - 1 and s - tR - 3: inside when 1 <= x <= n1
      const unsigned ok = (xm1[1] + (unsigned)q - 1u < nn ? 0x0000ffffu : 0u) |
                          (xm1[1] + (unsigned)q - 3u < nn ? 0xffff0000u : 0u);
      v1 = (v1 & ok) | (cur[1] & ~ok);
    }
    if (PADROWS) v1 = (v1 & ~pm[1]) | (cur[0] & pm[1]);
    if (KIND == K_SW) {
      bool keep_hi, keep_lo;  // smax >= v: keep the step recorded for that half
      smax[1] = __vibmax_s16x2(smax[1], v1, &keep_hi, &keep_lo);
      const unsigned take = (keep_lo ? 0u : 0x0000ffffu) | (keep_hi ? 0u : 0xffff0000u);
      sstep[1] = (sstep[1] & ~take) | (S & take);
    }
    // lane 31 feeds the incoming row to lane 0 through the same shuffle
    const unsigned send = (lane == 31) ? ((unsigned)inv[q + 1 < CH ? q + 1 : CH - 1] << 16) : v1;
    recv = __shfl_sync(FULL, send, (lane + 31) & 31);
    recv_prev = rcv;
    const unsigned up0 = __byte_perm(rcv, cur[1], 0x5432);
    unsigned v0 = rec.cell(up0, cur[0], D0);
    if (CHECKED) {
      const unsigned ok = (xm1[0] + (unsigned)q < nn ? 0x0000ffffu : 0u) |
                          (xm1[0] + (unsigned)q - 2u < nn ? 0xffff0000u : 0u);
      v0 = (v0 & ok) | (cur[0] & ~ok);
    }
    if (PADROWS) v0 = (v0 & ~pm[0]) | (up0 & pm[0]);
    if (KIND == K_SW) {
      bool keep_hi, keep_lo;
      smax[0] = __vibmax_s16x2(smax[0], v0, &keep_hi, &keep_lo);
      const unsigned take = (keep_lo ? 0u : 0x0000ffffu) | (keep_hi ? 0u : 0xffff0000u);
      sstep[0] = (sstep[0] & ~take) | (S & take);
    }
    prv[0] = cur[0];
    prv[1] = cur[1];
    cur[0] = v0;
    cur[1] = v1;
    pk_prev = pk0;

  }
}

}  // namespace gme
