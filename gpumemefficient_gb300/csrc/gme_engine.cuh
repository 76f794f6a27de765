// gme_engine.cuh -- the wavefront step engine shared by the plain and batched kernels.
//
// A warp owns 32*R rows of the table; lane t holds rows t*R..t*R+R-1.  At warp
// step s, lane t row r computes column x = s - t*R - r, so the warp sweeps one
// anti-diagonal per step and the R cells of a lane are independent.  The only
// value crossing lanes per step is the bottom cell of the lane above, carried by
// one __shfl_sync (the LCS-SHFL carry, LCS-SHFL/GPU_Hyperlane_Share.cu:339-361);
// lane 31 feeds the incoming row to lane 0 through the same shuffle.  Over a run
// of steps a warp's cells form a parallelogram: the reference's "hyperlane" tile
// (EditDistance/GPU_Hyperlane_Share.cu:320-496), kept in registers.
#pragma once

#include <type_traits>

#include "gme_common.cuh"

namespace gme {

constexpr unsigned FULL = 0xffffffffu;
constexpr int RING = 512;   // columns per ring (power of two)
constexpr int PADL = 261;   // left pad of the staged a[]: >= 32*8+5 and == 1 (mod 4)
constexpr int PADR = 352;   // right pad: reads reach base + C*j_end + 2C - 1 <= PADL + N + 32R + 2C

struct SwBest {
  int v;
  int pad;
  long long y, x;
};

__device__ __forceinline__ bool better(const SwBest &a, const SwBest &b) {
  // larger value first; among equals the first cell in row-major order
  if (a.v != b.v) return a.v > b.v;
  if (a.y != b.y) return a.y < b.y;
  return a.x < b.x;
}

// Shared-memory rings between the warps of a band: plain int32 values plus one
// tag word per C-column chunk (chunk index + 1), written with st.release after
// the chunk's values and read with ld.acquire before them.  The producer
// releases right after it has consumed its own symbol prefetch and the consumer
// acquires before issuing the next one, so no fence waits on a global load in
// flight.  Only the consumer's position is published back, for back-pressure.
// Tags are zeroed when a band starts.
constexpr int C = 16;  // wavefront steps (columns) per ring transaction
__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void lds_u64x4(const unsigned long long *p, unsigned long long (&e)[4]) {
  asm volatile("ld.volatile.shared.v2.u64 {%0,%1}, [%2];" : "=l"(e[0]), "=l"(e[1]) : "r"(smem_addr(p)));
  asm volatile("ld.volatile.shared.v2.u64 {%0,%1}, [%2+16];" : "=l"(e[2]), "=l"(e[3]) : "r"(smem_addr(p)));
}
__device__ __forceinline__ void sts_u64x4(unsigned long long *p, const unsigned long long (&e)[4]) {
  asm volatile("st.volatile.shared.v2.u64 [%0], {%1,%2};" :: "r"(smem_addr(p)), "l"(e[0]), "l"(e[1]) : "memory");
  asm volatile("st.volatile.shared.v2.u64 [%0+16], {%1,%2};" :: "r"(smem_addr(p)), "l"(e[2]), "l"(e[3]) : "memory");
}
__device__ __forceinline__ int lds_vol(const int *p) {
  int v;
  asm volatile("ld.volatile.shared.b32 %0, [%1];" : "=r"(v) : "r"(smem_addr(p)));
  return v;
}
__device__ __forceinline__ void sts_vol(int *p, int v) {
  asm volatile("st.volatile.shared.b32 [%0], %1;" :: "r"(smem_addr(p)), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long entry(int pos, int v) {
  return ((unsigned long long)(unsigned)(pos + 1) << 32) | (unsigned)v;
}

// Symbol loads: plain (coherent) global loads, cached in L1.  Not the read-only path:
// the served kernel runs while the host copies new pairs' symbols into its arena, and
// the read-only path may only read data that stays constant for a kernel's lifetime.
// Volatile, so that no load is moved ahead of the acquire that published its data.
__device__ __forceinline__ int4 ldg4(const int *p) {
  int4 v;
  asm volatile("ld.global.v4.b32 {%0,%1,%2,%3}, [%4];" : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w) : "l"(p));
  return v;
}
__device__ __forceinline__ int2 ldg2(const int *p) {
  int2 v;
  asm volatile("ld.global.v2.b32 {%0,%1}, [%2];" : "=r"(v.x), "=r"(v.y) : "l"(p));
  return v;
}

// n consecutive symbols from p into d[0..n): 16-byte loads when the lane's symbol base
// is 16-byte aligned (R a multiple of 4), else 8-byte loads (R = 2).
template <int R, int n>
__device__ __forceinline__ void ld_syms(const int *p, int *d) {
  if constexpr (R % 4 == 0) {
#pragma unroll
    for (int k = 0; k < n; k += 4) {
      const int4 q = ldg4(p + k);
      d[k] = q.x; d[k + 1] = q.y; d[k + 2] = q.z; d[k + 3] = q.w;
    }
  } else {
    static_assert(R % 2 == 0 && n % 2 == 0, "8-byte symbol loads need even R and n");
#pragma unroll
    for (int k = 0; k < n; k += 2) {
      const int2 q = ldg2(p + k);
      d[k] = q.x; d[k + 1] = q.y;
    }
  }
}

// ---------------------------------------------------------------------------
// C wavefront steps of one lane (R rows): one ring transaction per C steps.
//
// State entering step s: cur[r] = cells after step s-1, prv[r] = after step s-2,
// recv = the cell above row 0 for step s (lane t: lane t-1's bottom cell after
// step s-1; lane 0: the incoming row at column s), recv_prev = recv of step s-1.
// The diagonal terms need only values two steps old, so they are formed first;
// the bottom row is computed next and shuffled to the lane below at once, and
// the other rows are computed while the shuffle is in flight.
//
// Symbols: a circular window of 2C registers; symbol i (relative to the lane's
// base, column x = i - r + 1 for row r) lives at win[i mod 2C].  Chunk j reads
// i in [Cj-R+1, Cj+C-1] and, at step R (after the last read of the previous
// chunk's tail), loads the next chunk's C symbols into the other half.  PAR is
// j & 1, so every index is a compile-time constant and nothing is shifted.
//
// CHECKED: some cells of the warp fall outside 1 <= x <= n1 (ramp-in/out) and
// hold their value.  PADROWS: rows beyond n2 copy the row above, so the warp's
// bottom row equals row n2.
// ---------------------------------------------------------------------------
template <int KIND, int R, int PAR, bool CHECKED, bool PADROWS, int CH = C>
__device__ __forceinline__ void steps_chunk(const Rec<KIND> &rec, int (&cur)[R], int (&prv)[R],
                                            int &recv, int &recv_prev, int (&win)[2 * CH],
                                            const int *sym_next, const int (&bs)[R],
                                            const int (&inv)[CH], int (&outq)[CH], int s0, int lane,
                                            int N, unsigned padmask, int (&smax)[R], int (&sstep)[R]) {
  static_assert(R < CH, "the window refill at step R needs R < CH");
#pragma unroll
  for (int q = 0; q < CH; ++q) {
    if (q == R) ld_syms<R, CH>(sym_next, &win[(PAR ^ 1) * CH]);
    const int s = s0 + q;
    const int rcv = recv;  // the cell above row 0 for this step
    outq[q] = cur[R - 1];  // lane 31: bottom cell after step s-1 (column s-32R)
    int D[R];
#pragma unroll
    for (int r = 0; r < R; ++r)
      D[r] = (r ? prv[r - 1] : recv_prev) +
             (win[(PAR * CH + q - r + 2 * CH) % (2 * CH)] == bs[r] ? rec.ceq : rec.cne);
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
        // lane 31 feeds the incoming row to lane 0 through the same shuffle; the
        // chunk's last step sends nothing useful: lane 0 re-latches the next
        // chunk's first column from the validated ring values
        const int send = (lane == 31) ? inv[q + 1 < CH ? q + 1 : CH - 1] : v;
        recv = __shfl_sync(FULL, send, (lane + 31) & 31);  // for step s+1
        recv_prev = rcv;
      }
    }
#pragma unroll
    for (int r = 0; r < R; ++r) { prv[r] = cur[r]; cur[r] = nv[r]; }
  }
}

}  // namespace gme
