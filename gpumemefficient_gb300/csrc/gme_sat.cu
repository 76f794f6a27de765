// gme_sat.cu -- the summed-area table (SAT/GPU_Hyperlane_Share.cu) as one persistent
// launch over column strips.
//
// The reference's `SOR(n1, n2, table, tX, tY)` (SAT/GPU_Hyperlane_Share.cu:241-338)
// updates, in place, rows 1..n2 and columns 1..n1 of a table of row length
// n1 + 3 (paddX1 = 1, paddX2 = 2) with
//     t[y][x] = t[y][x-1] + t[y-1][x] + t[y][x] - t[y-1][x-1]        (:169, :196, :231)
// in int arithmetic (wrapping on the GPU); row 0 and column 0 keep their inputs.
//
// The recurrence telescopes.  With D_y(x) = t[y][x] - t[y-1][x] (the new table):
//     D_y(x) = D_y(0) + sum_{j=1..x} A[y][j],   D_y(0) = A[y][0] - A[y-1][0],
//     t[y][x] = t[y-1][x] + D_y(x).
// So a CTA that owns a strip of W = 128 columns needs, for each row, a single
// number from the strips to its left (D_y at the last column before the strip) and
// keeps its own columns' running sums t[y-1][x] in registers.  Per block of 32 rows:
//   1. the block's 32 x 128 values arrive in shared memory by 4-byte cp.async (any
//      row stride), four blocks ahead of the one being computed;
//   2. four lanes per row scan it serially, 32 columns each, and combine their
//      segment totals with two shuffles; the lane holding the row total publishes
//      it (an "aggregate" word), looks back over the strips to its left -- adding
//      their aggregates until it meets an "inclusive" word, a strip whose carry is
//      complete -- and publishes its own inclusive carry.  Strip 0 starts from
//      D_y(0), formed from column 0.  This is the decoupled look-back of single-pass
//      prefix scans (Merrill and Garland, 2016) applied along each row: no strip
//      waits for the whole chain of strips to its left, only for their aggregates,
//      which every strip publishes without waiting for anything.  The lanes write
//      D_y(x) back in place;
//   3. one lane per column walks the block's rows: t += D, stored to the table.
// A pad word per 32 columns keeps both shared-memory patterns free of bank
// conflicts.  Words are 64 bits: {tag, value}, one per strip and row.  Each call
// takes two fresh tags from the context's counter, T for aggregates and T + 1 for
// inclusive carries, stored as the word's whole high half: the same format and the
// same counter as the plain kernel's band words, which share this scratch, so no
// word left by one call can pass for a word of a later call of either kind and
// nothing needs clearing.  The table is read and written once: 8 bytes per cell of
// HBM traffic.
#include <algorithm>

#include "gme_common.cuh"
#include "gme_internal.h"

namespace gme {

namespace {

#ifndef GME_SAT_WIDTH
#define GME_SAT_WIDTH 128
#endif
#ifndef GME_SAT_STAGES
#define GME_SAT_STAGES 5
#endif
constexpr int SAT_W = GME_SAT_WIDTH;         // strip width: one column per thread (64 or 128)
constexpr int SAT_THREADS = SAT_W;
constexpr int SAT_SEG = SAT_W / 32;          // 32-column segments per row
#ifndef GME_SAT_ROWS
#define GME_SAT_ROWS 32
#endif
// rows per block (measured at 32768 x 32768: 64 rows with 2 or 3 stages 2.82-2.84 ms
// against 2.57 ms for 32 rows with 5)
constexpr int SAT_RB = GME_SAT_ROWS;
constexpr int SAT_RPT = SAT_RB / (SAT_THREADS / SAT_SEG);  // rows per row-scan lane group
// blocks in shared memory (measured at 32768 x 32768: 3 stages 2.76 ms, 5 stages
// 2.58 ms; 64-column strips 2.94-2.95 ms, their carries double)
constexpr int SAT_STAGES = GME_SAT_STAGES;
constexpr int SAT_PITCH = SAT_W + SAT_W / 32;  // a pad word per 32 columns
static_assert(SAT_W == 64 || SAT_W == 128, "strip width 64 or 128");
static_assert(SAT_RB == 32 || SAT_RB == 64, "32 or 64 rows per block");
constexpr unsigned FULL = 0xffffffffu;

struct SatParams {
  int *table;
  long long ld, n1, n2;
  int strips;
  unsigned long long *carry;  // carry[s * cstride + y]: strip s's word for row y
  long long cstride;
  unsigned tag;  // aggregates carry tag, inclusive carries tag + 1
  int *ctrl;     // [0] strip ticket, [1] status
  unsigned long long timeout_ns;
};

constexpr size_t SAT_SMEM = (size_t)SAT_STAGES * SAT_RB * SAT_PITCH * sizeof(int);

__device__ __forceinline__ int sat_col(int c) { return c + (c >> 5); }

__device__ __forceinline__ void cp_async4(int *dst, const int *src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

__global__ void __launch_bounds__(SAT_THREADS) sat_kernel(SatParams P) {
  extern __shared__ __align__(16) int sat_smem[];
  __shared__ int s_strip, s_abort;
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  if (tid == 0) s_abort = 0;
  Waiter W(P.timeout_ns, &P.ctrl[1], &s_abort);
  const long long n1 = P.n1, n2 = P.n2, ld = P.ld;
  const long long nblk = (n2 + SAT_RB - 1) / SAT_RB;
  // row-scan role: row rr of the block, segment g (columns 32g .. 32g+31)
  const int rr = tid / SAT_SEG, g = tid % SAT_SEG;
  for (;;) {
    __syncthreads();
    // strips are claimed in order: the strips to the left are always held by running CTAs
    if (tid == 0) s_strip = s_abort ? P.strips : atomicAdd(&P.ctrl[0], 1);
    __syncthreads();
    const int s = s_strip;
    if (s >= P.strips) break;
    const long long x0 = (long long)s * SAT_W;  // the strip's columns are x0 + 1 .. x0 + W
    const long long x = x0 + 1 + tid;           // this thread's column (load and column pass)
    const bool xok = x <= n1;
    unsigned col = xok ? (unsigned)P.table[x] : 0u;  // row 0
    unsigned long long *own = P.carry + (long long)s * P.cstride;
    const bool publish = s + 1 < P.strips;
    const unsigned tag_agg = P.tag, tag_inc = P.tag + 1u;  // the words' high halves
    auto issue = [&](long long b) {
      if (b < nblk) {
        int *t = sat_smem + (int)(b % SAT_STAGES) * (SAT_RB * SAT_PITCH) + sat_col(tid);
        const long long y0 = 1 + b * SAT_RB;
        const int *src = P.table + y0 * ld + x;
#pragma unroll 8
        for (int r = 0; r < SAT_RB; ++r, src += ld) {
          const bool ok = xok && y0 + r <= n2;
          cp_async4(t + r * SAT_PITCH, ok ? src : P.table, ok);
        }
      }
      cp_async_commit();  // one group per block (empty past the end) keeps the count uniform
    };
#pragma unroll
    for (int b = 0; b < SAT_STAGES - 1; ++b) issue(b);
    bool failed = false;
    for (long long b = 0; b < nblk; ++b) {
      cp_async_wait<SAT_STAGES - 2>();  // this thread's copies of block b have landed
      __syncthreads();                  // (1) everyone's have; the stage of block b-1 is free
      // (no abort test here: the abort word is only set inside the look-back wait,
      // between barriers (1) and (2), and barrier (2) decides for the whole CTA)
      issue(b + SAT_STAGES - 1);
      int *tile = sat_smem + (int)(b % SAT_STAGES) * (SAT_RB * SAT_PITCH);
      const long long y0 = 1 + b * SAT_RB;
      // 2. rows rr + 32q, segment g: serial prefix, then the row's segments combined
      unsigned pv[SAT_RPT][32], inc[SAT_RPT], seg_excl[SAT_RPT], c[SAT_RPT];
      bool live[SAT_RPT], done[SAT_RPT];
      long long yq[SAT_RPT], jq[SAT_RPT];
#pragma unroll
      for (int q = 0; q < SAT_RPT; ++q) {
        const int *rowp = tile + (rr + 32 * q) * SAT_PITCH + 33 * g;
        unsigned acc = 0;
#pragma unroll
        for (int i = 0; i < 32; ++i) { acc += (unsigned)rowp[i]; pv[q][i] = acc; }
        unsigned t = acc;
#pragma unroll
        for (int d = 1; d < SAT_SEG; d <<= 1) {
          const unsigned u = __shfl_up_sync(FULL, t, d, SAT_SEG);
          if (g >= d) t += u;
        }
        inc[q] = t;
        seg_excl[q] = t - acc;
        // the row's last segment holds the row total (rows beyond n2 and the other
        // lanes read nothing and always agree)
        yq[q] = y0 + rr + 32 * q;
        live[q] = g == SAT_SEG - 1 && yq[q] <= n2;
        c[q] = 0;
        done[q] = !live[q];
        jq[q] = s - 1;
        if (s == 0) {
          if (live[q]) c[q] = (unsigned)P.table[yq[q] * ld] - (unsigned)P.table[(yq[q] - 1) * ld];
        } else if (live[q] && publish) {
          st_relaxed_gpu_u64(own + yq[q], ((unsigned long long)tag_agg << 32) | inc[q]);
        }
      }
      // look back for every row of this lane at once
      if (s > 0) {
        const bool ok = W.wait([&] {
#pragma unroll
          for (int q = 0; q < SAT_RPT; ++q) {
            if (!done[q]) {
              const unsigned long long wv = ld_relaxed_gpu_u64(P.carry + jq[q] * P.cstride + yq[q]);
              const unsigned hi = (unsigned)(wv >> 32);
              if (hi == tag_inc) {
                c[q] += (unsigned)wv;
                done[q] = true;
              } else if (hi == tag_agg) {
                c[q] += (unsigned)wv;
                --jq[q];  // an aggregate: strip j's own total; keep looking left
              }
            }
          }
          bool all = true;
#pragma unroll
          for (int q = 0; q < SAT_RPT; ++q) all = all && done[q];
          return __all_sync(FULL, all);
        });
        if (!ok) failed = true;
      }
#pragma unroll
      for (int q = 0; q < SAT_RPT; ++q) {
        if (live[q] && publish && !failed)
          st_relaxed_gpu_u64(own + yq[q], ((unsigned long long)tag_inc << 32) | (c[q] + inc[q]));
        const unsigned off = __shfl_sync(FULL, c[q], (lane & ~(SAT_SEG - 1)) | (SAT_SEG - 1)) + seg_excl[q];
        int *rowp = tile + (rr + 32 * q) * SAT_PITCH + 33 * g;
#pragma unroll
        for (int i = 0; i < 32; ++i) rowp[i] = (int)(pv[q][i] + off);
      }
      // (2) D_y(x) in place.  The barrier also ORs every thread's own failure, so all
      // warps take the same branch even when one gives up while another is between
      // the barriers
      if (__syncthreads_or(failed)) break;
      // 3. column pass: t[y][x] = t[y-1][x] + D_y(x)
      const int *cp = tile + sat_col(tid);
      int *dst = P.table + y0 * ld + x;
      const int rows = (int)(n2 - y0 + 1 < SAT_RB ? n2 - y0 + 1 : SAT_RB);
      if (xok) {
        if (rows == SAT_RB) {
#pragma unroll 8
          for (int r = 0; r < SAT_RB; ++r, dst += ld) {
            col += (unsigned)cp[r * SAT_PITCH];
            __stcs(dst, (int)col);
          }
        } else {
          for (int r = 0; r < rows; ++r, dst += ld) {
            col += (unsigned)cp[r * SAT_PITCH];
            __stcs(dst, (int)col);
          }
        }
      }
    }
    cp_async_wait<0>();  // nothing of this strip still in flight into shared memory
  }
}

__global__ void sat_status_kernel(const int *ctrl, int *d_status) { *d_status = ctrl[1]; }

}  // namespace

long long sat_scratch_words(long long n1, long long n2) {
  const long long W = SAT_W;
  const long long strips = (n1 + W - 1) / W;
  return strips * ((n2 + 1 + 3) / 4 * 4);
}

// In place on a table of (n2 + 1) rows (0..n2) of `ld` ints, columns 0..n1 read,
// rows 1..n2 x columns 1..n1 rewritten.  d_status (optional) receives the run's
// status (0, or ST_TIMEOUT when a bounded wait gave up).
int sat_run(Workspace &ws, int *d_table, long long n1, long long n2, long long ld, int *d_status,
            cudaStream_t st, unsigned long long timeout_ns) {
  cudaError_t e;
  if (n1 < 0 || n2 < 0 || ld < n1 + 1) return ws.fail_msg(ST_INVALID, "sat: need n1, n2 >= 0 and ld >= n1 + 1");
  if (n1 == 0 || n2 == 0) {
    if (d_status && (e = cudaMemsetAsync(d_status, 0, sizeof(int), st)) != cudaSuccess)
      return ws.fail(e, "cudaMemsetAsync(sat status)");
    return ST_OK;
  }
  const long long W = SAT_W;
  const long long strips = (n1 + W - 1) / W;
  if (strips > (1ll << 30)) return ws.fail_msg(ST_INVALID, "sat: table too wide");
  const long long cstride = (n2 + 1 + 3) / 4 * 4;
  int rc = ws.reserve(0, 0, strips * cstride, 0);
  if (rc != ST_OK) return rc;
  // two tags per call from the counter the plain kernel's band words use: clear the
  // words before the 32-bit counter wraps
  if ((unsigned long long)ws.tag_next + 3ull >= 0xffffffffull) {
    if ((e = cudaMemsetAsync(ws.slots, 0, ws.slots_bytes, st)) != cudaSuccess)
      return ws.fail(e, "cudaMemsetAsync(slots)");
    ws.tag_next = 1;
  }
  SatParams P;
  P.table = d_table;
  P.ld = ld;
  P.n1 = n1;
  P.n2 = n2;
  P.strips = (int)strips;
  P.carry = ws.slots;
  P.cstride = cstride;
  P.tag = ws.tag_next;
  ws.tag_next += 2;
  P.ctrl = ws.ctrl;
  P.timeout_ns = timeout_ns;
  if ((e = cudaMemsetAsync(ws.ctrl, 0, 2 * sizeof(int), st)) != cudaSuccess)
    return ws.fail(e, "cudaMemsetAsync(sat ctrl)");
  // the shared-memory opt-in is per device (set again when the flag cannot tell)
  static bool attr_set[64] = {};
  const bool known = ws.device >= 0 && ws.device < 64;
  if (!known || !attr_set[ws.device]) {
    if ((e = cudaFuncSetAttribute(sat_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SAT_SMEM)) != cudaSuccess)
      return ws.fail(e, "cudaFuncSetAttribute(sat_kernel)");
    if (known) attr_set[ws.device] = true;
  }
  int occ = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sat_kernel, SAT_THREADS, SAT_SMEM);
  const int grid = (int)std::min<long long>(strips, (long long)ws.sms * std::max(occ, 1));
  sat_kernel<<<grid, SAT_THREADS, SAT_SMEM, st>>>(P);
  ws.launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "sat_kernel");
  if (d_status) {
    sat_status_kernel<<<1, 1, 0, st>>>(ws.ctrl, d_status);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "sat_status_kernel");
  }
  return ST_OK;
}

}  // namespace gme
