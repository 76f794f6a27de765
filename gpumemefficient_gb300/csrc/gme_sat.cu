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
//   1. the block's 32 x 128 values arrive in shared memory;
//   2. four lanes per row scan it serially, 32 columns each, and combine their
//      segment totals with shuffles; the lane holding the row total publishes it
//      (an "aggregate" word), looks back over the strips to its left -- adding their
//      aggregates until it meets an "inclusive" word, a strip whose carry is
//      complete -- and publishes its own inclusive carry.  Strip 0 starts from
//      D_y(0), formed from column 0.  This is the decoupled look-back of single-pass
//      prefix scans (Merrill and Garland, 2016) applied along each row: no strip
//      waits for the whole chain of strips to its left, only for their aggregates,
//      which every strip publishes without waiting for anything;
//   3. one lane per column walks the block's rows: t += prefix + the row's offset.
// Each step is latency-bound, so a CTA has two roles of 4 warps: the scan warps run
// step 2 for block k (its look-back one block later, from a word requested before
// the scan) while the column warps run step 3 for an earlier block, handing stages
// over through mbarriers.  Words are 64 bits: {tag, value}, one per strip and row.
// Each call takes two fresh tags from the context's counter, T for aggregates and
// T + 1 for inclusive carries, stored as the word's whole high half: the same format
// and the same counter as the plain kernel's band words, which share this scratch,
// so no word left by one call can pass for a word of a later call of either kind and
// nothing needs clearing.  The table is read and written once: 8 bytes per cell of
// HBM traffic.
//
// Two kernels move the blocks.  Any row stride (the reference's n1 + 3 is odd):
// sat_ws_kernel, the column warps loading their own columns by 4-byte cp.async into
// rows padded by a word per 32 columns (no bank conflicts).  Rows of a multiple of
// 16 bytes (ld % 4 == 0, the table 16-byte aligned): sat_tma_kernel on a 2D tensor
// map: the strips are then 16-byte aligned (columns 128 s .. 128 s + 127; strip 0
// holds the border column 0, written back unchanged), each 32 x 128 block arrives as
// four 32 x 32 boxes by cp.async.bulk.tensor with 128-byte swizzle (one thread issues
// them, an mbarrier per stage counts their bytes), the row scan reads 16-byte chunks
// of the swizzled rows and the column pass single words, both without bank
// conflicts, and the finished block leaves by four tensor stores from shared memory.
// Padding columns past n1 are written back as they were read; rows past n2 and
// columns past ld lie outside the map, so loads fill them with zeros and stores skip
// them.
#include <algorithm>
#include <cstdint>

#include <cuda.h>  // CUtensorMap and its enums; the encoder is fetched from the driver at run time

#include "gme_common.cuh"
#include "gme_internal.h"

namespace gme {

namespace {

// strip width (one column per column-pass thread) and rows per block: 128 x 32
// (measured before the two roles, at 32768 x 32768: 64-column strips 2.94 ms, their
// carries double; 64-row blocks 2.82 ms; 128 x 32 2.57 ms)
constexpr int SAT_W = 128;
constexpr int SAT_SEG = SAT_W / 32;            // 32-column segments per row
constexpr int SAT_RB = 32;
constexpr int SAT_PITCH = SAT_W + SAT_W / 32;  // a pad word per 32 columns
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


__device__ __forceinline__ int sat_col(int c) { return c + (c >> 5); }

__device__ __forceinline__ void cp_async4(int *dst, const int *src, bool valid) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(d), "l"(src), "r"(valid ? 4 : 0)
               : "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }


// ---------------------------------------------------------------------------
// The tensor-map kernel (16-byte rows).
// ---------------------------------------------------------------------------
constexpr int TMA_W = 128;                     // strip width: 4 boxes of 32 columns
constexpr int TMA_RB = 32;                     // rows per block
#ifndef GME_SAT_TMA_STAGES
#define GME_SAT_TMA_STAGES 6
#endif
constexpr int TMA_STAGES = GME_SAT_TMA_STAGES;
// blocks loaded ahead of the scan (a load also waits until its stage's last block has
// been stored).  Measured at 32768 x 32768 (stages, ahead): (6, 2) 1.97 ms; (6, 3) and
// (5, 2) 2.70 ms, the loads then wait on the stores; 7 stages leave room for one CTA per
// SM only, 3.03 ms
#ifndef GME_SAT_TMA_AHEAD
#define GME_SAT_TMA_AHEAD 2
#endif
constexpr int TMA_AHEAD = GME_SAT_TMA_AHEAD;
constexpr int TMA_BOX = 32 * 32 * 4;           // bytes of a 32 x 32 box
constexpr int TMA_STAGE = 4 * TMA_BOX;         // bytes of a block
constexpr size_t TMA_SMEM = (size_t)TMA_STAGES * TMA_STAGE + 1024;  // + alignment to 1024 bytes
static_assert(TMA_STAGES >= TMA_AHEAD + 3, "stages for the loads ahead, the scan, the finish, a store");

struct SatTmaParams {
  int *table;
  long long ld, n1, n2;
  int strips;                 // ceil((n1 + 1) / 128)
  unsigned long long *carry;  // as SatParams
  long long cstride;
  unsigned tag;
  int *ctrl;
  unsigned long long timeout_ns;
};

__device__ __forceinline__ unsigned su32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(su32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void tma_load(void *dst, const CUtensorMap *map, int x, int y, unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          su32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(su32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_store(const CUtensorMap *map, int x, int y, const void *src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(map), "r"(x),
               "r"(y), "r"(su32(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read1() { asm volatile("cp.async.bulk.wait_group.read 1;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Byte offset of element (r, c) of a 32 x 32 box loaded with 128-byte swizzle: the
// 16-byte chunk c / 4 of row r sits at chunk (c / 4) ^ (r % 8) of the row.
__device__ __forceinline__ int swz(int r, int c) { return r * 128 + ((((c >> 2) ^ (r & 7))) << 4) + ((c & 3) << 2); }

__device__ __forceinline__ void mbar_arrive(unsigned long long *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void bar_named(int id, int n) { asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory"); }

// Two roles of 4 warps each, so that one block's row scan and look-back overlap an
// earlier block's column pass.  Scan warps (0-3): request the left neighbour's word
// for block k - 1's rows, wait for block k's boxes, scan its rows in place and
// publish their aggregates, then look back for block k - 1 from that word, publish
// its inclusive carries, write its per-row offsets and arrive on scanned[stage];
// warp 0 also loads blocks ahead once the column warps have freed their stages.
// (Measured at 32768 x 32768: looking back right after the scan, 2.16 ms; one block
// later, 1.96 ms; two blocks later, 3.03 ms -- each strip's inclusive words then come
// so late that every strip to its right waits on them.)  Column warps (4-7): wait for scanned[stage],
// run the column pass, and their leader issues the block's tensor stores, then marks
// the previous block's stage free once its store has read it.
__global__ void __launch_bounds__(256) sat_tma_kernel(const __grid_constant__ CUtensorMap map, SatTmaParams P) {
  extern __shared__ __align__(16) unsigned char tma_raw[];
  __shared__ __align__(8) unsigned long long full[TMA_STAGES], scanned[TMA_STAGES], freed[TMA_STAGES];
  __shared__ unsigned s_off[TMA_STAGES][TMA_RB][4];  // per stage, row, box: carry + the box's row prefix
  __shared__ int s_strip, s_abort;
  unsigned char *smem = tma_raw + ((1024u - (su32(tma_raw) & 1023u)) & 1023u);
  const int tid = threadIdx.x, lane = tid & 31;
  const bool scan_role = tid < 128;
  if (tid == 0) {
    s_abort = 0;
    for (int i = 0; i < TMA_STAGES; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&scanned[i], 128);
      mbar_init(&freed[i], 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  Waiter W(P.timeout_ns, &P.ctrl[1], &s_abort);
  const long long n1 = P.n1, n2 = P.n2, ld = P.ld;
  const long long nblk = (n2 + TMA_RB - 1) / TMA_RB;
  // scan role: row rr of the block, box g.  The 8 lanes of a quarter-warp take 8 rows
  // of one box, so their 16-byte chunks (chunk ^ row % 8 under the swizzle) fall in 8
  // different bank groups; a row's 4 boxes are lanes l, l + 8, l + 16, l + 24
  const int rr = (lane & 7) + 8 * ((tid & 127) >> 5), g = lane >> 3;
  // column role: column ct of the strip, box cq, its column cc
  const int ct = tid & 127, cq = ct >> 5, cc = ct & 31;
  unsigned long long kbase = 0;   // blocks this CTA loaded before this strip
  unsigned long long issued = 0;  // blocks loaded (thread 0), consumed (scan role), in global count
  unsigned long long consumed = 0;
  bool failed = false;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_strip = s_abort ? P.strips : atomicAdd(&P.ctrl[0], 1);
    __syncthreads();
    const int s = s_strip;
    if (s >= P.strips) break;
    const long long X0 = (long long)s * TMA_W;
    unsigned long long *own = P.carry + (long long)s * P.cstride;
    const unsigned long long *left = P.carry + (long long)(s > 0 ? s - 1 : 0) * P.cstride;
    const bool publish = s + 1 < P.strips;
    const unsigned tag_agg = P.tag, tag_inc = P.tag + 1u;
    int nbox = 0;  // boxes of the strip inside the map (the others are never moved)
    while (nbox < 4 && X0 + 32 * nbox < ld) ++nbox;
    if (scan_role) {
      // loads block b once the stage's previous block has been stored and read: warp 0
      // waits (a bounded wait takes the whole warp), its lane 0 issues
      auto issue = [&](long long b) -> bool {
        const unsigned long long k = kbase + b;
        const int st = (int)(k % TMA_STAGES);
        if (k >= (unsigned long long)TMA_STAGES &&
            !W.wait([&] { return __all_sync(FULL, mbar_test(&freed[st], (unsigned)((k / TMA_STAGES - 1) & 1ull))); }))
          return false;
        if (lane == 0) {
          unsigned char *dst = smem + st * TMA_STAGE;
          mbar_expect_tx(&full[st], (unsigned)(nbox * TMA_BOX));
          for (int q = 0; q < nbox; ++q)
            tma_load(dst + q * TMA_BOX, &map, (int)(X0 + 32 * q), (int)(1 + b * TMA_RB), &full[st]);
        }
        issued = k + 1;
        return true;
      };
      if (tid < 32)
        for (long long b = 0; b < TMA_AHEAD && b < nblk && !failed; ++b) failed = !issue(b);
      // the block scanned last iteration and not yet looked back (its look-back runs
      // after this iteration's scan, from a word requested before it)
      unsigned p_inc = 0, p_excl = 0;  // this lane's row total, its box's exclusive prefix
      bool p_live = false;             // whether the lane holds a row total to publish
      long long p_y = 0;               // its row
      for (long long b = 0; b <= nblk && !failed; ++b) {
        const unsigned long long pre = (b >= 1 && s > 0 && p_live) ? ld_relaxed_gpu_u64(left + p_y) : 0ull;
        unsigned c_inc = 0, c_excl = 0;
        bool c_live = false;
        long long c_y = 0;
        if (b < nblk) {
          const unsigned long long k = kbase + b;
          const int st = (int)(k % TMA_STAGES);
          const unsigned par = (unsigned)((k / TMA_STAGES) & 1ull);
          if (!W.wait([&] { return __all_sync(FULL, mbar_test(&full[st], par)); })) {
            failed = true;
            break;
          }
          consumed = k + 1;
          if (tid < 32 && b + TMA_AHEAD < nblk && !issue(b + TMA_AHEAD)) {
            failed = true;
            break;
          }
          // row rr, columns X0 + 32 g .. + 31: serial prefix over 16-byte chunks, in place
          unsigned char *row = smem + st * TMA_STAGE + g * TMA_BOX;
          const long long xs = X0 + 32 * g;
          const bool interior = xs >= 1 && xs + 31 <= n1;
          unsigned pv[32];
          unsigned acc = 0;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            const int4 v = *reinterpret_cast<const int4 *>(row + swz(rr, 4 * q));
            const unsigned e[4] = {(unsigned)v.x, (unsigned)v.y, (unsigned)v.z, (unsigned)v.w};
#pragma unroll
            for (int w = 0; w < 4; ++w) {
              const long long xx = xs + 4 * q + w;
              acc += (interior || (xx >= 1 && xx <= n1)) ? e[w] : 0u;  // border and padding add nothing
              pv[4 * q + w] = acc;
            }
          }
          if (interior || xs + 31 <= n1) {
#pragma unroll
            for (int q = 0; q < 8; ++q)
              *reinterpret_cast<int4 *>(row + swz(rr, 4 * q)) =
                  make_int4((int)pv[4 * q], (int)pv[4 * q + 1], (int)pv[4 * q + 2], (int)pv[4 * q + 3]);
          } else {
#pragma unroll
            for (int i = 0; i < 32; ++i)
              if (xs + i <= n1) *reinterpret_cast<int *>(row + swz(rr, i)) = (int)pv[i];  // padding keeps its value
          }
          unsigned t = acc;
#pragma unroll
          for (int d = 1; d < 4; d <<= 1) {
            const unsigned u = __shfl_up_sync(FULL, t, 8 * d);
            if (g >= d) t += u;
          }
          c_inc = t;
          c_excl = t - acc;
          c_y = 1 + b * TMA_RB + rr;
          c_live = g == 3 && c_y <= n2;
          if (s > 0 && c_live && publish) st_relaxed_gpu_u64(own + c_y, ((unsigned long long)tag_agg << 32) | c_inc);
        }
        if (b >= 1) {
          // look-back for block b - 1, starting from the word requested above
          unsigned c = 0;
          bool done = !p_live;
          long long jq = s - 1;
          if (s == 0) {
            if (p_live) c = (unsigned)P.table[p_y * ld] - (unsigned)P.table[(p_y - 1) * ld];
          } else if (p_live) {
            const unsigned hi = (unsigned)(pre >> 32);
            if (hi == tag_inc) {
              c = (unsigned)pre;
              done = true;
            } else if (hi == tag_agg) {
              c = (unsigned)pre;
              --jq;
            }
          }
          if (s > 0 && !W.wait([&] {
                if (!done) {
                  const unsigned long long wv = ld_relaxed_gpu_u64(P.carry + jq * P.cstride + p_y);
                  const unsigned hi = (unsigned)(wv >> 32);
                  if (hi == tag_inc) {
                    c += (unsigned)wv;
                    done = true;
                  } else if (hi == tag_agg) {
                    c += (unsigned)wv;
                    --jq;
                  }
                }
                return __all_sync(FULL, done);
              })) {
            failed = true;
            break;
          }
          if (p_live && publish) st_relaxed_gpu_u64(own + p_y, ((unsigned long long)tag_inc << 32) | (c + p_inc));
          const int pst = (int)((kbase + b - 1) % TMA_STAGES);
          s_off[pst][rr][g] = __shfl_sync(FULL, c, (lane & 7) | 24) + p_excl;
          mbar_arrive(&scanned[pst]);  // (release: this thread's prefix row and offset)
        }
        p_inc = c_inc;
        p_excl = c_excl;
        p_live = c_live;
        p_y = c_y;
      }
    } else {
      const long long x = X0 + ct;  // 0 = the border, rewritten as read
      unsigned col = x <= n1 ? (unsigned)P.table[x] : 0u;  // row 0
      const bool leader = ct == 0;
      for (long long b = 0; b < nblk; ++b) {
        const unsigned long long k = kbase + b;
        const int st = (int)(k % TMA_STAGES);
        if (!W.wait([&] { return __all_sync(FULL, mbar_test(&scanned[st], (unsigned)((k / TMA_STAGES) & 1ull))); })) {
          failed = true;
          break;
        }
        // column pass: t[y][x] = t[y-1][x] + prefix + offset, in place
        const long long y0 = 1 + b * TMA_RB;
        const int rows = (int)(n2 - y0 + 1 < TMA_RB ? n2 - y0 + 1 : TMA_RB);
        unsigned char *tile = smem + st * TMA_STAGE;
        if (x <= n1) {
          unsigned char *cb = tile + cq * TMA_BOX;
#pragma unroll 8
          for (int r = 0; r < rows; ++r) {
            int *pt = reinterpret_cast<int *>(cb + swz(r, cc));
            col += (unsigned)*pt + s_off[st][r][cq];
            *pt = (int)col;
          }
        }
        fence_async_smem();  // these writes before the tensor stores read them
        bar_named(1, 128);   // the column warps' writes are all in
        if (leader) {
          for (int q = 0; q < nbox; ++q) tma_store(&map, (int)(X0 + 32 * q), (int)y0, tile + q * TMA_BOX);
          bulk_commit();
          if (b >= 1) {
            bulk_wait_read1();  // the previous block's store has read its stage
            mbar_arrive(&freed[(int)((k - 1) % TMA_STAGES)]);
          }
        }
      }
      if (leader && !failed && nblk >= 1) {
        bulk_wait_read0();
        mbar_arrive(&freed[(int)((kbase + nblk - 1) % TMA_STAGES)]);
      }
    }
    if (__syncthreads_or(failed)) {
      // a wait gave up: loads issued but not consumed must land before the CTA leaves
      // (bounded), and the stores must have read shared memory
      if (tid == 0)
        for (unsigned long long k = consumed; k < issued; ++k)
          for (int it = 0; it < (1 << 22) && !mbar_test(&full[k % TMA_STAGES], (unsigned)((k / TMA_STAGES) & 1ull)); ++it) {
          }
      if (tid == 128) bulk_wait_all();
      __syncthreads();
      break;
    }
    kbase += nblk;
  }
  if (tid == 128) bulk_wait_all();  // no store still reading shared memory at exit
}

// ---------------------------------------------------------------------------
// Any row stride (the reference's n1 + 3 included): the same two roles over the
// cp.async layout.  Column warps load their own columns of a block by 4-byte
// cp.async (zero-filled past n1 and n2) and let an mbarrier count the copies
// (cp.async.mbarrier.arrive); after a block's column pass, each thread reloads its
// column of that stage with the block WS_STAGES further on.  Scan warps scan the
// padded rows (a pad word per 32 columns: conflict-free) and look back as in the
// tensor-map kernel.
// ---------------------------------------------------------------------------
#ifndef GME_SAT_WS_STAGES
#define GME_SAT_WS_STAGES 6
#endif
constexpr int WS_STAGES = GME_SAT_WS_STAGES;
constexpr size_t WS_SMEM = (size_t)WS_STAGES * SAT_RB * SAT_PITCH * sizeof(int);
static_assert(SAT_W == 128 && SAT_RB == 32, "the two roles take 128 columns x 32 rows per block");

__device__ __forceinline__ void cp_async_mbar_arrive(unsigned long long *bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(su32(bar)) : "memory");
}

__global__ void __launch_bounds__(256) sat_ws_kernel(SatParams P) {
  extern __shared__ __align__(16) int ws_smem[];
  __shared__ __align__(8) unsigned long long full[WS_STAGES], scanned[WS_STAGES];
  __shared__ unsigned s_off[WS_STAGES][SAT_RB][SAT_SEG];
  __shared__ int s_strip, s_abort;
  __shared__ unsigned long long s_issued, s_consumed;  // blocks loaded / waited for (global count)
  const int tid = threadIdx.x, lane = tid & 31;
  const bool scan_role = tid < 128;
  if (tid == 0) {
    s_abort = 0;
    s_issued = s_consumed = 0;
    for (int i = 0; i < WS_STAGES; ++i) {
      mbar_init(&full[i], 128);
      mbar_init(&scanned[i], 128);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  Waiter W(P.timeout_ns, &P.ctrl[1], &s_abort);
  const long long n1 = P.n1, n2 = P.n2, ld = P.ld;
  const long long nblk = (n2 + SAT_RB - 1) / SAT_RB;
  const int rr = (tid & 127) >> 2, g = tid & 3;  // scan role: row rr, segment g (4 lanes per row)
  const int ct = tid & 127;                      // column role: the strip's column ct
  unsigned long long kbase = 0;
  bool failed = false;
  for (;;) {
    __syncthreads();
    if (tid == 0) s_strip = s_abort ? P.strips : atomicAdd(&P.ctrl[0], 1);
    __syncthreads();
    const int s = s_strip;
    if (s >= P.strips) break;
    const long long x0 = (long long)s * SAT_W;  // the strip's columns are x0 + 1 .. x0 + W
    unsigned long long *own = P.carry + (long long)s * P.cstride;
    const unsigned long long *left = P.carry + (long long)(s > 0 ? s - 1 : 0) * P.cstride;
    const bool publish = s + 1 < P.strips;
    const unsigned tag_agg = P.tag, tag_inc = P.tag + 1u;
    if (scan_role) {
      unsigned p_inc = 0, p_excl = 0;
      bool p_live = false;
      long long p_y = 0;
      for (long long b = 0; b <= nblk && !failed; ++b) {
        const unsigned long long pre = (b >= 1 && s > 0 && p_live) ? ld_relaxed_gpu_u64(left + p_y) : 0ull;
        unsigned c_inc = 0, c_excl = 0;
        bool c_live = false;
        long long c_y = 0;
        if (b < nblk) {
          const unsigned long long k = kbase + b;
          const int st = (int)(k % WS_STAGES);
          const unsigned par = (unsigned)((k / WS_STAGES) & 1ull);
          if (!W.wait([&] { return __all_sync(FULL, mbar_test(&full[st], par)); })) {
            failed = true;
            break;
          }
          if (tid == 0) s_consumed = k + 1;
          int *rowp = ws_smem + st * (SAT_RB * SAT_PITCH) + rr * SAT_PITCH + 33 * g;
          unsigned pv[32];
          unsigned acc = 0;
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            acc += (unsigned)rowp[i];  // zero past n1 (the copies zero-fill)
            pv[i] = acc;
          }
#pragma unroll
          for (int i = 0; i < 32; ++i) rowp[i] = (int)pv[i];
          unsigned t = acc;
#pragma unroll
          for (int d = 1; d < SAT_SEG; d <<= 1) {
            const unsigned u = __shfl_up_sync(FULL, t, d, SAT_SEG);
            if (g >= d) t += u;
          }
          c_inc = t;
          c_excl = t - acc;
          c_y = 1 + b * SAT_RB + rr;
          c_live = g == SAT_SEG - 1 && c_y <= n2;
          if (s > 0 && c_live && publish) st_relaxed_gpu_u64(own + c_y, ((unsigned long long)tag_agg << 32) | c_inc);
        }
        if (b >= 1) {
          unsigned c = 0;
          bool done = !p_live;
          long long jq = s - 1;
          if (s == 0) {
            if (p_live) c = (unsigned)P.table[p_y * ld] - (unsigned)P.table[(p_y - 1) * ld];
          } else if (p_live) {
            const unsigned hi = (unsigned)(pre >> 32);
            if (hi == tag_inc) {
              c = (unsigned)pre;
              done = true;
            } else if (hi == tag_agg) {
              c = (unsigned)pre;
              --jq;
            }
          }
          if (s > 0 && !W.wait([&] {
                if (!done) {
                  const unsigned long long wv = ld_relaxed_gpu_u64(P.carry + jq * P.cstride + p_y);
                  const unsigned hi = (unsigned)(wv >> 32);
                  if (hi == tag_inc) {
                    c += (unsigned)wv;
                    done = true;
                  } else if (hi == tag_agg) {
                    c += (unsigned)wv;
                    --jq;
                  }
                }
                return __all_sync(FULL, done);
              })) {
            failed = true;
            break;
          }
          if (p_live && publish) st_relaxed_gpu_u64(own + p_y, ((unsigned long long)tag_inc << 32) | (c + p_inc));
          const int pst = (int)((kbase + b - 1) % WS_STAGES);
          s_off[pst][rr][g] = __shfl_sync(FULL, c, (lane & ~(SAT_SEG - 1)) | (SAT_SEG - 1)) + p_excl;
          mbar_arrive(&scanned[pst]);
        }
        p_inc = c_inc;
        p_excl = c_excl;
        p_live = c_live;
        p_y = c_y;
      }
    } else {
      const long long x = x0 + 1 + ct;
      const bool xok = x <= n1;
      unsigned col = xok ? (unsigned)P.table[x] : 0u;  // row 0
      const int seg = ct >> 5;
      auto issue = [&](long long b) {
        const unsigned long long k = kbase + b;
        const int st = (int)(k % WS_STAGES);
        int *t = ws_smem + st * (SAT_RB * SAT_PITCH) + sat_col(ct);
        const long long y0 = 1 + b * SAT_RB;
        const int *src = P.table + y0 * ld + x;
#pragma unroll 8
        for (int r = 0; r < SAT_RB; ++r, src += ld) {
          const bool ok = xok && y0 + r <= n2;
          cp_async4(t + r * SAT_PITCH, ok ? src : P.table, ok);
        }
        cp_async_mbar_arrive(&full[st]);  // counts once this thread's copies have landed
        if (ct == 0) s_issued = k + 1;
      };
      for (long long b = 0; b < WS_STAGES && b < nblk; ++b) issue(b);
      for (long long b = 0; b < nblk; ++b) {
        const unsigned long long k = kbase + b;
        const int st = (int)(k % WS_STAGES);
        if (!W.wait([&] { return __all_sync(FULL, mbar_test(&scanned[st], (unsigned)((k / WS_STAGES) & 1ull))); })) {
          failed = true;
          break;
        }
        const long long y0 = 1 + b * SAT_RB;
        const int rows = (int)(n2 - y0 + 1 < SAT_RB ? n2 - y0 + 1 : SAT_RB);
        const int *cp = ws_smem + st * (SAT_RB * SAT_PITCH) + sat_col(ct);
        int *dst = P.table + y0 * ld + x;
        if (xok) {
          if (rows == SAT_RB) {
#pragma unroll 8
            for (int r = 0; r < SAT_RB; ++r, dst += ld) {
              col += (unsigned)cp[r * SAT_PITCH] + s_off[st][r][seg];
              __stcs(dst, (int)col);
            }
          } else {
            for (int r = 0; r < rows; ++r, dst += ld) {
              col += (unsigned)cp[r * SAT_PITCH] + s_off[st][r][seg];
              __stcs(dst, (int)col);
            }
          }
        }
        if (b + WS_STAGES < nblk) issue(b + WS_STAGES);  // this thread's column of the stage is read
      }
      cp_async_wait<0>();  // no copy of this strip still landing
    }
    if (__syncthreads_or(failed)) {
      // a wait gave up: every thread's copies land, and their arrivals on the stage
      // barriers (bounded), before the CTA leaves
      cp_async_wait<0>();
      __syncthreads();
      if (tid == 0)
        for (unsigned long long k = s_consumed; k < s_issued; ++k)
          for (int it = 0; it < (1 << 22) && !mbar_test(&full[k % WS_STAGES], (unsigned)((k / WS_STAGES) & 1ull)); ++it) {
          }
      __syncthreads();
      break;
    }
    kbase += nblk;
  }
}

using EncodeTiledFn = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                   const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// The driver's tensor-map encoder, or null (then every table takes the cp.async kernel).
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

__global__ void sat_status_kernel(const int *ctrl, int *d_status) { *d_status = ctrl[1]; }

}  // namespace

long long sat_scratch_words(long long n1, long long n2) {
  const long long W = SAT_W;
  const long long strips = std::max((n1 + W - 1) / W, (n1 + TMA_W) / TMA_W);  // either kernel's
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
  // 16-byte rows take the tensor-map kernel (its strips start at column 0)
  CUtensorMap map;
  bool tma = ld % 4 == 0 && (reinterpret_cast<uintptr_t>(d_table) & 15u) == 0 && encode_tiled() != nullptr &&
             ld < (1ll << 31) && n2 + 1 < (1ll << 31);
  if (tma) {
    const cuuint64_t dims[2] = {(cuuint64_t)ld, (cuuint64_t)(n2 + 1)};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 4};
    const cuuint32_t box[2] = {32, 32};
    const cuuint32_t estr[2] = {1, 1};
    tma = encode_tiled()(&map, CU_TENSOR_MAP_DATA_TYPE_INT32, 2, d_table, dims, strides, box, estr,
                         CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                         CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
  }
  const long long W = tma ? TMA_W : SAT_W;
  const long long strips = tma ? (n1 + W) / W : (n1 + W - 1) / W;
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
  const unsigned tag = ws.tag_next;
  ws.tag_next += 2;
  if ((e = cudaMemsetAsync(ws.ctrl, 0, 2 * sizeof(int), st)) != cudaSuccess)
    return ws.fail(e, "cudaMemsetAsync(sat ctrl)");
  // the shared-memory opt-in is per device (set again when the flag cannot tell)
  static bool attr_set[64] = {};
  const bool known = ws.device >= 0 && ws.device < 64;
  if (!known || !attr_set[ws.device]) {
    if ((e = cudaFuncSetAttribute(sat_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WS_SMEM)) !=
        cudaSuccess)
      return ws.fail(e, "cudaFuncSetAttribute(sat_ws_kernel)");
    if ((e = cudaFuncSetAttribute(sat_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TMA_SMEM)) !=
        cudaSuccess)
      return ws.fail(e, "cudaFuncSetAttribute(sat_tma_kernel)");
    if (known) attr_set[ws.device] = true;
  }
  int occ = 0;
  if (tma) {
    SatTmaParams P;
    P.table = d_table;
    P.ld = ld;
    P.n1 = n1;
    P.n2 = n2;
    P.strips = (int)strips;
    P.carry = ws.slots;
    P.cstride = cstride;
    P.tag = tag;
    P.ctrl = ws.ctrl;
    P.timeout_ns = timeout_ns;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sat_tma_kernel, 256, TMA_SMEM);
    const int grid = (int)std::min<long long>(strips, (long long)ws.sms * std::max(occ, 1));
    sat_tma_kernel<<<grid, 256, TMA_SMEM, st>>>(map, P);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "sat_tma_kernel");
  } else {
    SatParams P;
    P.table = d_table;
    P.ld = ld;
    P.n1 = n1;
    P.n2 = n2;
    P.strips = (int)strips;
    P.carry = ws.slots;
    P.cstride = cstride;
    P.tag = tag;
    P.ctrl = ws.ctrl;
    P.timeout_ns = timeout_ns;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sat_ws_kernel, 256, WS_SMEM);
    const int grid = (int)std::min<long long>(strips, (long long)ws.sms * std::max(occ, 1));
    sat_ws_kernel<<<grid, 256, WS_SMEM, st>>>(P);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "sat_ws_kernel");
  }
  if (d_status) {
    sat_status_kernel<<<1, 1, 0, st>>>(ws.ctrl, d_status);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "sat_status_kernel");
  }
  return ST_OK;
}

}  // namespace gme
