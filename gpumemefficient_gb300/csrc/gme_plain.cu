// gme_plain.cu -- one alignment per call: a single persistent wavefront kernel.
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
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <type_traits>

#include "gme_engine.cuh"
#include "gme_internal.h"
#include "gme_tuned_plain.h"

namespace gme {

struct PlainParams {
  const int *a_pad;  // a_pad[PADL + i] = a[i]
  const int *b_pad;  // b_pad[i] = b[i], length nbands*H
  int N, M;          // n1 (columns, over a), n2 (rows, over b)
  int H, nbands;
  int nslot;
  long long slot_stride;          // u64 words per slot
  unsigned long long *slots;      // nslot * slot_stride tagged words
  unsigned tag0;                  // tag of band b = tag0 + b
  int *ctrl;                      // [0] ticket, [1] status
  int *last_col;                  // optional, device, n2+1 values
  SwBest *best;                   // one per CTA
  Scoring sc;
  unsigned long long timeout_ns;
};

template <int NW> struct __align__(16) PlainSmem {
  int ring[NW + 1][RING];
  int tag[NW + 1][RING / C];
  int cons[NW + 1];
  int band;
  int abort;
  SwBest best[NW + 1];
};

// One compute warp sweeping its 32*R rows of a band across all N columns.  Every
// warp hands its bottom row to the next ring (the last active warp's ring is
// drained to global memory by the band's I/O warp).
//
// The incoming row runs one chunk ahead: during chunk j the warp already reads
// the tag and values of chunk j+1, so at the start of chunk j+1 the check is a
// register compare.  In steady state this makes each warp trail the one above
// by one extra chunk (C steps), which buys the latency of the shared loads.
template <int KIND, int R, int NW>
__device__ void compute_band(const PlainParams &P, PlainSmem<NW> &S, int band, int warp, int lane,
                             Waiter &W, SwBest &tb) {
  const Rec<KIND> rec(P.sc);
  const int N = P.N, M = P.M;
  const int yl = band * P.H + warp * 32 * R + lane * R + 1;  // first row of this lane
  int bs[R], cur[R], prv[R], smax[R], sstep[R];
  ld_syms<R, R>(P.b_pad + (yl - 1), bs);
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

  // Symbol window for chunk 0: i in [0, C) at win[0..C), i in [-R, 0) at win[2C-R..2C).
  const int *sym = P.a_pad + (PADL - 1 - lane * R);  // sym[i]: symbol index i of this lane
  int win[2 * C];
  ld_syms<R, C>(sym, win);
  ld_syms<R, R>(sym - R, &win[2 * C - R]);
#pragma unroll
  for (int k = C; k < 2 * C - R; ++k) win[k] = 0;

  const int *ring_in = S.ring[warp];
  int *ring_out = S.ring[warp + 1];
  int *tag_in = S.tag[warp], *tag_out = S.tag[warp + 1];
  int *cons_in = &S.cons[warp], *cons_out = &S.cons[warp + 1];
  int cons_seen = 0;
  int recv = 0, recv_prev = 0;

  // incoming-row buffers by chunk parity: ib[PAR] holds chunk j, ib[PAR^1] chunk j+1
  int ib[2][C];
  int tag_next;
  auto load_in = [&](int j, int (&dst)[C]) {
#pragma unroll
    for (int k = 0; k < C; k += 4) {
      const int4 q = *reinterpret_cast<const int4 *>(&ring_in[(C * j + k) & (RING - 1)]);
      dst[k] = q.x; dst[k + 1] = q.y; dst[k + 2] = q.z; dst[k + 3] = q.w;
    }
  };
  tag_next = ld_acquire_cta(&tag_in[0]);
  load_in(0, ib[0]);

  auto chunk = [&](int j, auto par, auto checked, auto padrows) -> bool {
    constexpr int PAR = decltype(par)::value;
    constexpr bool CK = decltype(checked)::value, PD = decltype(padrows)::value;
    int(&inv)[C] = ib[PAR];
    const int s0 = C * j;
    __syncwarp();
    if (s0 <= N && !__all_sync(FULL, tag_next == j + 1)) {
      // the read-ahead found the chunk not yet written: wait for it, then reread.
      // Lanes may read the tag at different moments; the decision is warp-uniform
      // so that no lane leaves the wait alone.
      auto ready = [&] { return __all_sync(FULL, ld_acquire_cta(&tag_in[j & (RING / C - 1)]) == j + 1); };
      if (!W.wait(ready)) return false;
      load_in(j, inv);
    }
    if (lane == 31) sts_vol(cons_in, s0 + C);
    if (lane == 0) recv = inv[0];  // the incoming row's column s0 (see steps_chunk)
    // read ahead: chunk j+1
    tag_next = ld_acquire_cta(&tag_in[(j + 1) & (RING / C - 1)]);
    load_in(j + 1, ib[PAR ^ 1]);

    int outq[C];
    steps_chunk<KIND, R, PAR, CK, PD>(rec, cur, prv, recv, recv_prev, win, sym + s0 + C, bs, inv,
                                      outq, s0, lane, N, padmask, smax, sstep);
    // outgoing row: columns pos..pos+C-1, pos = s0 - 32R (chunk j - 2R)
    const int pos = s0 - 32 * R;
    if (pos >= 0) {
      if (pos + C - RING > cons_seen) {
        if (!W.wait([&] {
              cons_seen = __shfl_sync(FULL, lds_vol(cons_out), 0);
              return cons_seen >= pos + C - RING;
            }))
          return false;
      }
      if (lane == 31) {
#pragma unroll
        for (int k = 0; k < C; k += 4)
          *reinterpret_cast<int4 *>(&ring_out[(pos + k) & (RING - 1)]) =
              make_int4(outq[k], outq[k + 1], outq[k + 2], outq[k + 3]);
        st_release_cta(&tag_out[(pos / C) & (RING / C - 1)], pos / C + 1);
      }
    }
    return true;
  };

  using T = std::true_type;
  using F = std::false_type;
  using P0 = std::integral_constant<int, 0>;
  using P1 = std::integral_constant<int, 1>;
  // chunks ja..jb (inclusive) in parity order
  auto range = [&](int ja, int jb, auto ck, auto pd) -> bool {
    int j = ja;
    if (j <= jb && (j & 1)) {
      if (!chunk(j, P1{}, ck, pd)) return false;
      ++j;
    }
    for (; j + 1 <= jb; j += 2) {
      if (!chunk(j, P0{}, ck, pd)) return false;
      if (!chunk(j + 1, P1{}, ck, pd)) return false;
    }
    if (j <= jb && !chunk(j, P0{}, ck, pd)) return false;
    return true;
  };
  // last chunk: its output covers column N (outputs lag the inputs by 32R columns)
  const int j_end = (N + 32 * R) / C;
  if (padwarp) {
    if (!range(0, j_end, T{}, T{})) return;
  } else {
    // steady chunks: every cell of the warp has 1 <= x <= N for all C steps
    const int j_lo = min((32 * R) / C, j_end + 1);
    const int j_hi = max(min((N - C + 1) / C, j_end), j_lo - 1);
    if (!range(0, j_lo - 1, T{}, F{})) return;
    if (!range(j_lo, j_hi, F{}, F{})) return;
    if (!range(j_hi + 1, j_end, T{}, F{})) return;
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

// The I/O warp of a band.  Incoming row: forwards the band above's tagged global
// words (or, for band 0, the table's top border) into ring 0 and releases each
// completed chunk.  Outgoing row: copies the chunks the last compute warp has
// released from ring `active` to the band's global slot as tagged words.  The
// global poll is issued first and consumed last, so its L2 round trip overlaps
// the drain.
template <int KIND, int NW>
__device__ void io_band(const PlainParams &P, PlainSmem<NW> &S, int band, int active, int lane) {
  const int N1 = P.N + 1;
  const unsigned long long *src =
      band > 0 ? P.slots + (long long)((band - 1) % P.nslot) * P.slot_stride : nullptr;
  unsigned long long *dst = P.slots + (long long)(band % P.nslot) * P.slot_stride;
  const unsigned src_tag = P.tag0 + (unsigned)(band - 1);
  const unsigned long long dst_tag = (unsigned long long)(P.tag0 + (unsigned)band) << 32;
  int *ring0 = S.ring[0];
  const int *ringo = S.ring[active];
  const int *tago = S.tag[active];
  int in_pos = 0, out_pos = 0;
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
    // (b) outgoing: lane k looks at chunk out_pos/C + k
    if (out_pos < N1) {
      const int c = out_pos / C + lane;
      bool ready = false;
      if (lane < 8 && c * C < N1) ready = ld_acquire_cta(&tago[c & (RING / C - 1)]) == c + 1;
      const unsigned rm = __ballot_sync(FULL, ready);
      const int nch = (rm == FULL) ? 32 : (__ffs(~rm) - 1);
      if (nch > 0) {
        if (lane < nch) {
#pragma unroll
          for (int k = 0; k < C; k += 4) {
            const int4 q = *reinterpret_cast<const int4 *>(&ringo[(c * C + k) & (RING - 1)]);
            volatile unsigned long long *dp = dst + c * C + k;
            const unsigned long long w0 = dst_tag | (unsigned)q.x, w1 = dst_tag | (unsigned)q.y;
            const unsigned long long w2 = dst_tag | (unsigned)q.z, w3 = dst_tag | (unsigned)q.w;
            asm volatile("st.volatile.global.v2.u64 [%0], {%1,%2};" :: "l"(dp), "l"(w0), "l"(w1) : "memory");
            asm volatile("st.volatile.global.v2.u64 [%0+16], {%1,%2};" :: "l"(dp), "l"(w2), "l"(w3) : "memory");
          }
        }
        out_pos = min(out_pos + nch * C, N1);
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
        const int c0 = in_pos / C;
        const int c1 = (in_pos + n >= N1) ? (N1 + C - 1) / C : (in_pos + n) / C;
        if (lane < c1 - c0) st_release_cta(&S.tag[0][(c0 + lane) & (RING / C - 1)], c0 + lane + 1);
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
      if (band == 0 || in_pos >= N1) __nanosleep(128);
    }
  }
}

template <int KIND, int R, int NW>
__global__ void __launch_bounds__((NW + 1) * 32, 1) plain_kernel(PlainParams P) {
  __shared__ PlainSmem<NW> S;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) S.abort = 0;
  __syncthreads();
  Waiter W(P.timeout_ns, &P.ctrl[1], &S.abort);
  SwBest tb = {0, 0, 0, 0};
  for (;;) {
    if (threadIdx.x == 0) {
      S.band = S.abort ? P.nbands : atomicAdd(&P.ctrl[0], 1);
#pragma unroll
      for (int k = 0; k <= NW; ++k) S.cons[k] = 0;
    }
    for (int i = threadIdx.x; i < (NW + 1) * (RING / C); i += blockDim.x) (&S.tag[0][0])[i] = 0;
    __syncthreads();
    const int band = S.band;
    if (band >= P.nbands) break;
    const int rows_left = P.M - band * P.H;
    const int active = min(NW, (rows_left + 32 * R - 1) / (32 * R));
    if (warp < NW) {
      if (warp < active) compute_band<KIND, R, NW>(P, S, band, warp, lane, W, tb);
    } else {
      io_band<KIND, NW>(P, S, band, active, lane);
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
      for (int k = 1; k <= NW; ++k)
        if (better(S.best[k], b)) b = S.best[k];
      P.best[blockIdx.x] = b;
    }
  }
}

// ---------------------------------------------------------------------------
// Staging, finishing and degenerate-size kernels.
// ---------------------------------------------------------------------------
__global__ void stage_kernel(const int *__restrict__ a, int N, const int *__restrict__ b, int M,
                             int *__restrict__ a_pad, long long a_pad_len, int *__restrict__ b_pad,
                             long long b_pad_len) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < a_pad_len; i += stride) {
    const long long k = i - PADL;
    a_pad[i] = (k >= 0 && k < N) ? a[k] : 0;
  }
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < b_pad_len; i += stride)
    b_pad[i] = (i < M) ? b[i] : 0;
}

template <int KIND>
__global__ void finish_row_kernel(const unsigned long long *__restrict__ last_slot, int N, int M,
                                  int *__restrict__ last_row) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x <= N) last_row[x] = Rec<KIND>::to_v((int)(unsigned)last_slot[x], x, M);
}

template <int KIND>
__global__ void finish_result_kernel(const unsigned long long *__restrict__ last_slot, int N, int M,
                                     int rule, const SwBest *__restrict__ best, int nbest,
                                     const int *ctrl, gme_result *out, int *last_col) {
  __shared__ SwBest sb[32];
  SwBest b = {0, 0, 0, 0};
  if (KIND == K_SW) {
    for (int i = threadIdx.x; i < nbest; i += blockDim.x)
      if (better(best[i], b)) b = best[i];
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    SwBest c;
    c.v = __shfl_down_sync(FULL, b.v, o);
    c.y = __shfl_down_sync(FULL, b.y, o);
    c.x = __shfl_down_sync(FULL, b.x, o);
    c.pad = 0;
    if (better(c, b)) b = c;
  }
  if (lane == 0) sb[warp] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 1; k < (int)(blockDim.x / 32); ++k)
      if (better(sb[k], b)) b = sb[k];
    gme_result r;
    r.score = Rec<KIND>::to_v((int)(unsigned)last_slot[N], N, M);
    r.sw_max = KIND == K_SW ? b.v : 0;
    r.sw_max_y = KIND == K_SW ? b.y : 0;
    r.sw_max_x = KIND == K_SW ? b.x : 0;
    r.status = ctrl[1];
    r.kind = KIND;
    *out = r;
    if (last_col) last_col[0] = Rec<KIND>::to_v(Rec<KIND>::top(N, rule), N, 0);  // row 0, column n1
  }
}

// n1 == 0 or n2 == 0: the table is its borders.
template <int KIND>
__global__ void degenerate_kernel(int N, int M, int rule, int *last_row, int *last_col, gme_result *out) {
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long stride = (long long)gridDim.x * blockDim.x;
  // row n2 when n2 == 0 is row 0; otherwise (n1 == 0) it is the single value column-0 at n2
  for (long long x = tid; x <= N && last_row; x += stride)
    last_row[x] = (M == 0) ? Rec<KIND>::to_v(Rec<KIND>::top(x, rule), x, 0)
                           : Rec<KIND>::to_v(Rec<KIND>::left(M), 0, M);
  for (long long y = tid; y <= M && last_col; y += stride)
    last_col[y] = (y == 0) ? Rec<KIND>::to_v(Rec<KIND>::top(N, rule), N, 0)
                           : Rec<KIND>::to_v(Rec<KIND>::left(y), 0, y);
  if (tid == 0) {
    gme_result r;
    r.score = (M == 0) ? Rec<KIND>::to_v(Rec<KIND>::top(N, rule), N, 0)
                       : Rec<KIND>::to_v(Rec<KIND>::left(M), 0, M);
    r.sw_max = 0; r.sw_max_y = 0; r.sw_max_x = 0; r.status = 0; r.kind = KIND;
    *out = r;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
template <int KIND, int R, int NW>
static cudaError_t launch_plain_t(const PlainParams &P, int grid, cudaStream_t st) {
  plain_kernel<KIND, R, NW><<<grid, (NW + 1) * 32, 0, st>>>(P);
  return cudaGetLastError();
}

template <int KIND>
static cudaError_t launch_plain_k(int R, int NW, const PlainParams &P, int grid, cudaStream_t st) {
  if (R == 2) {
    switch (NW) {
      case 4: return launch_plain_t<KIND, 2, 4>(P, grid, st);
      case 8: return launch_plain_t<KIND, 2, 8>(P, grid, st);
    }
  }
  if (R == 4) {
    switch (NW) {
      case 1: return launch_plain_t<KIND, 4, 1>(P, grid, st);
      case 2: return launch_plain_t<KIND, 4, 2>(P, grid, st);
      case 3: return launch_plain_t<KIND, 4, 3>(P, grid, st);
      case 4: return launch_plain_t<KIND, 4, 4>(P, grid, st);
      case 6: return launch_plain_t<KIND, 4, 6>(P, grid, st);
      case 8: return launch_plain_t<KIND, 4, 8>(P, grid, st);
    }
  }
  return cudaErrorInvalidValue;
}

bool plain_config_valid(int R, int NW) {
  return (R == 4 && (NW == 1 || NW == 2 || NW == 3 || NW == 4 || NW == 6 || NW == 8)) ||
         (R == 2 && (NW == 4 || NW == 8));
}

// Automatic shape.  Every band boundary costs one L2 hand-off on the critical
// path and a band that has to wait for a free CTA doubles the sweep, so take the
// shortest band (most SMs busy) for which all bands run at once, one per SM.
// Rows per lane and warps per band: the tuned table's entry for the nearest table
// height (gme_tuned_plain.h, swept by gpumemefficient_gb300/tune.py), else the
// smallest band that keeps every band on its own SM.
void plain_auto_config(int sms, long long n1, long long n2, int *R, int *NW, int *grid) {
  (void)n1;
  static const int cand[][2] = {{4, 1}, {4, 2}, {4, 3}, {4, 4}, {4, 6}, {4, 8}};
  int r = 4, nw = 8;
  if (TUNED_PLAIN > 0) {
    double best = 1e30;
    for (int k = 0; k < TUNED_PLAIN; ++k) {
      const double d = std::fabs(std::log((double)std::max<long long>(n2, 1) / TUNED_PLAIN_TABLE[k].n));
      if (d < best) { best = d; r = TUNED_PLAIN_TABLE[k].rows_per_lane; nw = TUNED_PLAIN_TABLE[k].warps_per_band; }
    }
  } else {
    for (const auto &c : cand) {
      const long long H = (long long)c[1] * 32 * c[0];
      if ((n2 + H - 1) / H <= sms) { r = c[0]; nw = c[1]; break; }
    }
  }
  *R = r;
  *NW = nw;
  const long long H = (long long)nw * 32 * r;
  const long long nb = (n2 + H - 1) / H;
  *grid = (int)std::min<long long>(nb, (long long)sms);
}

int plain_run(Workspace &ws, int kind, const int *d_a, long long n1, const int *d_b, long long n2,
              const Scoring &sc, gme_result *d_out, int *d_last_row, int *d_last_col,
              cudaStream_t st, int R, int NW, int grid, unsigned long long timeout_ns) {
  const int N = (int)n1, M = (int)n2;
  cudaError_t e;
  if (N == 0 || M == 0) {
    const int threads = 256;
    const long long mx = std::max<long long>(n1, n2) + 1;
    const int blocks = (int)std::min<long long>((mx + threads - 1) / threads, 1024);
    switch (kind) {
      case K_LCS: degenerate_kernel<K_LCS><<<blocks, threads, 0, st>>>(N, M, sc.ed_rule, d_last_row, d_last_col, d_out); break;
      case K_ED: degenerate_kernel<K_ED><<<blocks, threads, 0, st>>>(N, M, sc.ed_rule, d_last_row, d_last_col, d_out); break;
      default: degenerate_kernel<K_SW><<<blocks, threads, 0, st>>>(N, M, sc.ed_rule, d_last_row, d_last_col, d_out); break;
    }
    ws.launches += 1;
    e = cudaGetLastError();
    return e == cudaSuccess ? ST_OK : ws.fail(e, "degenerate_kernel");
  }
  const long long H = (long long)NW * 32 * R;
  const long long nbands = (n2 + H - 1) / H;
  if (grid <= 0 || grid > nbands) grid = (int)std::min<long long>(nbands, ws.sms);
  const int nslot = grid + 2;
  // the last warp writes C-column groups: a group starting at column <= n1 ends at < stride
  const long long stride = ((n1 + 1 + C - 1) / C) * C + C;
  const long long a_pad_len = PADL + n1 + PADR;
  const long long b_pad_len = nbands * H;
  int rc = ws.reserve(a_pad_len, b_pad_len, (long long)nslot * stride, grid);
  if (rc != ST_OK) return rc;
  // unique 32-bit tags per band since the slots were last cleared
  if ((unsigned long long)ws.tag_next + (unsigned long long)nbands + 2ull >= 0xffffffffull) {
    e = cudaMemsetAsync(ws.slots, 0, ws.slots_bytes, st);
    if (e != cudaSuccess) return ws.fail(e, "cudaMemsetAsync(slots)");
    ws.tag_next = 1;
  }
  const unsigned tag0 = ws.tag_next;
  ws.tag_next += (unsigned)nbands + 1;

  {
    const int threads = 256;
    const long long mx = std::max(a_pad_len, b_pad_len);
    const int blocks = (int)std::min<long long>((mx + threads - 1) / threads, 2 * ws.sms);
    stage_kernel<<<blocks, threads, 0, st>>>(d_a, N, d_b, M, ws.a_pad, a_pad_len, ws.b_pad, b_pad_len);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "stage_kernel");
  }
  if ((e = cudaMemsetAsync(ws.ctrl, 0, 4 * sizeof(int), st)) != cudaSuccess)
    return ws.fail(e, "cudaMemsetAsync(ctrl)");

  PlainParams P;
  P.a_pad = ws.a_pad;
  P.b_pad = ws.b_pad;
  P.N = N;
  P.M = M;
  P.H = (int)H;
  P.nbands = (int)nbands;
  P.nslot = nslot;
  P.slot_stride = stride;
  P.slots = ws.slots;
  P.tag0 = tag0;
  P.ctrl = ws.ctrl;
  P.last_col = d_last_col;
  P.best = reinterpret_cast<SwBest *>(ws.best);
  P.sc = sc;
  P.timeout_ns = timeout_ns;
  switch (kind) {
    case K_LCS: e = launch_plain_k<K_LCS>(R, NW, P, grid, st); break;
    case K_ED: e = launch_plain_k<K_ED>(R, NW, P, grid, st); break;
    default: e = launch_plain_k<K_SW>(R, NW, P, grid, st); break;
  }
  ws.launches += 1;
  if (e != cudaSuccess) return ws.fail(e, "plain_kernel");

  const unsigned long long *last_slot = ws.slots + (long long)((nbands - 1) % nslot) * stride;
  if (d_last_row) {
    const int threads = 256;
    const int blocks = (int)((n1 + 1 + threads - 1) / threads);
    switch (kind) {
      case K_LCS: finish_row_kernel<K_LCS><<<blocks, threads, 0, st>>>(last_slot, N, M, d_last_row); break;
      case K_ED: finish_row_kernel<K_ED><<<blocks, threads, 0, st>>>(last_slot, N, M, d_last_row); break;
      default: finish_row_kernel<K_SW><<<blocks, threads, 0, st>>>(last_slot, N, M, d_last_row); break;
    }
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "finish_row_kernel");
  }
  switch (kind) {
    case K_LCS: finish_result_kernel<K_LCS><<<1, 256, 0, st>>>(last_slot, N, M, sc.ed_rule, P.best, grid, ws.ctrl, d_out, d_last_col); break;
    case K_ED: finish_result_kernel<K_ED><<<1, 256, 0, st>>>(last_slot, N, M, sc.ed_rule, P.best, grid, ws.ctrl, d_out, d_last_col); break;
    default: finish_result_kernel<K_SW><<<1, 256, 0, st>>>(last_slot, N, M, sc.ed_rule, P.best, grid, ws.ctrl, d_out, d_last_col); break;
  }
  ws.launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "finish_result_kernel");
  return ST_OK;
}

}  // namespace gme
