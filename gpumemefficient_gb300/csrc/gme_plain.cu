// gme_plain.cu -- one alignment per call: the host side of the plain path.
//
// Replaces the reference's host schedulers (EditDistance/GPU_Hyperlane_Share.cu:689-789
// and their LCS/SW twins): instead of allocating the full (n+pad)^2 int table
// (:698-713) and launching one <<<1,1024>>> kernel per tile row on SM-count streams
// (:752-764), a call stages the pair, launches the single persistent wavefront
// kernel (gme_plain_kernel.cuh, one translation unit per kind) and two small
// kernels that turn the last band's row into the caller's outputs.  Memory is O(n)
// per band in flight; nothing of the table is kept.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <type_traits>

#include "gme_plain_kernel.cuh"
#include "gme_tuned_plain.h"

namespace gme {

extern template cudaError_t launch_plain_k<K_LCS>(int, int, const PlainParams &, int, cudaStream_t);
extern template cudaError_t launch_plain_k<K_ED>(int, int, const PlainParams &, int, cudaStream_t);
extern template cudaError_t launch_plain_k<K_SW>(int, int, const PlainParams &, int, cudaStream_t);

// ---------------------------------------------------------------------------
// Staging, finishing and degenerate-size kernels.
// ---------------------------------------------------------------------------
// The range of the pair's symbols, as two maxima over unsigned keys (cleared to 0 by
// the caller): ctrl[2] = max of (s ^ 0x80000000) and ctrl[3] = max of ~(s ^ 0x80000000).
__global__ void plain_range_kernel(const int *__restrict__ a, int N, const int *__restrict__ b, int M, int *ctrl) {
  unsigned hi = 0, lo = 0;
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)N + M; i += stride) {
    const unsigned k = (unsigned)(i < N ? a[i] : b[i - N]) ^ 0x80000000u;
    hi = max(hi, k);
    lo = max(lo, ~k);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    hi = max(hi, __shfl_xor_sync(FULL, hi, o));
    lo = max(lo, __shfl_xor_sync(FULL, lo, o));
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMax(reinterpret_cast<unsigned *>(&ctrl[2]), hi);
    atomicMax(reinterpret_cast<unsigned *>(&ctrl[3]), lo);
  }
}

// Stages the pair in the form the range allows (see COST_TABLE): a into a_pad (and
// a_pad2, the same shifted right by two), b into b_pad, and the choice into ctrl[4].
// table_ok: the scoring constants fit the table's signed bytes (and SW's gap <= 0).
__global__ void plain_stage_kernel(const int *__restrict__ a, int N, const int *__restrict__ b, int M,
                                   int *__restrict__ a_pad, int *__restrict__ a_pad2, long long a_pad_len,
                                   int *__restrict__ b_pad, long long b_pad_len, int *ctrl, int table_ok) {
  const unsigned hi = (unsigned)ctrl[2] ^ 0x80000000u, lo = ~(unsigned)ctrl[3] ^ 0x80000000u;
  const long long span = (long long)(int)hi - (long long)(int)lo;  // max - min (no symbols: negative)
  const bool table = table_ok && span >= 0 && span < SENTINEL;
  const int mn = (int)lo;
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long t0 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t0 == 0) ctrl[4] = table ? 1 : 0;
  auto col = [&](long long i) -> int {  // a_pad[i]
    const long long k = i - PADL;
    if (k >= 0 && k < N) return table ? cost_selector(a[k] - mn) : a[k];
    return table ? cost_selector(SENTINEL) : 0;
  };
  for (long long i = t0; i < a_pad_len; i += stride) {
    a_pad[i] = col(i);
    a_pad2[i] = col(i - 2);
  }
  for (long long i = t0; i < b_pad_len; i += stride)
    b_pad[i] = (i < M) ? (table ? b[i] - mn : b[i]) : 0;
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
bool plain_config_valid(int R, int NW) { return (R == 2 || R == 4) && (NW == 4 || NW == 8); }

// Automatic shape.  Every band boundary costs one L2 hand-off on the critical
// path and a band that has to wait for a free CTA doubles the sweep, so take the
// shortest band (most SMs busy) for which all bands run at once, one per SM.
// Rows per lane and warps per band: the tuned table's entry for the nearest table
// height (gme_tuned_plain.h, swept by gpumemefficient_gb300/tune.py), else the
// smallest band that keeps every band on its own SM.
void plain_auto_config(int sms, long long n1, long long n2, int *R, int *NW, int *grid) {
  (void)n1;
  static const int cand[][2] = {{2, 4}, {4, 4}, {4, 8}};
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
  // the I/O warp writes PLAIN_C-column groups: a group starting at column <= n1 ends at < stride
  const long long stride = ((n1 + 1 + PLAIN_C - 1) / PLAIN_C) * PLAIN_C + PLAIN_C;
  // a_pad and its copy shifted by two, each a whole number of 16-byte groups
  const long long a_pad_len = (PADL + n1 + PADR + 3) / 4 * 4;
  const long long b_pad_len = nbands * H;
  int rc = ws.reserve(2 * a_pad_len, b_pad_len, (long long)nslot * stride, grid);
  if (rc != ST_OK) return rc;
  // unique 32-bit tags per band since the slots were last cleared
  if ((unsigned long long)ws.tag_next + (unsigned long long)nbands + 2ull >= 0xffffffffull) {
    e = cudaMemsetAsync(ws.slots, 0, ws.slots_bytes, st);
    if (e != cudaSuccess) return ws.fail(e, "cudaMemsetAsync(slots)");
    ws.tag_next = 1;
  }
  const unsigned tag0 = ws.tag_next;
  ws.tag_next += (unsigned)nbands + 1;

  // ticket, status, symbol range and cost form start cleared
  if ((e = cudaMemsetAsync(ws.ctrl, 0, 8 * sizeof(int), st)) != cudaSuccess)
    return ws.fail(e, "cudaMemsetAsync(ctrl)");
  {
    const int threads = 256;
    const long long n = n1 + n2;
    const int blocks = (int)std::min<long long>((n + threads - 1) / threads, 2 * ws.sms);
    plain_range_kernel<<<blocks, threads, 0, st>>>(d_a, N, d_b, M, ws.ctrl);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "plain_range_kernel");
  }
  {
    // the table form holds costs as signed bytes, and its ramp cells rely on gap <= 0
    int table_ok = 1;
    if (kind == K_SW)
      table_ok = sc.match >= -128 && sc.match <= 127 && sc.mismatch >= -128 && sc.mismatch <= 127 && sc.gap <= 0;
    const int threads = 256;
    const long long mx = std::max(a_pad_len, b_pad_len);
    const int blocks = (int)std::min<long long>((mx + threads - 1) / threads, 2 * ws.sms);
    plain_stage_kernel<<<blocks, threads, 0, st>>>(d_a, N, d_b, M, ws.a_pad, ws.a_pad + a_pad_len, a_pad_len,
                                                   ws.b_pad, b_pad_len, ws.ctrl, table_ok);
    ws.launches += 1;
    if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "plain_stage_kernel");
  }

  PlainParams P;
  P.a_pad = ws.a_pad;
  P.a_pad2 = ws.a_pad + a_pad_len;
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
