// gme_baselines.cu -- comparison baselines: the reference's two table-based strategies
// for the same recurrences, run on this GPU so that the plain path can be timed beside
// them (bench.py --workload baselines).  Not the product path.
//
//   tiles: the whole (n2 + 1) x (n1 + 1) table in device memory, cut into tiles of
//          tile_y x tile_x cells, one launch per anti-diagonal of tiles; a CTA loads its
//          tile's top row and left column from the table, sweeps the tile by cell
//          anti-diagonals in shared memory (a thread per tile row, a barrier per step)
//          and writes the tile back (the strategy of LCS/GPU_TILE_SHARE.cu:12-207);
//   cells: the same table, one launch per anti-diagonal of cells, a thread per cell
//          reading its three neighbours from the table (EditDistance/GPU.cu:20-60).
//
// The recurrences and borders are the reference's as the oracle restates them
// (LCS/LCS.cpp:59-63, EditDistance/ED.cpp:48-65, SmithWaterman/SW.cpp:45-65): plain
// cell values, no transformed forms.  SW's maximum is the first strict maximum in
// row-major order, kept as one 64-bit key {value, ~(y (n1 + 1) + x)} per call.
#include <algorithm>
#include <climits>

#include "gme_common.cuh"
#include "gme_internal.h"

namespace gme {

namespace {

__device__ __forceinline__ int bl_top(int kind, int rule, long long x) {
  if (kind != K_ED) return 0;
  if (rule == 1) return (int)x;        // the standard border
  return x == 0 ? 0 : (int)(x - 1);    // ED.cpp's CPU border: row 0 = 0, 0, 1, 2, ...
}
__device__ __forceinline__ int bl_left(int kind, long long y) { return kind == K_ED ? (int)y : 0; }

__device__ __forceinline__ int bl_cell(int kind, int up, int left, int diag, bool eq, const Scoring &sc) {
  if (kind == K_LCS) return eq ? diag + 1 : max(left, up);
  if (kind == K_ED) return eq ? diag : min(up + 1, min(left + 1, diag + 1));
  return max(left + sc.gap, max(up + sc.gap, max(diag + (eq ? sc.match : sc.mismatch), 0)));
}

__device__ __forceinline__ unsigned long long bl_key(int v, long long y, long long x, long long n1) {
  return ((unsigned long long)(unsigned)v << 32) | (0xffffffffu - (unsigned)(y * (n1 + 1) + x));
}

__global__ void bl_border_kernel(int *t, long long n1, long long n2, int kind, int rule) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n1) t[i] = bl_top(kind, rule, i);
  if (i >= 1 && i <= n2) t[i * (n1 + 1)] = bl_left(kind, i);
}

// One tile per CTA: tile row ty = first_ty + blockIdx.x, tile column tx = d - ty.
__global__ void bl_tile_kernel(int *t, const int *__restrict__ a, const int *__restrict__ b, long long n1,
                               long long n2, int kind, Scoring sc, int TX, int TY, int d, int first_ty,
                               unsigned long long *best) {
  extern __shared__ int s[];  // (TY + 1) x (TX + 1)
  const int ty = first_ty + blockIdx.x, tx = d - ty;
  const long long y0 = 1 + (long long)ty * TY, x0 = 1 + (long long)tx * TX;
  const int W = TX + 1;
  const int r = threadIdx.x;  // this thread's tile row
  // borders: row y0 - 1 (columns x0 - 1 .. x0 + TX - 1) and column x0 - 1
  for (int c = r; c <= TX; c += blockDim.x) {
    const long long x = x0 - 1 + c;
    s[c] = x <= n1 ? t[(y0 - 1) * (n1 + 1) + x] : 0;
  }
  const long long y = y0 + r;
  if (r < TY) s[(r + 1) * W] = y <= n2 ? t[y * (n1 + 1) + x0 - 1] : 0;
  const int sy = (r < TY && y <= n2) ? b[y - 1] : INT_MIN;
  int bv = 0;
  long long bx = 0;
  __syncthreads();
  for (int k = 0; k < TX + TY - 1; ++k) {
    const int c = k - r;
    if (r < TY && c >= 0 && c < TX) {
      const long long x = x0 + c;
      if (y <= n2 && x <= n1) {
        const int v = bl_cell(kind, s[r * W + c + 1], s[(r + 1) * W + c], s[r * W + c], a[x - 1] == sy, sc);
        s[(r + 1) * W + c + 1] = v;
        if (kind == K_SW && v > bv) { bv = v; bx = x; }
      }
    }
    __syncthreads();
  }
  if (kind == K_SW && bv > 0) atomicMax(best, bl_key(bv, y, bx, n1));
  // the tile back to the table, row by row
  for (int i = threadIdx.x; i < TY * TX; i += blockDim.x) {
    const int rr = i / TX, cc = i % TX;
    const long long yy = y0 + rr, xx = x0 + cc;
    if (yy <= n2 && xx <= n1) t[yy * (n1 + 1) + xx] = s[(rr + 1) * W + cc + 1];
  }
}

// One cell per thread on anti-diagonal x + y = d.
__global__ void bl_cell_kernel(int *t, const int *__restrict__ a, const int *__restrict__ b, long long n1,
                               long long n2, int kind, Scoring sc, long long d, long long ylo, long long count,
                               unsigned long long *best) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= count) return;
  const long long y = ylo + i, x = d - y;
  const long long w = n1 + 1;
  const int v = bl_cell(kind, t[(y - 1) * w + x], t[y * w + x - 1], t[(y - 1) * w + x - 1], a[x - 1] == b[y - 1], sc);
  t[y * w + x] = v;
  if (kind == K_SW && v > 0) {
    // only a value above the current best can win; the key orders equal values
    const unsigned long long k = bl_key(v, y, x, n1);
    if (k > *(volatile unsigned long long *)best) atomicMax(best, k);
  }
}

__global__ void bl_finish_kernel(const int *t, long long n1, long long n2, int kind, const unsigned long long *best,
                                 gme_result *out) {
  gme_result r;
  r.score = t[n2 * (n1 + 1) + n1];
  const unsigned long long k = kind == K_SW ? *best : 0ull;
  r.sw_max = (int)(k >> 32);
  const long long lin = r.sw_max ? (long long)(0xffffffffu - (unsigned)k) : 0;
  r.sw_max_y = r.sw_max ? lin / (n1 + 1) : 0;
  r.sw_max_x = r.sw_max ? lin % (n1 + 1) : 0;
  r.status = 0;
  r.kind = kind;
  *out = r;
}

}  // namespace

// The whole table in d_table ((n2 + 1) x (n1 + 1) ints); strategy 0 = tiles, 1 = cells.
int baseline_run(Workspace &ws, int strategy, int kind, const int *d_a, long long n1, const int *d_b, long long n2,
                 const Scoring &sc, int *d_table, int TX, int TY, gme_result *d_out, cudaStream_t st) {
  if (n1 < 1 || n2 < 1 || (n1 + 1) * (n2 + 1) >= (1ll << 32))
    return ws.fail_msg(ST_INVALID, "baseline: need 1 <= n1, n2 and (n1 + 1)(n2 + 1) < 2^32");
  if (strategy == 0 && (TX < 1 || TY < 1 || TY > 1024 || (size_t)(TX + 1) * (TY + 1) * 4 > 200 * 1024))
    return ws.fail_msg(ST_INVALID, "baseline: tile_y 1..1024 threads, (tile_x + 1)(tile_y + 1) ints in shared memory");
  int rc = ws.reserve(0, 0, 0, 0);
  if (rc != ST_OK) return rc;
  cudaError_t e;
  unsigned long long *best = reinterpret_cast<unsigned long long *>(ws.ctrl);  // ctrl[0..1]
  if ((e = cudaMemsetAsync(ws.ctrl, 0, 2 * sizeof(int), st)) != cudaSuccess) return ws.fail(e, "cudaMemsetAsync(best)");
  const long long m = std::max(n1 + 1, n2 + 1);
  bl_border_kernel<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(d_table, n1, n2, kind, sc.ed_rule);
  ws.launches += 1;
  if (strategy == 0) {
    const int nty = (int)((n2 + TY - 1) / TY), ntx = (int)((n1 + TX - 1) / TX);
    const size_t smem = (size_t)(TX + 1) * (TY + 1) * 4;
    if ((e = cudaFuncSetAttribute(bl_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) !=
        cudaSuccess)
      return ws.fail(e, "cudaFuncSetAttribute(bl_tile_kernel)");
    for (int d = 0; d < nty + ntx - 1; ++d) {
      const int lo = std::max(0, d - (ntx - 1)), hi = std::min(nty - 1, d);
      bl_tile_kernel<<<hi - lo + 1, TY, smem, st>>>(d_table, d_a, d_b, n1, n2, kind, sc, TX, TY, d, lo, best);
      ws.launches += 1;
    }
  } else {
    for (long long d = 2; d <= n1 + n2; ++d) {
      const long long ylo = std::max(1ll, d - n1), yhi = std::min(n2, d - 1);
      const long long count = yhi - ylo + 1;
      bl_cell_kernel<<<(unsigned)((count + 255) / 256), 256, 0, st>>>(d_table, d_a, d_b, n1, n2, kind, sc, d, ylo,
                                                                       count, best);
      ws.launches += 1;
    }
  }
  bl_finish_kernel<<<1, 1, 0, st>>>(d_table, n1, n2, kind, best, d_out);
  ws.launches += 1;
  if ((e = cudaGetLastError()) != cudaSuccess) return ws.fail(e, "baseline kernels");
  return ST_OK;
}

}  // namespace gme
