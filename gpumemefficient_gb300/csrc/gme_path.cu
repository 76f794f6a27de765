// gme_path.cu -- optimal alignment paths in linear memory (Hirschberg).
//
// The score-only kernels export the last row of a table; that is all a
// divide-and-conquer traceback needs.  A subproblem (a[i0, i1), b[j0, j1)) is cut at
// its middle row m: the last row F of the table of (a[i0, i1), b[j0, m)) and the last
// row G of the table of the two reversed remainders (a[i0, i1) and b[m, j1) read
// backwards) give, for each column k, the best score of a path through (m, k):
// F[k] + G[cols - k].  The best k splits the problem into (a[i0, i0+k), b[j0, m)) and
// (a[i0+k, i1), b[m, j1)), which are solved the same way, level by level: all halves
// of a level go to the GPU as one batch (gme_align_batch_device_rows, each half's
// last row written at its offset), one kernel picks every node's split, and one copy
// brings the split columns back.
// Subproblems of at most LEAF_ROWS rows and LEAF_CELLS cells are solved whole, one
// CTA each in a single launch: an anti-diagonal sweep that keeps 2-bit directions in
// shared memory, then the walk back from the corner.
//
// Paths are edit scripts: 'M' aligns a[i] with b[j] (for LCS only where they are
// equal), 'D' takes a[i] against a gap (one column), 'I' takes b[j] against a gap
// (one row).  LCS maximises the number of 'M'; ED (the standard border, row 0 =
// 0, 1, 2, ...) minimises 'D' + 'I' + mismatched 'M'.  Ties go diagonal, then up
// ('I'), then left ('D').  The reference computes scores only (its GPU host
// functions return the corner cell, EditDistance/GPU_Hyperlane_Share.cu:689-789);
// this is the traceback its boundary outputs make possible.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gme.h"
#include "gme_common.cuh"
#include "gme_internal.h"

namespace gme {

constexpr int LEAF_ROWS = 256;
constexpr long long LEAF_CELLS = 1ll << 19;

struct PathNode {
  int i0, i1, j0, j1;  // a[i0, i1) x b[j0, j1)
};

struct Leaf {
  int i0, i1, j0, j1;
  long long out;  // offset of its script in the ops buffer (rows + cols characters)
};

// One inner node of a level: its two halves' last rows and where its split goes.
struct NodeJob {
  long long F, G;  // offsets of the forward and backward last rows (cols + 1 values each)
  int cols;
};

// Reverses segment s (len[s] symbols at src[s]) into dst[s], one CTA per segment.
__global__ void reverse_kernel(int *__restrict__ sym, const long long *__restrict__ src,
                               const long long *__restrict__ dst, const int *__restrict__ len, int nseg) {
  for (int s = blockIdx.x; s < nseg; s += gridDim.x) {
    const int n = len[s];
    const int *from = sym + src[s];
    int *to = sym + dst[s];
    for (int i = threadIdx.x; i < n; i += blockDim.x) to[i] = from[n - 1 - i];
  }
}

// The best split column of each node (one CTA per node): k in [0, cols] optimising
// F[k] + G[cols - k] (ED: the smallest sum, LCS: the largest), the smallest k among
// equals.
__global__ void split_kernel(const int *__restrict__ rows, const NodeJob *__restrict__ nodes, int kind,
                             int *__restrict__ out) {
  __shared__ long long best[32];
  const NodeJob nd = nodes[blockIdx.x];
  const int *F = rows + nd.F, *G = rows + nd.G;
  const int cols = nd.cols;
  long long b = LLONG_MAX;
  for (int k = threadIdx.x; k <= cols; k += blockDim.x) {
    const long long s = (long long)F[k] + G[cols - k];
    const long long key = ((kind == K_ED ? s : -s) << 24) | k;  // cols < 2^24
    b = min(b, key);
  }
  for (int o = 16; o > 0; o >>= 1) b = min(b, __shfl_down_sync(0xffffffffu, b, o));
  if ((threadIdx.x & 31) == 0) best[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long m = best[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = min(m, best[w]);
    out[blockIdx.x] = (int)(m & 0xffffff);
  }
}

// One leaf per CTA: thread t owns row t+1; at step d it computes column x = d - t.
// Values of the row above come through shared memory (double-buffered by step
// parity); each cell's direction (0 diagonal, 1 up, 2 left) is kept in 2 bits.
__global__ void __launch_bounds__(LEAF_ROWS) leaf_kernel(const int *__restrict__ a, const int *__restrict__ b,
                                                         const Leaf *__restrict__ leaves, int kind,
                                                         char *__restrict__ ops) {
  extern __shared__ unsigned dirs[];  // (rows * cols * 2 + 31) / 32 words
  __shared__ int last[2][LEAF_ROWS + 1];  // [parity][row]: the row's value after its last step
  const Leaf L = leaves[blockIdx.x];
  const int rows = L.j1 - L.j0, cols = L.i1 - L.i0, t = threadIdx.x;
  const int y = t + 1;
  const bool mine = y <= rows;
  const int by = mine ? b[L.j0 + y - 1] : 0;
  for (int i = t; i < (rows * cols * 2 + 31) / 32; i += blockDim.x) dirs[i] = 0;
  // column 0 of every row, and row 0 (index 0) of the value buffers
  const int col0 = kind == K_ED ? y : 0;
  int left = col0;  // this row's value at column x-1
  if (t <= LEAF_ROWS) last[0][t] = last[1][t] = 0;
  __syncthreads();
  for (int d = 1; d <= rows + cols - 1 + 1; ++d) {
    const int x = d - t;
    // the row above at columns x and x-1: row 0 is the border, else the other thread's
    // values of steps d-1 (its column x) and d-2 (its column x-1)
    int up = 0, diag = 0;
    if (mine && x >= 1 && x <= cols) {
      if (y == 1) {
        up = kind == K_ED ? x : 0;
        diag = kind == K_ED ? x - 1 : 0;
      } else {
        up = last[(d - 1) & 1][t];       // thread t-1's value at column x (row y-1)
        diag = last[d & 1][t];           // its value at column x-1 (two steps back)
        if (x == 1) diag = kind == K_ED ? y - 1 : 0;
      }
    }
    __syncthreads();
    if (mine && x >= 1 && x <= cols) {
      const bool eq = a[L.i0 + x - 1] == by;
      int v, dir;
      if (kind == K_ED) {
        const int dg = diag + (eq ? 0 : 1), u = up + 1, l = left + 1;
        v = dg; dir = 0;
        if (u < v) { v = u; dir = 1; }
        if (l < v) { v = l; dir = 2; }
      } else {
        if (eq) { v = diag + 1; dir = 0; }
        else if (up >= left) { v = up; dir = 1; }
        else { v = left; dir = 2; }
      }
      left = v;
      const long long c = (long long)(y - 1) * cols + (x - 1);
      atomicOr(&dirs[c >> 4], (unsigned)dir << ((c & 15) * 2));
      last[d & 1][t + 1] = v;  // read by thread t+1 (row y+1) at steps d+1 and d+2
    } else if (mine && x < 1) {
      last[d & 1][t + 1] = col0;  // column 0, for the row below's diagonal
    }
    __syncthreads();
  }
  if (t == 0) {
    // walk back from the corner; the script is written backwards, then reversed
    char *o = ops + L.out;
    int n = 0, yy = rows, xx = cols;
    while (yy > 0 && xx > 0) {
      const long long c = (long long)(yy - 1) * cols + (xx - 1);
      const int dir = (dirs[c >> 4] >> ((c & 15) * 2)) & 3;
      if (dir == 0) { o[n++] = 'M'; --yy; --xx; }
      else if (dir == 1) { o[n++] = 'I'; --yy; }
      else { o[n++] = 'D'; --xx; }
    }
    while (xx > 0) { o[n++] = 'D'; --xx; }
    while (yy > 0) { o[n++] = 'I'; --yy; }
    for (int i = 0; i < n / 2; ++i) { const char c = o[i]; o[i] = o[n - 1 - i]; o[n - 1 - i] = c; }
  }
}

}  // namespace gme

using gme::Leaf;
using gme::PathNode;
using gme::NodeJob;

extern "C" gme_status gme_align_path(gme_context *ctx, gme_kind kind, const int32_t *a, int64_t n1,
                                     const int32_t *b, int64_t n2, const gme_scoring *sc, char *ops,
                                     int64_t ops_cap, int64_t *n_ops, int32_t *score) {
  if (!ctx || !n_ops || (n1 && !a) || (n2 && !b) || n1 < 0 || n2 < 0 || (kind != GME_LCS && kind != GME_ED))
    return GME_ERR_INVALID;
  if (kind == GME_ED && sc && sc->ed_boundary != GME_ED_STANDARD) return GME_ERR_INVALID;
  if (n1 >= (1 << 24) - 1 || n2 >= (1 << 30)) return GME_ERR_OVERFLOW;
  *n_ops = n1 + n2;  // an upper bound until the script is known
  gme_scoring s = gme_default_scoring();
  s.ed_boundary = GME_ED_STANDARD;
  cudaSetDevice(gme::ctx_device(ctx));
  cudaStream_t st = nullptr;
  cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  auto fail = [&](gme_status rc) {
    if (st) cudaStreamDestroy(st);
    return rc;
  };
  // one symbol buffer: a, then b, then the reversed remainders of a level
  const long long sym_len = 2 * (n1 + n2) + 16;
  int *d_sym = nullptr, *d_rows = nullptr, *d_split = nullptr;
  gme_result *d_res = nullptr;
  long long *d_rsrc = nullptr, *d_rdst = nullptr;
  int *d_rlen = nullptr;
  NodeJob *d_nodes = nullptr;
  auto release = [&] {
    cudaFree(d_sym); cudaFree(d_rows); cudaFree(d_split); cudaFree(d_res);
    cudaFree(d_rsrc); cudaFree(d_rdst); cudaFree(d_rlen); cudaFree(d_nodes);
  };
  if (cudaMalloc(&d_sym, (size_t)sym_len * 4) || cudaMalloc(&d_res, sizeof(gme_result))) {
    release();
    return fail(GME_ERR_NOMEM);
  }
  int *d_a = d_sym, *d_b = d_sym + n1;
  if (n1) cudaMemcpyAsync(d_a, a, (size_t)n1 * 4, cudaMemcpyHostToDevice, st);
  if (n2) cudaMemcpyAsync(d_b, b, (size_t)n2 * 4, cudaMemcpyHostToDevice, st);
  // the optimal score, from the score-only path
  gme_result root{};
  {
    const gme_status r0 = gme_align_device(ctx, kind, d_a, n1, d_b, n2, &s, d_res, nullptr, nullptr, st);
    if (r0 != GME_OK || cudaMemcpyAsync(&root, d_res, sizeof(root), cudaMemcpyDeviceToHost, st) ||
        cudaStreamSynchronize(st)) {
      release();
      return fail(r0 != GME_OK ? r0 : GME_ERR_CUDA);
    }
    if (root.status != 0) {
      release();
      return fail((gme_status)root.status);
    }
  }

  std::vector<PathNode> level{{0, (int)n1, 0, (int)n2}};
  std::vector<Leaf> leaves;
  // the script is the leaves' scripts in order; order is kept by the recursion tree:
  // each node records its two children, leaves record their slot
  struct Item { int leaf; int left, right; };
  std::vector<Item> tree;            // tree node per processed node
  std::vector<int> level_ids{0};
  tree.push_back({-1, -1, -1});
  long long ops_total = 0;
  gme_status rc = GME_OK;
  long long rows_cap = 0, nodes_cap = 0;
  while (!level.empty() && rc == GME_OK) {
    std::vector<PathNode> inner;
    std::vector<int> inner_ids;
    for (size_t k = 0; k < level.size(); ++k) {
      const PathNode &p = level[k];
      const long long rows = p.j1 - p.j0, cols = p.i1 - p.i0;
      if ((rows <= gme::LEAF_ROWS && rows * cols <= gme::LEAF_CELLS) || rows == 0 || cols == 0) {
        tree[level_ids[k]].leaf = (int)leaves.size();
        leaves.push_back({p.i0, p.i1, p.j0, p.j1, ops_total});
        ops_total += rows + cols;
      } else {
        inner.push_back(p);
        inner_ids.push_back(level_ids[k]);
      }
    }
    if (inner.empty()) break;
    // the level's batch: per node, its top half forward and its bottom half reversed
    const long long nn = (long long)inner.size();
    std::vector<gme_pair> pairs(2 * nn);
    std::vector<int64_t> row_off(2 * nn);
    std::vector<NodeJob> nodes(nn);
    std::vector<long long> rsrc, rdst;
    std::vector<int> rlen;
    long long roff = 0, rev = n1 + n2;
    for (long long k = 0; k < nn; ++k) {
      const PathNode &p = inner[k];
      const int cols = p.i1 - p.i0, m = p.j0 + (p.j1 - p.j0) / 2, rb = p.j1 - m;
      pairs[2 * k] = gme_pair{(int64_t)p.i0, (int64_t)(n1 + p.j0), cols, m - p.j0, (int32_t)kind, 0};
      rsrc.push_back(p.i0); rdst.push_back(rev); rlen.push_back(cols);
      rsrc.push_back(n1 + m); rdst.push_back(rev + cols); rlen.push_back(rb);
      pairs[2 * k + 1] = gme_pair{(int64_t)rev, (int64_t)(rev + cols), cols, rb, (int32_t)kind, 0};
      rev += cols + rb;
      nodes[k] = {roff, roff + cols + 1, cols};
      row_off[2 * k] = roff;
      row_off[2 * k + 1] = roff + cols + 1;
      roff += 2 * (long long)(cols + 1);
    }
    if (roff > rows_cap) {
      cudaFree(d_rows);
      d_rows = nullptr;
      rows_cap = roff + roff / 4;
      if (cudaMalloc(&d_rows, (size_t)rows_cap * 4)) { rc = GME_ERR_NOMEM; break; }
    }
    if (nn > nodes_cap) {
      cudaFree(d_split); cudaFree(d_nodes); cudaFree(d_rsrc); cudaFree(d_rdst); cudaFree(d_rlen);
      d_split = nullptr; d_nodes = nullptr; d_rsrc = d_rdst = nullptr; d_rlen = nullptr;
      nodes_cap = nn + nn / 4 + 16;
      if (cudaMalloc(&d_split, nodes_cap * 4) || cudaMalloc(&d_nodes, nodes_cap * sizeof(NodeJob)) ||
          cudaMalloc(&d_rsrc, 2 * nodes_cap * 8) || cudaMalloc(&d_rdst, 2 * nodes_cap * 8) ||
          cudaMalloc(&d_rlen, 2 * nodes_cap * 4)) {
        rc = GME_ERR_NOMEM;
        break;
      }
    }
    // pageable sources: each copy has taken its bytes before it returns
    cudaMemcpyAsync(d_rsrc, rsrc.data(), rsrc.size() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_rdst, rdst.data(), rdst.size() * 8, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_rlen, rlen.data(), rlen.size() * 4, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(d_nodes, nodes.data(), nodes.size() * sizeof(NodeJob), cudaMemcpyHostToDevice, st);
    gme::reverse_kernel<<<(unsigned)std::min<long long>(2 * nn, 65535), 256, 0, st>>>(d_sym, d_rsrc, d_rdst,
                                                                                    d_rlen, (int)(2 * nn));
    gme_result *d_lres = nullptr;
    if (cudaMalloc(&d_lres, 2 * nn * sizeof(gme_result))) { rc = GME_ERR_NOMEM; break; }
    rc = gme_align_batch_device_rows(ctx, d_sym, sym_len, pairs.data(), 2 * nn, &s, d_lres, d_rows,
                                     row_off.data(), nullptr, nullptr, st);
    if (rc == GME_OK) {
      gme::split_kernel<<<(unsigned)nn, 256, 0, st>>>(d_rows, d_nodes, (int)kind, d_split);
    }
    std::vector<int> split(nn);
    std::vector<gme_result> lres(2 * nn);
    if (rc == GME_OK && (cudaMemcpyAsync(split.data(), d_split, nn * 4, cudaMemcpyDeviceToHost, st) ||
                         cudaMemcpyAsync(lres.data(), d_lres, 2 * nn * sizeof(gme_result),
                                         cudaMemcpyDeviceToHost, st) ||
                         cudaStreamSynchronize(st)))
      rc = GME_ERR_CUDA;
    cudaFree(d_lres);
    for (const gme_result &r : lres)
      if (rc == GME_OK && r.status != 0) rc = (gme_status)r.status;  // a wait gave up: no path
    if (rc != GME_OK) break;
    std::vector<PathNode> next;
    std::vector<int> next_ids;
    for (long long k = 0; k < nn; ++k) {
      const PathNode &p = inner[k];
      const int m = p.j0 + (p.j1 - p.j0) / 2, c = p.i0 + split[k];
      const int l = (int)tree.size(), r = l + 1;
      tree.push_back({-1, -1, -1});
      tree.push_back({-1, -1, -1});
      tree[inner_ids[k]].left = l;
      tree[inner_ids[k]].right = r;
      next.push_back({p.i0, c, p.j0, m});
      next_ids.push_back(l);
      next.push_back({c, p.i1, m, p.j1});
      next_ids.push_back(r);
    }
    level.swap(next);
    level_ids.swap(next_ids);
  }
  // the leaves, one CTA each
  char *d_ops = nullptr;
  Leaf *d_leaves = nullptr;
  std::vector<char> h_ops((size_t)ops_total + 1);
  if (rc == GME_OK && !leaves.empty()) {
    long long smem = 0;
    for (const Leaf &L : leaves)
      smem = std::max(smem, ((long long)(L.j1 - L.j0) * (L.i1 - L.i0) * 2 + 31) / 32 * 4);
    cudaFuncSetAttribute(gme::leaf_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)std::max(smem, 4ll));
    if (cudaMalloc(&d_ops, (size_t)ops_total + 1) || cudaMalloc(&d_leaves, leaves.size() * sizeof(Leaf))) {
      rc = GME_ERR_NOMEM;
    } else {
      cudaMemcpyAsync(d_leaves, leaves.data(), leaves.size() * sizeof(Leaf), cudaMemcpyHostToDevice, st);
      gme::leaf_kernel<<<(unsigned)leaves.size(), gme::LEAF_ROWS, (size_t)std::max(smem, 4ll), st>>>(
          d_a, d_b, d_leaves, (int)kind, d_ops);
      if (cudaGetLastError() != cudaSuccess ||
          cudaMemcpyAsync(h_ops.data(), d_ops, (size_t)ops_total, cudaMemcpyDeviceToHost, st) ||
          cudaStreamSynchronize(st))
        rc = GME_ERR_CUDA;
    }
  }
  cudaFree(d_ops);
  cudaFree(d_leaves);
  release();
  cudaStreamDestroy(st);
  st = nullptr;
  if (rc != GME_OK) return rc;
  // the script: leaves in tree order (left child before right child)
  std::string script;
  script.reserve((size_t)(n1 + n2));
  std::vector<int> stack{0};
  while (!stack.empty()) {
    const int id = stack.back();
    stack.pop_back();
    const Item &it = tree[id];
    if (it.leaf >= 0) {
      const Leaf &L = leaves[it.leaf];
      const long long len = (L.j1 - L.j0) + (L.i1 - L.i0);
      // a leaf's script is shorter than rows + cols when it has diagonal steps
      long long k = 0;
      int yy = 0, xx = 0;
      while (k < len && (yy < L.j1 - L.j0 || xx < L.i1 - L.i0)) {
        const char c = h_ops[L.out + k++];
        script.push_back(c);
        if (c == 'M') { ++yy; ++xx; } else if (c == 'I') ++yy; else ++xx;
      }
    } else {
      stack.push_back(it.right);
      stack.push_back(it.left);
    }
  }
  *n_ops = (int64_t)script.size();
  if (score) *score = root.score;
  if (!ops) return GME_OK;
  if ((int64_t)script.size() > ops_cap) return GME_ERR_INVALID;
  std::memcpy(ops, script.data(), script.size());
  return GME_OK;
}
