/*
 * oracle.c -- CPU restatement of the reference's alignment recurrences.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA path is
 * compared against; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline legs load it.  The product library never links or calls it.
 *
 * Table convention (identical to the reference's GPU host functions, which
 * put arr1 along x and arr2 along y, e.g. EditDistance/GPU_Hyperlane_Share.cu
 * :696-697 and the kernel's dev_arr1[idxx]==dev_arr2[idxy] at :409):
 *   rows    y = 0..n2 run over b = arr2,
 *   columns x = 0..n1 run over a = arr1,
 *   cell (y,x) for y,x >= 1 compares a[x-1] with b[y-1].
 * The CPU programs LCS.cpp/ED.cpp/SW.cpp loop y<n1, x<n2 but index arr1[x],
 * arr2[y] (LCS/LCS.cpp:54-63), which is only in bounds when n1 == n2; for
 * n1 == n2 this convention is exactly theirs.  Memory is O(n1) (one rolling
 * row) and indices are 64-bit, so sizes beyond the reference's int table
 * (n ~ 46340) are fine.
 *
 * Pinned against the unmodified reference binaries built by oracle/build_ref.sh
 * on the reference's square fixtures (tests/golden/kat.json).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <pthread.h>
#include <stdatomic.h>
#include <sched.h>

#define ORC_LCS 0
#define ORC_ED 1
#define ORC_SW 2

#define ORC_ED_REF_CPU 0  /* ED.cpp:48-54: row0 = [0,0,1,2,...], col0 = [0,1,2,...] */
#define ORC_ED_STANDARD 1 /* GPU_setInit (EditDistance/GPU_Hyperlane_Share.cu:16-22) */

static inline int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }
static inline int32_t imin(int32_t a, int32_t b) { return a < b ? a : b; }

/* Boundary row 0 value at column x (x = 0..n1). */
static inline int32_t top_value(int kind, int rule, int64_t x) {
    if (kind != ORC_ED) return 0;                      /* LCS.cpp:48-52, SW.cpp:51-55 */
    if (rule == ORC_ED_STANDARD) return (int32_t)x;     /* GPU_setInit */
    return x == 0 ? 0 : (int32_t)(x - 1);              /* ED.cpp:48-49 then :51-54 sets [0]=0 */
}

/* Boundary column 0 value at row y (y = 0..n2). */
static inline int32_t left_value(int kind, int64_t y) {
    return kind == ORC_ED ? (int32_t)y : 0;            /* ED.cpp:51-54; zero for LCS/SW */
}

typedef struct {
    int32_t match, mismatch, gap; /* SW only: SW.cpp:45-47 (+3/-3) and :63-65 (-2) */
} orc_sw_scoring;

/* One cell of each recurrence, as the reference writes it. */
static inline int32_t cell(int kind, int32_t up, int32_t left, int32_t diag, int eq,
                           const orc_sw_scoring *sc) {
    if (kind == ORC_LCS) {
        /* LCS/LCS.cpp:59-63 */
        return eq ? diag + 1 : imax(left, up);
    } else if (kind == ORC_ED) {
        /* EditDistance/ED.cpp:63-65: min of the three +1, then diag on a match */
        int32_t t = imin(up + 1, imin(left + 1, diag + 1));
        return eq ? diag : t;
    } else {
        /* SmithWaterman/SW.cpp:63-65 */
        int32_t s = eq ? sc->match : sc->mismatch;
        return imax(left + sc->gap, imax(up + sc->gap, imax(diag + s, 0)));
    }
}

/*
 * Rows [y0, y1] (1-based, inclusive) of one alignment, given row y0-1 in
 * `row` (n1+1 values, overwritten in place with row y1).  Optionally records
 * column n1 of every row into last_col[y], and for SW the first strict maximum
 * in row-major order over the rows processed.
 */
static void sweep_rows(int kind, int rule, const int32_t *a, int64_t n1, const int32_t *b,
                       int64_t y0, int64_t y1, int32_t *row, int32_t *last_col,
                       const orc_sw_scoring *sc, int32_t *best, int64_t *by, int64_t *bx) {
    for (int64_t y = y0; y <= y1; ++y) {
        int32_t diag = row[0];
        int32_t left = left_value(kind, y);
        row[0] = left;
        const int32_t sy = b[y - 1];
        for (int64_t x = 1; x <= n1; ++x) {
            int32_t up = row[x];
            int32_t v = cell(kind, up, left, diag, a[x - 1] == sy, sc);
            if (kind == ORC_SW && v > *best) { *best = v; *by = y; *bx = x; }
            row[x] = v;
            diag = up;
            left = v;
        }
        if (last_col) last_col[y] = row[n1];
    }
    (void)rule;
}

/*
 * Full single-threaded alignment.  Returns the bottom-right cell (what the
 * reference returns: LCS.cpp:78, ED.cpp:79, SW.cpp:80).  last_row (n1+1) and
 * last_col (n2+1) are optional.  For SW, sw_max, sw_y and sw_x receive the first
 * strict maximum in row-major order over y = 1..n2, x = 1..n1 (0 at (0,0)
 * when no cell is positive); this extension is not in the reference.
 */
int32_t orc_align(int kind, int rule, const int32_t *a, int64_t n1, const int32_t *b, int64_t n2,
                  int32_t match, int32_t mismatch, int32_t gap,
                  int32_t *last_row, int32_t *last_col,
                  int32_t *sw_max, int64_t *sw_y, int64_t *sw_x) {
    orc_sw_scoring sc = {match, mismatch, gap};
    int32_t *row = (int32_t *)malloc((size_t)(n1 + 1) * sizeof(int32_t));
    if (!row) return INT32_MIN;
    for (int64_t x = 0; x <= n1; ++x) row[x] = top_value(kind, rule, x);
    if (last_col) last_col[0] = row[n1];
    int32_t best = 0; int64_t by = 0, bx = 0;
    if (n2 > 0) sweep_rows(kind, rule, a, n1, b, 1, n2, row, last_col, &sc, &best, &by, &bx);
    int32_t corner = row[n1];
    if (last_row) memcpy(last_row, row, (size_t)(n1 + 1) * sizeof(int32_t));
    if (sw_max) *sw_max = best;
    if (sw_y) *sw_y = by;
    if (sw_x) *sw_x = bx;
    free(row);
    return corner;
}

/*
 * Full table, for tiny cases only: (n2+1) x (n1+1) row-major, the reference's
 * DEBUG dump layout without its padding columns.
 */
void orc_table(int kind, int rule, const int32_t *a, int64_t n1, const int32_t *b, int64_t n2,
               int32_t match, int32_t mismatch, int32_t gap, int32_t *table) {
    orc_sw_scoring sc = {match, mismatch, gap};
    int64_t w = n1 + 1;
    for (int64_t x = 0; x <= n1; ++x) table[x] = top_value(kind, rule, x);
    for (int64_t y = 1; y <= n2; ++y) {
        table[y * w] = left_value(kind, y);
        for (int64_t x = 1; x <= n1; ++x)
            table[y * w + x] = cell(kind, table[(y - 1) * w + x], table[y * w + x - 1],
                                    table[(y - 1) * w + x - 1], a[x - 1] == b[y - 1], &sc);
    }
}

/* ------------------------------------------------------------------------- */
/* Multi-threaded forms (CPU baselines and large-test checkers).              */
/* ------------------------------------------------------------------------- */

/*
 * One alignment on T threads: the CPU analogue of the reference's per-tile-row
 * scheduling with dev_lock counters (EditDistance/GPU_Hyperlane_Share.cu
 * :110-129, :736-764).  Rows are cut into bands of H rows; band k is swept by
 * thread k % T in column chunks of C; band k may start chunk j once band k-1
 * has published chunk j (an atomic progress counter per band).  Each band
 * boundary row lives in its own buffer, so results equal orc_align exactly.
 */
typedef struct {
    int kind, rule;
    const int32_t *a, *b;
    int64_t n1, n2, H, C, nbands;
    int nthreads, tid;
    int32_t **bnd;          /* bnd[0] = row 0; bnd[k+1] = bottom row of band k (n1+1) */
    _Atomic int64_t *prog;  /* prog[k] = columns of bnd[k] published */
    int32_t *last_col;
    orc_sw_scoring sc;
    int32_t best; int64_t by, bx;
} mt_arg;

static void *mt_worker(void *p) {
    mt_arg *g = (mt_arg *)p;
    int64_t n1 = g->n1;
    int32_t *colv = (int32_t *)malloc((size_t)g->H * sizeof(int32_t));
    g->best = 0; g->by = 0; g->bx = 0;
    for (int64_t k = g->tid; k < g->nbands; k += g->nthreads) {
        int64_t y0 = k * g->H + 1, y1 = y0 + g->H - 1;
        if (y1 > g->n2) y1 = g->n2;
        int64_t h = y1 - y0 + 1;
        const int32_t *in = g->bnd[k];       /* row y0-1 */
        int32_t *out = g->bnd[k + 1];        /* row y1 */
        _Atomic int64_t *pin = &g->prog[k];
        _Atomic int64_t *pout = &g->prog[k + 1];
        /* left column of the band: colv[i] = value at (y0+i, x-1) */
        for (int64_t i = 0; i < h; ++i) colv[i] = left_value(g->kind, y0 + i);
        while (atomic_load_explicit(pin, memory_order_acquire) < 1) sched_yield();
        out[0] = colv[h - 1];
        int32_t diag_top = in[0];
        for (int64_t x0 = 1; x0 <= n1; x0 += g->C) {
            int64_t x1 = x0 + g->C - 1;
            if (x1 > n1) x1 = n1;
            while (atomic_load_explicit(pin, memory_order_acquire) < x1 + 1) sched_yield();
            for (int64_t x = x0; x <= x1; ++x) {
                int32_t up = in[x];
                int32_t diag = diag_top;
                const int32_t sx = g->a[x - 1];
                for (int64_t i = 0; i < h; ++i) {
                    int32_t left = colv[i];
                    int32_t v = cell(g->kind, up, left, diag, sx == g->b[y0 + i - 1], &g->sc);
                    if (g->kind == ORC_SW && v > g->best) {
                        /* row-major first maximum: compare (y, x) order */
                        g->best = v; g->by = y0 + i; g->bx = x;
                    } else if (g->kind == ORC_SW && v == g->best && v > 0 &&
                               (y0 + i < g->by || (y0 + i == g->by && x < g->bx))) {
                        g->by = y0 + i; g->bx = x;
                    }
                    diag = left;
                    colv[i] = v;
                    up = v;
                }
                diag_top = in[x];
                out[x] = colv[h - 1];
            }
            atomic_store_explicit(pout, x1 + 1, memory_order_release);
        }
        if (n1 == 0) atomic_store_explicit(pout, 1, memory_order_release);
        if (g->last_col)
            for (int64_t i = 0; i < h; ++i) g->last_col[y0 + i] = colv[i];
    }
    free(colv);
    return NULL;
}

int32_t orc_align_mt(int kind, int rule, const int32_t *a, int64_t n1, const int32_t *b, int64_t n2,
                     int32_t match, int32_t mismatch, int32_t gap,
                     int32_t *last_row, int32_t *last_col,
                     int32_t *sw_max, int64_t *sw_y, int64_t *sw_x,
                     int nthreads, int64_t band_rows, int64_t chunk_cols) {
    if (nthreads <= 1 || n2 <= band_rows)
        return orc_align(kind, rule, a, n1, b, n2, match, mismatch, gap, last_row, last_col,
                         sw_max, sw_y, sw_x);
    int64_t H = band_rows > 0 ? band_rows : 256;
    int64_t C = chunk_cols > 0 ? chunk_cols : 1024;
    int64_t nb = (n2 + H - 1) / H;
    int32_t **bnd = (int32_t **)malloc((size_t)(nb + 1) * sizeof(int32_t *));
    _Atomic int64_t *prog = (_Atomic int64_t *)malloc((size_t)(nb + 1) * sizeof(_Atomic int64_t));
    for (int64_t k = 0; k <= nb; ++k) {
        bnd[k] = (int32_t *)malloc((size_t)(n1 + 1) * sizeof(int32_t));
        atomic_init(&prog[k], 0);
    }
    for (int64_t x = 0; x <= n1; ++x) bnd[0][x] = top_value(kind, rule, x);
    atomic_store(&prog[0], n1 + 1);
    if (last_col) last_col[0] = bnd[0][n1];
    if (nthreads > nb) nthreads = (int)nb;
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    mt_arg *args = (mt_arg *)malloc((size_t)nthreads * sizeof(mt_arg));
    for (int t = 0; t < nthreads; ++t) {
        mt_arg g = {kind, rule, a, b, n1, n2, H, C, nb, nthreads, t, bnd, prog, last_col,
                    {match, mismatch, gap}, 0, 0, 0};
        args[t] = g;
        pthread_create(&th[t], NULL, mt_worker, &args[t]);
    }
    int32_t best = 0; int64_t by = 0, bx = 0;
    for (int t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        mt_arg *g = &args[t];
        if (g->best > best || (g->best == best && g->best > 0 &&
                               (g->by < by || (g->by == by && g->bx < bx)))) {
            best = g->best; by = g->by; bx = g->bx;
        }
    }
    int32_t corner = bnd[nb][n1];
    if (last_row) memcpy(last_row, bnd[nb], (size_t)(n1 + 1) * sizeof(int32_t));
    if (sw_max) *sw_max = best;
    if (sw_y) *sw_y = by;
    if (sw_x) *sw_x = bx;
    for (int64_t k = 0; k <= nb; ++k) free(bnd[k]);
    free(bnd); free((void *)prog); free(th); free(args);
    return corner;
}

/*
 * Many independent alignments on T threads (pairs claimed from an atomic
 * counter).  Pair i: kinds[i], a = seq + a_off[i] (a_len[i]), b = seq +
 * b_off[i] (b_len[i]).  Writes score[i] (corner) and, for SW pairs, sw_max[i],
 * sw_y[i], sw_x[i].
 */
typedef struct {
    const int32_t *kinds, *seq;
    const int64_t *a_off, *a_len, *b_off, *b_len;
    int64_t npairs;
    int rule; int32_t match, mismatch, gap;
    int32_t *score, *sw_max; int64_t *sw_y, *sw_x;
    _Atomic int64_t *next;
} batch_arg;

static void *batch_worker(void *p) {
    batch_arg *g = (batch_arg *)p;
    for (;;) {
        int64_t i = atomic_fetch_add(g->next, 1);
        if (i >= g->npairs) break;
        int32_t m = 0; int64_t y = 0, x = 0;
        g->score[i] = orc_align(g->kinds[i], g->rule, g->seq + g->a_off[i], g->a_len[i],
                                g->seq + g->b_off[i], g->b_len[i], g->match, g->mismatch, g->gap,
                                NULL, NULL, &m, &y, &x);
        if (g->sw_max) { g->sw_max[i] = m; g->sw_y[i] = y; g->sw_x[i] = x; }
    }
    return NULL;
}

void orc_align_batch_mt(const int32_t *kinds, const int32_t *seq,
                        const int64_t *a_off, const int64_t *a_len,
                        const int64_t *b_off, const int64_t *b_len, int64_t npairs,
                        int rule, int32_t match, int32_t mismatch, int32_t gap,
                        int32_t *score, int32_t *sw_max, int64_t *sw_y, int64_t *sw_x,
                        int nthreads) {
    _Atomic int64_t next;
    atomic_init(&next, 0);
    if (nthreads < 1) nthreads = 1;
    batch_arg g = {kinds, seq, a_off, a_len, b_off, b_len, npairs, rule, match, mismatch, gap,
                   score, sw_max, sw_y, sw_x, &next};
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, batch_worker, &g);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(th);
}

/*
 * Summed-area table, in place: the recurrence of the reference's SAT kernels,
 *   t[y][x] = t[y][x-1] + t[y-1][x] + t[y][x] - t[y-1][x-1]
 * (SAT/GPU_Hyperlane_Share.cu:169 first tiles, :231 last tiles; the same
 * expression at :196 for the hyperlane tiles), over rows 1..n2 and columns 1..n1
 * of a table with row stride ld (the reference's host function allocates rows of
 * n1 + 3 ints, SAT/GPU_Hyperlane_Share.cu:245-248, and its tiles start at row 1,
 * column 1 and end at column n1, :155-162, :210-214).  Row 0 and column 0 keep their
 * values.  Evaluated row after row, left to right, in 32-bit unsigned arithmetic
 * (the int wrap-around of the GPU).
 */
void orc_sat(int32_t *t, int64_t n1, int64_t n2, int64_t ld) {
    for (int64_t y = 1; y <= n2; ++y) {
        uint32_t *row = (uint32_t *)t + y * ld;
        const uint32_t *up = (const uint32_t *)t + (y - 1) * ld;
        for (int64_t x = 1; x <= n1; ++x)
            row[x] = row[x - 1] + up[x] + row[x] - up[x - 1];
    }
}

/*
 * The same table with all host threads, for the CPU baselines: the recurrence above
 * telescopes to t[y][x] = A[y][0] + A[0][x] - A[0][0] + sum_{1<=i<=y, 1<=j<=x} A[i][j]
 * (mod 2^32), so pass 1 turns each row into its prefix sums (rows across threads) and
 * pass 2 accumulates them down each column and adds the borders (column blocks across
 * threads).  Equal to orc_sat bit for bit; tested against it.
 */
typedef struct {
    uint32_t *t;
    int64_t n1, n2, ld;
    int pass, nthreads, id;
} sat_arg;

static void *sat_worker(void *p) {
    sat_arg *g = (sat_arg *)p;
    if (g->pass == 1) {
        for (int64_t y = 1 + g->id; y <= g->n2; y += g->nthreads) {
            uint32_t *row = g->t + y * g->ld, acc = 0;
            for (int64_t x = 1; x <= g->n1; ++x) { acc += row[x]; row[x] = acc; }
        }
    } else {
        const int64_t blk = 1024;
        const uint32_t *top = g->t;
        for (int64_t x0 = 1 + g->id * blk; x0 <= g->n1; x0 += g->nthreads * blk) {
            const int64_t x1 = x0 + blk - 1 < g->n1 ? x0 + blk - 1 : g->n1;
            for (int64_t y = 1; y <= g->n2; ++y) {
                uint32_t *row = g->t + y * g->ld;
                const uint32_t *up = g->t + (y - 1) * g->ld;
                const uint32_t left = row[0] - top[0];  /* A[y][0] - A[0][0] */
                if (y == 1) {
                    for (int64_t x = x0; x <= x1; ++x) row[x] = top[x] + left + row[x];
                } else {
                    const uint32_t upleft = up[0] - top[0];  /* A[y-1][0] - A[0][0] */
                    for (int64_t x = x0; x <= x1; ++x) row[x] = up[x] - upleft + left + row[x];
                }
            }
        }
    }
    return NULL;
}

void orc_sat_mt(int32_t *t, int64_t n1, int64_t n2, int64_t ld, int nthreads) {
    if (n1 <= 0 || n2 <= 0) return;
    if (nthreads < 1) nthreads = 1;
    pthread_t *th = (pthread_t *)malloc((size_t)nthreads * sizeof(pthread_t));
    sat_arg *args = (sat_arg *)malloc((size_t)nthreads * sizeof(sat_arg));
    for (int pass = 1; pass <= 2; ++pass) {
        for (int i = 0; i < nthreads; ++i) {
            sat_arg a = {(uint32_t *)t, n1, n2, ld, pass, nthreads, i};
            args[i] = a;
            pthread_create(&th[i], NULL, sat_worker, &args[i]);
        }
        for (int i = 0; i < nthreads; ++i) pthread_join(th[i], NULL);
    }
    free(th);
    free(args);
}
