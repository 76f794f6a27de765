// gme_reference.cpp -- the reference's host-function signatures (include/gme_reference.h)
// implemented on the C ABI.
#include <climits>
#include <mutex>

#include "gme_reference.h"

namespace {
std::mutex g_mu;
gme_context *g_ctx = nullptr;
thread_local gme_status g_last = GME_OK;

bool ensure_ctx() {
  if (!g_ctx) {
    gme_status s = gme_create(0, &g_ctx);
    if (s != GME_OK) {
      g_ctx = nullptr;
      g_last = s;
      return false;
    }
  }
  return true;
}

int32_t run(gme_kind kind, int32_t n1, int32_t n2, const int32_t *a, const int32_t *b) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!ensure_ctx()) return INT_MIN;
  gme_scoring sc = gme_default_scoring();
  sc.ed_boundary = GME_ED_STANDARD;  // GPU_setInit
  gme_result r;
  gme_status s = gme_align(g_ctx, kind, a, n1, b, n2, &sc, &r, nullptr, nullptr);
  g_last = s;
  return s == GME_OK ? r.score : INT_MIN;
}

// the reference's layout: rows 0..n2 of n1 + 3 ints (SAT/GPU_Hyperlane_Share.cu:245-248)
int32_t run_sat(int32_t n1, int32_t n2, int32_t *table) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!ensure_ctx()) return (int32_t)g_last;
  g_last = gme_sat(g_ctx, table, n1, n2, (int64_t)n1 + 3);
  return (int32_t)g_last;
}
}  // namespace

int LCS(int n1, int n2, int *arr1, int *arr2, int, int, int *) { return run(GME_LCS, n1, n2, arr1, arr2); }
int LCS(int n1, int n2, int *arr1, int *arr2) { return run(GME_LCS, n1, n2, arr1, arr2); }
int ED(int n1, int n2, int *arr1, int *arr2, int, int, int *, int, int) { return run(GME_ED, n1, n2, arr1, arr2); }
int ED(int n1, int n2, int *arr1, int *arr2, int, int, int *) { return run(GME_ED, n1, n2, arr1, arr2); }
int ED(int n1, int n2, int *arr1, int *arr2) { return run(GME_ED, n1, n2, arr1, arr2); }
int SW(int n1, int n2, int *arr1, int *arr2, int, int, int *, int, int) { return run(GME_SW, n1, n2, arr1, arr2); }
int SW(int n1, int n2, int *arr1, int *arr2, int, int, int *) { return run(GME_SW, n1, n2, arr1, arr2); }
int SW(int n1, int n2, int *arr1, int *arr2) { return run(GME_SW, n1, n2, arr1, arr2); }
void SOR(int n1, int n2, int *table, int, int) { run_sat(n1, n2, table); }
void SOR(int n1, int n2, int *table) { run_sat(n1, n2, table); }

extern "C" {
gme_status gme_reference_last_status(void) { return g_last; }
int32_t gme_ref_lcs(int32_t n1, int32_t n2, const int32_t *a, const int32_t *b) { return run(GME_LCS, n1, n2, a, b); }
int32_t gme_ref_ed(int32_t n1, int32_t n2, const int32_t *a, const int32_t *b) { return run(GME_ED, n1, n2, a, b); }
int32_t gme_ref_sw(int32_t n1, int32_t n2, const int32_t *a, const int32_t *b) { return run(GME_SW, n1, n2, a, b); }
int32_t gme_ref_sor(int32_t n1, int32_t n2, int32_t *table) { return run_sat(n1, n2, table); }
}
