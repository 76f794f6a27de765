// gme_common.cuh -- pieces shared by the plain, batched and served kernels.
//
// Recurrences (bit-exact with the reference CPU programs):
//   LCS  LCS/LCS.cpp:59-63            t = a==b ? diag+1 : max(left, up)
//   ED   EditDistance/ED.cpp:63-65     t = a==b ? diag : min(up, left, diag) + 1
//   SW   SmithWaterman/SW.cpp:63-65    t = max(left+gap, up+gap, diag+s(a,b), 0)
// Each is evaluated in a form with a single 3-input DPX min/max on the path from
// the two neighbours that were produced one anti-diagonal earlier (up, left):
//
//   LCS: t = max3(up, left, diag + eq).  Equal to the reference form because in an
//        LCS table with zero borders adjacent cells differ by 0 or 1, so on a match
//        diag+1 >= max(up, left), and off a match diag <= max(up, left).
//   ED:  stored as w = v - (x + y);  w = min3(up_w, left_w, diag_w + (eq ? -2 : -1)).
//        Equal to the reference form because, for both boundary conventions
//        (row 0 [0,0,1,2,..] or [0,1,2,..], column 0 [0,1,2,..]), neighbouring
//        cells differ by at most 1, so on a match diag <= up+1 and diag <= left+1
//        and "diag on a match" equals min(up+1, left+1, diag).  The induction: the
//        borders have steps in {-1,0,1}; if the row above and the cell to the left
//        do, min(up+1, left+1, diag+c) with c in {0,1} is within 1 of both.
//   SW:  t = max(max(up + gap, max(left + gap, diag + s)), 0), two DPX add-max ops.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gme {

enum : int { K_LCS = 0, K_ED = 1, K_SW = 2 };

// Status codes shared with include/gme.h (gme_status).
enum : int { ST_OK = 0, ST_INVALID = 1, ST_CUDA = 2, ST_NOMEM = 3, ST_TIMEOUT = 4 };

struct Scoring {
  int match, mismatch, gap, ed_rule;  // ed_rule: 0 = ED.cpp boundary, 1 = standard
};

// ---------------------------------------------------------------------------
// Cell recurrences.  `D` is the diagonal term, formed one step early.
// ---------------------------------------------------------------------------
template <int KIND> struct Rec;

template <> struct Rec<K_LCS> {
  int ceq, cne;
  __device__ __forceinline__ explicit Rec(const Scoring &) : ceq(1), cne(0) {}
  __device__ __forceinline__ int cell(int up, int left, int D) const {
    return __vimax3_s32(up, left, D);
  }
  // stored value -> table value at (x, y)
  __device__ __forceinline__ static int to_v(int w, long long, long long) { return w; }
  __device__ __forceinline__ static int top(long long, int) { return 0; }
  __device__ __forceinline__ static int left(long long) { return 0; }
};

template <> struct Rec<K_ED> {
  int ceq, cne;
  __device__ __forceinline__ explicit Rec(const Scoring &) : ceq(-2), cne(-1) {}
  __device__ __forceinline__ int cell(int up, int left, int D) const {
    return __vimin3_s32(up, left, D);
  }
  __device__ __forceinline__ static int to_v(int w, long long x, long long y) {
    return (int)(w + x + y);
  }
  // stored form of row 0 at column x: ED.cpp gives [0,0,1,2,..] (w = 0,-1,-1,..),
  // the GPU_setInit convention gives [0,1,2,..] (w = 0).
  __device__ __forceinline__ static int top(long long x, int rule) {
    return (rule == 0 && x > 0) ? -1 : 0;
  }
  __device__ __forceinline__ static int left(long long) { return 0; }  // v = y
};

template <> struct Rec<K_SW> {
  int ceq, cne, gap;
  __device__ __forceinline__ explicit Rec(const Scoring &s) : ceq(s.match), cne(s.mismatch), gap(s.gap) {}
  __device__ __forceinline__ int cell(int up, int left, int D) const {
    return __viaddmax_s32_relu(up, gap, __viaddmax_s32(left, gap, D));
  }
  __device__ __forceinline__ static int to_v(int w, long long, long long) { return w; }
  __device__ __forceinline__ static int top(long long, int) { return 0; }
  __device__ __forceinline__ static int left(long long) { return 0; }
};

// ---------------------------------------------------------------------------
// Memory-order helpers (PTX scopes written out so the intent is explicit).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int ld_acquire_cta(const int *p) {
  int v;
  asm volatile("ld.acquire.cta.shared.b32 %0, [%1];" : "=r"(v) : "r"((unsigned)__cvta_generic_to_shared(p)) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_cta(int *p, int v) {
  asm volatile("st.release.cta.shared.b32 [%0], %1;" :: "r"((unsigned)__cvta_generic_to_shared(p)), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_gpu_u64(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed_gpu_u64(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" :: "l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_acquire_gpu_s32(const int *p) {
  int v;
  asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_relaxed_gpu_s32(const int *p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// A bounded wait.  `poll()` is re-evaluated until it returns true; the deadline
// (now + timeout) starts at the first failed poll, and every 64 polls the clock,
// the block-wide abort word and the grid-wide status word are checked.
// Returns false (after recording ST_TIMEOUT in *status) when the deadline passes
// or another warp has already given up; the caller then abandons its work.
// Called by all 32 lanes of a warp; poll() must return the same value in each.
struct Waiter {
  unsigned long long timeout, deadline;
  int *status;          // global status word (0 = fine)
  volatile int *abort;  // block-local abort flag in shared memory
  __device__ __forceinline__ Waiter(unsigned long long timeout_ns, int *st, volatile int *ab)
      : timeout(timeout_ns), deadline(0), status(st), abort(ab) {}
  template <class F>
  __device__ __forceinline__ bool wait(F poll, int sleep_ns = 0) {
    if (poll()) return true;  // fast path: no clock read
    deadline = globaltimer_ns() + timeout;
    unsigned it = 0;
    while (!poll()) {
      if ((++it & 63u) == 0) {
        // decide once per warp so that every lane leaves the loop together
        int give = 0;
        if (*abort) give = 1;
        else if (ld_relaxed_gpu_s32(status) != 0) give = 2;
        else if (globaltimer_ns() > deadline) give = 3;
        give = __shfl_sync(0xffffffffu, give, 0);
        if (give) {
          if (give == 3) atomicCAS(status, 0, ST_TIMEOUT);
          *abort = 1;
          return false;
        }
      }
      if (sleep_ns) __nanosleep(sleep_ns);
    }
    return true;
  }
};

}  // namespace gme
