// gme_internal.h -- host-side declarations shared by the library's translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>

#include "gme.h"

namespace gme {

struct Scoring;

// Device workspace owned by one context.  Grows on demand, never shrinks, and is
// reused across calls so that a steady stream of calls allocates nothing.
struct Workspace {
  int device = 0;
  int sms = 0;
  int *a_pad = nullptr;
  long long a_pad_cap = 0;
  int *b_pad = nullptr;
  long long b_pad_cap = 0;
  unsigned long long *slots = nullptr;  // tagged band-boundary rows
  long long slots_cap = 0;              // words
  size_t slots_bytes = 0;
  void *best = nullptr;                 // per-CTA SW maxima (32 bytes each)
  int best_cap = 0;
  int *ctrl = nullptr;                  // ticket, status, spare
  unsigned tag_next = 1;                // next unused band tag since slots were cleared
  long long launches = 0;               // kernels launched (counted by the host)
  std::string last_error;
  cudaStream_t sync_stream = nullptr;   // stream drained before a workspace is regrown

  int reserve(long long a_len, long long b_len, long long slot_words, int nbest);
  int fail(cudaError_t e, const char *what);
  int fail_msg(int status, const std::string &msg);
  void release();
};

// plain path (gme_plain.cu)
bool plain_config_valid(int R, int NW);
void plain_auto_config(int sms, long long n1, long long n2, int *R, int *NW, int *grid);
int plain_run(Workspace &ws, int kind, const int *d_a, long long n1, const int *d_b, long long n2,
              const Scoring &sc, gme_result *d_out, int *d_last_row, int *d_last_col,
              cudaStream_t st, int R, int NW, int grid, unsigned long long timeout_ns);
int debug_wait_timeout(Workspace &ws, unsigned long long timeout_ns, int *kernel_status,
                       cudaStream_t st);

}  // namespace gme
