// gme_noalloc.cu -- gme_align_device_noalloc: the plain alignment with no allocation.
//
// Some callers cannot call cudaMalloc: code running inside another runtime's
// memory pool or arena, a driver or plugin that must not allocate on its hot path,
// or a process whose allocator is fenced off while a graph or a real-time loop is
// live.  For them this entry point runs the same persistent wavefront kernel as
// gme_align_device, with its scratch memory (staged sequences, band-boundary rows,
// per-CTA maxima, ticket/status words) in one file-scope __device__ array below,
// sized for sequences of up to GME_NOALLOC_MAX_LEN symbols each.  The caller still
// passes its own input and output buffers.
//
// In host code `g_noalloc_scratch` names a host-side stand-in, not a device
// address: a kernel given it would fault or silently use the wrong memory.  So the
// first call on each device (with that device current) asks the runtime for the
// array's device address with cudaGetSymbolAddress, checks the result and keeps
// it; every later call on that device passes that pointer.  The first call should
// therefore come before any stream capture.
//
// Every call on a device shares the one array and the array keeps the last call's
// contents.  The ticket/status words are cleared on the stream at every call, and
// band-boundary rows carry per-band tags, so stale contents are never read.  Calls
// that overlap on the GPU (two streams, or two host threads) race on the array and
// must be serialised by the caller.
#include <cstdlib>
#include <mutex>

#include "gme_common.cuh"
#include "gme_internal.h"

namespace gme {
namespace {

constexpr long long kMaxLen = GME_NOALLOC_MAX_LEN;
constexpr int kMaxGrid = 64;  // CTAs, hence band-boundary slots (grid + 2)
constexpr int kMaxDevices = 64;
constexpr long long kPadL = 261, kPadR = 352;  // the plain kernel's pads of the staged a[]
constexpr long long kMaxBandRows = 1024;       // largest band the automatic shape picks
constexpr long long kChunk = PLAIN_C;          // columns per ring transaction

constexpr long long words(long long bytes) { return (bytes + 255) / 256 * 32; }  // 256-byte granules
constexpr long long kCtrlWords = words(16 * sizeof(int));
constexpr long long kBestWords = words(kMaxGrid * 32);
// the staged a[] and its copy shifted by two, each rounded to whole 16-byte groups
constexpr long long kAWords = words(2 * ((kPadL + kMaxLen + kPadR + 3) / 4 * 4) * sizeof(int));
constexpr long long kBWords = words((kMaxLen + kMaxBandRows) * sizeof(int));
constexpr long long kStride = ((kMaxLen + 1 + kChunk - 1) / kChunk) * kChunk + kChunk;
constexpr long long kSlotWords = (kMaxGrid + 2) * kStride;
constexpr long long kTotalWords = kCtrlWords + kBestWords + kAWords + kBWords + kSlotWords;

// The scratch: about 4.4 MB, held by every GPU that loads the library until exit.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kTotalWords];

struct DeviceScratch {
  bool ready = false;
  Workspace ws;
};
std::mutex g_mu;
DeviceScratch g_dev[kMaxDevices];

// Set-up for the current device: resolve the array's device address once.
int setup(int dev, DeviceScratch &d) {
  if (d.ready) return ST_OK;
  unsigned long long *base = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void **)&base, g_noalloc_scratch);
  if (e != cudaSuccess || base == nullptr) return ST_CUDA;
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ST_CUDA;
  Workspace &ws = d.ws;
  ws.device = dev;
  ws.sms = sms;
  unsigned long long *p = base;
  ws.ctrl = reinterpret_cast<int *>(p);
  p += kCtrlWords;
  ws.best = p;
  ws.best_cap = kMaxGrid;
  p += kBestWords;
  ws.a_pad = reinterpret_cast<int *>(p);
  ws.a_pad_cap = kAWords * 2;
  p += kAWords;
  ws.b_pad = reinterpret_cast<int *>(p);
  ws.b_pad_cap = kBWords * 2;
  p += kBWords;
  ws.slots = p;
  ws.slots_cap = kSlotWords;
  ws.slots_bytes = (size_t)kSlotWords * 8;
  // the array starts zeroed (device globals are zero-initialised), so every tag is unused
  ws.tag_next = 1;
  ws.sync_stream = nullptr;
  d.ready = true;
  return ST_OK;
}

}  // namespace
}  // namespace gme

extern "C" gme_status gme_align_device_noalloc(gme_kind kind, const int32_t *d_a, int64_t n1,
                                               const int32_t *d_b, int64_t n2,
                                               const gme_scoring *sc, gme_result *d_out,
                                               int32_t *d_last_row, int32_t *d_last_col,
                                               void *stream) {
  using namespace gme;
  if (kind < GME_LCS || kind > GME_SW || !d_out || n1 < 0 || n2 < 0 || (n1 > 0 && !d_a) ||
      (n2 > 0 && !d_b))
    return GME_ERR_INVALID;
  if (n1 > kMaxLen || n2 > kMaxLen) return GME_ERR_INVALID;  // beyond the static scratch
  gme_scoring def = gme_default_scoring();
  if (!sc) sc = &def;
  if (kind == GME_ED && sc->ed_boundary != GME_ED_REF_CPU && sc->ed_boundary != GME_ED_STANDARD)
    return GME_ERR_INVALID;
  if (kind == GME_SW) {
    long long m = llabs(sc->match);
    if (llabs(sc->mismatch) > m) m = llabs(sc->mismatch);
    if (llabs(sc->gap) > m) m = llabs(sc->gap);
    if (m * (long long)(n1 + n2 + 2) >= (1ll << 30)) return GME_ERR_OVERFLOW;
  }
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return GME_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_mu);
  DeviceScratch &d = g_dev[dev];
  int rc = setup(dev, d);
  if (rc != ST_OK) return (gme_status)rc;
  int R, NW, grid;
  plain_auto_config(d.ws.sms, n1, n2, &R, &NW, &grid);
  if (grid > kMaxGrid) grid = kMaxGrid;
  Scoring s;
  s.match = sc->match;
  s.mismatch = sc->mismatch;
  s.gap = sc->gap;
  s.ed_rule = sc->ed_boundary;
  rc = plain_run(d.ws, (int)kind, d_a, n1, d_b, n2, s, d_out, d_last_row, d_last_col,
                 (cudaStream_t)stream, R, NW, grid, 10ull * 1000 * 1000 * 1000);
  return (gme_status)rc;
}
