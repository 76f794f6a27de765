// gme_batch_r2.cu -- the batched work-queue kernel at 2 rows per lane (64-row bands),
// which the autotuner may pick for a length range; its own translation unit, so that it
// compiles beside gme_batch.cu.  The 16-bit packed engine exists only at 4 rows per lane.
// Only the 8-warp CTA is built: the 4-warp one (register-capped for 3 CTAs per SM) let
// warps read the job word before thread 0 had written it, so that its warps ran
// different jobs and a bounded wait gave up; the 8-warp one passes every batch test.
#include "gme_batch_kernel.cuh"

namespace gme {

template <int NW>
static cudaError_t launch_r2_t(const BatchParams &P, int grid, cudaStream_t st) {
  batch_kernel<2, NW><<<grid, NW * 32, sizeof(BatchSmem<NW>), st>>>(P);
  return cudaGetLastError();
}

cudaError_t batch_launch_r2(int NW, const BatchParams &P, int grid, cudaStream_t st) {
  return NW == 8 ? launch_r2_t<8>(P, grid, st) : cudaErrorInvalidValue;
}

template <int NW>
static int occupancy_r2_t() {
  int n = 0;
  const size_t smem = sizeof(BatchSmem<NW>);
  cudaFuncSetAttribute(batch_kernel<2, NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, batch_kernel<2, NW>, NW * 32, smem);
  return n;
}

int batch_occupancy_r2(int NW) { return NW == 8 ? occupancy_r2_t<8>() : 0; }

}  // namespace gme
