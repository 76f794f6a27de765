// gme_plain_sw.cu -- the plain wavefront kernel for Smith-Waterman (one translation
// unit per kind, so the three compile in parallel).
#include "gme_plain_kernel.cuh"

namespace gme {
template cudaError_t launch_plain_k<K_SW>(int R, int NW, const PlainParams &P, int grid, cudaStream_t st);
}  // namespace gme
