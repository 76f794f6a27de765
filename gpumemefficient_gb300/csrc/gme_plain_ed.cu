// gme_plain_ed.cu -- the plain wavefront kernel for edit distance (one translation
// unit per kind, so the three compile in parallel).
#include "gme_plain_kernel.cuh"

namespace gme {
template cudaError_t launch_plain_k<K_ED>(int R, int NW, const PlainParams &P, int grid, cudaStream_t st);
}  // namespace gme
