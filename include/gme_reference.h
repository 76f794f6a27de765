/*
 * gme_reference.h -- the reference's own host-function signatures, served by libgme.so.
 *
 * A reference driver (e.g. EditDistance/GPU_Hyperlane_Share.cpp) that includes this
 * header instead of its GPU_*.h and links against libgme.so computes the same value
 * with the GB300 wavefront kernel.  These are C++ functions (C++ linkage, overloaded
 * exactly as the reference's headers declare them), built on the C ABI in gme.h.
 *
 * Semantics kept from the reference:
 *   - arr1 (length n1) runs along x, arr2 (length n2) along y; the return value is
 *     the bottom-right cell (EditDistance/GPU_Hyperlane_Share.cu:765).
 *   - ED uses the boundary the reference GPU code initialises with GPU_setInit
 *     (row 0 = 0,1,2,..; EditDistance/GPU_Hyperlane_Share.cu:16-22,
 *     EditDistance/GPU.cu:12-18), i.e. GME_ED_STANDARD.
 *   - SW uses match +3, mismatch -3, gap -2 (SmithWaterman/GPU_Hyperlane_Share.cu:16-18,
 *     :402-404) and returns the corner cell, not the maximum.
 *   - `table` is not written: the reference fills it only in its -DDEBUG build
 *     (EditDistance/GPU_Hyperlane_Share.cu:766-777).  paddX/paddY/tX/tY are accepted
 *     and ignored; tile shapes are chosen by the library.
 * Differences, on purpose:
 *   - Errors never call exit() (the reference's checkGPUError does, :682-687).  A failed
 *     call returns INT_MIN and gme_reference_last_status() reports why.
 *   - The reference's ED/SW directories ship a GPU_TILE_SHARE.cu that computes LCS under
 *     the name LCS; the 4-argument ED/SW here compute ED/SW as their names say.
 *   - All device state lives in one process-wide context on device 0 (the reference
 *     hard-codes cudaSetDevice(0)); calls are serialised by a mutex.
 */
#ifndef GME_REFERENCE_H
#define GME_REFERENCE_H

#include "gme.h"

#ifdef __cplusplus
/* LCS/GPU_Hyperlane_Share.h:5, LCS/GPU_Hyperlane_Cache.h:5 */
int LCS(int n1, int n2, int *arr1, int *arr2, int paddX, int paddY, int *table);
/* LCS/GPU_TILE_SHARE.h:5, LCS/GPU_TILE_NOSHARE.h:5, LCS/GPU.h:5 */
int LCS(int n1, int n2, int *arr1, int *arr2);
/* EditDistance/GPU_Hyperlane_Share.h:5 */
int ED(int n1, int n2, int *arr1, int *arr2, int paddX, int paddY, int *table, int tX, int tY);
/* EditDistance/GPU_Hyperlane_Cache.h:5 */
int ED(int n1, int n2, int *arr1, int *arr2, int paddX, int paddY, int *table);
/* EditDistance/GPU.h:5 */
int ED(int n1, int n2, int *arr1, int *arr2);
/* SmithWaterman/GPU_Hyperlane_Share.h:5 */
int SW(int n1, int n2, int *arr1, int *arr2, int paddX, int paddY, int *table, int tX, int tY);
/* SmithWaterman/GPU_Hyperlane_Cache.h:5 */
int SW(int n1, int n2, int *arr1, int *arr2, int paddX, int paddY, int *table);
/* SmithWaterman/GPU.h:5 */
int SW(int n1, int n2, int *arr1, int *arr2);
/* SAT/GPU_Hyperlane_Share.h:5: the summed-area table of the reference's layout (rows
 * 0..n2, row length n1 + 3; gme_sat).  Unlike the reference, which leaves `table`
 * untouched (its copy back is commented out, SAT/GPU_Hyperlane_Share.cu:321), rows
 * 1..n2 x columns 1..n1 of `table` receive the result.  tX, tY are accepted and
 * ignored. */
void SOR(int n1, int n2, int *table, int tX, int tY);
/* SAT/GPU_Hyperlane_Cache.h:5: the same, in the Cache driver's three-argument form. */
void SOR(int n1, int n2, int *table);
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* Status of the last reference-signature call made by this thread. */
gme_status gme_reference_last_status(void);
/* C-callable forms of the same three computations (for FFI users). */
int32_t gme_ref_lcs(int32_t n1, int32_t n2, const int32_t *arr1, const int32_t *arr2);
int32_t gme_ref_ed(int32_t n1, int32_t n2, const int32_t *arr1, const int32_t *arr2);
int32_t gme_ref_sw(int32_t n1, int32_t n2, const int32_t *arr1, const int32_t *arr2);
/* SOR for FFI users: 0 on success, else the gme_status. */
int32_t gme_ref_sor(int32_t n1, int32_t n2, int32_t *table);
#ifdef __cplusplus
}
#endif

#endif /* GME_REFERENCE_H */
