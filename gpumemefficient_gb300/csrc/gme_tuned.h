// gme_tuned.h -- batched-kernel settings per length range, written by
// gpumemefficient_gb300/tune.py from a sweep on GB300 (the sweep table is kept
// beside the profiles).  A batch is planned with the entry whose range [lo, hi]
// is nearest (in log scale) to the batch's own -- both the 2nd..98th percentile
// of sqrt(n1*n2) + 1 over the pairs, for an entry those of the batch it was
// tuned on -- unless the caller set its own.
#pragma once

namespace gme {

struct TunedBucket {
  float lo, hi;
  int warps_per_block, blocks_per_sm;
  long long block_min_cells, team_min_cells;
  int team_split;
  int rows_per_lane;  // 4 or 2
  int packed16;       // 1: packed 16-bit cells where values fit
};

constexpr int TUNED_BUCKETS = 6;
constexpr TunedBucket TUNED[TUNED_BUCKETS > 0 ? TUNED_BUCKETS : 1] = {
    {43.0f, 388.9f, 4, 0, 4194304ll, -1ll, 2, 4, 1},  // short: 847 GCUPS
    {587.9f, 1788.1f, 4, 0, 8388608ll, -1ll, 2, 4, 1},  // mid: 2052 GCUPS
    {2355.9f, 7059.6f, 8, 0, 2097152ll, -1ll, 2, 4, 1},  // long: 1648 GCUPS
    {8535.6f, 14944.5f, 8, 0, 4194304ll, 67108864ll, 3, 4, 1},  // wide: 1435 GCUPS
    {99.3f, 2669.9f, 4, 0, 4194304ll, 33554432ll, 4, 4, 1},  // mixed_64_4096: 1784 GCUPS
    {60.0f, 8309.6f, 4, 0, 4194304ll, 33554432ll, 4, 4, 0},  // mixed_32_16384: 1196 GCUPS
};

}  // namespace gme
