// gme_tuned.h -- batched-kernel settings per length range, written by
// gpumemefficient_gb300/tune.py from a sweep on GB300 (the sweep table is kept
// beside the profiles).  A batch is planned with the entry whose length range
// [lo, hi] is nearest (in log scale) to the batch's own: the 2nd..98th
// percentile of sqrt(n1*n2) over its pairs -- unless the caller set its own.
#pragma once

namespace gme {

struct TunedBucket {
  int lo, hi;
  int warps_per_block, blocks_per_sm;
  long long block_min_cells, team_min_cells;
};

constexpr int TUNED_BUCKETS = 6;
constexpr TunedBucket TUNED[TUNED_BUCKETS > 0 ? TUNED_BUCKETS : 1] = {
    {32, 512, 4, 0, 1048576ll, 33554432ll},  // short: 785 GCUPS
    {512, 2048, 4, 0, 2097152ll, 16777216ll},  // mid: 1710 GCUPS
    {2048, 8192, 4, 0, 2097152ll, 16777216ll},  // long: 1250 GCUPS
    {8192, 16384, 4, 2, 8388608ll, 16777216ll},  // wide: 1119 GCUPS
    {64, 4096, 4, 0, 2097152ll, 33554432ll},  // mixed_64_4096: 1501 GCUPS
    {32, 16384, 4, 0, 2097152ll, 16777216ll},  // mixed_32_16384: 1098 GCUPS
};

}  // namespace gme
