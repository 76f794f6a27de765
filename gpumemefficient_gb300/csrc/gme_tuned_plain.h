// gme_tuned_plain.h -- plain-path shape per table height, written by
// gpumemefficient_gb300/tune.py (sweep_plain) from a sweep on GB300: edit distance
// on square pairs.  plain_auto_config takes the entry whose n is nearest (in log
// scale) to the pair's row count n2.
#pragma once

namespace gme {

struct TunedPlain {
  int n, rows_per_lane, warps_per_band;
};

constexpr int TUNED_PLAIN = 6;
constexpr TunedPlain TUNED_PLAIN_TABLE[TUNED_PLAIN > 0 ? TUNED_PLAIN : 1] = {
    {2048, 2, 4},  // 32 GCUPS
    {4096, 2, 4},  // 67 GCUPS
    {8192, 2, 4},  // 139 GCUPS
    {16384, 2, 4},  // 283 GCUPS
    {32768, 2, 4},  // 570 GCUPS
    {65536, 2, 4},  // 1154 GCUPS
};

}  // namespace gme
