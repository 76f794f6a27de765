// gme-refcheck -- calls every one of the reference's host-function signatures, as the
// reference drivers call them, through libgme.so (include/gme_reference.h).
//
//   gme-refcheck SEQFILE [SATFILE]
//
// SEQFILE is a sequence data file in the reference's layout (gme_datafile.h).  Each of
// the eight LCS/ED/SW overloads runs on its two sequences with the arguments the
// reference drivers pass: paddX = 3, paddY = 1, a caller-owned table of
// (n2 + paddX) * (n1 + paddY) ints, tX = 32, tY = 128
// (EditDistance/GPU_Hyperlane_Share.cpp:86-108 and its LCS/SW twins; the 4-argument forms
// are the TILE_SHARE / naive drivers', LCS/GPU_TILE_SHARE.cpp, EditDistance/GPU.cpp).
// SATFILE, if given, is a summed-area-table data file in the reference's layout; SOR
// (SAT/GPU_Hyperlane_Share.cpp) runs on its table.
//
// Output, one line per call: the overload's name and argument count, then the value it
// returned (SOR, in both its forms: the sum of rows 1..n2 x columns 1..n1 of the result
// modulo 2^32, then the bottom-right cell).  Exit status 1 if a call reports an error.
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "gme_datafile.h"
#include "gme_reference.h"

int main(int argc, char **argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: gme-refcheck SEQFILE [SATFILE]\n");
    return 1;
  }
  std::vector<int32_t> a, b;
  std::string err;
  if (!gme_tools::read_data_file(argv[1], a, b, &err)) {
    std::fprintf(stderr, "gme-refcheck: %s\n", err.c_str());
    return 1;
  }
  const int n1 = (int)a.size(), n2 = (int)b.size();
  const int paddX = 3, paddY = 1, tX = 32, tY = 128;
  std::vector<int> table((size_t)(n2 + paddX) * (n1 + paddY), 0);
  int bad = 0;
  auto report = [&](const char *name, int v) {
    const gme_status s = gme_reference_last_status();
    std::printf("%s %d\n", name, v);
    if (s != GME_OK) {
      std::fprintf(stderr, "gme-refcheck: %s: %s\n", name, gme_status_string(s));
      bad = 1;
    }
  };
  report("LCS/7", LCS(n1, n2, a.data(), b.data(), paddX, paddY, table.data()));
  report("LCS/4", LCS(n1, n2, a.data(), b.data()));
  report("ED/9", ED(n1, n2, a.data(), b.data(), paddX, paddY, table.data(), tX, tY));
  report("ED/7", ED(n1, n2, a.data(), b.data(), paddX, paddY, table.data()));
  report("ED/4", ED(n1, n2, a.data(), b.data()));
  report("SW/9", SW(n1, n2, a.data(), b.data(), paddX, paddY, table.data(), tX, tY));
  report("SW/7", SW(n1, n2, a.data(), b.data(), paddX, paddY, table.data()));
  report("SW/4", SW(n1, n2, a.data(), b.data()));
  if (argc > 2) {
    long long s1 = 0, s2 = 0;
    std::vector<int32_t> t;
    if (!gme_tools::read_sat_file(argv[2], s1, s2, t, &err)) {
      std::fprintf(stderr, "gme-refcheck: %s\n", err.c_str());
      return 1;
    }
    const long long ld = s1 + 3;
    // both forms, each on its own copy of the file's table
    for (int form = 5; form >= 3; form -= 2) {
      std::vector<int32_t> u = t;
      if (form == 5) SOR((int)s1, (int)s2, u.data(), tX, tY);
      else SOR((int)s1, (int)s2, u.data());
      uint32_t sum = 0;
      for (long long y = 1; y <= s2; ++y)
        for (long long x = 1; x <= s1; ++x) sum += (uint32_t)u[y * ld + x];
      std::printf("SOR/%d %u %d\n", form, sum, u[s2 * ld + s1]);
      if (gme_reference_last_status() != GME_OK) {
        std::fprintf(stderr, "gme-refcheck: SOR: %s\n", gme_status_string(gme_reference_last_status()));
        bad = 1;
      }
    }
  }
  return bad;
}
