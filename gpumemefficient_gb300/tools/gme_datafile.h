// gme_datafile.h -- the reference's sequence data files, read and written.
//
// Layout (EditDistance/GPU_Hyperlane_Share.cpp:13-31 reads it, EditDistance/
// generator.cpp:50-66 writes it):
//   line 1: "n1 n2"
//   line 2: n1 symbols, each followed by one space
//   line 3: n2 symbols, each followed by one space
// The files are named DIR/str1_2_<e1>_str2_2_<e2>.txt for sequences of 2^e1 and
// 2^e2 symbols (EditDistance/GPU_Hyperlane_Share.cpp:62-82).
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace gme_tools {

inline std::string data_file(const std::string &dir, int e1, int e2) {
  return dir + "/str1_2_" + std::to_string(e1) + "_str2_2_" + std::to_string(e2) + ".txt";
}

// Reads a data file; false (and a message in *err) if it cannot be read or is short.
inline bool read_data_file(const std::string &path, std::vector<int32_t> &a, std::vector<int32_t> &b,
                           std::string *err) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) {
    if (err) *err = "ERROR: Input file cannot be opened!";
    return false;
  }
  long long n1 = -1, n2 = -1;
  bool ok = std::fscanf(f, "%lld %lld", &n1, &n2) == 2 && n1 >= 0 && n2 >= 0;
  a.assign(ok ? (size_t)n1 : 0, 0);
  b.assign(ok ? (size_t)n2 : 0, 0);
  for (long long i = 0; ok && i < n1; ++i) ok = std::fscanf(f, "%d", &a[(size_t)i]) == 1;
  for (long long i = 0; ok && i < n2; ++i) ok = std::fscanf(f, "%d", &b[(size_t)i]) == 1;
  std::fclose(f);
  if (!ok && err) *err = "ERROR: malformed data file " + path;
  return ok;
}

inline bool write_data_file(const std::string &path, const int32_t *a, long long n1, const int32_t *b,
                            long long n2) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  std::fprintf(f, "%lld %lld\n", n1, n2);
  for (long long i = 0; i < n1; ++i) std::fprintf(f, "%d ", a[i]);
  std::fprintf(f, "\n");
  for (long long i = 0; i < n2; ++i) std::fprintf(f, "%d ", b[i]);
  std::fprintf(f, "\n");
  return std::fclose(f) == 0;
}

// ---- summed-area-table data files ---------------------------------------------
// Layout (SAT/GPU_Hyperlane_Share.cpp:14-32 reads it, SAT/generator.cpp:48-61 writes
// it): line 1 "n1 n2", then n2 + 3 lines of n1 + 3 values, each followed by one
// space.  Named DIR/x_2_<e1>_y_2_<e2>.txt (SAT/GPU_Hyperlane_Share.cpp:70-87).

inline std::string sat_file(const std::string &dir, int e1, int e2) {
  return dir + "/x_2_" + std::to_string(e1) + "_y_2_" + std::to_string(e2) + ".txt";
}

// Reads the (n1 + 3) x (n2 + 3) values row after row; false (and *err) if short.
inline bool read_sat_file(const std::string &path, long long &n1, long long &n2, std::vector<int32_t> &t,
                          std::string *err) {
  FILE *f = std::fopen(path.c_str(), "r");
  if (!f) {
    if (err) *err = "ERROR: Input file cannot be opened!";
    return false;
  }
  n1 = n2 = -1;
  bool ok = std::fscanf(f, "%lld %lld", &n1, &n2) == 2 && n1 >= 0 && n2 >= 0;
  const long long cnt = ok ? (n1 + 3) * (n2 + 3) : 0;
  t.assign((size_t)cnt, 0);
  for (long long i = 0; ok && i < cnt; ++i) ok = std::fscanf(f, "%d", &t[(size_t)i]) == 1;
  std::fclose(f);
  if (!ok && err) *err = "ERROR: malformed data file " + path;
  return ok;
}

inline bool write_sat_file(const std::string &path, long long n1, long long n2, const int32_t *t) {
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  std::fprintf(f, "%lld %lld\n", n1, n2);
  for (long long y = 0; y < n2 + 3; ++y) {
    for (long long x = 0; x < n1 + 3; ++x) std::fprintf(f, "%d ", t[y * (n1 + 3) + x]);
    std::fprintf(f, "\n");
  }
  return std::fclose(f) == 0;
}

}  // namespace gme_tools
