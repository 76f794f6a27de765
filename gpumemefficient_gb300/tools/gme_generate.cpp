// gme-generate -- writes the reference's data files from a seeded PRNG.
//
//   gme-generate E1 E2 [--seed S] [--dir DIR] [--alphabet A]
//   gme-generate --sat E1 E2 [--seed S] [--dir DIR] [--min E]
//
// Like EditDistance/generator.cpp:10-77: draws 2^E1 and 2^E2 symbols uniform over
// {0..A-1} (A = 4 there: rand()%4) and writes DIR/str1_2_<e1>_str2_2_<e2>.txt for
// (e1, e2) = (E1, E2), (E1-1, E2-1), ... while e1 >= 8, each file holding prefixes of
// the same two sequences.  The reference seeds with srand(time(NULL)), so its files
// are not reproducible; here the seed is an argument (default 0x9E3779B9), drawn
// with std::mt19937_64.
//
// --sat: like SAT/generator.cpp:10-74, one array of (2^E1 + 3) x (2^E2 + 3) values
// uniform over 0..9999 (rand() % 10000 there), written as DIR/x_2_<e1>_y_2_<e2>.txt
// for (e1, e2) = (E1, E2), (E1-1, E2-1), ... while e1 >= --min (13 there); each file
// holds the array's first (2^e1 + 3) x (2^e2 + 3) values in rows of 2^e1 + 3, as the
// reference writes them.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <random>
#include <string>
#include <vector>

#include "gme_datafile.h"

int main(int argc, char **argv) {
  std::vector<std::string> pos;
  unsigned long long seed = 0x9E3779B9ull;
  std::string dir = "./Data";
  int alphabet = 4, min_e = 13;
  bool sat = false;
  for (int i = 1; i < argc; ++i) {
    const std::string s = argv[i];
    if (s == "--seed" && i + 1 < argc) seed = std::strtoull(argv[++i], nullptr, 0);
    else if (s == "--dir" && i + 1 < argc) dir = argv[++i];
    else if (s == "--alphabet" && i + 1 < argc) alphabet = std::atoi(argv[++i]);
    else if (s == "--min" && i + 1 < argc) min_e = std::atoi(argv[++i]);
    else if (s == "--sat") sat = true;
    else pos.push_back(s);
  }
  if (pos.size() != 2 || alphabet < 1) {
    std::cout << "Incorrect parameters have been passed." << std::endl;
    std::cout << "usage: gme-generate E1 E2 [--seed S] [--dir DIR] [--alphabet A]" << std::endl;
    return 1;
  }
  int e1 = std::atoi(pos[0].c_str()), e2 = std::atoi(pos[1].c_str());
  if (e1 < 0 || e2 < 0 || e1 > 30 || e2 > 30) {
    std::cout << "sizes must be powers 0..30" << std::endl;
    return 1;
  }
  if (sat) {
    if (e1 > 16 || e2 > 16) {
      std::cout << "SAT sizes must be powers 0..16" << std::endl;
      return 1;
    }
    std::mt19937_64 rng(seed);
    std::uniform_int_distribution<int> val(0, 9999);
    std::vector<int32_t> t((size_t)(((1ll << e1) + 3) * ((1ll << e2) + 3)));
    for (auto &x : t) x = val(rng);
    do {
      const std::string path = gme_tools::sat_file(dir, e1, e2);
      if (!gme_tools::write_sat_file(path, 1ll << e1, 1ll << e2, t.data())) {
        std::cout << "ERROR: cannot write " << path << std::endl;
        return 1;
      }
      --e1;
      --e2;
    } while (e1 >= min_e && e2 >= 0);
    return 0;
  }
  const long long s1 = 1ll << e1, s2 = 1ll << e2;
  std::mt19937_64 rng(seed);
  std::uniform_int_distribution<int> sym(0, alphabet - 1);
  std::vector<int32_t> a((size_t)s1), b((size_t)s2);
  for (auto &x : a) x = sym(rng);
  for (auto &x : b) x = sym(rng);
  do {
    const std::string path = gme_tools::data_file(dir, e1, e2);
    if (!gme_tools::write_data_file(path, a.data(), 1ll << e1, b.data(), e2 >= 0 ? 1ll << e2 : 0)) {
      std::cout << "ERROR: cannot write " << path << std::endl;
      return 1;
    }
    --e1;
    --e2;
  } while (e1 >= 8 && e2 >= 0);
  return 0;
}
