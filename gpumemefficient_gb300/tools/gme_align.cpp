// gme-align -- the reference's command-line drivers on the GB300 library.
//
//   gme-align KIND E1 E2                  the CPU programs' form   (LCS/LCS.cpp:86-,
//                                         EditDistance/ED.cpp:84-, SmithWaterman/SW.cpp)
//   gme-align KIND E1 E2 TX TY ITR        the GPU drivers' form    (EditDistance/
//                                         GPU_Hyperlane_Share.cpp:47-115 and twins)
//   gme-align SAT E1 E2 [TX TY ITR]       the SAT driver's form    (SAT/
//                                         GPU_Hyperlane_Share.cpp:49-123)
//   options: --dir DIR (default ./Data)  --border cpu|gpu  --out FILE (SAT)
//
// KIND is LCS, ED or SW.  Reads DIR/str1_2_<E1>_str2_2_<E2>.txt as the reference
// does, aligns it ITR times (default 1) and prints what the reference prints:
//   input data loaded            (GPU-driver form)
//   last: <score>                (ED, SW; "lcs length: <score>" for LCS)
//   execution time: <ms> ms.     (mean wall time per alignment)
// The ED border follows the program being replaced: the CPU form computes ED.cpp's
// row 0 = [0,0,1,2,...] (ED.cpp:48-54), the GPU form GPU_setInit's [0,1,2,...]
// (EditDistance/GPU_Hyperlane_Share.cu:16-22); --border overrides it.  TX/TY are
// accepted and ignored: tiling is the library's.  Errors print a message and exit
// with status 1 (the reference calls exit(EXIT_FAILURE)).
//
// SAT reads DIR/x_2_<E1>_y_2_<E2>.txt, computes the summed-area table of its first
// n2 + 2 rows ITR times (each time from the file's values, as the reference's SOR,
// which never writes the table back, does) and prints what the reference prints:
//   execution time: <ms> ms.     (mean wall time per table, host table in and out)
// --out FILE writes the resulting table in the same file layout.
#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <vector>

#include "gme.h"
#include "gme_datafile.h"

static int run_sat(const std::vector<std::string> &pos, const std::string &dir, const std::string &out) {
  if (pos.size() != 3 && pos.size() != 6) {
    std::cout << "Incorrect Input Parameters. Must be two string sizes, two tile sizes, and one "
                 "iteration step."
              << std::endl;
    return 1;
  }
  const int e1 = std::atoi(pos[1].c_str()), e2 = std::atoi(pos[2].c_str());
  const int itr = pos.size() == 6 ? std::atoi(pos[5].c_str()) : 1;
  if (itr < 1) {
    std::cout << "The iteration step must be at least 1." << std::endl;
    return 1;
  }
  long long n1 = 0, n2 = 0;
  std::vector<int32_t> t;
  std::string err;
  if (!gme_tools::read_sat_file(gme_tools::sat_file(dir, e1, e2), n1, n2, t, &err)) {
    std::cout << err << std::endl;
    return 1;
  }
  const long long ld = n1 + 3, cells = (n2 + 1) * ld;  // rows 0..n2 are read
  std::vector<int32_t> work(t.begin(), t.begin() + cells);
  gme_context *ctx = nullptr;
  gme_status st = gme_create(0, &ctx);
  if (st != GME_OK) {
    std::cout << "ERROR: " << gme_status_string(st) << std::endl;
    return 1;
  }
  st = gme_sat(ctx, work.data(), n1, n2, ld);  // untimed warm-up
  double ms = 0.0;
  for (int i = 0; st == GME_OK && i < itr; ++i) {
    std::copy(t.begin(), t.begin() + cells, work.begin());
    const auto t0 = std::chrono::steady_clock::now();
    st = gme_sat(ctx, work.data(), n1, n2, ld);
    ms += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
  if (st != GME_OK) {
    std::cout << "ERROR: " << gme_status_string(st) << ": " << gme_last_error(ctx) << std::endl;
    gme_destroy(ctx);
    return 1;
  }
  std::cout << "execution time: " << ms / itr << " ms." << std::endl;
  gme_destroy(ctx);
  if (!out.empty()) {
    std::copy(work.begin(), work.end(), t.begin());
    if (!gme_tools::write_sat_file(out, n1, n2, t.data())) {
      std::cout << "ERROR: cannot write " << out << std::endl;
      return 1;
    }
  }
  return 0;
}

int main(int argc, char **argv) {
  std::vector<std::string> pos;
  std::string dir = "./Data", border, out;
  for (int i = 1; i < argc; ++i) {
    const std::string s = argv[i];
    if (s == "--dir" && i + 1 < argc) dir = argv[++i];
    else if (s == "--border" && i + 1 < argc) border = argv[++i];
    else if (s == "--out" && i + 1 < argc) out = argv[++i];
    else pos.push_back(s);
  }
  if (!pos.empty() && (pos[0] == "SAT" || pos[0] == "sat")) return run_sat(pos, dir, out);
  if (pos.size() != 3 && pos.size() != 6) {
    std::cout << "Incorrect Input Parameters. Must be a kind (LCS, ED, SW), two string sizes, "
                 "and optionally two tile sizes and one total iteration step."
              << std::endl;
    return 1;
  }
  gme_kind kind;
  if (pos[0] == "LCS" || pos[0] == "lcs") kind = GME_LCS;
  else if (pos[0] == "ED" || pos[0] == "ed") kind = GME_ED;
  else if (pos[0] == "SW" || pos[0] == "sw") kind = GME_SW;
  else {
    std::cout << "Unknown kind " << pos[0] << " (LCS, ED or SW)." << std::endl;
    return 1;
  }
  const int e1 = std::atoi(pos[1].c_str()), e2 = std::atoi(pos[2].c_str());
  const bool gpu_form = pos.size() == 6;
  const int itr = gpu_form ? std::atoi(pos[5].c_str()) : 1;
  if (itr < 1) {
    std::cout << "The iteration step must be at least 1." << std::endl;
    return 1;
  }
  std::vector<int32_t> a, b;
  std::string err;
  if (!gme_tools::read_data_file(gme_tools::data_file(dir, e1, e2), a, b, &err)) {
    std::cout << err << std::endl;
    return 1;
  }
  if (gpu_form) std::cout << "input data loaded" << std::endl;

  gme_scoring sc = gme_default_scoring();
  const bool gpu_border = border.empty() ? gpu_form : border == "gpu";
  sc.ed_boundary = gpu_border ? GME_ED_STANDARD : GME_ED_REF_CPU;
  gme_context *ctx = nullptr;
  gme_status st = gme_create(0, &ctx);
  if (st != GME_OK) {
    std::cout << "ERROR: " << gme_status_string(st) << std::endl;
    return 1;
  }
  gme_result r{};
  // one untimed call first: the reference's timed loop also runs on a warm device
  st = gme_align(ctx, kind, a.data(), (int64_t)a.size(), b.data(), (int64_t)b.size(), &sc, &r, nullptr,
                 nullptr);
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; st == GME_OK && i < itr; ++i)
    st = gme_align(ctx, kind, a.data(), (int64_t)a.size(), b.data(), (int64_t)b.size(), &sc, &r,
                   nullptr, nullptr);
  const double ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() / itr;
  if (st != GME_OK) {
    std::cout << "ERROR: " << gme_status_string(st) << ": " << gme_last_error(ctx) << std::endl;
    gme_destroy(ctx);
    return 1;
  }
  if (kind == GME_LCS) std::cout << "lcs length: " << r.score << std::endl;
  else std::cout << "last: " << r.score << std::endl;
  std::cout << "execution time: " << ms << " ms." << std::endl;
  gme_destroy(ctx);
  return 0;
}
