// logf_table.cu — builds the exception table that makes the device's logf
// agree bit for bit with this machine's C library logf (see flye_logf in
// common.cuh).  For every float x in [1, 2^24) it compares logf(x) with
// log_wide(x) rounded to float and writes the disagreements as
// (x bits, logf bits) pairs, sorted by x:  u32 count, then count pairs.
// Host-only program; compiled with -ffp-contract=off so log_wide rounds here
// exactly as its explicit-intrinsic device form does.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <thread>
#include <vector>

#include "common.cuh"

int main(int argc, char** argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: %s OUT\n", argv[0]);
    return 2;
  }
  const float lo_f = 1.0f, hi_f = 16777216.0f;
  uint32_t lo, hi;
  std::memcpy(&lo, &lo_f, 4);
  std::memcpy(&hi, &hi_f, 4);
  unsigned nt = std::thread::hardware_concurrency();
  if (nt == 0) nt = 4;
  if (nt > 64) nt = 64;
  std::vector<std::vector<uint32_t>> parts(nt);
  std::vector<std::thread> pool;
  const uint64_t span = hi - lo;
  for (unsigned t = 0; t < nt; ++t) {
    pool.emplace_back([&, t]() {
      const uint32_t a = lo + static_cast<uint32_t>(span * t / nt);
      const uint32_t b = lo + static_cast<uint32_t>(span * (t + 1) / nt);
      for (uint32_t u = a; u < b; ++u) {
        float x;
        std::memcpy(&x, &u, 4);
        const float ref = logf(x);
        const float mine = cuflye::logf_wide(x);
        if (std::memcmp(&ref, &mine, 4) != 0) {
          uint32_t r;
          std::memcpy(&r, &ref, 4);
          parts[t].push_back(u);
          parts[t].push_back(r);
        }
      }
    });
  }
  for (auto& th : pool) th.join();
  uint32_t n = 0;
  for (auto& p : parts) n += static_cast<uint32_t>(p.size() / 2);
  FILE* f = std::fopen(argv[1], "wb");
  if (!f) return 1;
  std::fwrite(&n, 4, 1, f);
  for (auto& p : parts) std::fwrite(p.data(), 4, p.size(), f);
  std::fclose(f);
  std::printf("logf exceptions: %u\n", n);
  return 0;
}
