// Randomised check of ooc::Extents, the free-block bookkeeping of the server's
// pinned result reserve (built and run by test_extents.py): blocks never overlap,
// stay inside the region and are grain-sized; free plus taken bytes always add up
// to the region; and once every block is back the region is one free extent.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

#include "ooc_extents.h"

static int fail(const char* what, unsigned seed) {
  std::printf("FAIL seed %u: %s\n", seed, what);
  return 1;
}

int main() {
  for (unsigned seed = 1; seed <= 64; seed++) {
    std::mt19937_64 rng(seed);
    const size_t grain = size_t(1) << (10 + seed % 8);
    const size_t total = grain * (64 + rng() % 4096);
    ooc::Extents e;
    e.reset(total, grain);
    std::vector<std::pair<size_t, size_t>> held;  // (offset, cap)
    std::vector<char> used(total / grain, 0);
    size_t taken = 0;
    for (int step = 0; step < 20000; step++) {
      const bool give = !held.empty() && (rng() % 100 < 45 || step > 15000);
      if (give) {
        const size_t i = rng() % held.size();
        const auto b = held[i];
        held[i] = held.back();
        held.pop_back();
        for (size_t g = b.first / grain; g < (b.first + b.second) / grain; g++) used[g] = 0;
        e.put(b.first, b.second);
        taken -= b.second;
      } else {
        // sizes from a byte to a tenth of the region, skewed small like octree results
        const size_t n = 1 + (size_t)(std::pow((double)(rng() % 1000000) / 1e6, 4.0) * (double)(total / 10));
        size_t off = 0, cap = 0;
        if (e.take(n, off, cap)) {
          if (cap < n || cap % grain || off % grain) return fail("block size or alignment", seed);
          if (off + cap > total) return fail("block outside the region", seed);
          for (size_t g = off / grain; g < (off + cap) / grain; g++) {
            if (used[g]) return fail("blocks overlap", seed);
            used[g] = 1;
          }
          held.push_back({off, cap});
          taken += cap;
        } else if (e.free_bytes() >= total && n <= total) {
          return fail("refused with the whole region free", seed);
        }
      }
      if (e.free_bytes() + taken != total) return fail("free plus taken is not the region", seed);
    }
    for (const auto& b : held) e.put(b.first, b.second);
    if (e.extents() != 1 || e.free_bytes() != total) return fail("region not whole after every put", seed);
  }
  std::printf("ok\n");
  return 0;
}
