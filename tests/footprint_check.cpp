// Prints ooc::voxel_bound (the serving loop's per-triangle voxel bound) for triangles
// read from stdin: a line "N unit_div", then 9 floats per triangle (test_footprint.py).
#include <cstdint>
#include <cstdio>

#include "ooc_footprint.h"

int main() {
  unsigned long long N = 0;
  float unit_div = 0.0f;
  if (std::scanf("%llu %f", &N, &unit_div) != 2) return 2;
  float v[9];
  for (;;) {
    for (int k = 0; k < 9; k++)
      if (std::scanf("%a", &v[k]) != 1) return 0;
    std::printf("%.17g\n", ooc::voxel_bound(v, unit_div, N));
  }
}
