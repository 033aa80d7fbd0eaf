// An upper bound on the voxels one triangle can set, used by the serving loop's
// admission footprint.  Header-only so that a host-side test can check it against
// the oracle's voxel counts.
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>

namespace ooc {

// Voxels of an N^3 grid that triangle v (9 floats; grid coordinates are v * unit_div)
// can set: the voxels of its clamped grid box (no other is tested), and, for a triangle
// with a plane, the voxels that overlap it.  Those lie within the triangle grown by a
// ball of radius sqrt(3) voxels (a voxel passing the overlap test has its centre within
// sqrt(3)/2 of the triangle, and all of it within sqrt(3)), whose volume is
// 2 r A + (pi / 2) r^2 L + (4 / 3) pi r^3 for area A and perimeter L (Steiner's formula
// for a flat convex body).  The smaller of the two.
inline double voxel_bound(const float* v, float unit_div, uint64_t N) {
  double box = 1.0;
  for (int a = 0; a < 3; a++) {
    const float lo = std::min(v[a], std::min(v[3 + a], v[6 + a])) * unit_div;
    const float hi = std::max(v[a], std::max(v[3 + a], v[6 + a])) * unit_div;
    // NaN or out-of-range coordinates count as the whole axis
    const double l = (lo >= 0.0f) ? std::min((double)lo, (double)N - 1) : 0.0;
    const double h = (hi < (float)N) ? std::max((double)hi, 0.0) : (double)N - 1;
    box *= (h >= l) ? std::floor(h) - std::floor(l) + 1.0 : (double)N;
  }
  // both are upper bounds: a small box (every small triangle of a fine mesh) is taken as
  // it is, sparing the submitting thread the area bound's square roots
  if (box <= 64.0) return box;
  // in voxel units
  double p[3][3];
  for (int k = 0; k < 3; k++)
    for (int a = 0; a < 3; a++) p[k][a] = (double)v[3 * k + a] * (double)unit_div;
  double e[3][3], len = 0.0;
  for (int k = 0; k < 3; k++) {
    double l2 = 0.0;
    for (int a = 0; a < 3; a++) {
      e[k][a] = p[(k + 1) % 3][a] - p[k][a];
      l2 += e[k][a] * e[k][a];
    }
    len += std::sqrt(l2);
  }
  const double cx = e[0][1] * e[1][2] - e[0][2] * e[1][1], cy = e[0][2] * e[1][0] - e[0][0] * e[1][2],
               cz = e[0][0] * e[1][1] - e[0][1] * e[1][0];
  const double area = 0.5 * std::sqrt(cx * cx + cy * cy + cz * cz);
  // a degenerate triangle has no plane test (its normal is NaN): only its box bounds it
  if (!(area > 1e-6) || !std::isfinite(area) || !std::isfinite(len)) return box;
  const double r = std::sqrt(3.0), pi = 3.14159265358979323846;
  const double grown = 2.0 * r * area + 0.5 * pi * r * r * len + 4.0 / 3.0 * pi * r * r * r;
  return std::min(box, 1.01 * grown + 1.0);
}

}  // namespace ooc
