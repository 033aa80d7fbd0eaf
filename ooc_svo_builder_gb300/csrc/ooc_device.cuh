// Device helpers shared by the voxelization and octree kernels.
//
// Every FP32 expression here is evaluated in the reference's order
// (voxelizer.cpp:189-299, BarycentricCoords.h:4-33, OctreeBuilder.cpp:81-99)
// with one rounding per operation: the translation units that include this
// file are compiled with -fmad=false, and IEEE division and square root
// (nvcc's defaults -prec-div=true -prec-sqrt=true, no fast-math).
#pragma once

#include <stdint.h>

namespace ooc {

// ---------------------------------------------------------------------------
// Morton codes: x -> bit 3i, y -> bit 3i+1, z -> bit 3i+2
// (libmorton morton3D_64_encode, morton.h:59-61).
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint32_t spread3_10(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
__host__ __device__ __forceinline__ uint32_t compact3_10(uint32_t v) {
  v &= 0x09249249u;
  v = (v ^ (v >> 2)) & 0x030c30c3u;
  v = (v ^ (v >> 4)) & 0x0300f00fu;
  v = (v ^ (v >> 8)) & 0x030000ffu;
  v = (v ^ (v >> 16)) & 0x3ffu;
  return v;
}
// Local Morton code inside a stripe (coordinates < 1024, code < 2^30).
__host__ __device__ __forceinline__ uint32_t morton_local(uint32_t x, uint32_t y, uint32_t z) {
  return spread3_10(x) | (spread3_10(y) << 1) | (spread3_10(z) << 2);
}
__host__ __device__ __forceinline__ void morton_local_decode(uint32_t m, uint32_t& x, uint32_t& y, uint32_t& z) {
  x = compact3_10(m);
  y = compact3_10(m >> 1);
  z = compact3_10(m >> 2);
}
__host__ __device__ __forceinline__ uint64_t spread3_21(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
__host__ __device__ __forceinline__ uint32_t compact3_21(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
  v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
  v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
  v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
  v = (v ^ (v >> 32)) & 0x1fffffull;
  return (uint32_t)v;
}
__host__ __device__ __forceinline__ uint64_t morton_global(uint32_t x, uint32_t y, uint32_t z) {
  return spread3_21(x) | (spread3_21(y) << 1) | (spread3_21(z) << 2);
}
__host__ __device__ __forceinline__ void morton_global_decode(uint64_t m, uint32_t& x, uint32_t& y, uint32_t& z) {
  x = compact3_21(m);
  y = compact3_21(m >> 1);
  z = compact3_21(m >> 2);
}

// std::min / std::max argument semantics (intersection.h:9-18; voxelizer.cpp:228).
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// glm-order dot products: (a.x*b.x + a.y*b.y) + a.z*b.z.
__device__ __forceinline__ float dot3(float ax, float ay, float az, float bx, float by, float bz) {
  const float px = __fmul_rn(ax, bx), py = __fmul_rn(ay, by), pz = __fmul_rn(az, bz);
  return __fadd_rn(__fadd_rn(px, py), pz);
}
__device__ __forceinline__ float dot2(float ax, float ay, float bx, float by) {
  return __fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by));
}

// Triangle vertices (the first nine floats of either record layout).
struct TriVerts {
  float v[3][3];
};

__device__ __forceinline__ TriVerts load_verts(const float* __restrict__ tris, uint64_t t, int stride) {
  TriVerts r;
  const float* p = tris + t * (uint64_t)stride;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    r.v[k][0] = __ldg(p + 3 * k);
    r.v[k][1] = __ldg(p + 3 * k + 1);
    r.v[k][2] = __ldg(p + 3 * k + 2);
  }
  return r;
}

// computeBoundingBox (intersection.h:9-18) followed by the grid-box truncation
// of voxelizer.cpp:189-196.
__device__ __forceinline__ void grid_box(const TriVerts& t, float unit_div, int gmin[3], int gmax[3]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float lo = smin(t.v[0][a], smin(t.v[1][a], t.v[2][a]));
    const float hi = smax(t.v[0][a], smax(t.v[1][a], t.v[2][a]));
    gmin[a] = __float2int_rz(__fmul_rn(lo, unit_div));
    gmax[a] = __float2int_rz(__fmul_rn(hi, unit_div));
  }
}

// Per-triangle constants of the Schwarz-Seidel test (voxelizer.cpp:207-254).
struct TriSetup {
  float n[3];
  float d1, d2;
  float xy[3][2], dxy[3];
  float yz[3][2], dyz[3];
  float zx[3][2], dzx[3];
};

__device__ __forceinline__ void normalize3(float& x, float& y, float& z) {
  const float r = __fdiv_rn(1.0f, __fsqrt_rn(dot3(x, y, z, x, y, z)));
  x = __fmul_rn(x, r);
  y = __fmul_rn(y, r);
  z = __fmul_rn(z, r);
}

__device__ __forceinline__ void tri_normal(const TriVerts& t, float n[3]) {
  const float e0x = __fsub_rn(t.v[1][0], t.v[0][0]), e0y = __fsub_rn(t.v[1][1], t.v[0][1]),
              e0z = __fsub_rn(t.v[1][2], t.v[0][2]);
  const float e1x = __fsub_rn(t.v[2][0], t.v[1][0]), e1y = __fsub_rn(t.v[2][1], t.v[1][1]),
              e1z = __fsub_rn(t.v[2][2], t.v[1][2]);
  // cross(e0, e1)
  n[0] = __fsub_rn(__fmul_rn(e0y, e1z), __fmul_rn(e0z, e1y));
  n[1] = __fsub_rn(__fmul_rn(e0z, e1x), __fmul_rn(e0x, e1z));
  n[2] = __fsub_rn(__fmul_rn(e0x, e1y), __fmul_rn(e0y, e1x));
  normalize3(n[0], n[1], n[2]);
}

__device__ __forceinline__ float edge_offset(float a, float b, float va, float vb, float u) {
  // (-1 * dot(ne, v.proj)) + max(0, u*ne[0]) + max(0, u*ne[1])
  return __fadd_rn(__fadd_rn(-dot2(a, b, va, vb), smax(0.0f, __fmul_rn(u, a))), smax(0.0f, __fmul_rn(u, b)));
}

__device__ __forceinline__ void tri_setup(const TriVerts& t, float u, TriSetup& s) {
  float e[3][3];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    e[0][a] = __fsub_rn(t.v[1][a], t.v[0][a]);
    e[1][a] = __fsub_rn(t.v[2][a], t.v[1][a]);
    e[2][a] = __fsub_rn(t.v[0][a], t.v[2][a]);
  }
  s.n[0] = __fsub_rn(__fmul_rn(e[0][1], e[1][2]), __fmul_rn(e[0][2], e[1][1]));
  s.n[1] = __fsub_rn(__fmul_rn(e[0][2], e[1][0]), __fmul_rn(e[0][0], e[1][2]));
  s.n[2] = __fsub_rn(__fmul_rn(e[0][0], e[1][1]), __fmul_rn(e[0][1], e[1][0]));
  normalize3(s.n[0], s.n[1], s.n[2]);
  // critical point and plane offsets
  const float cx = (s.n[0] > 0.0f) ? u : 0.0f;
  const float cy = (s.n[1] > 0.0f) ? u : 0.0f;
  const float cz = (s.n[2] > 0.0f) ? u : 0.0f;
  s.d1 = dot3(s.n[0], s.n[1], s.n[2], __fsub_rn(cx, t.v[0][0]), __fsub_rn(cy, t.v[0][1]), __fsub_rn(cz, t.v[0][2]));
  s.d2 = dot3(s.n[0], s.n[1], s.n[2], __fsub_rn(__fsub_rn(u, cx), t.v[0][0]), __fsub_rn(__fsub_rn(u, cy), t.v[0][1]),
              __fsub_rn(__fsub_rn(u, cz), t.v[0][2]));
  const float fz = (s.n[2] < 0.0f) ? -1.0f : 1.0f;
  const float fx = (s.n[0] < 0.0f) ? -1.0f : 1.0f;
  const float fy = (s.n[1] < 0.0f) ? -1.0f : 1.0f;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    // XY: (-e.y, e.x), YZ: (-e.z, e.y), ZX: (-e.x, e.z); sign-flipped by n.
    // Multiplying by +-1 is exact, like the reference's -1.0f * vec2.
    s.xy[k][0] = __fmul_rn(fz, -e[k][1]);
    s.xy[k][1] = __fmul_rn(fz, e[k][0]);
    s.yz[k][0] = __fmul_rn(fx, -e[k][2]);
    s.yz[k][1] = __fmul_rn(fx, e[k][1]);
    s.zx[k][0] = __fmul_rn(fy, -e[k][0]);
    s.zx[k][1] = __fmul_rn(fy, e[k][2]);
    s.dxy[k] = edge_offset(s.xy[k][0], s.xy[k][1], t.v[k][0], t.v[k][1], u);
    s.dyz[k] = edge_offset(s.yz[k][0], s.yz[k][1], t.v[k][1], t.v[k][2], u);
    s.dzx[k] = edge_offset(s.zx[k][0], s.zx[k][1], t.v[k][2], t.v[k][0], u);
  }
}

// XY projection tests for a column (x, y): they do not depend on z.
__device__ __forceinline__ bool pass_xy(const TriSetup& s, float px, float py) {
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (__fadd_rn(dot2(s.xy[k][0], s.xy[k][1], px, py), s.dxy[k]) < 0.0f) return false;
  return true;
}

// Plane test + YZ and ZX projection tests at one voxel (voxelizer.cpp:266-287);
// the XY tests are evaluated once per column by pass_xy.
__device__ __forceinline__ bool pass_z(const TriSetup& s, float nxy, float px, float py, float pz) {
  const float nDOTp = __fadd_rn(nxy, __fmul_rn(s.n[2], pz));
  if (__fmul_rn(__fadd_rn(nDOTp, s.d1), __fadd_rn(nDOTp, s.d2)) > 0.0f) return false;
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (__fadd_rn(dot2(s.yz[k][0], s.yz[k][1], py, pz), s.dyz[k]) < 0.0f) return false;
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (__fadd_rn(dot2(s.zx[k][0], s.zx[k][1], pz, px), s.dzx[k]) < 0.0f) return false;
  return true;
}

// n.x*p.x + n.y*p.y, the part of dot(n, p) that is constant along a z column.
__device__ __forceinline__ float plane_xy(const TriSetup& s, float px, float py) {
  return __fadd_rn(__fmul_rn(s.n[0], px), __fmul_rn(s.n[1], py));
}

// The projection tests that do not depend on x (YZ) and on y (ZX).
__device__ __forceinline__ bool pass_yz(const TriSetup& s, float py, float pz) {
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (__fadd_rn(dot2(s.yz[k][0], s.yz[k][1], py, pz), s.dyz[k]) < 0.0f) return false;
  return true;
}
__device__ __forceinline__ bool pass_zx(const TriSetup& s, float pz, float px) {
#pragma unroll
  for (int k = 0; k < 3; k++)
    if (__fadd_rn(dot2(s.zx[k][0], s.zx[k][1], pz, px), s.dzx[k]) < 0.0f) return false;
  return true;
}

// Where the plane test of voxel p stands along axis w, whose normal component is nw:
// 0 it passes, -1 the passing run lies at larger w, +1 at smaller w.  Every
// operand of the test is a rounded sum or product of one monotone input, so
// along any line the rounded plane value moves monotonically with the sign of
// nw, the two offsets keep their order, and the passing voxels form one run;
// outside it both factors have the sign that says which side it is on.
__device__ __forceinline__ int plane_side(const TriSetup& s, float px, float py, float pz, float nw) {
  const float nDOTp = __fadd_rn(plane_xy(s, px, py), __fmul_rn(s.n[2], pz));
  const float a = __fadd_rn(nDOTp, s.d1), b = __fadd_rn(nDOTp, s.d2);
  if (!(__fmul_rn(a, b) > 0.0f)) return 0;
  return ((a > 0.0f) == (nw > 0.0f)) ? 1 : -1;
}

// True when the monotone-run argument above holds for this triangle: every
// constant of the test finite and small enough that no sum or product of the
// test overflows or turns into NaN (voxel coordinates are below 2^60 too).
__device__ __forceinline__ bool monotone_setup(const TriSetup& s, float coord_max) {
  const float lim = 1.0e18f;
  bool ok = fabsf(s.d1) < lim && fabsf(s.d2) < lim && coord_max < lim;
#pragma unroll
  for (int a = 0; a < 3; a++) ok = ok && fabsf(s.n[a]) < lim;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    ok = ok && fabsf(s.xy[k][0]) < lim && fabsf(s.xy[k][1]) < lim && fabsf(s.dxy[k]) < lim;
    ok = ok && fabsf(s.yz[k][0]) < lim && fabsf(s.yz[k][1]) < lim && fabsf(s.dyz[k]) < lim;
    ok = ok && fabsf(s.zx[k][0]) < lim && fabsf(s.zx[k][1]) < lim && fabsf(s.dzx[k]) < lim;
  }
  return ok;  // NaN fails every comparison
}

}  // namespace ooc
