/*
 * CPU oracle: plain-C restatement of ooc_svo_builder's partition -> voxelize ->
 * SVO-build path (svo_builder / svo_builder_binary, v1.6.4).
 *
 * TEST INFRASTRUCTURE ONLY (see ooc_oracle.h).  Compile with
 * -ffp-contract=off: the reference is built for x86-64 without -march, so it
 * never fuses a multiply and an add, and every FP32 expression below is
 * evaluated in the same order as the reference's source (and the glm
 * stand-in, oracle/glm_shim/glm/glm.hpp).
 *
 * References are file:line within the reference project.
 */
#include "ooc_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* Small FP32 vector helpers, in the evaluation order of the glm stand-in.   */
/* ------------------------------------------------------------------------ */
typedef struct { float x, y, z; } v3;

static inline v3 mk(float x, float y, float z) { v3 r; r.x = x; r.y = y; r.z = z; return r; }
static inline v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline float dot3(v3 a, v3 b) {
  float px = a.x * b.x, py = a.y * b.y, pz = a.z * b.z;
  return (px + py) + pz;
}
static inline float dot2(float ax, float ay, float bx, float by) {
  float px = ax * bx, py = ay * by;
  return px + py;
}
static inline v3 cross3(v3 a, v3 b) {
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline v3 normalize3(v3 v) {
  float r = 1.0f / sqrtf(dot3(v, v));
  return mk(v.x * r, v.y * r, v.z * r);
}
/* std::min / std::max argument semantics (intersection.h:9-18, voxelizer.cpp:228) */
static inline float smin(float a, float b) { return (b < a) ? b : a; }
static inline float smax(float a, float b) { return (a < b) ? b : a; }
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

/* ------------------------------------------------------------------------ */
/* Morton codes (libmorton morton3D_64_encode/decode, morton.h:59-61,102-104): */
/* bit 3i = x_i, bit 3i+1 = y_i, bit 3i+2 = z_i.                             */
/* ------------------------------------------------------------------------ */
static inline uint64_t spread3(uint64_t v) {
  v &= 0x1fffffull;
  v = (v | (v << 32)) & 0x1f00000000ffffull;
  v = (v | (v << 16)) & 0x1f0000ff0000ffull;
  v = (v | (v << 8)) & 0x100f00f00f00f00full;
  v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}
static inline uint32_t compact3(uint64_t v) {
  v &= 0x1249249249249249ull;
  v = (v ^ (v >> 2)) & 0x10c30c30c30c30c3ull;
  v = (v ^ (v >> 4)) & 0x100f00f00f00f00full;
  v = (v ^ (v >> 8)) & 0x1f0000ff0000ffull;
  v = (v ^ (v >> 16)) & 0x1f00000000ffffull;
  v = (v ^ (v >> 32)) & 0x1fffffull;
  return (uint32_t)v;
}
uint64_t oracle_morton_encode(uint32_t x, uint32_t y, uint32_t z) {
  return spread3(x) | (spread3(y) << 1) | (spread3(z) << 2);
}
void oracle_morton_decode(uint64_t m, uint32_t* x, uint32_t* y, uint32_t* z) {
  *x = compact3(m);
  *y = compact3(m >> 1);
  *z = compact3(m >> 2);
}

/* ------------------------------------------------------------------------ */
/* Growable byte arrays for the node and data files.                        */
/* ------------------------------------------------------------------------ */
typedef struct { unsigned char* p; uint64_t n, cap; size_t rec; } recbuf;

static int rb_push(recbuf* b, const void* rec) {
  if (b->n == b->cap) {
    uint64_t nc = b->cap ? b->cap * 2 : 1024;
    unsigned char* np = (unsigned char*)realloc(b->p, (size_t)(nc * b->rec));
    if (!np) return -1;
    b->p = np;
    b->cap = nc;
  }
  memcpy(b->p + b->n * b->rec, rec, b->rec);
  b->n++;
  return 0;
}

/* VoxelData memory order: morton, color, normal (VoxelData.h:9-13). */
typedef struct { uint64_t morton; float color[3]; float normal[3]; } vdata;
/* Node record: data, children_base, children_offset[8] (Node.h:16-18). */
typedef struct { uint64_t data; uint64_t children_base; int8_t off[8]; } noderec;

/* ------------------------------------------------------------------------ */
/* Streaming octree builder (OctreeBuilder.h:16-90, OctreeBuilder.cpp).      */
/* ------------------------------------------------------------------------ */
typedef struct {
  noderec rec;
  float color[3], normal[3]; /* data_cache (Node.h:20) */
} onode;

typedef struct {
  int D;
  int levels;
  int binary;
  onode buf[22][8];
  int cnt[22];
  uint64_t cursor; /* b_current_morton */
  uint64_t total;  /* gridsize^3 */
  recbuf nodes, data;
  int err;
} obuilder;

static int onode_is_null(const onode* n) {
  /* isNull = isLeaf && !hasData (Node.h:45-47) */
  for (int k = 0; k < 8; k++)
    if (n->rec.off[k] != -1) return 0;
  return n->rec.data == 0;
}

static onode onode_empty(void) {
  onode n;
  memset(&n, 0, sizeof(n));
  memset(n.rec.off, 0xff, 8);
  return n;
}

static uint64_t ob_write_node(obuilder* b, const noderec* r) {
  if (rb_push(&b->nodes, r)) b->err = 1;
  return b->nodes.n - 1;
}
static uint64_t ob_write_data(obuilder* b, const vdata* d) {
  if (rb_push(&b->data, d)) b->err = 1;
  return b->data.n - 1;
}

/* groupNodes (OctreeBuilder.cpp:58-102) */
static onode ob_group(obuilder* b, const onode* g) {
  onode parent = onode_empty();
  int first = 1;
  for (int k = 0; k < 8; k++) {
    if (!onode_is_null(&g[k])) {
      uint64_t pos = ob_write_node(b, &g[k].rec);
      if (first) {
        parent.rec.children_base = pos;
        parent.rec.off[k] = 0;
        first = 0;
      } else {
        parent.rec.off[k] = (int8_t)(pos - parent.rec.children_base);
      }
    } else {
      parent.rec.off[k] = -1;
    }
  }
  if (b->levels) {
    /* SIMPLE LEVEL CONSTRUCTION (OctreeBuilder.cpp:81-99) */
    vdata d;
    memset(&d, 0, sizeof(d));
    float notnull = 0.0f;
    for (int i = 0; i < 8; i++) {
      if (!onode_is_null(&g[i])) notnull = notnull + 1.0f;
      for (int c = 0; c < 3; c++) d.color[c] = d.color[c] + g[i].color[c];
      for (int c = 0; c < 3; c++) d.normal[c] = d.normal[c] + g[i].normal[c];
    }
    for (int c = 0; c < 3; c++) d.color[c] = d.color[c] / notnull;
    v3 t = mk(d.normal[0] / notnull, d.normal[1] / notnull, d.normal[2] / notnull);
    v3 nn = normalize3(t);
    d.normal[0] = nn.x; d.normal[1] = nn.y; d.normal[2] = nn.z;
    parent.rec.data = ob_write_data(b, &d);
    memcpy(parent.color, d.color, sizeof(d.color));
    memcpy(parent.normal, d.normal, sizeof(d.normal));
  }
  return parent;
}

/* push + refineBuffers (OctreeBuilder.cpp:104-128) */
static void ob_push(obuilder* b, int level, const onode* n) {
  b->buf[level][b->cnt[level]++] = *n;
  while (level > 0 && b->cnt[level] == 8) {
    onode parent;
    int all_null = 1;
    for (int k = 0; k < 8; k++)
      if (!onode_is_null(&b->buf[level][k])) { all_null = 0; break; }
    parent = all_null ? onode_empty() : ob_group(b, b->buf[level]);
    b->cnt[level] = 0;
    level--;
    b->buf[level][b->cnt[level]++] = parent;
  }
}

/* fastAddEmpty / computeBestFillBuffer (OctreeBuilder.h:73-90): an empty node
 * is added at the coarsest level that is both aligned at the cursor and no
 * larger than the remaining gap. */
static void ob_pad(obuilder* b, uint64_t count) {
  while (count > 0) {
    int tz = 0;
    if (b->cursor == 0) {
      tz = b->D;
    } else {
      uint64_t c = b->cursor;
      while ((c & 7) == 0 && tz < b->D) { c >>= 3; tz++; }
    }
    int lp = 0;
    { uint64_t c = count; int hb = 0; while (c >>= 1) hb++; lp = hb / 3; } /* findPowerOf8 */
    int s = tz < lp ? tz : lp;
    onode e = onode_empty();
    ob_push(b, b->D - s, &e);
    uint64_t step = 1ull << (3 * s);
    b->cursor += step;
    count -= step;
  }
}

static void ob_init(obuilder* b, uint64_t gridsize, int levels, int binary) {
  memset(b, 0, sizeof(*b));
  int D = 0;
  while ((1ull << D) < gridsize) D++;
  b->D = D;
  b->levels = levels;
  b->binary = binary;
  b->total = gridsize * gridsize * gridsize;
  b->nodes.rec = sizeof(noderec);
  b->data.rec = sizeof(vdata);
  vdata z;
  memset(&z, 0, sizeof(z));
  ob_write_data(b, &z); /* first data point is NULL (OctreeBuilder.cpp:22) */
  if (binary) {
    /* white voxel that every binary leaf refers to (OctreeBuilder.cpp:25-27) */
    vdata w;
    memset(&w, 0, sizeof(w));
    w.color[0] = w.color[1] = w.color[2] = 1.0f;
    ob_write_data(b, &w);
  }
}

/* addVoxel (OctreeBuilder.cpp:130-167) */
static void ob_add(obuilder* b, const vdata* v) {
  if (v->morton != b->cursor) ob_pad(b, v->morton - b->cursor);
  onode n = onode_empty();
  if (b->binary) {
    n.rec.data = 1;
  } else {
    n.rec.data = ob_write_data(b, v);
    memcpy(n.color, v->color, sizeof(n.color));
    memcpy(n.normal, v->normal, sizeof(n.normal));
  }
  ob_push(b, b->D, &n);
  b->cursor++;
}

/* finalizeTree (OctreeBuilder.cpp:34-55).  The reference pads only while
 * b_current_morton < gridsize^3 - 1, which leaves the tree unfinished when the
 * last set voxel is gridsize^3 - 2; the restatement pads to the end. */
static void ob_finalize(obuilder* b) {
  if (b->cursor < b->total) ob_pad(b, b->total - b->cursor);
  ob_write_node(b, &b->buf[0][0].rec);
}

/* ------------------------------------------------------------------------ */
/* Partitioning (partitioner.cpp:12-149).                                   */
/* ------------------------------------------------------------------------ */
uint64_t oracle_estimate_partitions(uint64_t gridsize, uint64_t memory_limit_mb) {
  uint64_t required = (gridsize * gridsize * gridsize) / 1024 / 1024;
  if (required <= memory_limit_mb) return 1;
  uint64_t n = 1, req = required;
  while (req > memory_limit_mb) {
    req /= 8;
    n *= 8;
  }
  return n;
}

typedef struct { uint64_t* idx; uint64_t n, cap; } idxlist;

static int il_push(idxlist* l, uint64_t v) {
  if (l->n == l->cap) {
    uint64_t nc = l->cap ? l->cap * 2 : 256;
    uint64_t* np = (uint64_t*)realloc(l->idx, (size_t)nc * sizeof(uint64_t));
    if (!np) return -1;
    l->idx = np;
    l->cap = nc;
  }
  l->idx[l->n++] = v;
  return 0;
}

static inline v3 tri_v(const float* t, int k) { return mk(t[3 * k], t[3 * k + 1], t[3 * k + 2]); }

/* computeBoundingBox (intersection.h:9-18) */
static inline void tri_bbox(const float* t, v3* lo, v3* hi) {
  v3 a = tri_v(t, 0), b = tri_v(t, 1), c = tri_v(t, 2);
  *lo = mk(smin(a.x, smin(b.x, c.x)), smin(a.y, smin(b.y, c.y)), smin(a.z, smin(b.z, c.z)));
  *hi = mk(smax(a.x, smax(b.x, c.x)), smax(a.y, smax(b.y, c.y)), smax(a.z, smax(b.z, c.z)));
}

/* ------------------------------------------------------------------------ */
/* Radix sort of (key, payload index) pairs by key.                          */
/* ------------------------------------------------------------------------ */
static int sort_by_key(uint64_t* keys, uint64_t* vals, uint64_t n, int key_bits) {
  if (n < 2) return 0;
  uint64_t* k2 = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
  uint64_t* v2 = (uint64_t*)malloc((size_t)n * sizeof(uint64_t));
  if (!k2 || !v2) { free(k2); free(v2); return -1; }
  for (int shift = 0; shift < key_bits; shift += 11) {
    uint64_t cnt[2049];
    memset(cnt, 0, sizeof(cnt));
    for (uint64_t i = 0; i < n; i++) cnt[((keys[i] >> shift) & 2047) + 1]++;
    for (int i = 0; i < 2048; i++) cnt[i + 1] += cnt[i];
    for (uint64_t i = 0; i < n; i++) {
      uint64_t d = cnt[(keys[i] >> shift) & 2047]++;
      k2[d] = keys[i];
      v2[d] = vals[i];
    }
    memcpy(keys, k2, (size_t)n * sizeof(uint64_t));
    memcpy(vals, v2, (size_t)n * sizeof(uint64_t));
  }
  free(k2);
  free(v2);
  return 0;
}

/* ------------------------------------------------------------------------ */
/* Whole path (main.cpp:294-392).                                            */
/* ------------------------------------------------------------------------ */
int oracle_build(const oracle_params* prm, const float* tris, uint64_t n_tris, oracle_result* out) {
  memset(out, 0, sizeof(*out));
  const uint64_t N = prm->gridsize;
  if (N == 0 || (N & (N - 1)) != 0 || N > (1ull << 20)) return -2;
  const int binary = prm->geometry_only ? 1 : 0;
  const int stride = binary ? 9 : 21;

  const uint64_t P = oracle_estimate_partitions(N, prm->memory_limit_mb);
  /* unitlength (main.cpp:311, partitioner.cpp:45) */
  const float unitlength = (prm->bbox_max[0] - prm->bbox_min[0]) / (float)N;
  const uint64_t M = (N * N * N) / P; /* morton_part (main.cpp:312) */

  /* ---- partition (partitioner.cpp:80-149) ---- */
  idxlist* parts = (idxlist*)calloc((size_t)P, sizeof(idxlist));
  if (!parts) return -1;
  if (P == 1) {
    /* partition_one copies every triangle (partitioner.cpp:80-98) */
    parts[0].idx = (uint64_t*)malloc((size_t)(n_tris ? n_tris : 1) * sizeof(uint64_t));
    if (!parts[0].idx) { free(parts); return -1; }
    for (uint64_t t = 0; t < n_tris; t++) parts[0].idx[t] = t;
    parts[0].n = parts[0].cap = n_tris;
  } else {
    /* createBuffers world boxes (partitioner.cpp:52-61) */
    float* wb = (float*)malloc((size_t)P * 6 * sizeof(float));
    if (!wb) { free(parts); return -1; }
    for (uint64_t i = 0; i < P; i++) {
      uint32_t a[3], c[3];
      oracle_morton_decode(M * i, &a[0], &a[1], &a[2]);
      oracle_morton_decode(M * (i + 1) - 1, &c[0], &c[1], &c[2]);
      for (int k = 0; k < 3; k++) {
        wb[6 * i + k] = (float)a[k] * unitlength;
        wb[6 * i + 3 + k] = (float)(c[k] + 1u) * unitlength;
      }
    }
    /* partition: every triangle against every box (partitioner.cpp:117-126,
     * BBoxBuffer.h:70-84, intersectBoxBox intersection.h:49-53) */
    for (uint64_t t = 0; t < n_tris; t++) {
      v3 lo, hi;
      tri_bbox(tris + t * stride, &lo, &hi);
      for (uint64_t j = 0; j < P; j++) {
        const float* b = wb + 6 * j;
        if (hi.x < b[0] || hi.y < b[1] || hi.z < b[2] || lo.x > b[3] || lo.y > b[4] || lo.z > b[5])
          continue;
        if (il_push(&parts[j], t)) { free(wb); return -1; }
      }
    }
    free(wb);
  }
  out->n_partitions = P;
  out->part_tricounts = (uint64_t*)malloc((size_t)P * sizeof(uint64_t));
  if (out->part_tricounts)
    for (uint64_t i = 0; i < P; i++) out->part_tricounts[i] = parts[i].n;

  /* ---- voxelize + build per partition (main.cpp:329-387) ---- */
  obuilder* ob = (obuilder*)malloc(sizeof(obuilder));
  unsigned char* voxels = (unsigned char*)malloc((size_t)M);
  if (!ob || !voxels) { free(ob); free(voxels); return -1; }
  ob_init(ob, N, prm->generate_levels, binary);

  /* collected voxels of one partition: Morton key and payload */
  idxlist keys = {0, 0, 0}, order = {0, 0, 0};
  float* vcol = NULL;
  float* vnrm = NULL;
  uint64_t vcap = 0;
  uint64_t nfilled = 0;
  int rc = 0;

  const float unit_div = 1.0f / unitlength;     /* voxelizer.cpp:164 */
  const v3 delta_p = mk(unitlength, unitlength, unitlength);

  for (uint64_t i = 0; i < P && rc == 0; i++) {
    if (parts[i].n == 0) continue; /* main.cpp:330 */
    const uint64_t mstart = i * M;
    memset(voxels, 0, (size_t)M); /* voxelizer.cpp:144 */
    keys.n = 0;
    /* partition box in grid coordinates (voxelizer.cpp:148-150) */
    uint32_t pa[3], pb[3];
    oracle_morton_decode(mstart, &pa[0], &pa[1], &pa[2]);
    oracle_morton_decode(mstart + M - 1, &pb[0], &pb[1], &pb[2]);

    for (uint64_t q = 0; q < parts[i].n; q++) {
      const uint64_t tid = parts[i].idx[q];
      const float* t = tris + tid * stride;
      v3 v0 = tri_v(t, 0), v1 = tri_v(t, 1), v2 = tri_v(t, 2);
      v3 wlo, whi;
      tri_bbox(t, &wlo, &whi);
      /* grid box by truncation, clamped to the partition (voxelizer.cpp:189-204) */
      int gmin[3], gmax[3];
      gmin[0] = (int)(wlo.x * unit_div); gmin[1] = (int)(wlo.y * unit_div); gmin[2] = (int)(wlo.z * unit_div);
      gmax[0] = (int)(whi.x * unit_div); gmax[1] = (int)(whi.y * unit_div); gmax[2] = (int)(whi.z * unit_div);
      for (int k = 0; k < 3; k++) {
        gmin[k] = clampi(gmin[k], (int)pa[k], (int)pb[k]);
        gmax[k] = clampi(gmax[k], (int)pa[k], (int)pb[k]);
      }
      /* triangle set-up (voxelizer.cpp:207-254) */
      v3 e0 = sub(v1, v0), e1 = sub(v2, v1), e2 = sub(v0, v2);
      v3 n = normalize3(cross3(e0, e1));
      v3 c = mk(0.0f, 0.0f, 0.0f);
      if (n.x > 0) c.x = unitlength;
      if (n.y > 0) c.y = unitlength;
      if (n.z > 0) c.z = unitlength;
      float d1 = dot3(n, sub(c, v0));
      float d2 = dot3(n, sub(sub(delta_p, c), v0));
      /* XY projection */
      float xy[3][2] = {{-e0.y, e0.x}, {-e1.y, e1.x}, {-e2.y, e2.x}};
      if (n.z < 0.0f)
        for (int k = 0; k < 3; k++) { xy[k][0] = -xy[k][0]; xy[k][1] = -xy[k][1]; }
      const v3 vv[3] = {v0, v1, v2};
      float dxy[3], dyz[3], dzx[3];
      for (int k = 0; k < 3; k++)
        dxy[k] = ((-dot2(xy[k][0], xy[k][1], vv[k].x, vv[k].y)) + smax(0.0f, unitlength * xy[k][0])) +
                 smax(0.0f, unitlength * xy[k][1]);
      /* YZ projection */
      float yz[3][2] = {{-e0.z, e0.y}, {-e1.z, e1.y}, {-e2.z, e2.y}};
      if (n.x < 0.0f)
        for (int k = 0; k < 3; k++) { yz[k][0] = -yz[k][0]; yz[k][1] = -yz[k][1]; }
      for (int k = 0; k < 3; k++)
        dyz[k] = ((-dot2(yz[k][0], yz[k][1], vv[k].y, vv[k].z)) + smax(0.0f, unitlength * yz[k][0])) +
                 smax(0.0f, unitlength * yz[k][1]);
      /* ZX projection */
      float zx[3][2] = {{-e0.x, e0.z}, {-e1.x, e1.z}, {-e2.x, e2.z}};
      if (n.y < 0.0f)
        for (int k = 0; k < 3; k++) { zx[k][0] = -zx[k][0]; zx[k][1] = -zx[k][1]; }
      for (int k = 0; k < 3; k++)
        dzx[k] = ((-dot2(zx[k][0], zx[k][1], vv[k].z, vv[k].x)) + smax(0.0f, unitlength * zx[k][0])) +
                 smax(0.0f, unitlength * zx[k][1]);

      /* candidate loop x -> y -> z (voxelizer.cpp:257-305) */
      for (int x = gmin[0]; x <= gmax[0]; x++) {
        for (int y = gmin[1]; y <= gmax[1]; y++) {
          for (int z = gmin[2]; z <= gmax[2]; z++) {
            const uint64_t index = oracle_morton_encode((uint32_t)x, (uint32_t)y, (uint32_t)z);
            if (voxels[index - mstart] == 1) continue;
            const v3 p = mk((float)x * unitlength, (float)y * unitlength, (float)z * unitlength);
            const float nDOTp = dot3(n, p);
            if ((nDOTp + d1) * (nDOTp + d2) > 0.0f) continue;
            if ((dot2(xy[0][0], xy[0][1], p.x, p.y) + dxy[0]) < 0.0f) continue;
            if ((dot2(xy[1][0], xy[1][1], p.x, p.y) + dxy[1]) < 0.0f) continue;
            if ((dot2(xy[2][0], xy[2][1], p.x, p.y) + dxy[2]) < 0.0f) continue;
            if ((dot2(yz[0][0], yz[0][1], p.y, p.z) + dyz[0]) < 0.0f) continue;
            if ((dot2(yz[1][0], yz[1][1], p.y, p.z) + dyz[1]) < 0.0f) continue;
            if ((dot2(yz[2][0], yz[2][1], p.y, p.z) + dyz[2]) < 0.0f) continue;
            if ((dot2(zx[0][0], zx[0][1], p.z, p.x) + dzx[0]) < 0.0f) continue;
            if ((dot2(zx[1][0], zx[1][1], p.z, p.x) + dzx[1]) < 0.0f) continue;
            if ((dot2(zx[2][0], zx[2][1], p.z, p.x) + dzx[2]) < 0.0f) continue;
            voxels[index - mstart] = 1;
            if (il_push(&keys, index)) { rc = -1; break; }
            if (!binary) {
              /* payload sample (voxelizer.cpp:295-299, BarycentricCoords.h:4-33) */
              if (keys.n > vcap) {
                uint64_t nc = vcap ? vcap * 2 : 1024;
                float* a = (float*)realloc(vcol, (size_t)nc * 3 * sizeof(float));
                if (!a) { rc = -1; break; }
                vcol = a;
                float* b2 = (float*)realloc(vnrm, (size_t)nc * 3 * sizeof(float));
                if (!b2) { rc = -1; break; }
                vnrm = b2;
                vcap = nc;
              }
              const v3 q3 = mk((float)x / unit_div, (float)y / unit_div, (float)z / unit_div);
              const float coeffD = -dot3(v0, n);
              const float k = (dot3(q3, n) + coeffD) / ((n.x * n.x + n.y * n.y) + n.z * n.z);
              const v3 pt = mk(q3.x - k * n.x, q3.y - k * n.y, q3.z - k * n.z);
              /* inverse(mat3(v0, v1, v2)) * pt, adjugate over determinant */
              const float a = v0.x, b = v1.x, cc = v2.x;
              const float d = v0.y, e = v1.y, f = v2.y;
              const float g = v0.z, h = v1.z, ii = v2.z;
              const float C00 = e * ii - f * h, C01 = f * g - d * ii, C02 = d * h - e * g;
              const float det = (a * C00 + b * C01) + cc * C02;
              const float r = 1.0f / det;
              const float C10 = cc * h - b * ii, C11 = a * ii - cc * g, C12 = b * g - a * h;
              const float C20 = b * f - cc * e, C21 = cc * d - a * f, C22 = a * e - b * d;
              const float i00 = C00 * r, i10 = C01 * r, i20 = C02 * r; /* column 0 */
              const float i01 = C10 * r, i11 = C11 * r, i21 = C12 * r; /* column 1 */
              const float i02 = C20 * r, i12 = C21 * r, i22 = C22 * r; /* column 2 */
              const float bx = (i00 * pt.x + i01 * pt.y) + i02 * pt.z;
              const float by = (i10 * pt.x + i11 * pt.y) + i12 * pt.z;
              const float bz = (i20 * pt.x + i21 * pt.y) + i22 * pt.z;
              float* col = vcol + 3 * (keys.n - 1);
              for (int cch = 0; cch < 3; cch++) {
                const float c0 = t[12 + cch], c1 = t[15 + cch], c2 = t[18 + cch];
                col[cch] = (bx * c0 + by * c1) + bz * c2;
              }
              float* nr = vnrm + 3 * (keys.n - 1);
              nr[0] = t[9]; nr[1] = t[10]; nr[2] = t[11];
            }
            nfilled++;
          }
          if (rc) break;
        }
        if (rc) break;
      }
      if (rc) break;
    }
    if (rc) break;

    /* sort by Morton (main.cpp:356, 371); keys are unique within a partition */
    order.n = 0;
    for (uint64_t q = 0; q < keys.n; q++)
      if (il_push(&order, q)) { rc = -1; break; }
    if (rc) break;
    int kb = 0;
    while ((1ull << kb) < M) kb++;
    uint64_t* rel = (uint64_t*)malloc((size_t)(keys.n ? keys.n : 1) * sizeof(uint64_t));
    if (!rel) { rc = -1; break; }
    for (uint64_t q = 0; q < keys.n; q++) rel[q] = keys.idx[q] - mstart;
    if (sort_by_key(rel, order.idx, keys.n, kb)) { free(rel); rc = -1; break; }
    free(rel);

    for (uint64_t q = 0; q < keys.n; q++) {
      const uint64_t src = order.idx[q];
      vdata v;
      memset(&v, 0, sizeof(v));
      v.morton = keys.idx[src];
      if (!binary) {
        memcpy(v.color, vcol + 3 * src, sizeof(v.color));
        memcpy(v.normal, vnrm + 3 * src, sizeof(v.normal));
        /* colour modes (main.cpp:373-382) */
        if (prm->color_mode == ORACLE_COLOR_FIXED) {
          v.color[0] = v.color[1] = v.color[2] = 1.0f;
        } else if (prm->color_mode == ORACLE_COLOR_LINEAR) {
          /* mortonToRGB (svo_builder_util.h:14-18) */
          uint32_t a0, a1, a2;
          oracle_morton_decode(v.morton, &a0, &a1, &a2);
          v.color[0] = (float)a2 / (float)N;
          v.color[1] = (float)a1 / (float)N;
          v.color[2] = (float)a0 / (float)N;
        } else if (prm->color_mode == ORACLE_COLOR_NORMAL) {
          v3 nn = normalize3(mk(v.normal[0], v.normal[1], v.normal[2]));
          v.color[0] = (nn.x + 1.0f) / 2.0f;
          v.color[1] = (nn.y + 1.0f) / 2.0f;
          v.color[2] = (nn.z + 1.0f) / 2.0f;
        }
      }
      ob_add(ob, &v);
    }
    if (ob->err) rc = -1;
  }

  if (rc == 0) {
    ob_finalize(ob);
    if (ob->err) rc = -1;
  }
  if (rc == 0) {
    out->nodes = ob->nodes.p;
    out->n_nodes = ob->nodes.n;
    out->data = ob->data.p;
    out->n_data = ob->data.n;
    out->n_filled = nfilled;
  } else {
    free(ob->nodes.p);
    free(ob->data.p);
  }
  for (uint64_t i = 0; i < P; i++) free(parts[i].idx);
  free(parts);
  free(keys.idx);
  free(order.idx);
  free(vcol);
  free(vnrm);
  free(voxels);
  free(ob);
  return rc;
}

void oracle_free(oracle_result* r) {
  if (!r) return;
  free(r->nodes);
  free(r->data);
  free(r->part_tricounts);
  memset(r, 0, sizeof(*r));
}
