// Host orchestration and the C ABI of libooc_svo_gpu.so.
//
// The grid is processed in stripes: Morton-aligned cubes of at most 8^10
// voxels inside one reference partition (or a whole partition when that is
// smaller).  Each stripe is voxelized into an occupancy bitfield on the GPU
// and turned into its complete subtree there; the few nodes above the stripes
// are grouped on the host in the reference's streaming order.  Because the
// reference writes every subtree as one contiguous run of the node and data
// files, a stripe's records land at global indices known before it starts.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ooc_device.cuh"
#include "ooc_internal.h"
#include "ooc_svo_gpu.h"

namespace {

struct OocError {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw OocError{code, msg}; }

void ck(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    int code = (e == cudaErrorMemoryAllocation) ? OOC_ERR_OOM : OOC_ERR_DEVICE;
    fail(code, std::string(what) + ": " + cudaGetErrorString(e));
  }
}

struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
};
struct PinBuf {
  void* p = nullptr;
  size_t cap = 0;
};

// Scratch buffer: contents are not preserved when it grows.
template <typename T>
T* ensure(DevBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes > b.cap) {
    const size_t want = std::max(bytes, b.cap + b.cap / 4);
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    ck(cudaMalloc(&b.p, want), "cudaMalloc");
    b.cap = want;
  }
  return static_cast<T*>(b.p);
}

// Growable buffer whose first `keep` bytes (at most its current capacity) survive growth.
template <typename T>
T* ensure_keep(DevBuf& b, size_t bytes, size_t keep, cudaStream_t st) {
  if (bytes == 0) bytes = 16;
  keep = std::min(keep, b.cap);
  if (bytes > b.cap) {
    size_t want = std::max(bytes, b.cap + b.cap / 2);
    void* np = nullptr;
    ck(cudaMalloc(&np, want), "cudaMalloc");
    if (b.p) {
      if (keep) ck(cudaMemcpyAsync(np, b.p, keep, cudaMemcpyDeviceToDevice, st), "cudaMemcpyAsync");
      ck(cudaStreamSynchronize(st), "cudaStreamSynchronize");
      cudaFree(b.p);
    }
    b.p = np;
    b.cap = want;
  }
  return static_cast<T*>(b.p);
}

template <typename T>
T* ensure_pinned(PinBuf& b, size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes > b.cap) {
    const size_t want = std::max(bytes, b.cap + b.cap / 4);
    if (b.p) cudaFreeHost(b.p);
    b.p = nullptr;
    b.cap = 0;
    ck(cudaMallocHost(&b.p, want), "cudaMallocHost");
    b.cap = want;
  }
  return static_cast<T*>(b.p);
}

constexpr int kPhases = 6;
enum Phase { PH_BIN = 0, PH_VOX = 1, PH_PYR = 2, PH_TREE = 3, PH_COPY = 4, PH_ALL = 5 };

}  // namespace

struct ooc_ctx {
  int device = 0;
  int num_sms = 152;
  cudaStream_t own_stream = nullptr;
  std::string err;
  bool timing = false;
  float phase_ms[kPhases] = {0, 0, 0, 0, 0, 0};
  unsigned long long launches = 0;
  DevBuf d_tris, d_items, d_hist, d_axis, d_bits, d_scan, d_scanpart, d_keys, d_size, d_dsize, d_start, d_dstart,
      d_cache, d_winners, d_taskoff, d_taskpart, d_counter, d_nodes, d_data, d_recs, d_rootinfo, d_itemmask,
      d_firstchild, d_itembox;
  PinBuf h_nodes, h_data, h_misc, h_recs;
  uint64_t res_nodes = 0, res_data = 0;
  bool res_valid = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<std::array<size_t, 3>> marks;  // phase, start event, end event
  // per-kernel timing: "" off, "*" every kernel, otherwise one kernel name
  std::string kfilter;
  std::vector<std::pair<const char*, std::array<size_t, 2>>> kmarks;
  size_t kopen = 0;
  std::vector<std::string> knames;
  std::vector<float> kms;
  std::vector<uint64_t> kcount;
};

namespace {

using namespace ooc;

cudaEvent_t next_event(ooc_ctx* c) {
  if (c->ev_used == c->ev_pool.size()) {
    cudaEvent_t e;
    ck(cudaEventCreate(&e), "cudaEventCreate");
    c->ev_pool.push_back(e);
  }
  return c->ev_pool[c->ev_used++];
}

struct PhaseScope {
  ooc_ctx* c;
  int phase;
  cudaStream_t st;
  size_t start_idx = 0;
  PhaseScope(ooc_ctx* c_, int ph, cudaStream_t s) : c(c_), phase(ph), st(s) {
    if (c->timing) {
      start_idx = c->ev_used;
      ck(cudaEventRecord(next_event(c), st), "cudaEventRecord");
    }
  }
  ~PhaseScope() {
    if (c->timing) {
      size_t end_idx = c->ev_used;
      if (cudaEventRecord(next_event(c), st) == cudaSuccess)
        c->marks.push_back({(size_t)phase, start_idx, end_idx});
    }
  }
};

// ---------------------------------------------------------------------------
// Node records and the host-side grouping above the stripes.
// ---------------------------------------------------------------------------
struct TNode {
  uint64_t data = 0;
  uint64_t cb = 0;
  uint64_t off = ~0ull;  // children_offset[8] packed little-endian, 0xff = no child
  float cache[6] = {0, 0, 0, 0, 0, 0};
  bool is_null() const { return off == ~0ull && data == 0; }  // Node::isNull (Node.h:45-47)
};

struct Emitter {
  bool device = false;
  // device mode: (index, words...) records scattered into the device files at the end
  std::vector<uint64_t> node_recs, data_recs;
  // host mode
  ooc_sink_fn sink = nullptr;
  void* user = nullptr;

  void node(uint64_t pos, const TNode& n) {
    if (device) {
      node_recs.insert(node_recs.end(), {pos, n.data, n.cb, n.off});
    } else {
      uint64_t rec[3] = {n.data, n.cb, n.off};
      if (sink(user, OOC_STREAM_NODES, rec, 24) != 0) fail(OOC_ERR_SINK, "node sink returned an error");
    }
  }
  void data(uint64_t pos, uint64_t morton, const float* v) {
    uint64_t w[4];
    w[0] = morton;
    std::memcpy(&w[1], v, 24);
    if (device) {
      data_recs.insert(data_recs.end(), {pos, w[0], w[1], w[2], w[3]});
    } else {
      if (sink(user, OOC_STREAM_DATA, w, 32) != 0) fail(OOC_ERR_SINK, "data sink returned an error");
    }
  }
};

// The reference's per-level 8-node buffers (OctreeBuilder.h:18, refineBuffers
// OctreeBuilder.cpp:112-128, groupNodes 58-102) for the levels above the stripes.
struct TopBuilder {
  int top;  // stripe-root level
  bool levels;
  std::vector<std::array<TNode, 8>> buf;
  std::vector<int> cnt;
  uint64_t node_pos = 0, data_pos = 0;
  Emitter* out = nullptr;

  TopBuilder(int top_level, bool lv, Emitter* o) : top(top_level), levels(lv), buf(top_level + 1), cnt(top_level + 1, 0), out(o) {}

  TNode group(const std::array<TNode, 8>& g) {
    bool all_null = true;
    for (const TNode& n : g) all_null = all_null && n.is_null();
    if (all_null) return TNode();
    TNode parent;
    parent.off = 0;
    bool first = true;
    for (int k = 0; k < 8; k++) {
      uint64_t byte = 0xff;
      if (!g[k].is_null()) {
        const uint64_t pos = node_pos++;
        out->node(pos, g[k]);
        if (first) {
          parent.cb = pos;
          byte = 0;
          first = false;
        } else {
          byte = pos - parent.cb;
        }
      }
      parent.off |= byte << (8 * k);
    }
    if (levels) {
      float acc[6] = {0, 0, 0, 0, 0, 0};
      float notnull = 0.0f;
      for (int k = 0; k < 8; k++) {
        if (!g[k].is_null()) notnull = notnull + 1.0f;
        for (int q = 0; q < 6; q++) acc[q] = acc[q] + g[k].cache[q];
      }
      float v[6];
      for (int q = 0; q < 3; q++) v[q] = acc[q] / notnull;
      float tx = acc[3] / notnull, ty = acc[4] / notnull, tz = acc[5] / notnull;
      const float px = tx * tx, py = ty * ty, pz = tz * tz;
      const float r = 1.0f / std::sqrt((px + py) + pz);
      v[3] = tx * r;
      v[4] = ty * r;
      v[5] = tz * r;
      const uint64_t di = data_pos++;
      out->data(di, 0, v);
      parent.data = di;
      std::memcpy(parent.cache, v, sizeof(v));
    }
    return parent;
  }

  void push(int level, const TNode& n) {
    buf[level][cnt[level]++] = n;
    while (level > 0 && cnt[level] == 8) {
      TNode parent = group(buf[level]);
      cnt[level] = 0;
      level--;
      buf[level][cnt[level]++] = parent;
    }
  }
};

uint64_t offsets_from_mask(uint32_t mask) {
  uint64_t off = 0;
  uint32_t r = 0;
  for (int k = 0; k < 8; k++) off |= (uint64_t)(((mask >> k) & 1u) ? r++ : 0xffu) << (8 * k);
  return off;
}

int ilog2(uint64_t v) {
  int r = 0;
  while ((1ull << r) < v) r++;
  return r;
}

void check_params(const ooc_build_params* p, uint64_t n_tris) {
  if (!p) fail(OOC_ERR_INVALID, "params is NULL");
  const uint64_t N = p->gridsize;
  if (N == 0 || (N & (N - 1)) != 0 || N > 65536) fail(OOC_ERR_INVALID, "gridsize must be a power of two in [1, 65536]");
  if (p->memory_limit_mb < 1) fail(OOC_ERR_INVALID, "memory limit must be >= 1");
  if (p->geometry_only != 0 && p->geometry_only != 1) fail(OOC_ERR_INVALID, "geometry_only must be 0 or 1");
  if (p->color_mode < 0 || p->color_mode > 3) fail(OOC_ERR_INVALID, "unknown colour mode");
  if (p->reserved != 0) fail(OOC_ERR_INVALID, "reserved field must be 0");
  if (n_tris >= (1ull << 32)) fail(OOC_ERR_INVALID, "at most 2^32-1 triangles per build");
}

// Everything one build needs to know about the grid decomposition.
struct Plan {
  uint64_t N, P, M;
  int D, kP, Dm, Ds, Ls;
  uint64_t S, stripes_per_part, n_stripes;
  int binary, levels;
  float u, unit_div;
};

Plan make_plan(const ooc_build_params* p) {
  Plan pl;
  pl.N = p->gridsize;
  pl.P = ooc_estimate_partitions(pl.N, p->memory_limit_mb);
  pl.D = ilog2(pl.N);
  pl.kP = ilog2(pl.P) / 3;
  if (pl.kP > 7) fail(OOC_ERR_INVALID, "memory limit gives more than 8^7 partitions");
  pl.M = (pl.N * pl.N * pl.N) / pl.P;
  pl.Dm = pl.D - pl.kP;
  pl.Ds = std::min(pl.Dm, kMaxStripeDepth);
  pl.S = 1ull << (3 * pl.Ds);
  pl.stripes_per_part = 1ull << (3 * (pl.Dm - pl.Ds));
  pl.n_stripes = pl.P * pl.stripes_per_part;
  pl.Ls = pl.D - pl.Ds;
  pl.binary = p->geometry_only;
  pl.levels = p->generate_levels ? 1 : 0;
  // unitlength (main.cpp:311) and unit_div (voxelizer.cpp:164)
  pl.u = (p->bbox_max[0] - p->bbox_min[0]) / (float)pl.N;
  pl.unit_div = 1.0f / pl.u;
  return pl;
}

struct StripeOut {
  bool empty = true;
  TNode root;
  uint64_t node_span = 0, data_span = 0, filled = 0;
};

StripeOut run_stripe(ooc_ctx* c, cudaStream_t st, const Plan& pl, const ooc_build_params* prm, const float* d_tris,
                     uint64_t n_tris_total, const uint32_t* items, uint64_t ibeg, uint64_t n_items, uint64_t part,
                     uint64_t stripe, uint64_t node_base, uint64_t data_base, bool device_mode) {
  StripeOut res;
  const int Ds = pl.Ds;
  const int stride = pl.binary ? 9 : 21;
  // Levels with at most this many 256-bit blocks (pyramid) or nodes (layout)
  // run together in one CTA instead of one launch each.
  constexpr uint64_t kSmallBlocks = 512, kSmallNodes = 256;
  // ---- pyramid layout ----
  Pyramid pyr;
  std::memset(&pyr, 0, sizeof(pyr));
  pyr.depth = Ds;
  uint64_t words = 0, blocks = 0;
  for (int l = 0; l <= Ds; l++) {
    const uint64_t nbits = 1ull << (3 * l);
    uint64_t nw = (nbits + 31) / 32;
    nw = (nw + 7) / 8 * 8;
    pyr.lv[l].off_w = words;
    pyr.lv[l].off_b = blocks;
    pyr.lv[l].nwords = nw;
    pyr.lv[l].nblocks = nw / 8;
    words += nw;
    blocks += nw / 8;
  }
  pyr.bits = ensure<uint32_t>(c->d_bits, words * 4);
  pyr.scan = ensure<uint32_t>(c->d_scan, (blocks + 1) * 4);
  uint32_t* scanpart = ensure<uint32_t>(c->d_scanpart, scan_partials_needed(blocks + 1) * 4);

  uint32_t pa[3], pb[3], sa[3];
  morton_global_decode(part * pl.M, pa[0], pa[1], pa[2]);
  morton_global_decode(stripe * pl.S, sa[0], sa[1], sa[2]);
  const uint32_t pside = 1u << pl.Dm, sside = 1u << Ds;

  VoxJob j;
  std::memset(&j, 0, sizeof(j));
  j.tris = d_tris;
  j.stride = stride;
  j.item_tri = items;
  j.ibeg = ibeg;
  j.n_items = n_items;
  for (int a = 0; a < 3; a++) {
    pb[a] = pa[a] + pside - 1;
    j.pa[a] = (int)pa[a];
    j.pb[a] = (int)pb[a];
    j.sa[a] = (int)sa[a];
    j.sb[a] = (int)(sa[a] + sside - 1);
  }
  j.u = pl.u;
  j.unit_div = pl.unit_div;
  j.small_vol = 64;
  j.leafbits = pyr.bits + pyr.lv[Ds].off_w;
  j.task_off = ensure<uint64_t>(c->d_taskoff, (n_items + 1) * 8);
  j.task_counter = ensure<unsigned long long>(c->d_counter, 16);
  j.item_mask = pl.binary ? nullptr : ensure<uint64_t>(c->d_itemmask, n_items * 8);
  j.item_box = pl.binary ? nullptr : ensure<uint64_t>(c->d_itembox, n_items * 8);
  uint64_t* taskpart = ensure<uint64_t>(c->d_taskpart, scan_partials_needed(n_items + 1) * 8);

  {
    PhaseScope ph(c, PH_VOX, st);
    ck(cudaMemsetAsync(pyr.bits, 0, words * 4, st), "memset bits");
    ck(cudaMemsetAsync(j.task_off + n_items, 0, 8, st), "memset task_off");
    launch_vox_small(j, 0, st);
    scan_u64_exclusive(j.task_off, n_items + 1, taskpart, st);
    launch_vox_large(j, 0, st, c->num_sms);
  }
  uint32_t* lvl = ensure_pinned<uint32_t>(c->h_misc, 64 * 4);
  uint32_t* d_root = ensure<uint32_t>(c->d_rootinfo, 64 * 4);
  {
    PhaseScope ph(c, PH_PYR, st);
    ck(cudaMemsetAsync(pyr.scan + blocks, 0, 4, st), "memset scan");
    int l = Ds;
    for (; l >= 0 && pyr.lv[l].nblocks > kSmallBlocks; l--) launch_pyramid(pyr, l, st);
    if (l >= 0) launch_pyramid_top(pyr, l, st);
    scan_u32_exclusive(pyr.scan, blocks + 1, scanpart, st);
    launch_level_bases(pyr, blocks, d_root + 16, st);
    ck(cudaMemcpyAsync(lvl, d_root + 16, (Ds + 2) * 4, cudaMemcpyDeviceToHost, st), "level bases");
  }
  ck(cudaStreamSynchronize(st), "stripe level counts");
  for (int l = 0; l <= Ds; l++) {
    pyr.lv[l].koff = lvl[l];
    pyr.lv[l].n = (uint64_t)lvl[l + 1] - lvl[l];
  }
  const uint64_t total = lvl[Ds + 1];
  const uint64_t n_leaf = pyr.lv[Ds].n;
  if (n_leaf == 0) return res;
  res.empty = false;
  res.filled = n_leaf;

  EmitJob e;
  std::memset(&e, 0, sizeof(e));
  e.binary = pl.binary;
  e.levels = pl.levels;
  e.color_mode = prm->color_mode;
  e.gridsize = pl.N;
  e.stripe_base = stripe * pl.S;
  for (int a = 0; a < 3; a++) e.origin[a] = (int)sa[a];
  e.tris = d_tris;
  e.stride = stride;
  e.unit_div = pl.unit_div;
  uint32_t* keys = ensure<uint32_t>(c->d_keys, total * 4);
  e.keys = keys;
  e.size = ensure<uint32_t>(c->d_size, total * 4);
  e.dsize = ensure<uint32_t>(c->d_dsize, total * 4);
  e.first_child = ensure<uint32_t>(c->d_firstchild, total * 4);
  e.start = ensure<uint64_t>(c->d_start, total * 8);
  e.dstart = ensure<uint64_t>(c->d_dstart, total * 8);
  e.cache = pl.levels ? ensure<float>(c->d_cache, total * 24) : nullptr;
  e.leaf_inline = (!pl.binary && !pl.levels) ? 1 : 0;

  const uint64_t node_span = total - 1;
  const uint64_t data_span = (pl.binary ? 0 : n_leaf) + (pl.levels ? total - n_leaf : 0);
  res.node_span = node_span;
  res.data_span = data_span;
  if (device_mode) {
    e.node_win = ensure_keep<uint64_t>(c->d_nodes, (node_base + node_span) * 24, node_base * 24, st);
    e.data_win = ensure_keep<unsigned char>(c->d_data, (data_base + data_span) * 32, data_base * 32, st);
    e.node_win_base = 0;
    e.data_win_base = 0;
    e.node_win_len = node_base + node_span;
    e.data_win_len = data_base + data_span;
  } else {
    e.node_win = ensure<uint64_t>(c->d_nodes, node_span * 24);
    e.data_win = ensure<unsigned char>(c->d_data, data_span * 32);
    e.node_win_base = node_base;
    e.data_win_base = data_base;
    e.node_win_len = node_span;
    e.data_win_len = data_span;
  }
  e.n_tris = n_tris_total;
  e.flag = d_root + 8;
  ck(cudaMemsetAsync(e.flag, 0, 4, st), "memset flag");

  {
    PhaseScope ph(c, PH_PYR, st);
    launch_compact(pyr, blocks, keys, st);
  }
  if (!pl.binary) {
    PhaseScope ph(c, PH_VOX, st);
    uint32_t* winners = ensure<uint32_t>(c->d_winners, n_leaf * 4);
    ck(cudaMemsetAsync(winners, 0xff, n_leaf * 4, st), "memset winners");
    j.winners = winners;
    j.leafscan = pyr.scan + pyr.lv[Ds].off_b;
    j.leafscan_base = (uint32_t)pyr.lv[Ds].koff;
    launch_vox_small(j, 1, st);
    launch_vox_large(j, 1, st, c->num_sms);
    e.winners = winners;
    if (pl.levels) launch_leaf_payload(pyr, e, st);
  }
  uint32_t* h_root = lvl + 32;
  {
    PhaseScope ph(c, PH_TREE, st);
    // levels 0 .. l_small hold at most kSmallNodes nodes each (counts grow with depth)
    int l_small = 0;
    while (l_small + 1 <= Ds - 1 && pyr.lv[l_small + 1].n <= kSmallNodes) l_small++;
    if (Ds >= 1) {
      for (int l = Ds - 1; l > l_small; l--) launch_bottom_up(pyr, e, l, st);
      launch_bottom_up_top(pyr, e, l_small, st);
      // parents of internal children: levels 0 .. Ds-2; the leaves get one thread each
      const int top_last = std::min(l_small, Ds - 2);
      launch_top_down_top(pyr, e, top_last, node_base, data_base, st);
      for (int l = top_last + 1; l <= Ds - 2; l++) launch_top_down(pyr, e, l, st);
      launch_top_down_leaves(pyr, e, st);
    }
    launch_root_info(pyr, e, data_base, d_root, st);
    ck(cudaMemcpyAsync(h_root, d_root, 9 * 4, cudaMemcpyDeviceToHost, st), "root info");
  }
  if (!device_mode) {
    PhaseScope ph(c, PH_COPY, st);
    void* hn = ensure_pinned<void>(c->h_nodes, node_span * 24);
    void* hd = ensure_pinned<void>(c->h_data, data_span * 32);
    if (node_span) ck(cudaMemcpyAsync(hn, e.node_win, node_span * 24, cudaMemcpyDeviceToHost, st), "D2H nodes");
    if (data_span) ck(cudaMemcpyAsync(hd, e.data_win, data_span * 32, cudaMemcpyDeviceToHost, st), "D2H data");
  }
  ck(cudaStreamSynchronize(st), "stripe");
  ck(cudaGetLastError(), "stripe kernels");
  if (h_root[8] != 0) fail(OOC_ERR_DEVICE, "internal layout check failed (flag " + std::to_string(h_root[8]) + ")");

  TNode& r = res.root;
  const uint32_t mask = h_root[0];
  float cache[6];
  std::memcpy(cache, h_root + 1, sizeof(cache));
  if (Ds >= 1) {
    r.data = pl.levels ? data_base + data_span - 1 : 0;
    r.cb = node_base + total - 1 - (uint64_t)__builtin_popcount(mask);
    r.off = offsets_from_mask(mask);
    if (pl.levels) std::memcpy(r.cache, cache, sizeof(cache));
  } else {
    r.data = pl.binary ? 1 : data_base;
    r.cb = 0;
    r.off = ~0ull;
    if (!pl.binary) std::memcpy(r.cache, cache, sizeof(cache));
  }
  return res;
}

void build_core(ooc_ctx* c, const ooc_build_params* prm, const float* d_tris, uint64_t n_tris, cudaStream_t st,
                Emitter& out, ooc_build_info* info) {
  const Plan pl = make_plan(prm);
  const int stride = pl.binary ? 9 : 21;

  // ---- partition binning (P > 1) ----
  std::vector<uint32_t> part_off;
  uint32_t* items = nullptr;
  uint64_t n_items = n_tris;
  if (pl.P > 1) {
    PhaseScope ph(c, PH_BIN, st);
    const int PA = 1 << pl.kP;
    const uint64_t side = pl.N / PA;
    std::vector<float> axis(6 * PA);
    for (int a = 0; a < 3; a++)
      for (int jj = 0; jj < PA; jj++) {
        // createBuffers world box (partitioner.cpp:56-61)
        axis[a * PA + jj] = (float)(uint32_t)(jj * side) * pl.u;
        axis[3 * PA + a * PA + jj] = (float)(uint32_t)((jj + 1) * side) * pl.u;
      }
    float* d_axis = ensure<float>(c->d_axis, axis.size() * 4);
    ck(cudaMemcpyAsync(d_axis, axis.data(), axis.size() * 4, cudaMemcpyHostToDevice, st), "axis boxes");
    uint32_t* hist = ensure<uint32_t>(c->d_hist, pl.P * 4);
    ck(cudaMemsetAsync(hist, 0, pl.P * 4, st), "memset hist");
    launch_part_count(d_tris, stride, n_tris, d_axis, d_axis + 3 * PA, pl.kP, pl.P, hist, st);
    std::vector<uint32_t> h(pl.P);
    ck(cudaMemcpyAsync(h.data(), hist, pl.P * 4, cudaMemcpyDeviceToHost, st), "hist");
    ck(cudaStreamSynchronize(st), "binning");
    part_off.assign(pl.P + 1, 0);
    uint64_t acc = 0;
    for (uint64_t i = 0; i < pl.P; i++) {
      part_off[i] = (uint32_t)acc;
      acc += h[i];
      if (acc >= (1ull << 32)) fail(OOC_ERR_INVALID, "more than 2^32 (triangle, partition) pairs");
    }
    part_off[pl.P] = (uint32_t)acc;
    n_items = acc;
    items = ensure<uint32_t>(c->d_items, n_items * 4);
    ck(cudaMemcpyAsync(hist, part_off.data(), pl.P * 4, cudaMemcpyHostToDevice, st), "cursors");
    launch_part_emit(d_tris, stride, n_tris, d_axis, d_axis + 3 * PA, pl.kP, pl.P, hist, items, st);
  }

  TopBuilder top(pl.Ls, pl.levels != 0, &out);
  // data file header records (OctreeBuilder.cpp:22-28)
  {
    float zero[6] = {0, 0, 0, 0, 0, 0};
    out.data(top.data_pos++, 0, zero);
    if (pl.binary) {
      float white[6] = {1, 1, 1, 0, 0, 0};
      out.data(top.data_pos++, 0, white);
    }
  }
  uint64_t filled = 0;
  for (uint64_t s = 0; s < pl.n_stripes; s++) {
    const uint64_t part = s / pl.stripes_per_part;
    const uint64_t ibeg = pl.P > 1 ? part_off[part] : 0;
    const uint64_t cnt = pl.P > 1 ? (uint64_t)part_off[part + 1] - part_off[part] : n_tris;
    if (cnt == 0) {  // main.cpp:330: partitions without triangles are skipped
      top.push(pl.Ls, TNode());
      continue;
    }
    StripeOut so = run_stripe(c, st, pl, prm, d_tris, n_tris, items, ibeg, cnt, part, s, top.node_pos, top.data_pos, out.device);
    if (so.empty) {
      top.push(pl.Ls, TNode());
      continue;
    }
    filled += so.filled;
    if (!out.device) {
      if (so.node_span && out.sink(out.user, OOC_STREAM_NODES, c->h_nodes.p, so.node_span * 24) != 0)
        fail(OOC_ERR_SINK, "node sink returned an error");
      if (so.data_span && out.sink(out.user, OOC_STREAM_DATA, c->h_data.p, so.data_span * 32) != 0)
        fail(OOC_ERR_SINK, "data sink returned an error");
    }
    top.node_pos += so.node_span;
    top.data_pos += so.data_span;
    top.push(pl.Ls, so.root);
  }
  // finalizeTree: the root is written last (OctreeBuilder.cpp:34-55)
  out.node(top.node_pos++, top.buf[0][0]);

  if (info) {
    info->n_nodes = top.node_pos;
    info->n_data = top.data_pos;
    info->n_filled = filled;
    info->n_partitions = pl.P;
    info->n_stripes = pl.n_stripes;
    info->n_items = n_items;
  }
  if (out.device) {
    uint64_t* nodes = ensure_keep<uint64_t>(c->d_nodes, top.node_pos * 24, (top.node_pos - 1) * 24, st);
    unsigned char* data = ensure_keep<unsigned char>(c->d_data, top.data_pos * 32, top.data_pos * 32, st);
    const uint64_t nr = out.node_recs.size() / 4, dr = out.data_recs.size() / 5;
    const size_t bytes = (out.node_recs.size() + out.data_recs.size()) * 8;
    uint64_t* h = ensure_pinned<uint64_t>(c->h_recs, bytes);
    std::memcpy(h, out.node_recs.data(), out.node_recs.size() * 8);
    std::memcpy(h + out.node_recs.size(), out.data_recs.data(), out.data_recs.size() * 8);
    uint64_t* d = ensure<uint64_t>(c->d_recs, bytes);
    ck(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st), "records");
    launch_scatter_records(d, nr, 3, nodes, st);
    launch_scatter_records(d + out.node_recs.size(), dr, 4, reinterpret_cast<uint64_t*>(data), st);
    c->res_nodes = top.node_pos;
    c->res_data = top.data_pos;
    c->res_valid = true;
  }
}

void finish_timing(ooc_ctx* c) {
  for (float& v : c->phase_ms) v = 0.0f;
  if (c->timing) {
    for (const auto& m : c->marks) {
      float ms = 0.0f;
      if (cudaEventElapsedTime(&ms, c->ev_pool[m[1]], c->ev_pool[m[2]]) == cudaSuccess) c->phase_ms[m[0]] += ms;
    }
  }
  c->knames.clear();
  c->kms.clear();
  c->kcount.clear();
  for (const auto& m : c->kmarks) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, c->ev_pool[m.second[0]], c->ev_pool[m.second[1]]) != cudaSuccess) continue;
    size_t i = 0;
    while (i < c->knames.size() && c->knames[i] != m.first) i++;
    if (i == c->knames.size()) {
      c->knames.push_back(m.first);
      c->kms.push_back(0.0f);
      c->kcount.push_back(0);
    }
    c->kms[i] += ms;
    c->kcount[i] += 1;
  }
}

void kernel_begin(void* user, const char* name, cudaStream_t st) {
  ooc_ctx* c = static_cast<ooc_ctx*>(user);
  if (c->kfilter != "*" && c->kfilter != name) return;
  c->kopen = c->ev_used;
  cudaEventRecord(next_event(c), st);
}

void kernel_end(void* user, const char* name, cudaStream_t st) {
  ooc_ctx* c = static_cast<ooc_ctx*>(user);
  if (c->kfilter != "*" && c->kfilter != name) return;
  const size_t e = c->ev_used;
  cudaEventRecord(next_event(c), st);
  c->kmarks.push_back({name, {c->kopen, e}});
}

void begin_build(ooc_ctx* c) {
  ck(cudaSetDevice(c->device), "cudaSetDevice");
  c->err.clear();
  c->marks.clear();
  c->kmarks.clear();
  c->ev_used = 0;
  c->res_valid = false;
  g_launches = 0;
  if (c->kfilter.empty()) {
    g_hooks = KernelHooks();
  } else {
    g_hooks.user = c;
    g_hooks.begin = kernel_begin;
    g_hooks.end = kernel_end;
  }
}

template <typename F>
int guarded(ooc_ctx* c, F&& f) {
  if (!c) return OOC_ERR_INVALID;
  try {
    f();
    c->launches = g_launches;
    return OOC_OK;
  } catch (const OocError& e) {
    c->err = e.msg;
    c->launches = g_launches;
    return e.code;
  } catch (const std::bad_alloc&) {
    c->err = "host allocation failed";
    return OOC_ERR_OOM;
  } catch (...) {
    c->err = "unexpected exception";
    return OOC_ERR_DEVICE;
  }
}

}  // namespace

// ===========================================================================
// C ABI
// ===========================================================================
extern "C" {

int ooc_ctx_create(int32_t device, ooc_ctx** out) {
  if (!out) return OOC_ERR_INVALID;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n) return OOC_ERR_DEVICE;
  ooc_ctx* c = new (std::nothrow) ooc_ctx();
  if (!c) return OOC_ERR_OOM;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return OOC_ERR_DEVICE;
  }
  *out = c;
  return OOC_OK;
}

void ooc_ctx_destroy(ooc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->own_stream) cudaStreamSynchronize(c->own_stream);
  DevBuf* bufs[] = {&c->d_tris, &c->d_items, &c->d_hist, &c->d_axis, &c->d_bits, &c->d_scan, &c->d_scanpart,
                    &c->d_keys, &c->d_size, &c->d_dsize, &c->d_start, &c->d_dstart, &c->d_cache, &c->d_winners,
                    &c->d_taskoff, &c->d_taskpart, &c->d_counter, &c->d_nodes, &c->d_data, &c->d_recs,
                    &c->d_rootinfo, &c->d_itemmask, &c->d_firstchild, &c->d_itembox};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  PinBuf* pins[] = {&c->h_nodes, &c->h_data, &c->h_misc, &c->h_recs};
  for (PinBuf* b : pins)
    if (b->p) cudaFreeHost(b->p);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  if (c->own_stream) cudaStreamDestroy(c->own_stream);
  delete c;
}

const char* ooc_last_error(const ooc_ctx* c) { return c ? c->err.c_str() : "null context"; }

uint64_t ooc_estimate_partitions(uint64_t gridsize, uint64_t memory_limit_mb) {
  // partitioner.cpp:12-28
  const uint64_t required = (gridsize * gridsize * gridsize) / 1024 / 1024;
  if (required <= memory_limit_mb) return 1;
  uint64_t n = 1, req = required;
  while (req > memory_limit_mb) {
    req /= 8;
    n *= 8;
  }
  return n;
}

int ooc_build(ooc_ctx* c, const ooc_build_params* prm, const float* tris_host, uint64_t n_tris, ooc_sink_fn sink,
              void* user, ooc_build_info* info) {
  return guarded(c, [&] {
    begin_build(c);
    check_params(prm, n_tris);
    if (!sink) fail(OOC_ERR_INVALID, "sink is NULL");
    if (n_tris && !tris_host) fail(OOC_ERR_INVALID, "triangles are NULL");
    cudaStream_t st = c->own_stream;
    const int stride = prm->geometry_only ? 9 : 21;
    const size_t bytes = n_tris * stride * sizeof(float);
    float* d_tris = ensure<float>(c->d_tris, bytes);
    {
      PhaseScope all(c, PH_ALL, st);
      {
        PhaseScope ph(c, PH_COPY, st);
        if (bytes) ck(cudaMemcpyAsync(d_tris, tris_host, bytes, cudaMemcpyHostToDevice, st), "H2D triangles");
      }
      Emitter out;
      out.device = false;
      out.sink = sink;
      out.user = user;
      build_core(c, prm, d_tris, n_tris, st, out, info);
    }
    ck(cudaStreamSynchronize(st), "build");
    finish_timing(c);
  });
}

int ooc_build_device(ooc_ctx* c, const ooc_build_params* prm, const float* tris_device, uint64_t n_tris,
                     void* stream, ooc_build_info* info) {
  return guarded(c, [&] {
    begin_build(c);
    check_params(prm, n_tris);
    if (n_tris && !tris_device) fail(OOC_ERR_INVALID, "triangles are NULL");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    {
      PhaseScope all(c, PH_ALL, st);
      Emitter out;
      out.device = true;
      build_core(c, prm, tris_device, n_tris, st, out, info);
    }
    ck(cudaStreamSynchronize(st), "build");
    ck(cudaGetLastError(), "build kernels");
    finish_timing(c);
  });
}

int ooc_result_device(ooc_ctx* c, const void** nodes_device, const void** data_device) {
  if (!c) return OOC_ERR_INVALID;
  if (!c->res_valid) {
    c->err = "no device result: run ooc_build_device first";
    return OOC_ERR_INVALID;
  }
  if (nodes_device) *nodes_device = c->d_nodes.p;
  if (data_device) *data_device = c->d_data.p;
  return OOC_OK;
}

int ooc_result_copy(ooc_ctx* c, void* nodes_host, void* data_host) {
  return guarded(c, [&] {
    if (!c->res_valid) fail(OOC_ERR_INVALID, "no device result: run ooc_build_device first");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    if (nodes_host && c->res_nodes)
      ck(cudaMemcpy(nodes_host, c->d_nodes.p, c->res_nodes * 24, cudaMemcpyDeviceToHost), "D2H nodes");
    if (data_host && c->res_data)
      ck(cudaMemcpy(data_host, c->d_data.p, c->res_data * 32, cudaMemcpyDeviceToHost), "D2H data");
  });
}

int ooc_set_phase_timing(ooc_ctx* c, int32_t enable) {
  if (!c) return OOC_ERR_INVALID;
  c->timing = enable != 0;
  return OOC_OK;
}

int ooc_phase_times(const ooc_ctx* c, float* ms, int32_t n) {
  if (!c || !ms || n < 0) return OOC_ERR_INVALID;
  for (int i = 0; i < n && i < kPhases; i++) ms[i] = c->phase_ms[i];
  return OOC_OK;
}

uint64_t ooc_kernel_launches(const ooc_ctx* c) { return c ? c->launches : 0; }

int ooc_set_kernel_timing(ooc_ctx* c, const char* kernel) {
  if (!c) return OOC_ERR_INVALID;
  c->kfilter = kernel ? kernel : "";
  return OOC_OK;
}

int ooc_kernel_time(const ooc_ctx* c, int32_t index, const char** name, float* total_ms, uint64_t* launches) {
  if (!c || index < 0 || (size_t)index >= c->knames.size()) return OOC_ERR_INVALID;
  if (name) *name = c->knames[index].c_str();
  if (total_ms) *total_ms = c->kms[index];
  if (launches) *launches = c->kcount[index];
  return OOC_OK;
}

}  // extern "C"
