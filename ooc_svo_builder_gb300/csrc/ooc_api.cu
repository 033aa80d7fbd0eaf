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
#include <functional>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <thread>
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

// Bounded pinned staging for the records a sub-batch copies back: its device
// bytes travel through kRingK chunks of kRingChunk bytes on the copy stream,
// and a chunk is refilled as soon as the host has handed it to the sink.  The
// pinned memory a context holds is therefore fixed, whatever a batch emits.
constexpr int kRingK = 4;
constexpr uint64_t kRingChunk = 32ull << 20;

struct D2HRing {
  PinBuf buf;
  cudaStream_t st = nullptr;  // the stream its copies go on (one per sub-batch slot)
  cudaEvent_t ev[kRingK] = {};
  const char* src = nullptr;
  uint64_t len = 0, n_chunks = 0;
  uint64_t issued = 0;    // chunks whose copy has been queued
  uint64_t released = 0;  // chunks handed to the sink and free again
  size_t t_begin = 0;     // timing event before the first chunk
};

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
  ooc::LaunchState lstate;  // this context's launch count and timing hooks, installed per API call
  DevBuf d_tris, d_hist, d_axis, d_bits, d_scan, d_scanpart, d_keys, d_size, d_dsize, d_start, d_dstart,
      d_cache, d_winners, d_taskoff, d_taskpart, d_counter, d_nodes, d_data, d_recs, d_rootinfo, d_itemmask,
      d_firstchild, d_itembox, d_leaf, d_touch, d_local, d_taskmap, d_woff;
  uint64_t max_tasks = 0;  // most large-item warp tasks a sub-batch has had (sizes the task map)
  // persistent phase A (ooc_tuning::persistent): its counters, its task map (all ones
  // between launches: every entry a launch fills is emptied by the warp that reads it)
  DevBuf d_pctr, d_pmap;
  bool pmap_empty = false;
  int persist_per_sm = -1;  // CTAs per SM of the persistent kernel for persist_lpl
  uint32_t persist_lpl = 0;
  bool leaf_zero = true;  // d_leaf and d_touch hold only zeros (no sub-batch left them dirty)
  PinBuf h_misc, h_recs, h_tables1, h_tables2, h_words;
  // double-buffered outputs of pipelined sub-batches
  DevBuf d_out_nodes[2], d_out_data[2];
  PinBuf h_root[2];
  D2HRing ring[2][2];  // [slot][OOC_STREAM_NODES / OOC_STREAM_DATA]
  cudaEvent_t ev_compute[2] = {nullptr, nullptr};
  cudaEvent_t ev_data[2] = {nullptr, nullptr};  // host output: a sub-batch's data file is final
  cudaStream_t copy_stream = nullptr;
  cudaStream_t ring_stream[2] = {nullptr, nullptr};  // host output: the copy back of each sub-batch slot
  cudaStream_t h2d_stream = nullptr;     // batch uploads, overlapping the sub-batches that do not need them yet
  std::vector<cudaEvent_t> up_events;    // recorded on h2d_stream as groups of meshes arrive
  DevBuf d_tables1, d_tables2;
  std::vector<DevBuf> d_mesh_items;
  ooc_tuning tuning = {64, 16, 256, 4, 4ull << 30, 0, 8, 1, 0};  // launch choices (ooc_set_tuning / ooc_autotune)
  // executable graphs of captured launch sequences, by shape (launch count and kernels)
  std::vector<std::pair<uint64_t, cudaGraphExec_t>> graph_execs;
  DevBuf d_tune_arena;                               // autotuner outputs
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
  // the last build's first mesh: triangles binned to each partition, voxels it filled
  std::vector<uint64_t> part_tris, part_filled;
  float file_ms[2] = {0, 0};  // ooc_build_files: input read and upload, output written (host ms)
  // out-of-core builds: device bytes for streamed triangle records (0: automatic), and their buffers
  uint64_t stream_budget = 0;
  DevBuf d_chunk[2], d_group[2], d_stream_mat, d_stream_part, d_stream_base, d_part_off;
  PinBuf h_stage[2];
  cudaEvent_t ev_stage[2] = {nullptr, nullptr};
  uint64_t stream_passes = 0;  // passes over the source in the last build (0: not streamed)
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

void ring_issue(ooc_ctx* c, D2HRing& r) {
  const uint64_t j = r.issued++;
  const uint64_t off = j * kRingChunk;
  const uint64_t n = std::min(kRingChunk, r.len - off);
  char* dst = static_cast<char*>(r.buf.p) + (j % kRingK) * kRingChunk;
  ck(cudaMemcpyAsync(dst, r.src + off, n, cudaMemcpyDeviceToHost, r.st), "D2H");
  ck(cudaEventRecord(r.ev[j % kRingK], r.st), "event");
  if (c->timing && r.issued == r.n_chunks) {
    const size_t e = c->ev_used;
    ck(cudaEventRecord(next_event(c), r.st), "cudaEventRecord");
    c->marks.push_back({(size_t)PH_COPY, r.t_begin, e});
  }
}

// Queue the first chunks of `len` device bytes on `st` (which already waits for their producer).
void ring_start(ooc_ctx* c, D2HRing& r, const void* src, uint64_t len, cudaStream_t st) {
  r.st = st;
  r.src = static_cast<const char*>(src);
  r.len = len;
  r.n_chunks = (len + kRingChunk - 1) / kRingChunk;
  r.issued = r.released = 0;
  if (!len) return;
  ensure_pinned<char>(r.buf, std::min<uint64_t>(len, kRingK * kRingChunk));
  for (int k = 0; k < kRingK; k++)
    if (!r.ev[k]) ck(cudaEventCreateWithFlags(&r.ev[k], cudaEventDisableTiming), "cudaEventCreate");
  if (c->timing) {
    r.t_begin = c->ev_used;
    ck(cudaEventRecord(next_event(c), st), "cudaEventRecord");
  }
  while (r.issued < r.n_chunks && r.issued < (uint64_t)kRingK) ring_issue(c, r);
}

// Hand bytes [a, b) to `out` in order; calls over one sub-batch cover its bytes in
// increasing order.  With `block` false it stops at the first chunk whose copy has
// not landed yet.  Returns how far it got (b when done).
template <typename F>
uint64_t ring_take(ooc_ctx* c, D2HRing& r, uint64_t a, uint64_t b, bool block, F&& out) {
  while (a < b) {
    const uint64_t j = a / kRingChunk;
    if (j >= r.issued || j < r.released) fail(OOC_ERR_DEVICE, "internal copy-back order");
    if (block) {
      ck(cudaEventSynchronize(r.ev[j % kRingK]), "D2H");
    } else {
      const cudaError_t e = cudaEventQuery(r.ev[j % kRingK]);
      if (e == cudaErrorNotReady) return a;
      ck(e, "D2H");
    }
    const uint64_t end = std::min(b, (j + 1) * kRingChunk);
    out(static_cast<const char*>(r.buf.p) + (j % kRingK) * kRingChunk + (a - j * kRingChunk), end - a);
    a = end;
    if (a == (j + 1) * kRingChunk || a == r.len) {
      r.released = j + 1;
      if (r.issued < r.n_chunks) ring_issue(c, r);
    }
  }
  return a;
}

// Run `launches` on `st`, directly or captured into a CUDA graph and replayed.
// Executable graphs are cached by shape (the sequence, its node count and its
// kernels) and updated in place with the new launch parameters, so repeated
// shapes skip instantiation.  The captured region neither allocates nor
// synchronises; phase and kernel timing launch directly.
template <typename F>
void run_launches(ooc_ctx* c, cudaStream_t st, int which, F&& launches, bool direct = false) {
  if (direct || !c->tuning.graphs || c->timing || c->lstate.hooks.begin) {
    launches();
    return;
  }
  ck(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
  cudaGraph_t graph = nullptr;
  const bool pdl = c->lstate.pdl;
  c->lstate.pdl = false;  // captured launches keep plain stream order
  try {
    launches();
  } catch (...) {
    c->lstate.pdl = pdl;
    cudaStreamEndCapture(st, &graph);
    if (graph) cudaGraphDestroy(graph);
    throw;
  }
  c->lstate.pdl = pdl;
  ck(cudaStreamEndCapture(st, &graph), "cudaStreamEndCapture");
  // shape key: which sequence, node count, and the kernels in capture order
  size_t count = 0;
  ck(cudaGraphGetNodes(graph, nullptr, &count), "cudaGraphGetNodes");
  std::vector<cudaGraphNode_t> nodes(count);
  if (count) ck(cudaGraphGetNodes(graph, nodes.data(), &count), "cudaGraphGetNodes");
  uint64_t key = 1469598103934665603ull ^ (uint64_t)which ^ ((uint64_t)count << 8);
  for (cudaGraphNode_t nd : nodes) {
    cudaGraphNodeType ty;
    ck(cudaGraphNodeGetType(nd, &ty), "cudaGraphNodeGetType");
    uint64_t v = (uint64_t)ty;
    if (ty == cudaGraphNodeTypeKernel) {
      cudaKernelNodeParams kp;
      ck(cudaGraphKernelNodeGetParams(nd, &kp), "cudaGraphKernelNodeGetParams");
      v ^= reinterpret_cast<uintptr_t>(kp.func) << 4;
    }
    key = (key ^ v) * 1099511628211ull;
  }
  cudaGraphExec_t exec = nullptr;
  for (auto& kv : c->graph_execs)
    if (kv.first == key) exec = kv.second;
  cudaError_t e = cudaSuccess;
  if (exec) {
    cudaGraphExecUpdateResultInfo info;
    e = cudaGraphExecUpdate(exec, graph, &info);
  }
  if (!exec || e != cudaSuccess) {
    cudaGetLastError();  // an update refused is a shape change, not an error
    for (auto it = c->graph_execs.begin(); it != c->graph_execs.end(); ++it)
      if (it->first == key) {
        cudaGraphExecDestroy(it->second);
        c->graph_execs.erase(it);
        break;
      }
    if (c->graph_execs.size() >= 64) {  // keep the cache bounded: drop the oldest shape
      cudaGraphExecDestroy(c->graph_execs.front().second);
      c->graph_execs.erase(c->graph_execs.begin());
    }
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e == cudaSuccess) c->graph_execs.push_back({key, exec});
  }
  cudaGraphDestroy(graph);
  ck(e, "cudaGraphInstantiate");
  ck(cudaGraphLaunch(exec, st), "cudaGraphLaunch");
}

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

// Where a mesh's records go: device files (records written on the host are
// collected and scattered at the end), a host sink in file order, or nowhere
// (the dry run that only computes positions).
struct Emitter {
  bool device = false;
  bool dry = false;
  // device mode: (index, words...) records scattered into the device files at the end
  std::vector<uint64_t> node_recs, data_recs;
  // host mode
  ooc_batch_sink_fn sink = nullptr;
  void* user = nullptr;
  uint64_t mesh = 0;

  void span(int32_t kind, const void* bytes, uint64_t n) {
    if (dry || device) return;
    if (sink(user, mesh, kind, bytes, n) != 0) fail(OOC_ERR_SINK, "sink returned an error");
  }
  void node(uint64_t pos, const TNode& n) {
    if (dry) return;
    if (device) {
      node_recs.insert(node_recs.end(), {pos, n.data, n.cb, n.off});
    } else {
      uint64_t rec[3] = {n.data, n.cb, n.off};
      if (sink(user, mesh, OOC_STREAM_NODES, rec, 24) != 0) fail(OOC_ERR_SINK, "sink returned an error");
    }
  }
  void data(uint64_t pos, uint64_t morton, const float* v) {
    if (dry) return;
    uint64_t w[4];
    w[0] = morton;
    std::memcpy(&w[1], v, 24);
    if (device) {
      data_recs.insert(data_recs.end(), {pos, w[0], w[1], w[2], w[3]});
    } else {
      if (sink(user, mesh, OOC_STREAM_DATA, w, 32) != 0) fail(OOC_ERR_SINK, "sink returned an error");
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

// Triangles of an out-of-core build, read again from the start for every pass:
// from host memory, or from a .tridata file (the reference streams each
// partition from its .tripdata file the same way, main.cpp:329-345).
struct StreamSource {
  const char* host = nullptr;
  std::string path;
  uint64_t n_tris = 0, rec = 0;  // records and bytes per record
  FILE* f = nullptr;
  StreamSource() = default;
  StreamSource(const StreamSource&) = delete;
  StreamSource& operator=(const StreamSource&) = delete;
  ~StreamSource() {
    if (f) std::fclose(f);
  }
};

// ---------------------------------------------------------------------------
// The batch engine.  A batch is a list of meshes; every mesh is split into
// stripes, and the stripes of all meshes run through one launch sequence (a
// sub-batch when their occupancy pyramids exceed the memory budget).  Each
// sub-batch synchronises with the host twice: after the level counts (to size
// the per-node arrays and place every stripe's records in its file), and at
// the end (root records for the host-side grouping).
// ---------------------------------------------------------------------------
struct MeshWork {
  const ooc_build_params* prm = nullptr;
  Plan pl;
  const float* d_tris = nullptr;
  uint64_t n_tris = 0;
  std::vector<uint32_t> part_off;  // P > 1: items of partition p are part_off[p] .. part_off[p+1)
  const uint32_t* items = nullptr;
  Emitter* out = nullptr;
  TopBuilder top;            // emits the records above the stripes, in file order
  uint64_t next_stripe = 0;  // stripes before this one have been pushed into `top`
  Emitter dry;
  TopBuilder layout;         // the same grouping run ahead on placeholders: file positions only
  uint64_t layout_next = 0;
  uint64_t filled = 0;
  std::vector<uint64_t> part_filled;  // voxels filled in each partition
  uint64_t n_items = 0;
  int64_t last_stripe = -1;  // last stripe with items (-1: none)
  cudaEvent_t uploaded = nullptr;  // the triangles are on the device once this has completed (null: already)
  // a one-partition mesh uploaded in pieces: (end item, event after its copy), so the
  // voxelization of each piece starts as soon as it is on the device
  std::vector<std::pair<uint64_t, cudaEvent_t>> pieces;
  uint64_t index = 0;        // in the batch
  // out-of-core: the triangles are read from `src` again for every group of partitions;
  // the resident group's records (each partition's in stream order) are in d_tris
  StreamSource* src = nullptr;
  std::vector<std::pair<uint64_t, uint64_t>> groups;  // consecutive partitions [p0, p1)
  size_t next_group = 0;
  uint64_t group_end = 0;         // partitions below this are resident or done
  uint64_t group_first_item = 0;  // part_off of the resident group's first partition
  uint64_t resident = 0;          // records in d_tris
  const float* d_axis = nullptr;  // the partitions' world slabs (stream_count)
  const uint32_t* d_part_off = nullptr;
  // caller-owned device destination (output to device destinations)
  void* dst_nodes = nullptr;
  void* dst_data = nullptr;
  bool dst_ready = false;
  uint64_t total_nodes = 0, total_data = 0;
  uint64_t carried_nodes = 0, carried_data = 0;  // records parked in the carry buffers
  MeshWork(const Plan& p, Emitter* o)
      : pl(p), out(o), top(p.Ls, p.levels != 0, o), layout(p.Ls, p.levels != 0, nullptr), part_filled(p.P, 0) {
    dry.dry = true;
  }
  MeshWork(const MeshWork&) = delete;
  MeshWork(MeshWork&& o) noexcept
      : prm(o.prm), pl(o.pl), d_tris(o.d_tris), n_tris(o.n_tris), part_off(std::move(o.part_off)), items(o.items),
        out(o.out), top(o.top), next_stripe(o.next_stripe), dry(o.dry), layout(o.layout),
        layout_next(o.layout_next), filled(o.filled), part_filled(std::move(o.part_filled)), n_items(o.n_items),
        last_stripe(o.last_stripe),
        uploaded(o.uploaded), pieces(std::move(o.pieces)),
        index(o.index), src(o.src), groups(std::move(o.groups)), next_group(o.next_group), group_end(o.group_end),
        group_first_item(o.group_first_item), resident(o.resident), d_axis(o.d_axis), d_part_off(o.d_part_off), dst_nodes(o.dst_nodes), dst_data(o.dst_data), dst_ready(o.dst_ready),
        total_nodes(o.total_nodes), total_data(o.total_data), carried_nodes(o.carried_nodes),
        carried_data(o.carried_data) {}
};

struct StripeRef {
  uint32_t mesh;
  uint64_t stripe, part, ibeg, n_items;
};

struct Placed {  // a stripe after the level counts
  bool empty = true;
  uint64_t total = 0, n_leaf = 0, node_span = 0, data_span = 0, node_base = 0, data_base = 0;
  uint64_t out_node_off = 0, out_data_off = 0;  // host mode: offsets in the batch output buffers
};

// Stripes of 512^3 voxels and more mark their leaf blocks; smaller leaf
// levels are read and zeroed whole (their marks would cost the voxelization
// more than they save).
constexpr int kMarkDepth = 9;

// Levels 0..Ds of a stripe appended to the buffers: the words of the levels
// kept zero between builds (the leaf level, and with marks the level above it)
// to `leaf_words`, the others to `words`, every level's scan entries to
// `entries` (one per group of kLeafGroup blocks for a marked leaf level).
int pyramid_levels(int Ds, Level* lv, uint64_t& words, uint64_t& leaf_words, uint64_t& entries, bool marked) {
  const int zl = marked ? Ds - 1 : Ds;
  for (int l = 0; l <= Ds; l++) {
    const uint64_t nbits = 1ull << (3 * l);
    uint64_t nw = (nbits + 31) / 32;
    nw = (nw + 7) / 8 * 8;
    uint64_t& acc = l >= zl ? leaf_words : words;
    lv[l].off_w = acc;
    lv[l].off_b = entries;
    lv[l].nwords = nw;
    lv[l].nblocks = nw / 8;
    lv[l].nscan = (l == Ds && marked) ? (lv[l].nblocks + kLeafGroup - 1) / kLeafGroup : lv[l].nblocks;
    acc += nw;
    entries += lv[l].nscan;
  }
  return Ds;
}

// CTA prefix of one batched launch: stripe s gets ceil(count(s) / per_cta) CTAs.
template <typename F>
std::vector<uint64_t> cta_prefix(uint32_t n, uint64_t per_cta, F count) {
  std::vector<uint64_t> beg(n + 1, 0);
  for (uint32_t s = 0; s < n; s++) beg[s + 1] = beg[s] + (count(s) + per_cta - 1) / per_cta;
  return beg;
}

// A per-block or per-node launch: its CTA prefix and the elements each thread
// takes.  A thread takes as many elements (up to the tuning's limit) as still
// leave about 16 CTAs per SM: few CTAs cost parallelism on small levels, many
// cost the per-CTA staging on large ones.
struct Light {
  std::vector<uint64_t> beg;
  uint32_t ept = 1;
};

template <typename F>
Light light_prefix(const ooc_ctx* c, uint32_t n, F count) {
  std::vector<uint64_t> cnt(n);
  uint64_t total = 0;
  for (uint32_t s = 0; s < n; s++) total += cnt[s] = count(s);
  Light L;
  const uint64_t fill = (uint64_t)c->num_sms * 16 * kChunk;
  L.ept = (uint32_t)std::min<uint64_t>(c->tuning.light_per_thread, std::max<uint64_t>(1, total / fill));
  L.beg = cta_prefix(n, (uint64_t)kChunk * L.ept, [&](uint32_t s) { return cnt[s]; });
  return L;
}

// Upload host vectors into one device buffer through pinned staging; returns device pointers.
struct Uploader {
  std::vector<std::pair<const void*, size_t>> parts;
  size_t add(const void* p, size_t bytes) {
    size_t off = 0;
    for (auto& q : parts) off += (q.second + 255) / 256 * 256;
    parts.push_back({p, bytes});
    return off;
  }
  unsigned char* run(ooc_ctx* c, DevBuf& dev, PinBuf& pin, cudaStream_t st) {
    size_t total = 0;
    for (auto& q : parts) total += (q.second + 255) / 256 * 256;
    unsigned char* h = ensure_pinned<unsigned char>(pin, total);
    unsigned char* d = ensure<unsigned char>(dev, total);
    size_t off = 0;
    for (auto& q : parts) {
      if (q.second) std::memcpy(h + off, q.first, q.second);
      off += (q.second + 255) / 256 * 256;
    }
    ck(cudaMemcpyAsync(d, h, total, cudaMemcpyHostToDevice, st), "upload tables");
    (void)c;
    return d;
  }
};

// Where the records of the stripes go: host sink (through the copy-back ring),
// the context's own device files (one mesh), or a device destination per mesh
// that the caller provides once the mesh's sizes are known.
enum OutMode { OUT_HOST, OUT_CTX, OUT_DEST };
struct OutSpec {
  OutMode mode = OUT_HOST;
  ooc_alloc_fn alloc = nullptr;
  ooc_ready_fn ready = nullptr;
  void* user = nullptr;
  mutable size_t alloc_next = 0;  // destinations are asked for in mesh order
};

// Sizes of a mesh's files from the placement run-ahead (every stripe with items
// already placed), then its destination from the caller.  Records parked in the
// carry buffers (stripes of earlier sub-batches) move there first.
void ensure_dest(ooc_ctx* c, cudaStream_t st, MeshWork& m, const OutSpec& os) {
  if (m.dst_ready) return;
  TopBuilder& tb = m.layout;
  tb.out = &m.dry;
  for (; m.layout_next < m.pl.n_stripes; m.layout_next++) tb.push(tb.top, TNode());
  m.total_nodes = tb.node_pos + 1;  // the root
  m.total_data = tb.data_pos;
  void* dn = nullptr;
  void* dd = nullptr;
  if (os.alloc(os.user, m.index, m.total_nodes * 24, m.total_data * 32, st, &dn, &dd) != 0 || !dn || !dd)
    fail(OOC_ERR_OOM, "destination allocation failed for mesh " + std::to_string(m.index));
  if ((reinterpret_cast<uintptr_t>(dn) | reinterpret_cast<uintptr_t>(dd)) & 7)
    fail(OOC_ERR_INVALID, "destinations must be 8-byte aligned");
  m.dst_nodes = dn;
  m.dst_data = dd;
  m.dst_ready = true;
  if (m.carried_nodes)
    ck(cudaMemcpyAsync(dn, c->d_nodes.p, m.carried_nodes * 24, cudaMemcpyDeviceToDevice, st), "carry");
  if (m.carried_data)
    ck(cudaMemcpyAsync(dd, c->d_data.p, m.carried_data * 32, cudaMemcpyDeviceToDevice, st), "carry");
}

// Destinations of meshes up to `idx`, in mesh order: the ones before it that
// have not had theirs are meshes without items (every stripe of a mesh with
// items precedes the stripes of later meshes, so it has been placed).
void alloc_through(ooc_ctx* c, cudaStream_t st, std::vector<MeshWork>& meshes, size_t idx, const OutSpec& os) {
  for (; os.alloc_next <= idx; os.alloc_next++) ensure_dest(c, st, meshes[os.alloc_next], os);
}

// A launched sub-batch whose records are still on their way to the host.
struct Pending {
  bool active = false;
  int slot = 0;
  std::vector<StripeRef> sb;
  std::vector<Placed> pl;
  std::vector<int> depth;
  // how far the hand-over has got (finish_sub_batch resumes from here)
  bool checked = false;  // the sub-batch's kernels are done and its layout flag is clear
  uint32_t at = 0;       // stripe being handed over
  int stage = 0;         // 0 not started, 1 node bytes, 2 data bytes
  uint64_t cur = 0;      // next byte of the current range
};

// Queues the read back of n device words into the context's pinned buffer (by a
// kernel's stores, so it does not wait behind copies on the copy engine); the
// returned host pointer holds them once `st` has reached this point.
const uint32_t* read_back_words(ooc_ctx* c, const uint32_t* src, uint64_t n, cudaStream_t st) {
  uint32_t* h = ensure_pinned<uint32_t>(c->h_words, std::max<uint64_t>(n, 1) * 4);
  uint32_t* d = nullptr;
  ck(cudaHostGetDevicePointer(reinterpret_cast<void**>(&d), h, 0), "mapped read back");
  launch_copy_words(src, n, d, st);
  return h;
}

// Waits for the level counts on `st`.  Meanwhile `idle` (if set) hands the previous
// sub-batch's landed copy-back chunks to the sink, so the copy stream keeps moving;
// it returns false once there is nothing left for it to do.
void wait_level_counts(cudaStream_t st, const std::function<bool()>& idle) {
  if (idle) {
    for (;;) {
      const cudaError_t e = cudaStreamQuery(st);
      if (e == cudaSuccess) return;
      if (e != cudaErrorNotReady) ck(e, "level counts");
      if (!idle()) break;
      std::this_thread::yield();
    }
  }
  ck(cudaStreamSynchronize(st), "level counts");
}

void run_sub_batch(ooc_ctx* c, cudaStream_t st, std::vector<MeshWork>& meshes, const std::vector<StripeRef>& sb,
                   const OutSpec& os, Pending& out_pending, int slot, const std::function<bool()>& idle = nullptr) {
  const uint32_t n = (uint32_t)sb.size();
  // a lone stripe of a mesh uploaded in pieces voxelizes each piece on arrival
  const std::vector<std::pair<uint64_t, cudaEvent_t>>* pieces =
      (n == 1 && !meshes[sb[0].mesh].pieces.empty()) ? &meshes[sb[0].mesh].pieces : nullptr;
  // ---- geometry of every stripe ----
  std::vector<Pyramid> pyr(n);
  std::vector<VoxJob> vj(n);
  std::vector<uint64_t> item_beg(n + 1, 0), touch_beg(n, 0), local_beg(n, 0), woff_beg(n, 0);
  uint64_t words = 0, leaf_words = 0, blocks = 0, tbytes = 0, nlocal = 0, items = 0, nwoff = 0;
  int max_depth = 0;
  for (uint32_t s = 0; s < n; s++) {
    const StripeRef& r = sb[s];
    const MeshWork& m = meshes[r.mesh];
    std::memset(&pyr[s], 0, sizeof(Pyramid));
    pyr[s].depth = m.pl.Ds;
    pyramid_levels(m.pl.Ds, pyr[s].lv, words, leaf_words, blocks, m.pl.Ds >= kMarkDepth);
    touch_beg[s] = tbytes;
    tbytes += touch_bytes(pyr[s].lv[m.pl.Ds]);
    local_beg[s] = nlocal;
    if (m.pl.Ds >= kMarkDepth) nlocal += pyr[s].lv[m.pl.Ds].nblocks;
    woff_beg[s] = nwoff;  // the winner pass's bit ranks: payload stripes only
    if (!m.pl.binary) nwoff += pyr[s].lv[m.pl.Ds].nblocks;
    max_depth = std::max(max_depth, m.pl.Ds);
    item_beg[s] = items;
    items += r.n_items;
  }
  item_beg[n] = items;
  uint32_t* bits = ensure<uint32_t>(c->d_bits, words * 4);
  // the leaf levels and their block marks are all zero between sub-batches
  if (leaf_words * 4 > c->d_leaf.cap || tbytes > c->d_touch.cap) c->leaf_zero = false;
  uint32_t* leaf = ensure<uint32_t>(c->d_leaf, leaf_words * 4);
  uint8_t* touch = ensure<uint8_t>(c->d_touch, tbytes);
  uint16_t* local = ensure<uint16_t>(c->d_local, nlocal * 2);
  uint64_t* woff = nwoff ? ensure<uint64_t>(c->d_woff, nwoff * 8) : nullptr;
  if (!c->leaf_zero) {
    ck(cudaMemsetAsync(leaf, 0, c->d_leaf.cap, st), "memset leaf levels");
    ck(cudaMemsetAsync(touch, 0, c->d_touch.cap, st), "memset leaf marks");
    c->leaf_zero = true;
  }
  uint32_t* scan = ensure<uint32_t>(c->d_scan, (blocks + 1) * 4);
  uint32_t* scanpart = ensure<uint32_t>(c->d_scanpart, scan_partials_needed(blocks + 1) * 4);
  uint64_t* task_off = ensure<uint64_t>(c->d_taskoff, (items + 1) * 8);
  uint64_t* taskpart = ensure<uint64_t>(c->d_taskpart, scan_partials_needed(items + 1) * 8);
  uint64_t* item_mask = ensure<uint64_t>(c->d_itemmask, items * 8);
  uint64_t* item_box = ensure<uint64_t>(c->d_itembox, items * 8);
  unsigned long long* counter = ensure<unsigned long long>(c->d_counter, 16);
  uint32_t* d_root = ensure<uint32_t>(c->d_rootinfo, ((uint64_t)n * 16 + 64) * 4);
  uint32_t* flag = d_root + (uint64_t)n * 16;

  constexpr int kTopPyramidLevel = 5;  // levels 0..5 have at most 512 blocks: one CTA per stripe
  for (uint32_t s = 0; s < n; s++) {
    const StripeRef& r = sb[s];
    const MeshWork& m = meshes[r.mesh];
    Pyramid& P = pyr[s];
    P.bits = bits;
    P.leaf = leaf;
    P.touch = P.depth >= kMarkDepth ? touch + touch_beg[s] : nullptr;
    P.zl = P.depth >= kMarkDepth ? P.depth - 1 : P.depth;
    P.local = P.depth >= kMarkDepth ? local + local_beg[s] : nullptr;
    P.scan = scan;
    P.woff = m.pl.binary ? nullptr : woff + woff_beg[s];
    VoxJob& j = vj[s];
    std::memset(&j, 0, sizeof(j));
    uint32_t pa[3], sa[3];
    morton_global_decode(r.part * m.pl.M, pa[0], pa[1], pa[2]);
    morton_global_decode(r.stripe * m.pl.S, sa[0], sa[1], sa[2]);
    const uint32_t pside = 1u << m.pl.Dm, sside = 1u << m.pl.Ds;
    j.tris = m.d_tris;
    j.stride = m.pl.binary ? 9 : 21;
    j.item_tri = m.items;
    j.ibeg = r.ibeg;
    j.n_items = r.n_items;
    for (int a = 0; a < 3; a++) {
      j.pa[a] = (int)pa[a];
      j.pb[a] = (int)(pa[a] + pside - 1);
      j.sa[a] = (int)sa[a];
      j.sb[a] = (int)(sa[a] + sside - 1);
    }
    j.u = m.pl.u;
    j.unit_div = m.pl.unit_div;
    j.small_vol = c->tuning.small_vol;
    j.lines_per_lane = c->tuning.lines_per_lane;
    j.leafbits = leaf + P.lv[P.depth].off_w;
    j.leaftouch = P.touch;
    j.task_off = task_off + item_beg[s];
    j.task_flag = task_off + items;
    j.task_counter = counter;
    j.item_mask = m.pl.binary ? nullptr : item_mask + item_beg[s];
    j.item_box = m.pl.binary ? nullptr : item_box + item_beg[s];
  }
  const std::vector<uint64_t> cp_items = cta_prefix(n, kChunk, [&](uint32_t s) { return sb[s].n_items; });
  std::vector<Light> cp_pyr;
  for (int r = 0; r <= max_depth - kTopPyramidLevel - 1; r++)
    cp_pyr.push_back(light_prefix(c, n, [&](uint32_t s) -> uint64_t {
      const int l = pyr[s].depth - r;
      return l > kTopPyramidLevel ? pyr[s].lv[l].nscan : 0;
    }));

  // keys of every level, launched as soon as the level counts are back (its prefix needs no count)
  const Light cp_compact = light_prefix(c, n, [&](uint32_t s) -> uint64_t {
    const uint64_t upper = pyr[s].lv[pyr[s].depth].off_b - pyr[s].lv[0].off_b;  // compact_elems
    return (upper + 31) / 32 * 32 + (pyr[s].lv[pyr[s].depth].nscan + 31) / 32 * 32;
  });

  // persistent phase A: 32-item chunks and pyramid units per stripe, and the
  // per-stripe counts of units not yet done that its waits read
  bool persist = c->tuning.persistent != 0 && !pieces;
  if (persist && (c->persist_per_sm < 0 || c->persist_lpl != c->tuning.lines_per_lane)) {
    c->persist_per_sm = persist_ctas_per_sm(c->tuning.lines_per_lane);
    c->persist_lpl = c->tuning.lines_per_lane;
  }
  persist = persist && c->persist_per_sm > 0;
  constexpr uint32_t kPersistEpt = 32;  // pyramid elements per lane of a unit (1,024 per unit)
  std::vector<uint64_t> p_chunk, p_unit;
  std::vector<uint32_t> p_occ, p_pyr;
  const uint32_t p_levels = (uint32_t)cp_pyr.size();
  if (persist) {
    p_chunk = cta_prefix(n, kPersistChunkItems, [&](uint32_t s) { return sb[s].n_items; });
    p_occ.resize(n);
    for (uint32_t s = 0; s < n; s++) p_occ[s] = (uint32_t)(p_chunk[s + 1] - p_chunk[s]);
    p_unit.assign(std::max<uint64_t>((uint64_t)p_levels * (n + 1), 1), 0);  // one entry at least: uploaded as is
    p_pyr.assign(std::max<uint64_t>((uint64_t)p_levels * n, 1), 0);
    uint64_t acc = 0;
    for (uint32_t r = 0; r < p_levels; r++) {
      for (uint32_t s = 0; s < n; s++) {
        p_unit[(uint64_t)r * (n + 1) + s] = acc;
        const int l = pyr[s].depth - (int)r;
        const uint64_t units = l > kTopPyramidLevel ? (pyr[s].lv[l].nscan + 32 * kPersistEpt - 1) / (32 * kPersistEpt) : 0;
        p_pyr[(uint64_t)r * n + s] = (uint32_t)units;
        acc += units;
      }
      p_unit[(uint64_t)r * (n + 1) + n] = acc;
    }
  }

  Uploader up1;
  const size_t o_vj = up1.add(vj.data(), n * sizeof(VoxJob));
  const size_t o_pyr = up1.add(pyr.data(), n * sizeof(Pyramid));
  const size_t o_beg = up1.add(item_beg.data(), (n + 1) * 8);
  const size_t o_cpi = up1.add(cp_items.data(), (n + 1) * 8);
  std::vector<size_t> o_cpp(cp_pyr.size());
  for (size_t r = 0; r < cp_pyr.size(); r++) o_cpp[r] = up1.add(cp_pyr[r].beg.data(), (n + 1) * 8);
  const size_t o_cc = up1.add(cp_compact.beg.data(), (n + 1) * 8);
  size_t o_pc = 0, o_pu = 0, o_po = 0, o_pp = 0;
  if (persist) {
    o_pc = up1.add(p_chunk.data(), (n + 1) * 8);
    o_pu = up1.add(p_unit.data(), p_unit.size() * 8);
    o_po = up1.add(p_occ.data(), n * 4);
    o_pp = up1.add(p_pyr.data(), p_pyr.size() * 4);
  }
  unsigned char* t1 = up1.run(c, c->d_tables1, c->h_tables1, st);
  auto dp1 = [&](size_t off) { return reinterpret_cast<const uint64_t*>(t1 + off); };
  const VoxJob* d_vj = reinterpret_cast<const VoxJob*>(t1 + o_vj);
  const Pyramid* d_pyr = reinterpret_cast<const Pyramid*>(t1 + o_pyr);
  const uint64_t* d_beg = reinterpret_cast<const uint64_t*>(t1 + o_beg);

  uint32_t* lvl = ensure_pinned<uint32_t>(c->h_misc, ((uint64_t)n * 16 + 64) * 4);  // level bases, then root info
  uint32_t* lvl_dev = nullptr;  // the same pinned memory as the kernels address it
  ck(cudaHostGetDevicePointer(reinterpret_cast<void**>(&lvl_dev), lvl, 0), "mapped level counts");
  // Warp task -> item map, sized by the items and the most tasks a sub-batch has had.
  // Built once the context has seen a sub-batch with many tasks: with few, the large
  // items' search of the task offsets costs less than the map's launch.
  constexpr uint64_t kMapMinTasks = 4096;
  uint64_t* task_map = nullptr;
  uint64_t map_cap = 0;
  if (c->max_tasks >= kMapMinTasks) {
    task_map = ensure<uint64_t>(c->d_taskmap, std::max<uint64_t>(items, c->max_tasks) * 8);
    map_cap = c->d_taskmap.cap / 8;
  }
  PersistJob pj;
  std::memset(&pj, 0, sizeof(pj));
  bool any_payload_stripe = false;
  for (uint32_t s = 0; s < n; s++) any_payload_stripe = any_payload_stripe || !meshes[sb[s].mesh].pl.binary;
  if (persist) {
    // task entries: room for the most tasks seen so far, twice over; a chunk whose tasks
    // do not fit walks them itself
    const uint64_t cap = std::max<uint64_t>(std::max<uint64_t>(2 * c->max_tasks, items), 4096);
    const size_t had = c->d_pmap.cap;
    unsigned long long* pmap = ensure<unsigned long long>(c->d_pmap, cap * 8);
    if (c->d_pmap.cap != had || !c->pmap_empty) {
      ck(cudaMemsetAsync(pmap, 0xff, c->d_pmap.cap, st), "memset task entries");
      c->pmap_empty = true;
    }
    pj.jobs = d_vj;
    pj.pyrs = d_pyr;
    pj.item_beg = d_beg;
    pj.n = n;
    pj.levels = p_levels;
    pj.chunk_beg = dp1(o_pc);
    pj.unit_beg = dp1(o_pu);
    pj.ept = kPersistEpt;
    pj.top_level = kTopPyramidLevel;
    pj.occ_left = reinterpret_cast<uint32_t*>(t1 + o_po);
    pj.pyr_left = reinterpret_cast<uint32_t*>(t1 + o_pp);
    pj.ctr = ensure<unsigned long long>(c->d_pctr, kPersistCtrWords * 8);
    pj.map = pmap;
    pj.cap = c->d_pmap.cap / 8;
    pj.scan_end = scan + blocks;
    pj.lines_per_lane = c->tuning.lines_per_lane;
    c->pmap_empty = false;  // until this launch is known to have ended without a timeout
  }
  c->leaf_zero = false;  // until the clean at the end of the sub-batch is queued
  run_launches(c, st, 0, [&] {
    if (persist) {
      PhaseScope ph(c, PH_VOX, st);
      ck(cudaMemsetAsync(task_off + items, 0, 8, st), "memset task_off");
      ck(cudaMemsetAsync(pj.ctr, 0, kPersistCtrWords * 8, st), "memset persistent counters");
      launch_b_persist(pj, c->num_sms, c->persist_per_sm, st);
      if (any_payload_stripe) {  // the winner pass numbers the tasks by item
        scan_u64_exclusive(task_off, items + 1, taskpart, st, true);
        if (map_cap) launch_b_task_map(dp1(o_cpi), n, cp_items[n], d_beg, task_off, items, task_map, map_cap, st);
      }
    } else {
      PhaseScope ph(c, PH_VOX, st);
      ck(cudaMemsetAsync(task_off + items, 0, 8, st), "memset task_off");
      if (pieces) {
        // each piece of the triangles as soon as its copy is done
        uint64_t beg = 0;
        for (const auto& pc : *pieces) {
          ck(cudaStreamWaitEvent(st, pc.second, 0), "wait piece");
          VoxJob jc = vj[0];
          jc.ibeg += beg;
          jc.n_items = pc.first - beg;
          jc.task_off += beg;
          if (jc.item_mask) jc.item_mask += beg;
          if (jc.item_box) jc.item_box += beg;
          launch_b_vox_small(nullptr, nullptr, 1, (jc.n_items + kChunk - 1) / kChunk, 0, &jc, st);
          beg = pc.first;
        }
      } else {
        launch_b_vox_small(d_vj, dp1(o_cpi), n, cp_items[n], 0, n == 1 ? &vj[0] : nullptr, st);
      }
      scan_u64_exclusive(task_off, items + 1, taskpart, st, true);
      if (map_cap) launch_b_task_map(dp1(o_cpi), n, cp_items[n], d_beg, task_off, items, task_map, map_cap, st);
      launch_b_vox_large(d_vj, d_beg, n, task_off, items, counter, 0, st, c->num_sms, (int)c->tuning.large_block,
                         (int)c->tuning.large_ctas_per_sm, c->tuning.lines_per_lane, task_map, map_cap);
    }
    {
      PhaseScope ph(c, PH_PYR, st);
      if (!persist) {
        for (size_t r = 0; r < cp_pyr.size(); r++)
          launch_b_pyramid(d_pyr, dp1(o_cpp[r]), n, cp_pyr[r].beg[n], cp_pyr[r].ept, (int)r,
                           n == 1 ? &pyr[0] : nullptr, st);
        launch_b_pyramid_top(d_pyr, n, kTopPyramidLevel, scan + blocks, st);
      }
      scan_u32_exclusive(scan, blocks + 1, scanpart, st);
      // the tasks of the sub-batch (sizes the task maps); the persistent kernel counts them itself
      const uint64_t* tasks = persist ? reinterpret_cast<const uint64_t*>(pj.ctr + kPersistTasksWord) : task_off + items;
      // The level counts go straight into pinned host memory, written by the kernel: a
      // copy on the copy engine would queue behind the previous sub-batch's copy back,
      // which the host keeps refilling while it waits, and hold up the whole pipeline.
      launch_b_level_bases(d_pyr, n, lvl_dev, tasks, reinterpret_cast<uint64_t*>(lvl_dev + (uint64_t)n * 16 + 8),
                           flag, persist ? reinterpret_cast<const uint64_t*>(pj.ctr + kPersistTimeoutWord) : nullptr,
                           reinterpret_cast<uint64_t*>(lvl_dev + (uint64_t)n * 16 + 12), st);
    }
  }, pieces != nullptr);  // waits on the upload stream are not captured
  wait_level_counts(st, idle);
  if (persist) {
    uint64_t code;
    std::memcpy(&code, lvl + (uint64_t)n * 16 + 12, 8);
    if (code != 0) fail(OOC_ERR_DEVICE, "persistent voxelization: a wait ran out (code " + std::to_string(code) + ")");
    c->pmap_empty = true;
  }
  uint64_t tasks_seen;
  std::memcpy(&tasks_seen, lvl + (uint64_t)n * 16 + 8, 8);
  c->max_tasks = std::max(c->max_tasks, tasks_seen);

  // ---- counts, placement in the files ----
  std::vector<Placed> pl(n);
  uint64_t total_nodes = 0, summed = 0;
  for (uint32_t s = 0; s < n; s++) {
    Pyramid& P = pyr[s];
    const uint32_t* o = lvl + (uint64_t)s * (kMaxLevels + 1);
    for (int l = 0; l <= P.depth; l++) {
      P.lv[l].koff = o[l];
      P.lv[l].n = (uint64_t)o[l + 1] - o[l];
    }
    const MeshWork& m = meshes[sb[s].mesh];
    Placed& q = pl[s];
    q.total = (uint64_t)o[P.depth + 1] - o[0];
    q.n_leaf = P.lv[P.depth].n;
    q.empty = q.n_leaf == 0;
    if (!q.empty) {
      q.node_span = q.total - 1;
      q.data_span = (m.pl.binary ? 0 : q.n_leaf) + (m.pl.levels ? q.total - q.n_leaf : 0);
    }
    total_nodes = std::max<uint64_t>(total_nodes, o[P.depth + 1]);
    summed += q.total;
  }
  // node indices are 32-bit within a sub-batch (the block scan is u32)
  if (summed != total_nodes) fail(OOC_ERR_LIMIT, "more than 2^32 nodes in one sub-batch; lower the batch budget");
  // the keys need only the phase-A tables: the GPU compacts while the host lays out the rest
  uint32_t* keys = ensure<uint32_t>(c->d_keys, total_nodes * 4);
  {
    PhaseScope ph(c, PH_PYR, st);
    launch_b_compact(d_pyr, dp1(o_cc), n, cp_compact.beg[n], cp_compact.ept, keys, n == 1 ? &pyr[0] : nullptr, st);
  }
  // the grouping above the stripes, run ahead on placeholders: where every stripe's records start
  for (uint32_t s = 0; s < n; s++) {
    MeshWork& m = meshes[sb[s].mesh];
    TopBuilder& tb = m.layout;
    tb.out = &m.dry;
    for (; m.layout_next < sb[s].stripe; m.layout_next++) tb.push(tb.top, TNode());
    m.layout_next++;
    pl[s].node_base = tb.node_pos;
    pl[s].data_base = tb.data_pos;
    if (pl[s].empty) {
      tb.push(tb.top, TNode());
    } else {
      tb.node_pos += pl[s].node_span;
      tb.data_pos += pl[s].data_span;
      TNode ph;
      ph.off = 0;  // any non-null node
      tb.push(tb.top, ph);
    }
  }
  // ---- per-node arrays and output windows ----
  bool any_levels = false, any_payload = false;
  for (auto& m : meshes) {
    any_levels = any_levels || m.pl.levels;
    any_payload = any_payload || !m.pl.binary;
  }
  uint32_t* size = ensure<uint32_t>(c->d_size, total_nodes * 4);
  uint32_t* dsize = ensure<uint32_t>(c->d_dsize, total_nodes * 4);
  uint32_t* first_child = ensure<uint32_t>(c->d_firstchild, total_nodes * 4);
  uint32_t* start = ensure<uint32_t>(c->d_start, total_nodes * 4);  // stripe-relative: a stripe spans < 2^32
  uint32_t* dstart = ensure<uint32_t>(c->d_dstart, total_nodes * 4);
  float* cache = any_levels ? ensure<float>(c->d_cache, total_nodes * 24) : nullptr;
  uint32_t* winners = any_payload ? ensure<uint32_t>(c->d_winners, total_nodes * 4) : nullptr;
  uint64_t out_nodes = 0, out_data = 0;
  if (os.mode == OUT_DEST) {
    // meshes whose last stripe is here get their destination; the others park
    // their records in the carry buffers until then
    for (uint32_t s = 0; s < n; s++) {
      MeshWork& m = meshes[sb[s].mesh];
      if ((int64_t)sb[s].stripe == m.last_stripe) alloc_through(c, st, meshes, sb[s].mesh, os);
    }
    uint64_t need_n = 0, need_d = 0;
    for (uint32_t s = 0; s < n; s++) {
      MeshWork& m = meshes[sb[s].mesh];
      if (m.dst_ready) continue;
      m.carried_nodes = std::max(m.carried_nodes, pl[s].node_base + pl[s].node_span);
      m.carried_data = std::max(m.carried_data, pl[s].data_base + pl[s].data_span);
      need_n = std::max(need_n, m.carried_nodes);
      need_d = std::max(need_d, m.carried_data);
    }
    if (need_n) ensure_keep<uint64_t>(c->d_nodes, need_n * 24, need_n * 24, st);
    if (need_d) ensure_keep<unsigned char>(c->d_data, need_d * 32, need_d * 32, st);
  } else if (os.mode == OUT_CTX) {
    uint64_t need_n = 0, need_d = 0;
    for (uint32_t s = 0; s < n; s++) {
      need_n = std::max(need_n, pl[s].node_base + pl[s].node_span);
      need_d = std::max(need_d, pl[s].data_base + pl[s].data_span);
    }
    ensure_keep<uint64_t>(c->d_nodes, need_n * 24, need_n * 24, st);
    ensure_keep<unsigned char>(c->d_data, need_d * 32, need_d * 32, st);
  } else {
    for (uint32_t s = 0; s < n; s++) {
      pl[s].out_node_off = out_nodes;
      pl[s].out_data_off = out_data;
      out_nodes += pl[s].node_span;
      out_data += pl[s].data_span;
    }
    ensure<uint64_t>(c->d_out_nodes[slot], out_nodes * 24);
    ensure<unsigned char>(c->d_out_data[slot], out_data * 32);
  }
  std::vector<EmitJob> ej(n);
  for (uint32_t s = 0; s < n; s++) {
    const MeshWork& m = meshes[sb[s].mesh];
    const Pyramid& P = pyr[s];
    const Placed& q = pl[s];
    EmitJob& e = ej[s];
    std::memset(&e, 0, sizeof(e));
    e.binary = m.pl.binary;
    e.levels = m.pl.levels;
    e.color_mode = m.prm->color_mode;
    e.gridsize = m.pl.N;
    e.stripe_base = sb[s].stripe * m.pl.S;
    for (int a = 0; a < 3; a++) e.origin[a] = vj[s].sa[a];
    e.tris = m.d_tris;
    e.stride = vj[s].stride;
    e.unit_div = m.pl.unit_div;
    e.keys = keys;
    e.size = size;
    e.dsize = dsize;
    e.first_child = first_child;
    e.start = start;
    e.dstart = dstart;
    e.cache = m.pl.levels ? cache : nullptr;
    e.leaf_inline = (!m.pl.binary && !m.pl.levels) ? 1 : 0;
    e.n_tris = m.resident;
    e.flag = flag;
    e.node_base = q.node_base;
    e.data_base = q.data_base;
    if (os.mode == OUT_DEST && m.dst_ready) {
      e.node_win = static_cast<uint64_t*>(m.dst_nodes);
      e.data_win = static_cast<unsigned char*>(m.dst_data);
      e.node_win_base = 0;
      e.data_win_base = 0;
      e.node_win_len = m.total_nodes;
      e.data_win_len = m.total_data;
    } else if (os.mode != OUT_HOST) {
      e.node_win = static_cast<uint64_t*>(c->d_nodes.p);
      e.data_win = static_cast<unsigned char*>(c->d_data.p);
      e.node_win_base = 0;
      e.data_win_base = 0;
      e.node_win_len = q.node_base + q.node_span;
      e.data_win_len = q.data_base + q.data_span;
    } else {
      e.node_win = static_cast<uint64_t*>(c->d_out_nodes[slot].p) + q.out_node_off * 3;
      e.data_win = static_cast<unsigned char*>(c->d_out_data[slot].p) + q.out_data_off * 32;
      e.node_win_base = q.node_base;
      e.data_win_base = q.data_base;
      e.node_win_len = q.node_span;
      e.data_win_len = q.data_span;
    }
    if (!m.pl.binary) {
      e.winners = winners + P.lv[P.depth].koff;
      vj[s].winners = winners + P.lv[P.depth].koff;
      vj[s].leafscan = scan + P.lv[P.depth].off_b;
      vj[s].leaflocal = P.local;
      vj[s].leafscan_base = (uint32_t)P.lv[P.depth].koff;
      vj[s].leafwoff = P.woff;
    }
    if (q.empty) continue;
    int ls = 0;
    while (ls + 1 <= P.depth - 1 && P.lv[ls + 1].n <= 256) ls++;
    e.l_small = ls;
  }
  auto live = [&](uint32_t s) { return !pl[s].empty; };
  const std::vector<uint64_t> cp_pay = cta_prefix(n, kChunk, [&](uint32_t s) -> uint64_t {
    return meshes[sb[s].mesh].pl.binary ? 0 : sb[s].n_items;
  });
  // leaf payloads: into the cache with -levels, else straight into the data file
  // (a depth-0 stripe's one voxel is written with its root)
  const Light cp_leafpay = light_prefix(c, n, [&](uint32_t s) -> uint64_t {
    const Plan& mp = meshes[sb[s].mesh].pl;
    if (!live(s) || mp.binary) return 0;
    return (mp.levels || pyr[s].depth >= 1) ? pl[s].n_leaf : 0;
  });
  // host output: without -levels the data file is final after the leaf payload pass,
  // so its copy back starts there, beside the node layout
  bool early_data = os.mode == OUT_HOST;
  for (uint32_t s = 0; s < n; s++) early_data = early_data && !meshes[sb[s].mesh].pl.levels;
  const Light cp_leaves = light_prefix(c, n, [&](uint32_t s) -> uint64_t {
    return (live(s) && pyr[s].depth >= 1) ? pl[s].n_leaf : 0;  // a depth-0 root is the leaf
  });
  const Light cp_clean = light_prefix(c, n, [&](uint32_t s) -> uint64_t { return touch_bytes(pyr[s].lv[pyr[s].depth]) / 16; });
  std::vector<Light> cp_bu(max_depth + 1), cp_td(max_depth + 1);
  for (int r = 1; r <= max_depth; r++)
    cp_bu[r] = light_prefix(c, n, [&](uint32_t s) -> uint64_t {
      const int l = pyr[s].depth - r;
      return (live(s) && l > ej[s].l_small && l >= 0) ? pyr[s].lv[l].n : 0;
    });
  for (int l = 0; l <= max_depth; l++)
    cp_td[l] = light_prefix(c, n, [&](uint32_t s) -> uint64_t {
      const int last_top = std::min(ej[s].l_small, pyr[s].depth - 2);
      return (live(s) && l > last_top && l <= pyr[s].depth - 2) ? pyr[s].lv[l + 1].n : 0;  // one thread per child
    });
  Uploader up2;
  const size_t o_vj2 = up2.add(vj.data(), n * sizeof(VoxJob));
  const size_t o_pyr2 = up2.add(pyr.data(), n * sizeof(Pyramid));
  const size_t o_ej = up2.add(ej.data(), n * sizeof(EmitJob));
  const size_t o_cpay = up2.add(cp_pay.data(), (n + 1) * 8);
  const size_t o_clp = up2.add(cp_leafpay.beg.data(), (n + 1) * 8);
  const size_t o_cl = up2.add(cp_leaves.beg.data(), (n + 1) * 8);
  const size_t o_cln = up2.add(cp_clean.beg.data(), (n + 1) * 8);
  std::vector<size_t> o_bu(cp_bu.size(), 0), o_td(cp_td.size(), 0);
  for (size_t r = 1; r < cp_bu.size(); r++) o_bu[r] = up2.add(cp_bu[r].beg.data(), (n + 1) * 8);
  for (size_t l = 0; l < cp_td.size(); l++) o_td[l] = up2.add(cp_td[l].beg.data(), (n + 1) * 8);
  unsigned char* t2 = up2.run(c, c->d_tables2, c->h_tables2, st);
  auto dp2 = [&](size_t off) { return reinterpret_cast<const uint64_t*>(t2 + off); };
  const VoxJob* d_vj2 = reinterpret_cast<const VoxJob*>(t2 + o_vj2);
  const Pyramid* d_pyr2 = reinterpret_cast<const Pyramid*>(t2 + o_pyr2);
  const EmitJob* d_ej = reinterpret_cast<const EmitJob*>(t2 + o_ej);
  const Pyramid* sp1 = n == 1 ? &pyr[0] : nullptr;  // one-stripe launches take the jobs as parameters
  const EmitJob* se1 = n == 1 ? &ej[0] : nullptr;

  uint32_t* hr = ensure_pinned<uint32_t>(c->h_root[slot], ((uint64_t)n * 16 + 1) * 4);
  uint32_t* hr_dev = nullptr;
  ck(cudaHostGetDevicePointer(reinterpret_cast<void**>(&hr_dev), hr, 0), "mapped root info");
  if (any_payload) run_launches(c, st, 1, [&] {
    {
      PhaseScope ph(c, PH_VOX, st);
      ck(cudaMemsetAsync(winners, 0xff, total_nodes * 4, st), "memset winners");
      launch_b_vox_small(d_vj2, dp2(o_cpay), n, cp_pay[n], 1, n == 1 ? &vj[0] : nullptr, st);
      if (tasks_seen)  // the count came back with the level counts
        launch_b_vox_large(d_vj2, d_beg, n, task_off, items, counter, 1, st, c->num_sms, (int)c->tuning.large_block,
                           (int)c->tuning.large_ctas_per_sm, c->tuning.lines_per_lane, task_map, map_cap);
      launch_b_leaf_payload(d_pyr2, d_ej, dp2(o_clp), n, cp_leafpay.beg[n], cp_leafpay.ept, sp1, se1, st);
    }
  });
  // recorded between the two launch sequences: an event recorded inside a captured
  // graph cannot be waited on from another stream
  if (early_data) ck(cudaEventRecord(c->ev_data[slot], st), "event");
  run_launches(c, st, 2, [&] {
    {
      PhaseScope ph(c, PH_TREE, st);
      for (size_t r = 1; r < cp_bu.size(); r++)
        launch_b_bottom_up(d_pyr2, d_ej, dp2(o_bu[r]), n, cp_bu[r].beg[n], cp_bu[r].ept, (int)r, sp1, se1, st);
      launch_b_bottom_up_top(d_pyr2, d_ej, n, st);
      launch_b_top_down_top(d_pyr2, d_ej, n, st);
      for (size_t l = 0; l < cp_td.size(); l++)
        launch_b_top_down(d_pyr2, d_ej, dp2(o_td[l]), n, cp_td[l].beg[n], cp_td[l].ept, (int)l, sp1, se1, st);
      launch_b_top_down_leaves(d_pyr2, d_ej, dp2(o_cl), n, cp_leaves.beg[n], cp_leaves.ept, sp1, se1, st);
      // into pinned host memory by the kernel, like the level counts: not behind the copy back
      launch_b_root_info(d_pyr2, d_ej, n, hr_dev, flag, st);
      // the last reader of the leaf levels is done: zero them for the next sub-batch
      launch_b_clean_leaves(d_pyr2, dp2(o_cln), n, cp_clean.beg[n], cp_clean.ept, sp1, st);
    }
  });
  c->leaf_zero = true;
  ck(cudaEventRecord(c->ev_compute[slot], st), "event");
  if (os.mode == OUT_HOST) {
    // The records travel to the host while the next sub-batch computes, on the slot's own
    // copy stream: the previous sub-batch's remaining chunks, refilled on the other slot's
    // stream, do not queue behind this one's wait for its compute.
    cudaStream_t cs = c->ring_stream[slot];
    if (early_data) {
      ck(cudaStreamWaitEvent(cs, c->ev_data[slot], 0), "wait");
      ring_start(c, c->ring[slot][OOC_STREAM_DATA], c->d_out_data[slot].p, out_data * 32, cs);
    }
    ck(cudaStreamWaitEvent(cs, c->ev_compute[slot], 0), "wait");
    ring_start(c, c->ring[slot][OOC_STREAM_NODES], c->d_out_nodes[slot].p, out_nodes * 24, cs);
    if (!early_data) ring_start(c, c->ring[slot][OOC_STREAM_DATA], c->d_out_data[slot].p, out_data * 32, cs);
  }
  out_pending.active = true;
  out_pending.slot = slot;
  out_pending.checked = false;
  out_pending.at = 0;
  out_pending.stage = 0;
  out_pending.cur = 0;
  out_pending.sb = sb;
  out_pending.pl = pl;
  out_pending.depth.resize(n);
  for (uint32_t s = 0; s < n; s++) out_pending.depth[s] = pyr[s].depth;
}

// Hand a sub-batch's stripes to their meshes, in file order.  With `block` it
// waits for every record; without, it stops (returning false) where the next
// record has not reached the host yet, and a later call resumes there.  Returns
// true once the whole sub-batch is handed over.
bool finish_sub_batch(ooc_ctx* c, std::vector<MeshWork>& meshes, Pending& pd, const OutSpec& os, bool block = true) {
  if (!pd.active) return true;
  const int slot = pd.slot;
  const uint32_t n = (uint32_t)pd.sb.size();
  if (!pd.checked) {
    if (block) {
      ck(cudaEventSynchronize(c->ev_compute[slot]), "sub-batch");
    } else {
      const cudaError_t e = cudaEventQuery(c->ev_compute[slot]);
      if (e == cudaErrorNotReady) return false;
      ck(e, "sub-batch");
    }
    ck(cudaGetLastError(), "sub-batch kernels");
    const uint32_t* hr = static_cast<const uint32_t*>(c->h_root[slot].p);
    if (hr[(uint64_t)n * 16] != 0)
      fail(OOC_ERR_DEVICE, "internal layout check failed (flag " + std::to_string(hr[(uint64_t)n * 16]) + ")");
    pd.checked = true;
    pd.at = 0;
    pd.stage = 0;
  }
  const uint32_t* hr = static_cast<const uint32_t*>(c->h_root[slot].p);
  for (; pd.at < n; pd.at++, pd.stage = 0) {
    const uint32_t s = pd.at;
    MeshWork& m = meshes[pd.sb[s].mesh];
    const Placed& q = pd.pl[s];
    if (pd.stage == 0) {
      for (; m.next_stripe < pd.sb[s].stripe; m.next_stripe++) m.top.push(m.top.top, TNode());
      m.next_stripe++;
      if (q.node_base != m.top.node_pos || q.data_base != m.top.data_pos)
        fail(OOC_ERR_DEVICE, "internal placement mismatch");
      if (q.empty) {
        m.top.push(m.top.top, TNode());
        continue;
      }
      m.filled += q.n_leaf;
      m.part_filled[pd.sb[s].part] += q.n_leaf;
      pd.stage = 1;
      pd.cur = q.out_node_off * 24;
    }
    if (os.mode == OUT_HOST) {
      if (pd.stage == 1) {
        const uint64_t end = (q.out_node_off + q.node_span) * 24;
        pd.cur = ring_take(c, c->ring[slot][OOC_STREAM_NODES], pd.cur, end, block,
                           [&](const void* p, uint64_t nb) { m.out->span(OOC_STREAM_NODES, p, nb); });
        if (pd.cur < end) return false;
        pd.stage = 2;
        pd.cur = q.out_data_off * 32;
      }
      const uint64_t end = (q.out_data_off + q.data_span) * 32;
      pd.cur = ring_take(c, c->ring[slot][OOC_STREAM_DATA], pd.cur, end, block,
                         [&](const void* p, uint64_t nb) { m.out->span(OOC_STREAM_DATA, p, nb); });
      if (pd.cur < end) return false;
    }
    m.top.node_pos += q.node_span;
    m.top.data_pos += q.data_span;
    const uint32_t* h_root = hr + (uint64_t)s * 16;
    TNode r;
    const uint32_t mask = h_root[0];
    float cf[6];
    std::memcpy(cf, h_root + 1, sizeof(cf));
    if (pd.depth[s] >= 1) {
      r.data = m.pl.levels ? q.data_base + q.data_span - 1 : 0;
      r.cb = q.node_base + q.total - 1 - (uint64_t)__builtin_popcount(mask);
      r.off = offsets_from_mask(mask);
      if (m.pl.levels) std::memcpy(r.cache, cf, sizeof(cf));
    } else {
      r.data = m.pl.binary ? 1 : q.data_base;
      r.cb = 0;
      r.off = ~0ull;
      if (!m.pl.binary) std::memcpy(r.cache, cf, sizeof(cf));
    }
    m.top.push(m.top.top, r);
  }
  pd.active = false;
  return true;
}

// Binning of a P > 1 mesh into per-partition item lists (K1).
void bin_mesh(ooc_ctx* c, cudaStream_t st, MeshWork& m, DevBuf& items_buf) {
  const Plan& pl = m.pl;
  const int stride = pl.binary ? 9 : 21;
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
  launch_part_count(m.d_tris, stride, m.n_tris, d_axis, d_axis + 3 * PA, pl.kP, pl.P, hist, st);
  const uint32_t* h = read_back_words(c, hist, pl.P, st);
  ck(cudaStreamSynchronize(st), "binning");
  m.part_off.assign(pl.P + 1, 0);
  uint64_t acc = 0;
  for (uint64_t i = 0; i < pl.P; i++) {
    m.part_off[i] = (uint32_t)acc;
    acc += h[i];
    if (acc >= (1ull << 32)) fail(OOC_ERR_INVALID, "more than 2^32 (triangle, partition) pairs");
  }
  m.part_off[pl.P] = (uint32_t)acc;
  m.n_items = acc;
  uint32_t* items = ensure<uint32_t>(items_buf, acc * 4);
  ck(cudaMemcpyAsync(hist, m.part_off.data(), pl.P * 4, cudaMemcpyHostToDevice, st), "cursors");
  ck(cudaStreamSynchronize(st), "cursors");  // part_off is reused on the host
  launch_part_emit(m.d_tris, stride, m.n_tris, d_axis, d_axis + 3 * PA, pl.kP, pl.P, hist, items, st);
  m.items = items;
}

// ---------------------------------------------------------------------------
// Out-of-core builds.  A mesh whose triangle records do not fit the device
// triangle budget is read in chunks: a first pass counts every partition's
// records (K1's box test), the partitions are cut into consecutive groups
// whose records fit half the budget, and before a group's stripes run, a pass
// over the source gathers that group's records into one of two device buffers,
// each partition's records contiguous and in stream order.  The sub-batches of
// a group read them there; the other buffer holds the previous group until its
// sub-batches are done (stream order on `st`).
// ---------------------------------------------------------------------------
constexpr uint64_t kStreamChunkBytes = 256ull << 20;  // one chunk of the source on the device
constexpr uint64_t kStreamMatMax = 1ull << 24;        // count-matrix entries of one chunk

uint64_t stream_budget(ooc_ctx* c) {
  if (c->stream_budget) return c->stream_budget;
  size_t free_b = 0, total_b = 0;
  ck(cudaMemGetInfo(&free_b, &total_b), "cudaMemGetInfo");
  return free_b / 2;
}

// Whether a one-mesh build of `bytes` of triangle records over P partitions streams.
bool wants_stream(ooc_ctx* c, uint64_t bytes, uint64_t P) { return P > 1 && bytes > stream_budget(c); }

// One pass over the source, chunk by chunk: each chunk is copied into one of two
// device buffers on `st` (a file through two pinned staging buffers) and handed
// to use(device chunk, records).
template <typename F>
void stream_pass(ooc_ctx* c, cudaStream_t st, StreamSource& src, uint64_t chunk, F&& use) {
  c->stream_passes++;
  const uint64_t max_bytes = std::max<uint64_t>(1, std::min(chunk, src.n_tris)) * src.rec;
  char* dev[2] = {ensure<char>(c->d_chunk[0], max_bytes), ensure<char>(c->d_chunk[1], max_bytes)};
  char* pin[2] = {nullptr, nullptr};
  if (!src.path.empty()) {
    if (!src.f) src.f = std::fopen(src.path.c_str(), "rb");
    if (!src.f) fail(OOC_ERR_IO, "cannot open " + src.path);
    std::rewind(src.f);
    for (int b = 0; b < 2; b++) {
      pin[b] = ensure_pinned<char>(c->h_stage[b], max_bytes);
      if (!c->ev_stage[b]) ck(cudaEventCreateWithFlags(&c->ev_stage[b], cudaEventDisableTiming), "cudaEventCreate");
    }
  }
  uint64_t i = 0;
  for (uint64_t t0 = 0; t0 < src.n_tris; t0 += chunk, i++) {
    const uint64_t n = std::min(chunk, src.n_tris - t0);
    const int b = (int)(i & 1);
    if (src.f) {
      ck(cudaEventSynchronize(c->ev_stage[b]), "staging");  // the buffer's last upload is done
      if (std::fread(pin[b], (size_t)src.rec, (size_t)n, src.f) != n) fail(OOC_ERR_IO, "short read of " + src.path);
      ck(cudaMemcpyAsync(dev[b], pin[b], n * src.rec, cudaMemcpyHostToDevice, st), "H2D");
      ck(cudaEventRecord(c->ev_stage[b], st), "event");
    } else {
      ck(cudaMemcpyAsync(dev[b], src.host + t0 * src.rec, n * src.rec, cudaMemcpyHostToDevice, st), "H2D");
    }
    use(reinterpret_cast<const float*>(dev[b]), n);
  }
}

// The partitions' world slabs along each axis (createBuffers, partitioner.cpp:56-61).
float* upload_axis_boxes(ooc_ctx* c, cudaStream_t st, const Plan& pl) {
  const int PA = 1 << pl.kP;
  const uint64_t side = pl.N / PA;
  std::vector<float> axis(6 * PA);
  for (int a = 0; a < 3; a++)
    for (int jj = 0; jj < PA; jj++) {
      axis[a * PA + jj] = (float)(uint32_t)(jj * side) * pl.u;
      axis[3 * PA + a * PA + jj] = (float)(uint32_t)((jj + 1) * side) * pl.u;
    }
  float* d_axis = ensure<float>(c->d_axis, axis.size() * 4);
  ck(cudaMemcpyAsync(d_axis, axis.data(), axis.size() * 4, cudaMemcpyHostToDevice, st), "axis boxes");
  ck(cudaStreamSynchronize(st), "axis boxes");  // `axis` is a local
  return d_axis;
}

// First pass: records per partition (the reference's part_tricounts) and the groups.
void stream_count(ooc_ctx* c, cudaStream_t st, MeshWork& m) {
  const Plan& pl = m.pl;
  PhaseScope ph(c, PH_BIN, st);
  const int PA = 1 << pl.kP;
  const float* d_axis = upload_axis_boxes(c, st, pl);
  uint32_t* hist = ensure<uint32_t>(c->d_hist, pl.P * 4);
  ck(cudaMemsetAsync(hist, 0, pl.P * 4, st), "memset hist");
  const int stride = pl.binary ? 9 : 21;
  stream_pass(c, st, *m.src, std::max<uint64_t>(1, kStreamChunkBytes / m.src->rec), [&](const float* d, uint64_t n) {
    launch_part_count(d, stride, n, d_axis, d_axis + 3 * PA, pl.kP, pl.P, hist, st);
  });
  const uint32_t* h = read_back_words(c, hist, pl.P, st);
  ck(cudaStreamSynchronize(st), "counts");
  m.part_off.assign(pl.P + 1, 0);
  uint64_t acc = 0;
  for (uint64_t i = 0; i < pl.P; i++) {
    m.part_off[i] = (uint32_t)acc;
    acc += h[i];
    if (acc >= (1ull << 32)) fail(OOC_ERR_INVALID, "more than 2^32 (triangle, partition) pairs");
  }
  m.part_off[pl.P] = (uint32_t)acc;
  m.n_items = acc;
  uint32_t* d_off = ensure<uint32_t>(c->d_part_off, (pl.P + 1) * 4);
  ck(cudaMemcpyAsync(d_off, m.part_off.data(), (pl.P + 1) * 4, cudaMemcpyHostToDevice, st), "partition offsets");
  ck(cudaStreamSynchronize(st), "partition offsets");
  m.d_part_off = d_off;
  m.d_axis = d_axis;
  // consecutive partitions whose records fit half the budget (the other half holds the previous group)
  const uint64_t half = stream_budget(c) / 2;
  m.groups.clear();
  uint64_t p0 = 0, bytes = 0;
  for (uint64_t p = 0; p < pl.P; p++) {
    const uint64_t b = (uint64_t)h[p] * m.src->rec;
    if (b > half)
      fail(OOC_ERR_LIMIT, "partition " + std::to_string(p) + " holds " + std::to_string(b) +
                              " bytes of triangles, more than half the device triangle budget");
    if (p > p0 && (bytes + b > half || p - p0 == kStreamMaxGroup)) {
      m.groups.push_back({p0, p});
      p0 = p;
      bytes = 0;
    }
    bytes += b;
  }
  m.groups.push_back({p0, pl.P});
  m.next_group = 0;
  m.group_end = 0;
}

// A later pass: the records of the group holding partition `part`, gathered into a device buffer.
void stream_group(ooc_ctx* c, cudaStream_t st, MeshWork& m, uint64_t part) {
  while (m.next_group < m.groups.size() && m.groups[m.next_group].second <= part) m.next_group++;
  if (m.next_group == m.groups.size()) fail(OOC_ERR_DEVICE, "internal: partition outside every group");
  const size_t g = m.next_group++;
  const uint64_t p0 = m.groups[g].first, p1 = m.groups[g].second;
  const uint32_t gp = (uint32_t)(p1 - p0);
  const Plan& pl = m.pl;
  PhaseScope ph(c, PH_BIN, st);
  const int PA = 1 << pl.kP;
  const int stride = pl.binary ? 9 : 21;
  const float* d_axis = m.d_axis;
  const uint64_t records = (uint64_t)m.part_off[p1] - m.part_off[p0];
  float* out = ensure<float>(c->d_group[g & 1], std::max<uint64_t>(records, 1) * m.src->rec);
  uint64_t* d_base = ensure<uint64_t>(c->d_stream_base, (uint64_t)gp * 8);
  launch_stream_bases(m.d_part_off, (uint32_t)p0, gp, d_base, st);
  const uint64_t chunk = std::max<uint64_t>(
      kStreamCtaTris, std::min(kStreamChunkBytes / m.src->rec, kStreamMatMax / gp * kStreamCtaTris));
  const uint64_t mat_n = (uint64_t)gp * stream_ctas(chunk) + 1;
  uint32_t* mat = ensure<uint32_t>(c->d_stream_mat, mat_n * 4);
  uint32_t* mat_part = ensure<uint32_t>(c->d_stream_part, scan_partials_needed(mat_n) * 4);
  stream_pass(c, st, *m.src, chunk, [&](const float* d, uint64_t n) {
    launch_stream_group_chunk(d, stride, n, d_axis, d_axis + 3 * PA, pl.kP, (uint32_t)p0, gp, mat, mat_part, d_base,
                              out, st);
  });
  m.d_tris = out;
  m.items = nullptr;
  m.group_first_item = m.part_off[p0];
  m.group_end = p1;
  m.resident = records;
}

// Last records of a mesh whose stripes are all done: empty stripes after the
// last one with items, then the root, written last (finalizeTree,
// OctreeBuilder.cpp:34-55).
void finalize_mesh(MeshWork& m) {
  for (; m.next_stripe < m.pl.n_stripes; m.next_stripe++) m.top.push(m.top.top, TNode());
  m.out->node(m.top.node_pos++, m.top.buf[0][0]);
}

// Whole path for a list of meshes (triangles already on the device).  Meshes
// complete in order, each as soon as the sub-batch holding its last stripe is
// finished; `on_done(list)` runs right after the last records of the meshes
// that have just completed.
void build_meshes(ooc_ctx* c, cudaStream_t st, std::vector<MeshWork>& meshes, const OutSpec& os,
                  const std::function<void(const std::vector<size_t>&)>& on_done = nullptr) {
  if (c->d_mesh_items.size() < meshes.size()) c->d_mesh_items.resize(meshes.size());
  for (size_t i = 0; i < meshes.size(); i++) {
    MeshWork& m = meshes[i];
    if (!m.src) m.resident = m.n_tris;
    if (m.pl.P > 1 && m.src) {
      stream_count(c, st, m);
    } else if (m.pl.P > 1) {
      if (m.uploaded) ck(cudaStreamWaitEvent(st, m.uploaded, 0), "wait upload");
      bin_mesh(c, st, m, c->d_mesh_items[i]);
    } else {
      m.n_items = m.n_tris;
    }
    // data file header records (OctreeBuilder.cpp:22-28)
    float zero[6] = {0, 0, 0, 0, 0, 0};
    m.out->data(m.top.data_pos++, 0, zero);
    if (m.pl.binary) {
      float white[6] = {1, 1, 1, 0, 0, 0};
      m.out->data(m.top.data_pos++, 0, white);
    }
    m.layout.data_pos = m.top.data_pos;
  }
  // stripes with items, in mesh order and Morton order, split by the pyramid budget
  std::vector<StripeRef> sb;
  uint64_t budget_words = 0;
  const uint64_t budget = c->tuning.batch_budget / 4;
  auto items_of = [&](const MeshWork& m, uint64_t s) -> uint64_t {
    const uint64_t part = s / m.pl.stripes_per_part;
    return m.pl.P > 1 ? (uint64_t)m.part_off[part + 1] - m.part_off[part] : m.n_tris;
  };
  for (MeshWork& m : meshes)
    for (int64_t s = (int64_t)m.pl.n_stripes - 1; s >= 0 && m.last_stripe < 0; s--)
      if (items_of(m, (uint64_t)s)) m.last_stripe = s;
  size_t n_done = 0;
  std::vector<size_t> just_done;
  auto complete = [&]() {
    just_done.clear();
    while (n_done < meshes.size() && (int64_t)meshes[n_done].next_stripe > meshes[n_done].last_stripe) {
      finalize_mesh(meshes[n_done]);
      just_done.push_back(n_done);
      n_done++;
    }
    if (on_done && !just_done.empty()) on_done(just_done);
  };
  complete();
  Pending pend[2];
  int k = 0;
  // launch sub-batch k, then finish k-1 while k computes
  auto flush = [&]() {
    // uploads arrive in mesh order: the sub-batch's last mesh being there covers the others
    // (a lone stripe of a mesh uploaded in pieces waits for each piece instead)
    const MeshWork& last = meshes[sb.back().mesh];
    if (last.uploaded && !(sb.size() == 1 && !last.pieces.empty()))
      ck(cudaStreamWaitEvent(st, last.uploaded, 0), "wait upload");
    // host output: while this sub-batch's level counts are pending, the previous
    // one's landed records go to the sink, so its copy back keeps the link busy
    Pending& prev = pend[(k + 1) & 1];
    std::function<bool()> pump;
    if (os.mode == OUT_HOST && prev.active)
      pump = [&]() { return !finish_sub_batch(c, meshes, prev, os, false); };
    run_sub_batch(c, st, meshes, sb, os, pend[k & 1], k & 1, pump);
    if (os.mode == OUT_CTX) finish_sub_batch(c, meshes, pend[k & 1], os);
    else finish_sub_batch(c, meshes, pend[(k + 1) & 1], os);
    complete();
    k++;
    sb.clear();
    budget_words = 0;
  };
  for (uint32_t mi = 0; mi < meshes.size(); mi++) {
    MeshWork& m = meshes[mi];
    for (uint64_t s = 0; s < m.pl.n_stripes; s++) {
      const uint64_t part = s / m.pl.stripes_per_part;
      const uint64_t cnt = items_of(m, s);
      if (cnt == 0) continue;  // main.cpp:330: partitions without triangles are skipped
      if (m.src && part >= m.group_end) {
        // out of core: the launched sub-batches read the previous group; gather the next
        if (!sb.empty()) flush();
        stream_group(c, st, m, part);
      }
      const uint64_t ibeg = m.pl.P > 1 ? m.part_off[part] - m.group_first_item : 0;
      Level tmp[kMaxLevels];
      uint64_t w = 0, b = 0;
      pyramid_levels(m.pl.Ds, tmp, w, w, b, false);
      // host output: the first sub-batch takes an eighth of the budget, so that the copy
      // back (the longer part of a large build) starts after a short first compute
      const uint64_t cap = (os.mode == OUT_HOST && k == 0) ? budget / 8 : budget;
      if (!sb.empty() && budget_words + w > cap) flush();
      sb.push_back(StripeRef{mi, s, part, ibeg, cnt});
      budget_words += w;
    }
  }
  if (!sb.empty()) flush();
  finish_sub_batch(c, meshes, pend[k & 1], os);  // the older of the two first
  finish_sub_batch(c, meshes, pend[(k + 1) & 1], os);
  complete();
  if (n_done != meshes.size()) fail(OOC_ERR_DEVICE, "internal: mesh left unfinished");
  // per-partition counts of the first mesh (the progress lines of the drop-in CLIs)
  const MeshWork& m0 = meshes[0];
  c->part_tris.assign(m0.pl.P, 0);
  for (uint64_t p = 0; p < m0.pl.P; p++)
    c->part_tris[p] = m0.pl.P > 1 ? (uint64_t)m0.part_off[p + 1] - m0.part_off[p] : m0.n_tris;
  c->part_filled = m0.part_filled;
}

void fill_info(const MeshWork& m, ooc_build_info* info) {
  if (!info) return;
  info->n_nodes = m.top.node_pos;
  info->n_data = m.top.data_pos;
  info->n_filled = m.filled;
  info->n_partitions = m.pl.P;
  info->n_stripes = m.pl.n_stripes;
  info->n_items = m.n_items;
}

// Device mode: scatter the host-written records (top levels, header records) into the device files.
void finish_device_output(ooc_ctx* c, cudaStream_t st, MeshWork& m, Emitter& out) {
  uint64_t* nodes = ensure_keep<uint64_t>(c->d_nodes, m.top.node_pos * 24, m.top.node_pos * 24, st);
  unsigned char* data = ensure_keep<unsigned char>(c->d_data, m.top.data_pos * 32, m.top.data_pos * 32, st);
  const uint64_t nr = out.node_recs.size() / 4, dr = out.data_recs.size() / 5;
  const size_t bytes = (out.node_recs.size() + out.data_recs.size()) * 8;
  uint64_t* h = ensure_pinned<uint64_t>(c->h_recs, bytes);
  std::memcpy(h, out.node_recs.data(), out.node_recs.size() * 8);
  std::memcpy(h + out.node_recs.size(), out.data_recs.data(), out.data_recs.size() * 8);
  uint64_t* d = ensure<uint64_t>(c->d_recs, bytes);
  ck(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, st), "records");
  launch_scatter_records(d, nr, 3, nodes, st);
  launch_scatter_records(d + out.node_recs.size(), dr, 4, reinterpret_cast<uint64_t*>(data), st);
  c->res_nodes = m.top.node_pos;
  c->res_data = m.top.data_pos;
  c->res_valid = true;
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
  c->stream_passes = 0;
  c->part_tris.clear();
  c->part_filled.clear();
  // a build that failed part-way may have left copies queued into the staging buffers
  ck(cudaStreamSynchronize(c->copy_stream), "cudaStreamSynchronize");
  ck(cudaStreamSynchronize(c->ring_stream[0]), "cudaStreamSynchronize");
  ck(cudaStreamSynchronize(c->ring_stream[1]), "cudaStreamSynchronize");
  ck(cudaStreamSynchronize(c->h2d_stream), "cudaStreamSynchronize");
  c->err.clear();
  c->marks.clear();
  c->kmarks.clear();
  c->ev_used = 0;
  c->res_valid = false;
  c->lstate.launches = 0;
  c->lstate.pdl = c->tuning.pdl != 0;
  if (c->kfilter.empty()) {
    c->lstate.hooks = KernelHooks();
  } else {
    c->lstate.hooks.user = c;
    c->lstate.hooks.begin = kernel_begin;
    c->lstate.hooks.end = kernel_end;
  }
}

// Runs one API call on `c`: its launches report to c's own launch state.
template <typename F>
int guarded(ooc_ctx* c, F&& f) {
  if (!c) return OOC_ERR_INVALID;
  LaunchScope scope(&c->lstate);
  try {
    f();
    c->launches = c->lstate.launches;
    return OOC_OK;
  } catch (const OocError& e) {
    c->err = e.msg;
    c->launches = c->lstate.launches;
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

namespace ooc {
void set_ctx_error(ooc_ctx* c, const std::string& msg) {
  if (c) c->err = msg;
}
void set_ctx_file_times(ooc_ctx* c, float read_ms, float write_ms) {
  if (!c) return;
  c->file_ms[0] = read_ms;
  c->file_ms[1] = write_ms;
}
}  // namespace ooc

namespace {
struct SingleSink {
  ooc_sink_fn sink;
  void* user;
};
int single_sink(void* user, uint64_t, int32_t kind, const void* bytes, uint64_t n) {
  SingleSink* s = static_cast<SingleSink*>(user);
  return kind == OOC_STREAM_END ? 0 : s->sink(s->user, kind, bytes, n);
}
}  // namespace

namespace ooc {
bool file_wants_stream(ooc_ctx* c, const ooc_build_params* prm, uint64_t n_tris) {
  if (!c || !prm) return false;
  try {
    return wants_stream(c, n_tris * (prm->geometry_only ? 36 : 84),
                        ooc_estimate_partitions(prm->gridsize, prm->memory_limit_mb));
  } catch (...) {
    return false;
  }
}

int build_from_file_stream(ooc_ctx* c, const ooc_build_params* prm, const char* tridata, uint64_t n_tris,
                           ooc_sink_fn sink, void* user, ooc_build_info* info) {
  return guarded(c, [&] {
    begin_build(c);
    check_params(prm, n_tris);
    if (!sink) fail(OOC_ERR_INVALID, "sink is NULL");
    cudaStream_t st = c->own_stream;
    SingleSink ss{sink, user};
    Emitter out;
    out.sink = single_sink;
    out.user = &ss;
    StreamSource src;
    src.path = tridata;
    src.n_tris = n_tris;
    src.rec = prm->geometry_only ? 36 : 84;
    std::vector<MeshWork> meshes;
    meshes.emplace_back(make_plan(prm), &out);
    meshes[0].prm = prm;
    meshes[0].n_tris = n_tris;
    meshes[0].src = &src;
    {
      PhaseScope all(c, PH_ALL, st);
      OutSpec os;
      os.mode = OUT_HOST;
      build_meshes(c, st, meshes, os);
    }
    ck(cudaStreamSynchronize(st), "build");
    ck(cudaGetLastError(), "build kernels");
    fill_info(meshes[0], info);
    finish_timing(c);
  });
}
}  // namespace ooc

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
      cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->ring_stream[0], cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->ring_stream[1], cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->h2d_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_compute[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_compute[1], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_data[0], cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&c->ev_data[1], cudaEventDisableTiming) != cudaSuccess) {
    ooc_ctx_destroy(c);  // frees whatever was created
    return OOC_ERR_DEVICE;
  }
  *out = c;
  return OOC_OK;
}

void ooc_ctx_destroy(ooc_ctx* c) {
  if (!c) return;
  cudaSetDevice(c->device);
  if (c->own_stream) cudaStreamSynchronize(c->own_stream);
  if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
  for (cudaStream_t rs : c->ring_stream)
    if (rs) cudaStreamSynchronize(rs);
  if (c->h2d_stream) cudaStreamSynchronize(c->h2d_stream);
  DevBuf* bufs[] = {&c->d_tris, &c->d_hist, &c->d_axis, &c->d_bits, &c->d_scan, &c->d_scanpart,
                    &c->d_keys, &c->d_size, &c->d_dsize, &c->d_start, &c->d_dstart, &c->d_cache, &c->d_winners,
                    &c->d_taskoff, &c->d_taskpart, &c->d_counter, &c->d_nodes, &c->d_data, &c->d_recs,
                    &c->d_rootinfo, &c->d_itemmask, &c->d_firstchild, &c->d_itembox, &c->d_leaf, &c->d_touch, &c->d_local,
                    &c->d_taskmap, &c->d_woff, &c->d_pctr, &c->d_pmap, &c->d_chunk[0], &c->d_chunk[1], &c->d_group[0],
                    &c->d_group[1], &c->d_stream_mat, &c->d_stream_part, &c->d_stream_base, &c->d_part_off};
  for (DevBuf* b : bufs)
    if (b->p) cudaFree(b->p);
  PinBuf* pins[] = {&c->h_misc, &c->h_recs, &c->h_tables1, &c->h_tables2, &c->h_words, &c->h_stage[0],
                    &c->h_stage[1]};
  for (PinBuf* b : pins)
    if (b->p) cudaFreeHost(b->p);
  for (cudaEvent_t e : c->ev_stage)
    if (e) cudaEventDestroy(e);
  for (int i = 0; i < 2; i++) {
    if (c->d_out_nodes[i].p) cudaFree(c->d_out_nodes[i].p);
    if (c->d_out_data[i].p) cudaFree(c->d_out_data[i].p);
    for (D2HRing& r : c->ring[i]) {
      if (r.buf.p) cudaFreeHost(r.buf.p);
      for (cudaEvent_t e : r.ev)
        if (e) cudaEventDestroy(e);
    }
    if (c->h_root[i].p) cudaFreeHost(c->h_root[i].p);
    if (c->ev_compute[i]) cudaEventDestroy(c->ev_compute[i]);
    if (c->ev_data[i]) cudaEventDestroy(c->ev_data[i]);
  }
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  for (cudaStream_t rs : c->ring_stream)
    if (rs) cudaStreamDestroy(rs);
  if (c->h2d_stream) cudaStreamDestroy(c->h2d_stream);
  for (auto& kv : c->graph_execs) cudaGraphExecDestroy(kv.second);
  for (cudaEvent_t e : c->up_events) cudaEventDestroy(e);
  if (c->d_tables1.p) cudaFree(c->d_tables1.p);
  if (c->d_tables2.p) cudaFree(c->d_tables2.p);
  for (DevBuf& b : c->d_mesh_items)
    if (b.p) cudaFree(b.p);
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
  if (!sink) {
    if (c) c->err = "sink is NULL";
    return OOC_ERR_INVALID;
  }
  ooc_mesh m;
  std::memset(&m, 0, sizeof(m));
  if (prm) m.params = *prm;
  m.tris = tris_host;
  m.n_tris = n_tris;
  SingleSink ss{sink, user};
  if (!prm) {
    if (c) c->err = "params is NULL";
    return OOC_ERR_INVALID;
  }
  return ooc_build_batch(c, &m, 1, single_sink, &ss, info);
}

namespace {
// The meshes of a batch call, their triangles in one device buffer (256-byte
// aligned slices); the H2D copies are queued on `st` by upload().
struct BatchInput {
  std::vector<uint64_t> off;
  std::vector<Emitter> outs;
  std::vector<MeshWork> meshes;
  unsigned char* d_all = nullptr;
  StreamSource src;  // a one-mesh call whose triangles exceed the device triangle budget

  BatchInput(ooc_ctx* c, const ooc_mesh* in, uint64_t n, bool device_records) : off(n + 1, 0), outs(n) {
    if (n && !in) fail(OOC_ERR_INVALID, "meshes are NULL");
    for (uint64_t i = 0; i < n; i++) {
      check_params(&in[i].params, in[i].n_tris);
      if (in[i].n_tris && !in[i].tris) fail(OOC_ERR_INVALID, "triangles are NULL");
      off[i + 1] = off[i] + (bytes(in[i]) + 255) / 256 * 256;
    }
    const bool streamed = n == 1 && wants_stream(c, bytes(in[0]), ooc_estimate_partitions(
                                                                       in[0].params.gridsize, in[0].params.memory_limit_mb));
    if (streamed) {
      src.host = static_cast<const char*>(static_cast<const void*>(in[0].tris));
      src.n_tris = in[0].n_tris;
      src.rec = in[0].params.geometry_only ? 36 : 84;
      std::fill(off.begin(), off.end(), 0);
    }
    d_all = ensure<unsigned char>(c->d_tris, off[n]);
    meshes.reserve(n);
    for (uint64_t i = 0; i < n; i++) {
      outs[i].device = device_records;
      outs[i].mesh = i;
      meshes.emplace_back(make_plan(&in[i].params), &outs[i]);
      meshes.back().prm = &in[i].params;
      meshes.back().d_tris = reinterpret_cast<const float*>(d_all + off[i]);
      meshes.back().n_tris = in[i].n_tris;
      meshes.back().index = i;
      if (streamed) {
        meshes.back().src = &src;
        meshes.back().d_tris = nullptr;
      }
    }
  }
  static uint64_t bytes(const ooc_mesh& m) { return m.n_tris * (m.params.geometry_only ? 9 : 21) * 4; }
  // Queue the uploads on the context's upload stream, with an event after
  // every group of about 16 MB, so each sub-batch waits only for its meshes.
  // A one-partition mesh of more than two groups goes up in pieces of about
  // 16 MB, each with its event, and its voxelization follows piece by piece.
  void upload(ooc_ctx* c, const ooc_mesh* in, cudaStream_t st) {
    ck(cudaEventRecord(c->ev_compute[0], st), "event");  // the device buffer is free once earlier work on st is done
    ck(cudaStreamWaitEvent(c->h2d_stream, c->ev_compute[0], 0), "wait");
    PhaseScope ph(c, PH_COPY, c->h2d_stream);
    constexpr uint64_t kGroup = 16ull << 20;
    size_t used = 0, group = 0;
    uint64_t acc = 0;
    auto event = [&]() {
      if (used == c->up_events.size()) {
        cudaEvent_t e;
        ck(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "cudaEventCreate");
        c->up_events.push_back(e);
      }
      cudaEvent_t e = c->up_events[used++];
      ck(cudaEventRecord(e, c->h2d_stream), "event");
      return e;
    };
    for (size_t i = 0; i < meshes.size(); i++) {
      const uint64_t nb = bytes(in[i]);
      MeshWork& m = meshes[i];
      m.pieces.clear();
      if (m.src) continue;  // out of core: read group by group during the build
      if (m.pl.P == 1 && nb > 2 * kGroup) {
        const uint64_t rec = nb / in[i].n_tris, per = kGroup / rec;  // triangles per piece
        for (uint64_t t0 = 0; t0 < in[i].n_tris; t0 += per) {
          const uint64_t t1 = std::min<uint64_t>(in[i].n_tris, t0 + per);
          ck(cudaMemcpyAsync(d_all + off[i] + t0 * rec, reinterpret_cast<const char*>(in[i].tris) + t0 * rec,
                             (t1 - t0) * rec, cudaMemcpyHostToDevice, c->h2d_stream), "H2D");
          m.pieces.emplace_back(t1, event());
        }
        for (; group <= i; group++) meshes[group].uploaded = m.pieces.back().second;
        acc = 0;
        continue;
      }
      if (nb) ck(cudaMemcpyAsync(d_all + off[i], in[i].tris, nb, cudaMemcpyHostToDevice, c->h2d_stream), "H2D");
      acc += nb;
      if (acc >= kGroup || i + 1 == meshes.size()) {
        const cudaEvent_t e = event();
        for (; group <= i; group++) meshes[group].uploaded = e;
        acc = 0;
      }
    }
  }
};
}  // namespace

int ooc_build_batch(ooc_ctx* c, const ooc_mesh* meshes_in, uint64_t n_meshes, ooc_batch_sink_fn sink, void* user,
                    ooc_build_info* infos) {
  return guarded(c, [&] {
    begin_build(c);
    if (!sink) fail(OOC_ERR_INVALID, "sink is NULL");
    cudaStream_t st = c->own_stream;
    BatchInput b(c, meshes_in, n_meshes, false);
    for (Emitter& e : b.outs) {
      e.sink = sink;
      e.user = user;
    }
    {
      PhaseScope all(c, PH_ALL, st);
      b.upload(c, meshes_in, st);
      OutSpec os;
      os.mode = OUT_HOST;
      build_meshes(c, st, b.meshes, os, [&](const std::vector<size_t>& done) {
        for (size_t i : done) {
          if (infos) fill_info(b.meshes[i], &infos[i]);
          if (sink(user, i, OOC_STREAM_END, nullptr, 0) != 0) fail(OOC_ERR_SINK, "sink returned an error");
        }
      });
    }
    ck(cudaStreamSynchronize(st), "build");
    finish_timing(c);
  });
}

int ooc_build_batch_device(ooc_ctx* c, const ooc_mesh* meshes_in, uint64_t n_meshes, ooc_alloc_fn alloc,
                           ooc_ready_fn ready, void* user, ooc_build_info* infos) {
  return guarded(c, [&] {
    begin_build(c);
    if (!alloc) fail(OOC_ERR_INVALID, "alloc is NULL");
    cudaStream_t st = c->own_stream;
    BatchInput b(c, meshes_in, n_meshes, true);
    OutSpec os;
    os.mode = OUT_DEST;
    os.alloc = alloc;
    os.ready = ready;
    os.user = user;
    {
      PhaseScope all(c, PH_ALL, st);
      b.upload(c, meshes_in, st);
      // records written on the host (levels above the stripes, header records,
      // the root) land in the destinations by one scatter per group of meshes
      build_meshes(c, st, b.meshes, os, [&](const std::vector<size_t>& done) {
        std::vector<uint64_t> nrec, drec;
        for (size_t i : done) {
          MeshWork& m = b.meshes[i];
          alloc_through(c, c->copy_stream, b.meshes, i, os);  // a mesh without items gets its destination here
          if (m.top.node_pos != m.total_nodes || m.top.data_pos != m.total_data)
            fail(OOC_ERR_DEVICE, "internal size mismatch for mesh " + std::to_string(i));
          Emitter& e = b.outs[i];
          const uint64_t dn = reinterpret_cast<uintptr_t>(m.dst_nodes), dd = reinterpret_cast<uintptr_t>(m.dst_data);
          for (size_t r = 0; r < e.node_recs.size(); r += 4) {
            if (e.node_recs[r] >= m.total_nodes) fail(OOC_ERR_DEVICE, "internal node record position");
            nrec.insert(nrec.end(), {dn + e.node_recs[r] * 24, e.node_recs[r + 1], e.node_recs[r + 2], e.node_recs[r + 3]});
          }
          for (size_t r = 0; r < e.data_recs.size(); r += 5) {
            if (e.data_recs[r] >= m.total_data) fail(OOC_ERR_DEVICE, "internal data record position");
            drec.insert(drec.end(), {dd + e.data_recs[r] * 32, e.data_recs[r + 1], e.data_recs[r + 2],
                                     e.data_recs[r + 3], e.data_recs[r + 4]});
          }
          std::vector<uint64_t>().swap(e.node_recs);
          std::vector<uint64_t>().swap(e.data_recs);
          if (infos) fill_info(m, &infos[i]);
        }
        const size_t words = nrec.size() + drec.size();
        if (words) {
          uint64_t* h = ensure_pinned<uint64_t>(c->h_recs, words * 8);
          std::memcpy(h, nrec.data(), nrec.size() * 8);
          std::memcpy(h + nrec.size(), drec.data(), drec.size() * 8);
          uint64_t* d = ensure<uint64_t>(c->d_recs, words * 8);
          ck(cudaMemcpyAsync(d, h, words * 8, cudaMemcpyHostToDevice, c->copy_stream), "records");
          launch_scatter_to(d, nrec.size() / 4, 3, c->copy_stream);
          launch_scatter_to(d + nrec.size(), drec.size() / 5, 4, c->copy_stream);
        }
        // the meshes' stripes were finished before their sub-batch's event; the scatter is this stream's
        ck(cudaStreamSynchronize(c->copy_stream), "records");
        ck(cudaGetLastError(), "scatter");
        if (ready)
          for (size_t i : done)
            if (ready(user, i) != 0) fail(OOC_ERR_SINK, "ready callback returned an error");
      });
    }
    ck(cudaStreamSynchronize(st), "build");
    finish_timing(c);
  });
}

int ooc_set_batch_budget(ooc_ctx* c, uint64_t bytes) {
  if (!c || bytes < 4096) return OOC_ERR_INVALID;
  c->tuning.batch_budget = bytes;
  return OOC_OK;
}

uint64_t ooc_batch_budget(const ooc_ctx* c) { return c ? c->tuning.batch_budget : 0; }

namespace {
bool tuning_ok(const ooc_tuning& t) {
  return t.small_vol >= 1 && t.small_vol <= 64 && t.lines_per_lane >= 1 && t.lines_per_lane <= 64 &&
         (t.large_block == 64 || t.large_block == 128 || t.large_block == 256) && t.large_ctas_per_sm >= 1 &&
         t.large_ctas_per_sm <= 16 && t.batch_budget >= 4096 && t.graphs <= 1 && t.light_per_thread >= 1 &&
         t.light_per_thread <= 16 && t.pdl <= 1 && t.persistent <= 1;
}

struct TuneArena {
  DevBuf* buf;
  uint64_t used;
};

int tune_alloc(void* user, uint64_t, uint64_t nodes_bytes, uint64_t data_bytes, void*, void** nodes, void** data) {
  TuneArena* a = static_cast<TuneArena*>(user);
  const uint64_t n = (nodes_bytes + 255) / 256 * 256, d = (data_bytes + 255) / 256 * 256;
  if (a->used + n + d > a->buf->cap) return 1;
  *nodes = static_cast<char*>(a->buf->p) + a->used;
  *data = static_cast<char*>(a->buf->p) + a->used + n;
  a->used += n + d;
  return 0;
}

int count_sink(void*, uint64_t, int32_t, const void*, uint64_t) { return 0; }
}  // namespace

int ooc_get_tuning(const ooc_ctx* c, ooc_tuning* out) {
  if (!c || !out) return OOC_ERR_INVALID;
  *out = c->tuning;
  return OOC_OK;
}

int ooc_set_tuning(ooc_ctx* c, const ooc_tuning* t) {
  if (!c || !t) return OOC_ERR_INVALID;
  if (!tuning_ok(*t)) {
    c->err = "tuning value out of range";
    return OOC_ERR_INVALID;
  }
  c->tuning = *t;
  return OOC_OK;
}

int ooc_autotune(ooc_ctx* c, const ooc_mesh* sample, uint64_t n, ooc_tuning* best) {
  if (!c || (n && !sample)) return OOC_ERR_INVALID;
  const ooc_tuning start = c->tuning;
  // sizes of the sample's files, then one arena that holds them all
  std::vector<ooc_build_info> infos(n > 0 ? n : 1);
  int rc = ooc_build_batch(c, sample, n, count_sink, nullptr, infos.data());
  if (rc != OOC_OK) return rc;
  uint64_t bytes = 0;
  for (uint64_t i = 0; i < n; i++)
    bytes += (infos[i].n_nodes * 24 + 255) / 256 * 256 + (infos[i].n_data * 32 + 255) / 256 * 256;
  rc = guarded(c, [&] { ensure<unsigned char>(c->d_tune_arena, bytes + 4096); });
  if (rc != OOC_OK) return rc;
  auto time_one = [&](const ooc_tuning& t, double& ms) -> int {
    c->tuning = t;
    double best_ms = 1e30;
    for (int rep = 0; rep < 2; rep++) {
      TuneArena a{&c->d_tune_arena, 0};
      const auto t0 = std::chrono::steady_clock::now();
      const int r = ooc_build_batch_device(c, sample, n, tune_alloc, nullptr, &a, infos.data());
      if (r != OOC_OK) return r;
      best_ms = std::min(best_ms, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
    }
    ms = best_ms;
    return OOC_OK;
  };
  ooc_tuning cur = start;
  double cur_ms = 0.0;
  rc = time_one(cur, cur_ms);  // warms the context's buffers too
  if (rc == OOC_OK) rc = time_one(cur, cur_ms);
  // one coordinate pass: each choice in turn, the others held at their best so far
  const uint32_t lpl[] = {4, 8, 16, 32}, cps[] = {2, 4, 8}, blk[] = {128, 256}, svol[] = {16, 32, 48, 64}, gr[] = {0, 1},
                 ept[] = {1, 2, 4, 8}, pdl[] = {0, 1}, per[] = {0, 1};
  const uint64_t bud[] = {1ull << 30, 2ull << 30, 4ull << 30, 8ull << 30};
  auto try_values = [&](auto setter, const auto& values) {
    for (const auto& v : values) {
      if (rc != OOC_OK) return;
      ooc_tuning t = cur;
      setter(t, v);
      if (std::memcmp(&t, &cur, sizeof(t)) == 0) continue;
      double ms = 0.0;
      rc = time_one(t, ms);
      if (rc == OOC_OK && ms < cur_ms) {
        cur = t;
        cur_ms = ms;
      }
    }
  };
  try_values([](ooc_tuning& t, uint32_t v) { t.lines_per_lane = v; }, lpl);
  try_values([](ooc_tuning& t, uint32_t v) { t.large_ctas_per_sm = v; }, cps);
  try_values([](ooc_tuning& t, uint32_t v) { t.large_block = v; }, blk);
  try_values([](ooc_tuning& t, uint32_t v) { t.small_vol = v; }, svol);
  try_values([](ooc_tuning& t, uint64_t v) { t.batch_budget = v; }, bud);
  try_values([](ooc_tuning& t, uint32_t v) { t.light_per_thread = v; }, ept);
  try_values([](ooc_tuning& t, uint32_t v) { t.graphs = v; }, gr);
  try_values([](ooc_tuning& t, uint32_t v) { t.pdl = v; }, pdl);
  try_values([](ooc_tuning& t, uint32_t v) { t.persistent = v; }, per);
  c->tuning = rc == OOC_OK ? cur : start;
  if (best) *best = c->tuning;
  return rc;
}

int ooc_arena_alloc(void* arena, uint64_t mesh, uint64_t nodes_bytes, uint64_t data_bytes, void* stream,
                    void** nodes, void** data) {
  (void)mesh;
  (void)stream;
  ooc_device_arena* a = static_cast<ooc_device_arena*>(arena);
  if (!a || !nodes || !data) return OOC_ERR_INVALID;
  const uint64_t n = (nodes_bytes + 255) / 256 * 256, d = (data_bytes + 255) / 256 * 256;
  if (a->used + n + d > a->capacity) return OOC_ERR_OOM;
  char* base = static_cast<char*>(a->base) + a->used;
  *nodes = base;
  *data = base + n;
  a->used += n + d;
  return OOC_OK;
}

int ooc_build_device(ooc_ctx* c, const ooc_build_params* prm, const float* tris_device, uint64_t n_tris,
                     void* stream, ooc_build_info* info) {
  return guarded(c, [&] {
    begin_build(c);
    check_params(prm, n_tris);
    if (n_tris && !tris_device) fail(OOC_ERR_INVALID, "triangles are NULL");
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : c->own_stream;
    Emitter out;
    out.device = true;
    std::vector<MeshWork> meshes;
    meshes.emplace_back(make_plan(prm), &out);
    meshes[0].prm = prm;
    meshes[0].d_tris = tris_device;
    meshes[0].n_tris = n_tris;
    {
      PhaseScope all(c, PH_ALL, st);
      OutSpec os;
      os.mode = OUT_CTX;
      build_meshes(c, st, meshes, os);
      finish_device_output(c, st, meshes[0], out);
    }
    ck(cudaStreamSynchronize(st), "build");
    ck(cudaGetLastError(), "build kernels");
    fill_info(meshes[0], info);
    finish_timing(c);
  });
}

int ooc_build_from_device(ooc_ctx* c, const ooc_build_params* prm, const float* tris_device, uint64_t n_tris,
                          ooc_sink_fn sink, void* user, ooc_build_info* info) {
  return guarded(c, [&] {
    begin_build(c);
    check_params(prm, n_tris);
    if (!sink) fail(OOC_ERR_INVALID, "sink is NULL");
    if (n_tris && !tris_device) fail(OOC_ERR_INVALID, "triangles are NULL");
    cudaStream_t st = c->own_stream;
    SingleSink ss{sink, user};
    Emitter out;
    out.sink = single_sink;
    out.user = &ss;
    std::vector<MeshWork> meshes;
    meshes.emplace_back(make_plan(prm), &out);
    meshes[0].prm = prm;
    meshes[0].d_tris = tris_device;
    meshes[0].n_tris = n_tris;
    {
      PhaseScope all(c, PH_ALL, st);
      OutSpec os;
      os.mode = OUT_HOST;
      build_meshes(c, st, meshes, os);
    }
    ck(cudaStreamSynchronize(st), "build");
    ck(cudaGetLastError(), "build kernels");
    fill_info(meshes[0], info);
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

uint64_t ooc_partition_counts(const ooc_ctx* c, uint64_t first, uint64_t n, uint64_t* triangles, uint64_t* filled) {
  if (!c) return 0;
  const uint64_t P = c->part_tris.size();
  for (uint64_t i = 0; i < n && first + i < P; i++) {
    if (triangles) triangles[i] = c->part_tris[first + i];
    if (filled) filled[i] = c->part_filled[first + i];
  }
  return P;
}

int ooc_set_stream_budget(ooc_ctx* c, uint64_t bytes) {
  if (!c) return OOC_ERR_INVALID;
  c->stream_budget = bytes;
  return OOC_OK;
}

uint64_t ooc_stream_budget(const ooc_ctx* c) { return c ? c->stream_budget : 0; }

uint64_t ooc_stream_passes(const ooc_ctx* c) { return c ? c->stream_passes : 0; }

int ooc_file_times(const ooc_ctx* c, float* ms, int32_t n) {
  if (!c || !ms || n < 0) return OOC_ERR_INVALID;
  for (int i = 0; i < n && i < 2; i++) ms[i] = c->file_ms[i];
  return OOC_OK;
}

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
