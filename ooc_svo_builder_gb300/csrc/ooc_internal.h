// Internal interfaces between the orchestration (ooc_api.cu) and the kernels
// (ooc_kernels.cu).  Not part of the public ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "ooc_svo_gpu.h"

namespace ooc {

// Maximum stripe: 8^10 = 2^30 voxels, a 1024^3 Morton-aligned cube whose
// occupancy bitfield (128 MiB) is about the size of the GB300's 129 MB L2, so
// the voxelization atomics mostly stay on chip.
constexpr int kMaxStripeDepth = 10;
constexpr int kMaxLevels = kMaxStripeDepth + 1;

// One level of the per-stripe occupancy pyramid.  Level l has 8^l bits; its
// words are padded to whole 256-bit blocks (8 words) and each block has a
// popcount entry in the concatenated scan array.
struct Level {
  uint64_t off_w;    // first word of this level in its buffer (`leaf` for the leaf level, `bits` above it)
  uint64_t off_b;    // first block entry of this level in the scan buffer
  uint64_t nwords;   // padded word count (multiple of 8)
  uint64_t nblocks;  // nwords / 8
  uint64_t nscan;    // scan entries: nblocks, or one per group of 16 blocks for a marked leaf level
  uint64_t koff;     // first node of this level in the per-node arrays
  uint64_t n;        // set bits (nodes) at this level, filled after the scan
};

// The leaf level (with a marked leaf level, also the level above it) lives in
// its own buffer, which is all zero between builds:
// the voxelization marks every 256-bit leaf block it sets a bit in (`touch`,
// one byte per block, written with plain stores), the passes over the leaf
// level read only marked blocks, and the last kernel of a sub-batch zeroes the
// marked blocks and the marks.  The levels above the leaf are written in full
// by the pyramid passes.
//
// A marked leaf level has one scan entry per group of kLeafGroup blocks (the
// group's node count) and, for each marked block, the count of the group's
// nodes before it (`local`), so the scan never visits unmarked blocks.
struct Pyramid {
  int depth;  // Ds: levels 0..Ds, level Ds = voxels of the stripe
  int zl;     // levels zl..Ds live in `leaf` (Ds, or Ds-1 when the leaf level is marked)
  Level lv[kMaxLevels];
  uint32_t* bits;   // words of levels 0..zl-1
  uint32_t* leaf;   // words of levels zl..Ds, zero between builds outside marked groups
  uint8_t* touch;   // byte b non-zero: leaf block b may have a set bit (NULL: every block is read)
  uint16_t* local;  // marked leaf level: nodes of block b's group before block b (written for marked blocks)
  uint32_t* scan;   // exclusive prefix popcount per 256-bit block, all levels (+1 total)
  uint64_t* woff;   // leaf level, payload stripes: per block, byte k = set bits in its words 0..k-1
                    // (written for every block of an unmarked level, for marked blocks otherwise); or NULL
};

constexpr uint64_t kLeafGroup = 16;  // leaf blocks per scan entry of a marked leaf level

// Mark bytes of a stripe's leaf level, padded to 16 bytes.
__host__ __device__ inline uint64_t touch_bytes(const Level& leaf) { return (leaf.nblocks + 15) / 16 * 16; }

// Inputs of the voxelization kernels for one stripe.
struct VoxJob {
  const float* tris;
  int stride;               // 9 (binary) or 21 (payload)
  const uint32_t* item_tri; // triangle of each item (NULL: item i is triangle ibeg + i)
  uint64_t ibeg;
  uint64_t n_items;
  int pa[3], pb[3];         // partition box in grid coordinates (inclusive)
  int sa[3], sb[3];         // stripe box in grid coordinates (inclusive)
  float u, unit_div;
  uint32_t small_vol;       // items with at most this many candidates (<= 64) run one per thread
  uint32_t lines_per_lane;  // lines of a large item each lane of a warp task walks (task = 32 x this)
  uint32_t* leafbits;       // level-Ds words
  uint8_t* leaftouch;       // byte per 256-bit block of leafbits, set when a bit of the block is (may be NULL)
  // pass B (payload winners)
  const uint32_t* leafscan; // scan entries of level Ds (exclusive, minus its base)
  const uint16_t* leaflocal;// marked leaf level: Pyramid::local (leafscan then has one entry per group)
  uint32_t leafscan_base;
  const uint64_t* leafwoff; // Pyramid::woff of the leaf level (the rank of a bit without a popcount per word)
  uint32_t* winners;        // per leaf: min triangle index
  uint64_t* task_off;       // per item: exclusive prefix of warp tasks (n_items + 1)
  uint64_t* task_flag;      // set to 1 by an item with tasks (the sub-batch's task_off[items]); may be NULL
  unsigned long long* task_counter;
  uint64_t* item_mask;      // per small item: which of its candidates passed (pass 0 -> pass 1); may be NULL
  uint64_t* item_box;       // per small item with a non-zero mask: its packed stripe-local box
};

struct EmitJob {
  int binary;
  int levels;
  int color_mode;
  uint64_t gridsize;
  uint64_t stripe_base;     // global Morton code of the stripe's first voxel
  int origin[3];            // stripe origin in grid coordinates
  const float* tris;
  int stride;
  float unit_div;
  const uint32_t* keys;     // per node: local key (Morton prefix within its level)
  uint32_t* size;           // per node: nodes in its subtree
  uint32_t* dsize;          // per node: data records in its subtree
  uint32_t* start;          // per node: first node written inside its subtree, minus node_base
  uint32_t* dstart;         // per node: its subtree's first data record, minus data_base
  float* cache;             // per node: 6 floats (colour, normal); only with -levels
  uint32_t* first_child;    // per internal node: global index of its first child
  int leaf_inline;          // payload without -levels: the leaf payload pass writes the leaves' data records
  const uint32_t* winners;
  uint64_t* node_win;       // node window (3 u64 per record)
  uint64_t node_win_base;   // global node index of node_win[0]
  unsigned char* data_win;  // data window (32 bytes per record)
  uint64_t data_win_base;
  uint64_t node_win_len;    // records the node window holds
  uint64_t data_win_len;    // records the data window holds
  uint64_t n_tris;          // triangles in `tris`
  uint32_t* flag;           // set non-zero by a kernel that finds an index out of range
  uint64_t node_base;       // file index of the stripe root's first written descendant
  uint64_t data_base;       // file index of the stripe's first data record
  int l_small;              // levels 0..l_small (at most 256 nodes each) run in one CTA
};

// Threads per CTA of the batched kernels; CTA b of a launch belongs to stripe s
// when cta_beg[s] <= b < cta_beg[s+1] and handles that stripe's elements
// kChunk * (b - cta_beg[s]) onward.
constexpr uint32_t kChunk = 256;

// The message ooc_last_error returns for `c` (for failures found outside ooc_api.cu).
void set_ctx_error(ooc_ctx* c, const std::string& msg);
// ooc_build_files' out-of-core path: whether a mesh of n_tris records streams, and the
// build that reads them from the .tridata file partition group by partition group.
bool file_wants_stream(ooc_ctx* c, const ooc_build_params* prm, uint64_t n_tris);
int build_from_file_stream(ooc_ctx* c, const ooc_build_params* prm, const char* tridata, uint64_t n_tris,
                           ooc_sink_fn sink, void* user, ooc_build_info* info);
// ooc_file_times' values for `c` (set by ooc_build_files).
void set_ctx_file_times(ooc_ctx* c, float read_ms, float write_ms);

// ---- launches (ooc_kernels.cu); all asynchronous on `st` ----

// Optional callbacks around every kernel launch (per-kernel CUDA-event timing).
struct KernelHooks {
  void* user = nullptr;
  void (*begin)(void* user, const char* kernel, cudaStream_t st) = nullptr;
  void (*end)(void* user, const char* kernel, cudaStream_t st) = nullptr;
};

// Launch accounting of one build: its kernel count and its timing callbacks.
// Every launch wrapper reports to the state installed on the calling host
// thread (none installed: nothing is counted or timed).  A context owns one
// and installs it with LaunchScope for the length of each API call, so builds
// of different contexts on different threads never share a counter or hooks,
// and a call made from inside another call's callback restores the outer
// call's state when it returns.
struct LaunchState {
  unsigned long long launches = 0;
  KernelHooks hooks;
  bool pdl = false;  // launch with programmatic stream serialization (ooc_tuning::pdl)
};
LaunchState* current_launch_state();
struct LaunchScope {
  LaunchState* prev;
  explicit LaunchScope(LaunchState* s);
  ~LaunchScope();
  LaunchScope(const LaunchScope&) = delete;
  LaunchScope& operator=(const LaunchScope&) = delete;
};

void scan_u32_exclusive(uint32_t* data, uint64_t n, uint32_t* partials, cudaStream_t st);
// flag_last: data[n-1] is not an input but a flag; zero means every element is zero,
// and the scan is left out.
void scan_u64_exclusive(uint64_t* data, uint64_t n, uint64_t* partials, cudaStream_t st, bool flag_last = false);
uint64_t scan_partials_needed(uint64_t n);

// n words from device memory into `dst`, mapped pinned host memory, by a kernel.
void launch_copy_words(const uint32_t* src, uint64_t n, uint32_t* dst, cudaStream_t st);
void launch_part_count(const float* tris, int stride, uint64_t n_tris, const float* axis_lo, const float* axis_hi,
                       int pa_bits, uint64_t n_parts, uint32_t* hist, cudaStream_t st);
void launch_part_emit(const float* tris, int stride, uint64_t n_tris, const float* axis_lo, const float* axis_hi,
                      int pa_bits, uint64_t n_parts, uint32_t* cursor, uint32_t* items, cudaStream_t st);

// Out-of-core binning of one chunk of the triangle stream for the partition group
// [p0, p0 + gp) (gp <= kStreamMaxGroup): the chunk's records of each group partition q
// are copied, in stream order, to out[base[q]...] (record indices), and base[q] moves
// past them.  `mat` holds gp * stream_ctas(n) + 1 entries, `mat_partials`
// scan_partials_needed of that.
constexpr uint32_t kStreamMaxGroup = 4096;
constexpr uint64_t kStreamCtaTris = 64;  // triangles per CTA of the group binning
uint32_t stream_ctas(uint64_t n);
// base[q] = part_off[p0 + q] - part_off[p0] for q < gp: where each group partition's records start.
void launch_stream_bases(const uint32_t* part_off, uint32_t p0, uint32_t gp, uint64_t* base, cudaStream_t st);
void launch_stream_group_chunk(const float* tris, int stride, uint64_t n, const float* axis_lo, const float* axis_hi,
                               int pa_bits, uint32_t p0, uint32_t gp, uint32_t* mat, uint32_t* mat_partials,
                               uint64_t* base, float* out, cudaStream_t st);

// One-stripe occupancy pass with the job as a kernel parameter (the allocation-free
// entry point's launches); each returns the status of its own launch calls.
cudaError_t launch_vox_small_occupancy(const VoxJob& j, cudaStream_t st);
cudaError_t launch_vox_large_occupancy(const VoxJob& j, cudaStream_t st, int num_sms);
cudaError_t scan_u64_exclusive_checked(uint64_t* data, uint64_t n, uint64_t* partials, cudaStream_t st);

// src holds n entries of (index, `words` u64 values); dst[index*words + q] = value q.
void launch_scatter_records(const uint64_t* src, uint64_t n, int words, uint64_t* dst, cudaStream_t st);
void launch_scatter_to(const uint64_t* src, uint64_t n, int words, cudaStream_t st);

// ---- batched launches: per-stripe jobs in device arrays; `cta_beg` (n + 1 entries) maps CTAs to stripes ----
// `single` (may be NULL): the job of a one-stripe launch, passed as a kernel parameter.
void launch_b_vox_small(const VoxJob* jobs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, int pass,
                        const VoxJob* single, cudaStream_t st);
// Large items of every stripe; task_off is the batch-wide exclusive scan (total_items + 1 entries),
// item_beg[s] the first batch item of stripe s (ascending).
// map[t] = item | stripe << 32 for every warp task t, if they all fit in `cap` entries
// (CTAs as for launch_b_vox_small: `cta_beg` over the stripes' items).
void launch_b_task_map(const uint64_t* cta_beg, uint32_t n, uint64_t ctas, const uint64_t* item_beg,
                       const uint64_t* task_off, uint64_t total_items, uint64_t* map, uint64_t cap, cudaStream_t st);
// `lines_per_lane` is every job's (it sizes each warp's shared list of lines); tasks find
// their item in `map` when the tasks fit in `cap`, else by searching task_off.
void launch_b_vox_large(const VoxJob* jobs, const uint64_t* item_beg, uint32_t n_stripes, const uint64_t* task_off,
                        uint64_t total_items, unsigned long long* counter, int pass, cudaStream_t st, int num_sms,
                        int block, int ctas_per_sm, uint32_t lines_per_lane, const uint64_t* map, uint64_t cap);
// Level depth - r of each stripe.
void launch_b_pyramid(const Pyramid* pyrs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept, int r,
                      const Pyramid* single, cudaStream_t st);
// One CTA per stripe: levels min(l_hi, depth) .. 0.
// Also zeroes *scan_end, the block scan's total entry, before the scan.
void launch_b_pyramid_top(const Pyramid* pyrs, uint32_t n_stripes, int l_hi, uint32_t* scan_end, cudaStream_t st);
// The persistent phase-A kernel's inputs (ooc_tuning::persistent).
struct PersistJob {
  const VoxJob* jobs;
  const Pyramid* pyrs;
  const uint64_t* item_beg;   // n + 1: first item of each stripe in the sub-batch
  uint32_t n;                 // stripes
  uint32_t levels;            // R: pyramid levels below the top ones, at most (over the stripes)
  const uint64_t* chunk_beg;  // n + 1: prefix of 256-item chunks per stripe
  const uint64_t* unit_beg;   // R x (n + 1): prefix of pyramid units per (level r, stripe), r-major, cumulative
  uint32_t ept;               // elements per lane of a pyramid unit
  int top_level;              // levels 0..top_level are the top levels
  uint32_t* occ_left;         // n: occupancy units of each stripe not yet done (chunks, then its queued tasks)
  uint32_t* pyr_left;         // R x n: pyramid units of (level r, stripe) not yet done
  unsigned long long* ctr;    // 64 counters, four used: tickets, chunks done, tasks reserved, timeout code
                              // (kCtr* in the kernel), each on its own 128-byte line
  unsigned long long* map;    // cap task entries (item | task << 32), all ones when empty
  uint64_t cap;
  uint32_t* scan_end;         // the pyramid scan's total entry
  uint32_t lines_per_lane;
};
// CTAs of the persistent kernel one SM holds (0 on an error).
int persist_ctas_per_sm(uint32_t lines_per_lane);
void launch_b_persist(const PersistJob& pj, int num_sms, int ctas_per_sm, cudaStream_t st);
constexpr uint64_t kPersistChunkItems = 256;  // items of a chunk unit
constexpr uint32_t kPersistCtrWords = 64;     // counters of the persistent kernel
constexpr uint32_t kPersistTimeoutWord = 48;  // where it records the code of a wait that ran out
constexpr uint32_t kPersistTasksWord = 32;    // where it counts the tasks it found (queued or not)
void launch_b_compact(const Pyramid* pyrs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept, uint32_t* keys,
                      const Pyramid* single, cudaStream_t st);
// Zero the marked leaf blocks of every stripe and the marks: one thread per 16 mark bytes.
void launch_b_clean_leaves(const Pyramid* pyrs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept,
                           const Pyramid* single, cudaStream_t st);
// out[s * (kMaxLevels + 1) + l] = global node index of level l's first node, l = 0..depth+1.
// Also *tasks_out = *tasks (the large-item task count travels back with the level counts)
// and *flag = 0 (the layout check flag the record kernels may set).
// Level counts of every stripe and the task count (and, when `code` is set, the
// persistent kernel's timeout code) into `out` (pinned host memory in the library's use).
void launch_b_level_bases(const Pyramid* pyrs, uint32_t n_stripes, uint32_t* out, const uint64_t* tasks,
                          uint64_t* tasks_out, uint32_t* flag, const uint64_t* code, uint64_t* code_out,
                          cudaStream_t st);
void launch_b_leaf_payload(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n,
                           uint64_t ctas, uint32_t ept, const Pyramid* sp, const EmitJob* se, cudaStream_t st);
// Level depth - r of each stripe.
void launch_b_bottom_up(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept,
                        int r, const Pyramid* sp, const EmitJob* se, cudaStream_t st);
void launch_b_bottom_up_top(const Pyramid* pyrs, const EmitJob* emits, uint32_t n_stripes, cudaStream_t st);
void launch_b_top_down_top(const Pyramid* pyrs, const EmitJob* emits, uint32_t n_stripes, cudaStream_t st);
// Parents of absolute level l.
void launch_b_top_down(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept,
                       int l, const Pyramid* sp, const EmitJob* se, cudaStream_t st);
void launch_b_top_down_leaves(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n,
                              uint64_t ctas, uint32_t ept, const Pyramid* sp, const EmitJob* se, cudaStream_t st);
// out[s * 16 + 0..6] = stripe s's root child mask and cache.
// Root information of every stripe, and the layout check flag after it, written into
// `out` (pinned host memory in the library's use).
void launch_b_root_info(const Pyramid* pyrs, const EmitJob* emits, uint32_t n_stripes, uint32_t* out,
                        const uint32_t* flag, cudaStream_t st);

}  // namespace ooc
