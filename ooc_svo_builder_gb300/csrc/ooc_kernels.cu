// CUDA kernels of the partition -> voxelize -> SVO-build path (sm_103a).
//
// Compiled with -fmad=false; FP32 arithmetic additionally goes through the
// __f*_rn intrinsics so that each operation rounds once, as in the
// reference's x86-64 build.
#include <cuda_runtime.h>

#include <cstring>
#include <utility>

#include "ooc_device.cuh"
#include "ooc_internal.h"

namespace ooc {

namespace {
thread_local LaunchState* t_launch = nullptr;  // the state of the call running on this thread
}  // namespace

LaunchState* current_launch_state() { return t_launch; }
LaunchScope::LaunchScope(LaunchState* s) : prev(t_launch) { t_launch = s; }
LaunchScope::~LaunchScope() { t_launch = prev; }

namespace {
constexpr unsigned FULL = 0xffffffffu;

// Counts one launch and brackets it with the timing hooks of the calling
// thread's launch state, when one is installed.
struct KScope {
  const char* name;
  cudaStream_t st;
  LaunchState* ls;
  KScope(const char* n, cudaStream_t s) : name(n), st(s), ls(t_launch) {
    if (!ls) return;
    ls->launches++;
    if (ls->hooks.begin) ls->hooks.begin(ls->hooks.user, name, st);
  }
  ~KScope() {
    if (ls && ls->hooks.end) ls->hooks.end(ls->hooks.user, name, st);
  }
};
// Programmatic dependent launch.  Every kernel here first waits until the
// grid before it on the stream has finished and its memory is visible, then
// lets the grid after it launch, so that grid's CTAs take the SMs this one's
// last CTAs free instead of waiting for the whole grid to drain.  Without the
// launch attribute (launch_k with ooc_tuning::pdl off) both are no-ops.
__device__ __forceinline__ void pdl_enter() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" :::);
}

// Launch `k` on `st`, with programmatic stream serialization when the calling
// thread's launch state asks for it.
template <typename... P, typename... A>
void launch_k(void (*k)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t st, A&&... args) {
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = st;
  cfg.attrs = at;
  cfg.numAttrs = (t_launch && t_launch->pdl) ? 1 : 0;
  cudaLaunchKernelEx(&cfg, k, std::forward<A>(args)...);
}

constexpr int SCAN_THREADS = 256;

inline unsigned grid_for(uint64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

// ===========================================================================
// Exclusive scan (three phases: per-CTA reduce, scan of CTA sums, down-sweep)
// ===========================================================================
template <typename T>
__device__ __forceinline__ T warp_inclusive(T v) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T y = __shfl_up_sync(FULL, v, o);
    if (lane >= o) v += y;
  }
  return v;
}

// Exclusive scan of one value per thread across the CTA; `total` gets the CTA sum.
template <typename T>
__device__ __forceinline__ T block_exclusive(T v, T& total) {
  __shared__ T warp_sums[33];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const T inc = warp_inclusive(v);
  if (lane == 31) warp_sums[warp] = inc;
  __syncthreads();
  if (warp == 0) {
    const T w = lane < nw ? warp_sums[lane] : T(0);
    const T wi = warp_inclusive(w);
    if (lane < nw) warp_sums[lane] = wi - w;
    if (lane == 31) warp_sums[32] = wi;
  }
  __syncthreads();
  const T r = inc - v + warp_sums[warp];
  total = warp_sums[32];
  __syncthreads();
  return r;
}

constexpr int SCAN_ITEMS = 16;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

// `skip` (may be NULL): when it points at a zero, every element is zero and the
// scan is left out (all zeros are their own exclusive scan).
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_reduce(const T* __restrict__ in, uint64_t n,
                                                              T* __restrict__ partials, const T* skip) {
  pdl_enter();
  if (skip && *skip == T(0)) return;
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
  T v = 0;
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const uint64_t i = base + (uint64_t)q * SCAN_THREADS + threadIdx.x;
    if (i < n) v += in[i];
  }
  T total;
  block_exclusive(v, total);
  if (threadIdx.x == 0) partials[blockIdx.x] = total;
}

// Also partials[np] = the grand total.
template <typename T>
__global__ void __launch_bounds__(1024) k_scan_partials(T* partials, uint64_t np, const T* skip) {
  pdl_enter();
  if (skip && *skip == T(0)) return;
  T carry = 0;
  for (uint64_t base = 0; base < np; base += blockDim.x) {
    const uint64_t i = base + threadIdx.x;
    const T v = i < np ? partials[i] : T(0);
    T total;
    const T ex = block_exclusive(v, total);
    if (i < np) partials[i] = ex + carry;
    carry += total;
  }
  if (threadIdx.x == 0) partials[np] = carry;
}

// Each thread scans SCAN_ITEMS consecutive elements staged through shared memory
// (`partials` NULL: a single tile, nothing before it).
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_down(T* data, uint64_t n, const T* __restrict__ partials,
                                                            const T* skip) {
  pdl_enter();
  // `skip` is read before any CTA writes: a scan that runs has a non-zero flag and a
  // non-zero total, so a late CTA reading the written total skips nothing either
  if (skip && *skip == T(0)) return;
  // the elements are counts: a zero total means all zero, which is already their scan
  if (partials && partials[gridDim.x] == T(0)) return;
  __shared__ T tile[SCAN_TILE + SCAN_TILE / 32];
  const uint64_t base = (uint64_t)blockIdx.x * SCAN_TILE;
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const uint32_t li = q * SCAN_THREADS + threadIdx.x;
    const uint64_t i = base + li;
    tile[li + li / 32] = i < n ? data[i] : T(0);
  }
  __syncthreads();
  T v[SCAN_ITEMS];
  T sum = 0;
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const uint32_t li = threadIdx.x * SCAN_ITEMS + q;
    v[q] = tile[li + li / 32];
    sum += v[q];
  }
  T total;
  T run = block_exclusive(sum, total) + (partials ? partials[blockIdx.x] : T(0));
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const uint32_t li = threadIdx.x * SCAN_ITEMS + q;
    tile[li + li / 32] = run;
    run += v[q];
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < SCAN_ITEMS; q++) {
    const uint32_t li = q * SCAN_THREADS + threadIdx.x;
    const uint64_t i = base + li;
    if (i < n) data[i] = tile[li + li / 32];
  }
}

template <typename T>
void scan_exclusive(T* data, uint64_t n, T* partials, cudaStream_t st, const T* skip = nullptr) {
  if (n == 0) return;
  const unsigned nb = (unsigned)((n + SCAN_TILE - 1) / SCAN_TILE);
  if (nb == 1) {  // one tile: one launch
    KScope k("scan_down", st);
    launch_k(k_scan_down<T>, dim3(1), dim3(SCAN_THREADS), 0, st, data, n, nullptr, skip);
    return;
  }
  {
    KScope k("scan_reduce", st);
    launch_k(k_scan_reduce<T>, dim3(nb), dim3(SCAN_THREADS), 0, st, data, n, partials, skip);
  }
  {
    KScope k("scan_partials", st);
    launch_k(k_scan_partials<T>, dim3(1), dim3(1024), 0, st, partials, nb, skip);
  }
  {
    KScope k("scan_down", st);
    launch_k(k_scan_down<T>, dim3(nb), dim3(SCAN_THREADS), 0, st, data, n, partials, skip);
  }
}

// ===========================================================================
// Partition binning (partitioner.cpp:101-149 with BBoxBuffer.h:70-84)
// ===========================================================================
struct WorldBox {
  float lo[3], hi[3];
};

__device__ __forceinline__ WorldBox tri_world_box(const float* __restrict__ tris, uint64_t t, int stride) {
  const TriVerts tv = load_verts(tris, t, stride);
  WorldBox b;
#pragma unroll
  for (int a = 0; a < 3; a++) {
    b.lo[a] = smin(tv.v[0][a], smin(tv.v[1][a], tv.v[2][a]));
    b.hi[a] = smax(tv.v[0][a], smax(tv.v[1][a], tv.v[2][a]));
  }
  return b;
}

// Per axis, the partitions j whose world slab [lo_j, hi_j] passes the
// reference's inclusive test form one contiguous run [j0, j1].
__device__ __forceinline__ bool axis_run(float lo, float hi, const float* __restrict__ alo,
                                         const float* __restrict__ ahi, int PA, int& j0, int& j1) {
  j0 = -1;
  j1 = -2;
  for (int j = 0; j < PA; j++) {
    const bool ok = !(hi < alo[j]) && !(lo > ahi[j]);
    if (ok) {
      if (j0 < 0) j0 = j;
      j1 = j;
    }
  }
  return j0 >= 0;
}

__global__ void k_part_count(const float* __restrict__ tris, int stride, uint64_t n_tris,
                             const float* __restrict__ axis_lo, const float* __restrict__ axis_hi, int pa_bits,
                             uint32_t n_parts, uint32_t* __restrict__ hist, int use_smem) {
  pdl_enter();
  extern __shared__ uint32_t sh[];
  if (use_smem) {
    for (uint32_t i = threadIdx.x; i < n_parts; i += blockDim.x) sh[i] = 0;
    __syncthreads();
  }
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n_tris) {
    const int PA = 1 << pa_bits;
    const WorldBox b = tri_world_box(tris, t, stride);
    int x0, x1, y0, y1, z0, z1;
    if (axis_run(b.lo[0], b.hi[0], axis_lo, axis_hi, PA, x0, x1) &&
        axis_run(b.lo[1], b.hi[1], axis_lo + PA, axis_hi + PA, PA, y0, y1) &&
        axis_run(b.lo[2], b.hi[2], axis_lo + 2 * PA, axis_hi + 2 * PA, PA, z0, z1)) {
      for (int jx = x0; jx <= x1; jx++)
        for (int jy = y0; jy <= y1; jy++)
          for (int jz = z0; jz <= z1; jz++) {
            const uint32_t p = morton_local(jx, jy, jz);
            if (use_smem) atomicAdd(&sh[p], 1u);
            else atomicAdd(&hist[p], 1u);
          }
    }
  }
  if (use_smem) {
    __syncthreads();
    for (uint32_t i = threadIdx.x; i < n_parts; i += blockDim.x)
      if (sh[i]) atomicAdd(&hist[i], sh[i]);
  }
}

__global__ void k_part_emit(const float* __restrict__ tris, int stride, uint64_t n_tris,
                            const float* __restrict__ axis_lo, const float* __restrict__ axis_hi, int pa_bits,
                            uint32_t n_parts, uint32_t* __restrict__ cursor, uint32_t* __restrict__ items,
                            int use_smem) {
  pdl_enter();
  extern __shared__ uint32_t sh[];  // [n_parts] counts, [n_parts] bases
  uint32_t* cnt = sh;
  uint32_t* base = sh + n_parts;
  if (use_smem) {
    for (uint32_t i = threadIdx.x; i < n_parts; i += blockDim.x) cnt[i] = 0;
    __syncthreads();
  }
  const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int PA = 1 << pa_bits;
  int x0 = 0, x1 = -1, y0 = 0, y1 = -1, z0 = 0, z1 = -1;
  bool hit = false;
  if (t < n_tris) {
    const WorldBox b = tri_world_box(tris, t, stride);
    hit = axis_run(b.lo[0], b.hi[0], axis_lo, axis_hi, PA, x0, x1) &&
          axis_run(b.lo[1], b.hi[1], axis_lo + PA, axis_hi + PA, PA, y0, y1) &&
          axis_run(b.lo[2], b.hi[2], axis_lo + 2 * PA, axis_hi + 2 * PA, PA, z0, z1);
  }
  if (!use_smem) {
    if (hit)
      for (int jx = x0; jx <= x1; jx++)
        for (int jy = y0; jy <= y1; jy++)
          for (int jz = z0; jz <= z1; jz++) {
            const uint32_t p = morton_local(jx, jy, jz);
            items[atomicAdd(&cursor[p], 1u)] = (uint32_t)t;
          }
    return;
  }
  if (hit)
    for (int jx = x0; jx <= x1; jx++)
      for (int jy = y0; jy <= y1; jy++)
        for (int jz = z0; jz <= z1; jz++) atomicAdd(&cnt[morton_local(jx, jy, jz)], 1u);
  __syncthreads();
  for (uint32_t i = threadIdx.x; i < n_parts; i += blockDim.x) {
    base[i] = cnt[i] ? atomicAdd(&cursor[i], cnt[i]) : 0u;
    cnt[i] = 0;
  }
  __syncthreads();
  if (hit)
    for (int jx = x0; jx <= x1; jx++)
      for (int jy = y0; jy <= y1; jy++)
        for (int jz = z0; jz <= z1; jz++) {
          const uint32_t p = morton_local(jx, jy, jz);
          items[base[p] + atomicAdd(&cnt[p], 1u)] = (uint32_t)t;
        }
}

// ---------------------------------------------------------------------------
// Out-of-core binning: the records of a group of consecutive partitions
// [p0, p0 + gp), gathered from one chunk of the triangle stream into the
// group's buffer, each partition's records contiguous and in stream order (the
// order of the reference's per-partition .tripdata files, partitioner.cpp:
// 101-149), so a smaller record index within a partition is an earlier
// triangle.  CTAs of kStreamCta triangles; mat[q * n_cta + cta] is CTA cta's
// count for group partition q, whose exclusive scan places every CTA's records.
// ---------------------------------------------------------------------------
constexpr int kStreamCta = (int)kStreamCtaTris;

// Per-axis partition runs of triangle t, packed 7 bits per bound with bit 63 set,
// or 0 when the triangle passes no partition's box test.
__device__ __forceinline__ uint64_t stream_runs(const float* __restrict__ tris, int stride, uint64_t t,
                                                const float* __restrict__ axis_lo, const float* __restrict__ axis_hi,
                                                int PA) {
  const WorldBox b = tri_world_box(tris, t, stride);
  int x0, x1, y0, y1, z0, z1;
  if (!(axis_run(b.lo[0], b.hi[0], axis_lo, axis_hi, PA, x0, x1) &&
        axis_run(b.lo[1], b.hi[1], axis_lo + PA, axis_hi + PA, PA, y0, y1) &&
        axis_run(b.lo[2], b.hi[2], axis_lo + 2 * PA, axis_hi + 2 * PA, PA, z0, z1)))
    return 0ull;
  return (uint64_t)x0 | ((uint64_t)x1 << 7) | ((uint64_t)y0 << 14) | ((uint64_t)y1 << 21) | ((uint64_t)z0 << 28) |
         ((uint64_t)z1 << 35) | (1ull << 63);
}

__device__ __forceinline__ int run_bound(uint64_t r, int k) { return (int)((r >> (7 * k)) & 127u); }

__global__ void __launch_bounds__(kStreamCta) k_stream_count(const float* __restrict__ tris, int stride, uint64_t n,
                                                             const float* __restrict__ axis_lo,
                                                             const float* __restrict__ axis_hi, int pa_bits,
                                                             uint32_t p0, uint32_t gp, uint32_t* __restrict__ mat,
                                                             uint32_t n_cta) {
  pdl_enter();
  extern __shared__ uint32_t cnt[];
  for (uint32_t q = threadIdx.x; q < gp; q += kStreamCta) cnt[q] = 0;
  if (blockIdx.x == 0 && threadIdx.x == 0) mat[(uint64_t)gp * n_cta] = 0;  // the scan's total entry
  __syncthreads();
  const uint64_t t = (uint64_t)blockIdx.x * kStreamCta + threadIdx.x;
  if (t < n) {
    const uint64_t r = stream_runs(tris, stride, t, axis_lo, axis_hi, 1 << pa_bits);
    if (r)
      for (int jx = run_bound(r, 0); jx <= run_bound(r, 1); jx++)
        for (int jy = run_bound(r, 2); jy <= run_bound(r, 3); jy++)
          for (int jz = run_bound(r, 4); jz <= run_bound(r, 5); jz++) {
            const uint32_t q = morton_local(jx, jy, jz) - p0;
            if (q < gp) atomicAdd(&cnt[q], 1u);
          }
  }
  __syncthreads();
  for (uint32_t q = threadIdx.x; q < gp; q += kStreamCta) mat[(uint64_t)q * n_cta + blockIdx.x] = cnt[q];
}

// Each record goes to base[q] + (its CTA's place among the chunk's records of q) +
// (the CTA's earlier triangles that are in q).
__global__ void __launch_bounds__(kStreamCta) k_stream_emit(const float* __restrict__ tris, int stride, uint64_t n,
                                                            const float* __restrict__ axis_lo,
                                                            const float* __restrict__ axis_hi, int pa_bits,
                                                            uint32_t p0, uint32_t gp, const uint32_t* __restrict__ mat,
                                                            uint32_t n_cta, const uint64_t* __restrict__ base,
                                                            float* __restrict__ out) {
  pdl_enter();
  __shared__ uint64_t runs[kStreamCta];
  const uint64_t t = (uint64_t)blockIdx.x * kStreamCta + threadIdx.x;
  const uint64_t r = t < n ? stream_runs(tris, stride, t, axis_lo, axis_hi, 1 << pa_bits) : 0ull;
  runs[threadIdx.x] = r;
  __syncthreads();
  if (!r) return;
  const float* src = tris + t * (uint64_t)stride;
  for (int jx = run_bound(r, 0); jx <= run_bound(r, 1); jx++)
    for (int jy = run_bound(r, 2); jy <= run_bound(r, 3); jy++)
      for (int jz = run_bound(r, 4); jz <= run_bound(r, 5); jz++) {
        const uint32_t q = morton_local(jx, jy, jz) - p0;
        if (q >= gp) continue;
        uint32_t rank = 0;
        for (uint32_t k = 0; k < threadIdx.x; k++) {
          const uint64_t o = runs[k];
          rank += (o >> 63) && run_bound(o, 0) <= jx && jx <= run_bound(o, 1) && run_bound(o, 2) <= jy &&
                  jy <= run_bound(o, 3) && run_bound(o, 4) <= jz && jz <= run_bound(o, 5);
        }
        const uint64_t row = (uint64_t)q * n_cta;
        const uint64_t dst = base[q] + (mat[row + blockIdx.x] - mat[row]) + rank;
        float* d = out + dst * (uint64_t)stride;
        for (int k = 0; k < stride; k++) d[k] = src[k];
      }
}

__global__ void k_stream_bases(const uint32_t* __restrict__ part_off, uint32_t p0, uint32_t gp,
                               uint64_t* __restrict__ base) {
  pdl_enter();
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < gp) base[q] = (uint64_t)(part_off[p0 + q] - part_off[p0]);
}

// After a chunk: every group partition's next record moves past the chunk's records of it.
__global__ void k_stream_advance(const uint32_t* __restrict__ mat, uint32_t n_cta, uint32_t gp,
                                 uint64_t* __restrict__ base) {
  pdl_enter();
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q < gp) base[q] += mat[(uint64_t)(q + 1) * n_cta] - mat[(uint64_t)q * n_cta];
}

// ===========================================================================
// Voxelization (voxelizer.cpp:168-306)
//
// Pass 0 sets the Morton-ordered occupancy bits of the stripe; pass 1 (payload
// mode) keeps, per set voxel, the smallest passing triangle index, which is
// the reference's first-writer-wins rule (voxelizer.cpp:263, 293-299).  For a
// small item pass 0 also stores which of its (at most 64) candidates passed,
// so pass 1 only ranks those voxels instead of testing again.
// ===========================================================================
__device__ __forceinline__ bool item_box(const VoxJob& j, const TriVerts& tv, int lo[3], int hi[3]) {
  int gmin[3], gmax[3];
  grid_box(tv, j.unit_div, gmin, gmax);
#pragma unroll
  for (int a = 0; a < 3; a++) {
    // clamp to the partition (voxelizer.cpp:199-204), then keep the part in this stripe
    lo[a] = clampi(gmin[a], j.pa[a], j.pb[a]);
    hi[a] = clampi(gmax[a], j.pa[a], j.pb[a]);
    lo[a] = lo[a] < j.sa[a] ? j.sa[a] : lo[a];
    hi[a] = hi[a] > j.sb[a] ? j.sb[a] : hi[a];
  }
  return lo[0] <= hi[0] && lo[1] <= hi[1] && lo[2] <= hi[2];
}

// Set bits before bit `b` inside its 256-bit block (`blk` points at the block's 8 words).
__device__ __forceinline__ uint32_t in_block_rank(const uint32_t* __restrict__ blk, uint64_t b) {
  const uint4* q = reinterpret_cast<const uint4*>(blk);
  const uint4 q0 = q[0], q1 = q[1];
  const uint32_t w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
  const uint32_t wi = (uint32_t)(b >> 5) & 7u;
  const uint32_t lowmask = (1u << (b & 31)) - 1u;
  uint32_t r = 0;
#pragma unroll
  for (uint32_t k = 0; k < 8; k++) r += __popc(k < wi ? w[k] : (k == wi ? (w[k] & lowmask) : 0u));
  return r;
}

// Sets `acc` in leaf word w and marks the word's 256-bit block, so every
// block with a set bit is marked.  The mark is a plain byte store: threads
// that mark the same block store the same value, and nothing reads the marks
// before the launch ends.
__device__ __forceinline__ void set_leaf(const VoxJob& j, uint32_t w, uint32_t acc) {
  atomicOr(&j.leafbits[w], acc);
  if (j.leaftouch) j.leaftouch[w >> 3] = 1;
}

// Rank of bit `b` among the set bits of the leaf level.
__device__ __forceinline__ uint32_t leaf_rank(const VoxJob& j, uint32_t b) {
  const uint32_t blk = b >> 8;
  const uint32_t base = j.leaflocal ? j.leafscan[blk / kLeafGroup] + j.leaflocal[blk] : j.leafscan[blk];
  if (j.leafwoff) {  // the set bits before the bit's word, from the pyramid pass, and one popcount
    const uint32_t wi = (b >> 5) & 7u;
    const uint32_t before = (uint32_t)(j.leafwoff[blk] >> (8 * wi)) & 0xffu;
    return base - j.leafscan_base + before + __popc(j.leafbits[b >> 5] & ((1u << (b & 31)) - 1u));
  }
  return base - j.leafscan_base + in_block_rank(j.leafbits + (uint64_t)blk * 8, b);
}

__device__ __forceinline__ uint64_t item_triangle(const VoxJob& j, uint64_t i) {
  return j.item_tri ? (uint64_t)j.item_tri[j.ibeg + i] : j.ibeg + i;
}

// ---------------------------------------------------------------------------
// Large items walk lines along the axis of their largest normal component.  On
// every line the voxels that pass the plane test form one run (plane_side), so
// a line costs its run plus a few probes instead of its whole length; every
// voxel of the run still gets the complete test, so the result is the
// reference's candidate loop (voxelizer.cpp:257-305) voxel for voxel.
// ---------------------------------------------------------------------------

// Axis of the largest component of cross(e0, e1); the item count and the tasks
// call this same function, so they agree on the lines of every item.
__device__ __forceinline__ int walk_axis(const TriVerts& t) {
  const float e0x = t.v[1][0] - t.v[0][0], e0y = t.v[1][1] - t.v[0][1], e0z = t.v[1][2] - t.v[0][2];
  const float e1x = t.v[2][0] - t.v[1][0], e1y = t.v[2][1] - t.v[1][1], e1z = t.v[2][2] - t.v[1][2];
  const float ax = fabsf(e0y * e1z - e0z * e1y), ay = fabsf(e0z * e1x - e0x * e1z), az = fabsf(e0x * e1y - e0y * e1x);
  if (az >= ax && az >= ay) return 2;
  return ax >= ay ? 0 : 1;
}

// Lines of a large item: the box extents across the walk axis.
__device__ __forceinline__ uint64_t item_lines(int W, const int lo[3], const int hi[3]) {
  const uint64_t ex = (uint64_t)(hi[0] - lo[0] + 1), ey = (uint64_t)(hi[1] - lo[1] + 1),
                 ez = (uint64_t)(hi[2] - lo[2] + 1);
  return W == 0 ? ey * ez : (W == 1 ? ex * ez : ex * ey);
}

// One line of a large item: pass 0 sets its bits, pass 1 offers the triangle
// to every voxel it passes.  `dir` is the sign-carrying slope of the plane
// value along the line (n_w * u) and `inv_dir` its reciprocal.
template <int PASS>
__device__ __forceinline__ void vox_line(const VoxJob& j, const TriSetup& s, uint32_t tri, int W, int ca, int cb,
                                         int w0, int w1, bool mono, float dir, float inv_dir) {
  const float fa = __fmul_rn((float)ca, j.u), fb = __fmul_rn((float)cb, j.u);
  float px, py, pz;
  auto corner = [&](int w) {
    const float fw = __fmul_rn((float)w, j.u);
    px = W == 0 ? fw : fa;
    py = W == 1 ? fw : (W == 0 ? fa : fb);
    pz = W == 2 ? fw : fb;
  };
  corner(w0);  // the caller has passed the projection test that does not depend on the walk coordinate
  // the two that do (with the plane test they complete the voxel test)
  auto rest = [&]() {
    return W == 2 ? (pass_yz(s, py, pz) && pass_zx(s, pz, px))
                  : (W == 0 ? (pass_xy(s, px, py) && pass_zx(s, pz, px)) : (pass_xy(s, px, py) && pass_yz(s, py, pz)));
  };
  // stripe-local Morton bits of the two fixed coordinates; the walk axis adds its own
  const int sw = W == 0 ? j.sa[0] : (W == 1 ? j.sa[1] : j.sa[2]);
  const uint32_t la = (uint32_t)(ca - (W == 0 ? j.sa[1] : j.sa[0])), lb = (uint32_t)(cb - (W == 2 ? j.sa[1] : j.sa[2]));
  const uint32_t mab = W == 0 ? (spread3_10(la) << 1) | (spread3_10(lb) << 2)
                              : (W == 1 ? spread3_10(la) | (spread3_10(lb) << 2) : spread3_10(la) | (spread3_10(lb) << 1));
  uint32_t cur_w = 0xffffffffu, acc = 0;
  auto emit = [&](int w) {
    const uint32_t m = mab | (spread3_10((uint32_t)(w - sw)) << W);
    if (PASS == 0) {
      const uint32_t wd = m >> 5;
      if (wd != cur_w) {
        if (acc) set_leaf(j, cur_w, acc);
        cur_w = wd;
        acc = 0;
      }
      acc |= 1u << (m & 31);
    } else {
      atomicMin(&j.winners[leaf_rank(j, m)], tri);  // pass 0 set this voxel's bit
    }
  };
  if (!mono) {  // every voxel of the line, complete test
    for (int w = w0; w <= w1; w++) {
      corner(w);
      if (pass_z(s, plane_xy(s, px, py), px, py, pz) && rest()) emit(w);
    }
  } else {
    auto side = [&](int w) {
      corner(w);
      return plane_side(s, px, py, pz, dir);
    };
    // start where the plane crosses the line's middle, then find one voxel of the run
    const float off = (W == 0 ? 0.0f : s.n[0] * px) + (W == 1 ? 0.0f : s.n[1] * py) + (W == 2 ? 0.0f : s.n[2] * pz);
    float west = -(off + 0.5f * (s.d1 + s.d2)) * inv_dir;
    west = fminf(fmaxf(west, (float)w0), (float)w1);  // NaN becomes w0
    int start = (int)west, walk = 0;                   // walk: +1 up only, -1 down only, 0 both ways
    const int g0 = side(start);
    if (g0 < 0) {  // the run lies above: first w with side >= 0
      int lo = start, hi = -1, step = 1;
      for (;;) {
        const int nx = min(lo + step, w1);
        if (side(nx) >= 0) {
          hi = nx;
          break;
        }
        if (nx == w1) return;
        lo = nx;
        step <<= 1;
      }
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (side(mid) >= 0) hi = mid;
        else lo = mid;
      }
      if (side(hi) != 0) return;  // the run falls between two voxels
      start = hi;
      walk = 1;
    } else if (g0 > 0) {  // below: last w with side <= 0
      int hi = start, lo = -1, step = 1;
      for (;;) {
        const int nx = max(hi - step, w0);
        if (side(nx) <= 0) {
          lo = nx;
          break;
        }
        if (nx == w0) return;
        hi = nx;
        step <<= 1;
      }
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (side(mid) <= 0) lo = mid;
        else hi = mid;
      }
      if (side(lo) != 0) return;
      start = lo;
      walk = -1;
    }
    // px/py/pz hold `start`'s corner and its plane test passed
    if (rest()) emit(start);
    if (walk >= 0)
      for (int w = start + 1; w <= w1 && side(w) == 0; w++)
        if (rest()) emit(w);
    if (walk <= 0)
      for (int w = start - 1; w >= w0 && side(w) == 0; w--)
        if (rest()) emit(w);
  }
  if (PASS == 0 && acc) set_leaf(j, cur_w, acc);
}

// ---------------------------------------------------------------------------
// Small items: the candidate tests by projection.  Of the seven tests of a
// candidate voxel (voxelizer.cpp:266-287) the three XY edge tests depend only
// on (x, y), the YZ tests only on (y, z), the ZX tests only on (z, x); only the
// plane test depends on all three.  Each is a pure function of its
// coordinates, so evaluating it once per distinct projection and reusing the
// result gives the reference's verdict for every candidate, bit for bit; the
// FP32 expressions are the reference's, operation by operation.  A candidate
// passes when all seven pass (the reference's order of early exits only saves
// work).  The pass mask of an item has bit (ix * by + iy) * bz + iz for box
// coordinates (ix, iy, iz).
// ---------------------------------------------------------------------------

// Sets a passing voxel's bit: bits of one leaf word are gathered in `acc`
// while consecutive voxels stay in it.
__device__ __forceinline__ void leaf_bit(const VoxJob& j, bool pass, uint32_t m, uint32_t& cur_w, uint32_t& acc) {
  if (!pass) return;
  const uint32_t w = m >> 5;
  if (w != cur_w) {
    if (acc) set_leaf(j, cur_w, acc);
    cur_w = w;
    acc = 0;
  }
  acc |= 1u << (m & 31);
}

__device__ __forceinline__ uint64_t bit_if(bool p, uint32_t pos) { return p ? (1ull << (pos & 63u)) : 0ull; }

// Boxes at most two voxels wide in x and y (the common small triangle): z is
// walked in 2 x 2 x 2 bricks, every test of a brick evaluated without
// branches; slots outside the box are masked.  The Morton bits of a
// coordinate + 1 come from the carry trick: setting every bit outside an
// axis' positions makes +1 carry across them.
__device__ __forceinline__ uint64_t vox_small_bricks(const VoxJob& j, const TriSetup& s, const int lo[3], uint32_t bx,
                                                     uint32_t by, uint32_t bz) {
  const float px0 = __fmul_rn((float)lo[0], j.u), px1 = __fmul_rn((float)(lo[0] + 1), j.u);
  const float py0 = __fmul_rn((float)lo[1], j.u), py1 = __fmul_rn((float)(lo[1] + 1), j.u);
  // XY over the four columns (x_i, y_j)
  bool c00 = true, c01 = by > 1, c10 = bx > 1, c11 = bx > 1 && by > 1;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const float a0 = __fmul_rn(s.xy[k][0], px0), a1 = __fmul_rn(s.xy[k][0], px1);
    const float b0 = __fmul_rn(s.xy[k][1], py0), b1 = __fmul_rn(s.xy[k][1], py1);
    c00 &= !(__fadd_rn(__fadd_rn(a0, b0), s.dxy[k]) < 0.0f);
    c01 &= !(__fadd_rn(__fadd_rn(a0, b1), s.dxy[k]) < 0.0f);
    c10 &= !(__fadd_rn(__fadd_rn(a1, b0), s.dxy[k]) < 0.0f);
    c11 &= !(__fadd_rn(__fadd_rn(a1, b1), s.dxy[k]) < 0.0f);
  }
  // n.x * p.x + n.y * p.y per column, and the halves of the YZ and ZX dot products
  // that do not depend on z
  const float n0x0 = __fmul_rn(s.n[0], px0), n0x1 = __fmul_rn(s.n[0], px1);
  const float n1y0 = __fmul_rn(s.n[1], py0), n1y1 = __fmul_rn(s.n[1], py1);
  const float q00 = __fadd_rn(n0x0, n1y0), q01 = __fadd_rn(n0x0, n1y1), q10 = __fadd_rn(n0x1, n1y0),
              q11 = __fadd_rn(n0x1, n1y1);
  float yz_y0[3], yz_y1[3], zx_x0[3], zx_x1[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    yz_y0[k] = __fmul_rn(s.yz[k][0], py0);
    yz_y1[k] = __fmul_rn(s.yz[k][0], py1);
    zx_x0[k] = __fmul_rn(s.zx[k][1], px0);
    zx_x1[k] = __fmul_rn(s.zx[k][1], px1);
  }
  constexpr uint32_t XBITS = 0x09249249u, YBITS = 0x12492492u, ZBITS = 0x24924924u;
  const uint32_t mx0 = spread3_10((uint32_t)(lo[0] - j.sa[0])), mx1 = ((mx0 | ~XBITS) + 1u) & XBITS;
  const uint32_t my0 = spread3_10((uint32_t)(lo[1] - j.sa[1])) << 1, my1 = ((my0 | ~YBITS) + 2u) & YBITS;
  uint32_t mz = spread3_10((uint32_t)(lo[2] - j.sa[2])) << 2;
  uint32_t cur_w = 0xffffffffu, acc = 0;
  uint64_t mask = 0;
  for (uint32_t zc = 0; zc < bz; zc += 2) {
    const bool z1ok = zc + 1 < bz;
    const float pz0 = __fmul_rn((float)(lo[2] + (int)zc), j.u), pz1 = __fmul_rn((float)(lo[2] + (int)zc + 1), j.u);
    bool y0z0 = true, y0z1 = z1ok, y1z0 = true, y1z1 = z1ok;  // YZ over (y_j, z_k)
    bool z0x0 = true, z0x1 = true, z1x0 = z1ok, z1x1 = z1ok;  // ZX over (z_k, x_i)
#pragma unroll
    for (int k = 0; k < 3; k++) {
      // dot((-e.z, e.y) * fx, (p.y, p.z)) + d and dot((-e.x, e.z) * fy, (p.z, p.x)) + d
      const float e0 = __fmul_rn(s.yz[k][1], pz0), e1 = __fmul_rn(s.yz[k][1], pz1);
      y0z0 &= !(__fadd_rn(__fadd_rn(yz_y0[k], e0), s.dyz[k]) < 0.0f);
      y0z1 &= !(__fadd_rn(__fadd_rn(yz_y0[k], e1), s.dyz[k]) < 0.0f);
      y1z0 &= !(__fadd_rn(__fadd_rn(yz_y1[k], e0), s.dyz[k]) < 0.0f);
      y1z1 &= !(__fadd_rn(__fadd_rn(yz_y1[k], e1), s.dyz[k]) < 0.0f);
      const float f0 = __fmul_rn(s.zx[k][0], pz0), f1 = __fmul_rn(s.zx[k][0], pz1);
      z0x0 &= !(__fadd_rn(__fadd_rn(f0, zx_x0[k]), s.dzx[k]) < 0.0f);
      z0x1 &= !(__fadd_rn(__fadd_rn(f0, zx_x1[k]), s.dzx[k]) < 0.0f);
      z1x0 &= !(__fadd_rn(__fadd_rn(f1, zx_x0[k]), s.dzx[k]) < 0.0f);
      z1x1 &= !(__fadd_rn(__fadd_rn(f1, zx_x1[k]), s.dzx[k]) < 0.0f);
    }
    // the plane test: (n.p + d1) (n.p + d2) > 0 fails
    const float g0 = __fmul_rn(s.n[2], pz0), g1 = __fmul_rn(s.n[2], pz1);
    auto plane = [&](float q, float g) {
      const float nd = __fadd_rn(q, g);
      return !(__fmul_rn(__fadd_rn(nd, s.d1), __fadd_rn(nd, s.d2)) > 0.0f);
    };
    const bool p000 = c00 & y0z0 & z0x0 & plane(q00, g0), p001 = c00 & y0z1 & z1x0 & plane(q00, g1);
    const bool p010 = c01 & y1z0 & z0x0 & plane(q01, g0), p011 = c01 & y1z1 & z1x0 & plane(q01, g1);
    const bool p100 = c10 & y0z0 & z0x1 & plane(q10, g0), p101 = c10 & y0z1 & z1x1 & plane(q10, g1);
    const bool p110 = c11 & y1z0 & z0x1 & plane(q11, g0), p111 = c11 & y1z1 & z1x1 & plane(q11, g1);
    const uint32_t mz1 = ((mz | ~ZBITS) + 4u) & ZBITS;
    mask |= bit_if(p000, zc) | bit_if(p001, zc + 1) | bit_if(p010, bz + zc) | bit_if(p011, bz + zc + 1) |
            bit_if(p100, by * bz + zc) | bit_if(p101, by * bz + zc + 1) | bit_if(p110, (by + 1) * bz + zc) |
            bit_if(p111, (by + 1) * bz + zc + 1);
    leaf_bit(j, p000, mx0 | my0 | mz, cur_w, acc);
    leaf_bit(j, p001, mx0 | my0 | mz1, cur_w, acc);
    leaf_bit(j, p010, mx0 | my1 | mz, cur_w, acc);
    leaf_bit(j, p011, mx0 | my1 | mz1, cur_w, acc);
    leaf_bit(j, p100, mx1 | my0 | mz, cur_w, acc);
    leaf_bit(j, p101, mx1 | my0 | mz1, cur_w, acc);
    leaf_bit(j, p110, mx1 | my1 | mz, cur_w, acc);
    leaf_bit(j, p111, mx1 | my1 | mz1, cur_w, acc);
    mz = ((mz1 | ~ZBITS) + 4u) & ZBITS;
  }
  if (acc) set_leaf(j, cur_w, acc);
  return mask;
}

// Other small boxes (at most 64 voxels): the YZ verdicts over (y, z) and the
// ZX verdicts over (z, x) as bit masks first, then per column the XY test and
// per candidate the plane test.
__device__ __forceinline__ uint64_t vox_small_factored(const VoxJob& j, const TriSetup& s, const int lo[3],
                                                       uint32_t bx, uint32_t by, uint32_t bz) {
  uint64_t yzm = 0;  // bit iy * bz + iz
  for (uint32_t iy = 0; iy < by; iy++) {
    const float py = __fmul_rn((float)(lo[1] + (int)iy), j.u);
    const float a0 = __fmul_rn(s.yz[0][0], py), a1 = __fmul_rn(s.yz[1][0], py), a2 = __fmul_rn(s.yz[2][0], py);
    for (uint32_t iz = 0; iz < bz; iz++) {
      const float pz = __fmul_rn((float)(lo[2] + (int)iz), j.u);
      const bool ok = !(__fadd_rn(__fadd_rn(a0, __fmul_rn(s.yz[0][1], pz)), s.dyz[0]) < 0.0f) &
                      !(__fadd_rn(__fadd_rn(a1, __fmul_rn(s.yz[1][1], pz)), s.dyz[1]) < 0.0f) &
                      !(__fadd_rn(__fadd_rn(a2, __fmul_rn(s.yz[2][1], pz)), s.dyz[2]) < 0.0f);
      yzm |= bit_if(ok, iy * bz + iz);
    }
  }
  uint64_t zxm = 0;  // bit ix * bz + iz
  for (uint32_t ix = 0; ix < bx; ix++) {
    const float px = __fmul_rn((float)(lo[0] + (int)ix), j.u);
    const float b0 = __fmul_rn(s.zx[0][1], px), b1 = __fmul_rn(s.zx[1][1], px), b2 = __fmul_rn(s.zx[2][1], px);
    for (uint32_t iz = 0; iz < bz; iz++) {
      const float pz = __fmul_rn((float)(lo[2] + (int)iz), j.u);
      const bool ok = !(__fadd_rn(__fadd_rn(__fmul_rn(s.zx[0][0], pz), b0), s.dzx[0]) < 0.0f) &
                      !(__fadd_rn(__fadd_rn(__fmul_rn(s.zx[1][0], pz), b1), s.dzx[1]) < 0.0f) &
                      !(__fadd_rn(__fadd_rn(__fmul_rn(s.zx[2][0], pz), b2), s.dzx[2]) < 0.0f);
      zxm |= bit_if(ok, ix * bz + iz);
    }
  }
  constexpr uint32_t XBITS = 0x09249249u, YBITS = 0x12492492u, ZBITS = 0x24924924u;
  const uint32_t mz0 = spread3_10((uint32_t)(lo[2] - j.sa[2])) << 2;
  const uint32_t my0 = spread3_10((uint32_t)(lo[1] - j.sa[1])) << 1;
  uint32_t mx = spread3_10((uint32_t)(lo[0] - j.sa[0]));
  const uint64_t zfull = bz >= 64 ? ~0ull : ((1ull << bz) - 1);
  uint32_t cur_w = 0xffffffffu, acc = 0;
  uint64_t mask = 0;
  for (uint32_t ix = 0; ix < bx; ix++, mx = ((mx | ~XBITS) + 1u) & XBITS) {
    const float px = __fmul_rn((float)(lo[0] + (int)ix), j.u);
    const float n0px = __fmul_rn(s.n[0], px);
    const uint64_t zx_col = (zxm >> ((ix * bz) & 63u)) & zfull;
    uint32_t my = my0;
    for (uint32_t iy = 0; iy < by; iy++, my = ((my | ~YBITS) + 2u) & YBITS) {
      const uint64_t zb = zx_col & (yzm >> ((iy * bz) & 63u));
      if (!zb) continue;
      const float py = __fmul_rn((float)(lo[1] + (int)iy), j.u);
      if (!pass_xy(s, px, py)) continue;
      const float nxy = __fadd_rn(n0px, __fmul_rn(s.n[1], py));
      const uint32_t mxy = mx | my;
      const uint32_t cbase = (ix * by + iy) * bz;
      uint32_t mz = mz0;
      for (uint32_t iz = 0; iz < bz; iz++, mz = ((mz | ~ZBITS) + 4u) & ZBITS) {
        if (!((zb >> iz) & 1u)) continue;
        const float pz = __fmul_rn((float)(lo[2] + (int)iz), j.u);
        const float nd = __fadd_rn(nxy, __fmul_rn(s.n[2], pz));
        if (__fmul_rn(__fadd_rn(nd, s.d1), __fadd_rn(nd, s.d2)) > 0.0f) continue;
        leaf_bit(j, true, mxy | mz, cur_w, acc);
        mask |= 1ull << (cbase + iz);
      }
    }
  }
  if (acc) set_leaf(j, cur_w, acc);
  return mask;
}

// Pass 0, one thread per item: items with at most small_vol (<= 64) candidates
// are voxelized here and leave their pass mask; larger ones get a warp-task
// count (32 x lines_per_lane lines per task).
__device__ __forceinline__ uint64_t vox_small_occ_item(const VoxJob& j, uint64_t i, const TriVerts& tv) {
  int lo[3], hi[3];
  uint64_t cost = 0, mask = 0;
  if (item_box(j, tv, lo, hi)) {
    const uint32_t bx = (uint32_t)(hi[0] - lo[0] + 1), by = (uint32_t)(hi[1] - lo[1] + 1),
                   bz = (uint32_t)(hi[2] - lo[2] + 1);
    // extents are at most a stripe's 1024: the product fits 64 bits
    if ((uint64_t)bx * by * bz <= j.small_vol) {
      TriSetup s;
      tri_setup(tv, j.u, s);
      mask = (bx <= 2 && by <= 2) ? vox_small_bricks(j, s, lo, bx, by, bz) : vox_small_factored(j, s, lo, bx, by, bz);
      if (j.item_mask && mask) {
        // stripe-local box origin (10 bits per axis) and extents - 1 (6 bits each)
        j.item_box[i] = (uint64_t)(lo[0] - j.sa[0]) | ((uint64_t)(lo[1] - j.sa[1]) << 10) |
                        ((uint64_t)(lo[2] - j.sa[2]) << 20) | ((uint64_t)(bx - 1) << 30) | ((uint64_t)(by - 1) << 36) |
                        ((uint64_t)(bz - 1) << 42);
      }
    } else {
      const uint64_t per_task = 32ull * j.lines_per_lane;
      cost = (item_lines(walk_axis(tv), lo, hi) + per_task - 1) / per_task;
    }
  }
  j.task_off[i] = cost;
  if (cost && j.task_flag) *j.task_flag = 1ull;  // the sub-batch has tasks: its scan runs
  if (j.item_mask) j.item_mask[i] = mask;
  return cost;
}

__device__ __forceinline__ uint64_t vox_small_occ_item(const VoxJob& j, uint64_t i) {
  return vox_small_occ_item(j, i, load_verts(j.tris, item_triangle(j, i), j.stride));
}

__global__ void k_vox_small_occ(VoxJob j) {
  pdl_enter();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < j.n_items) vox_small_occ_item(j, i);
}

// Pass 1 for small items: rank the voxels their pass mask names.
__device__ __forceinline__ void vox_small_win_item(const VoxJob& j, uint64_t i) {
  uint64_t mask = j.item_mask[i];
  if (!mask) return;
  const uint32_t t = (uint32_t)item_triangle(j, i);
  const uint64_t box = j.item_box[i];
  const uint32_t lx = (uint32_t)box & 1023u, ly = (uint32_t)(box >> 10) & 1023u, lz = (uint32_t)(box >> 20) & 1023u;
  const uint32_t by = (uint32_t)(box >> 36 & 63u) + 1u, bz = (uint32_t)(box >> 42 & 63u) + 1u;
  // q / d for q < 64, d <= 64 as (q * ceil(2^16 / d)) >> 16: the error of the rounded-up
  // reciprocal adds less than q / 2^16 < 1/d, which never carries past the next integer
  const uint32_t rz = (65535u + bz) / bz, ry = (65535u + by) / by;
  while (mask) {
    const uint32_t q = (uint32_t)(__ffsll((long long)mask) - 1);
    mask &= mask - 1;
    const uint32_t col = (q * rz) >> 16, z = q - col * bz;
    const uint32_t x = (col * ry) >> 16, y = col - x * by;
    const uint32_t m = morton_local(lx + x, ly + y, lz + z);
    atomicMin(&j.winners[leaf_rank(j, m)], t);
  }
}


// Lines 32*L*k .. 32*L*(k+1)-1 of large item i, L = lines_per_lane (lane, lane+32, ...).
// The projection test that does not depend on the walk coordinate, for line (ca, cb).
__device__ __forceinline__ bool line_passes(const VoxJob& j, const TriSetup& s, int W, int ca, int cb) {
  const float fa = __fmul_rn((float)ca, j.u), fb = __fmul_rn((float)cb, j.u);
  return W == 2 ? pass_xy(s, fa, fb) : (W == 0 ? pass_yz(s, fa, fb) : pass_zx(s, fb, fa));
}

// Lines of a task, first tested by every lane against the projection that does not
// depend on the walk coordinate; the lines that pass are packed into the warp's list
// (`lines_smem`, 32 x lines_per_lane entries) and then walked one per lane, so lanes
// do not idle beside lines outside the triangle.
template <int PASS>
__device__ __forceinline__ void vox_large_task(const VoxJob& j, uint64_t i, uint64_t k, int lane,
                                               uint32_t* __restrict__ lines_smem) {
  if (PASS == 1 && !j.winners) return;  // binary-mode stripe in a mixed batch: no winner pass
  const uint64_t t = item_triangle(j, i);
  const TriVerts tv = load_verts(j.tris, t, j.stride);
  int lo[3], hi[3];
  if (!item_box(j, tv, lo, hi)) return;  // cannot happen: the task count came from the same box
  const int W = walk_axis(tv);
  // lines of one item number at most 1024^2 (a stripe's face): 32-bit arithmetic
  const uint32_t ea = (uint32_t)(W == 0 ? hi[1] - lo[1] + 1 : hi[0] - lo[0] + 1);  // first axis across the walk
  const uint32_t lines = (uint32_t)item_lines(W, lo, hi);
  const uint32_t c0 = (uint32_t)k * 32u * j.lines_per_lane + (uint32_t)lane;
  TriSetup s;
  tri_setup(tv, j.u, s);
  const int top = max(hi[0], max(hi[1], hi[2]));
  const bool mono = monotone_setup(s, fabsf(__fmul_rn((float)(top + 1), j.u)));
  const float dir = (W == 0 ? s.n[0] : (W == 1 ? s.n[1] : s.n[2])) * j.u;
  const float inv_dir = 1.0f / dir;
  const int wlo = W == 0 ? lo[0] : (W == 1 ? lo[1] : lo[2]);
  const int whi = W == 0 ? hi[0] : (W == 1 ? hi[1] : hi[2]);
  const int alo = W == 0 ? lo[1] : lo[0], blo = W == 2 ? lo[1] : lo[2];
  // all 32 lanes: test, then pack the passing lines as (ca - alo) | (cb - blo) << 16
  const uint32_t lt = (1u << lane) - 1u;
  const uint32_t first = (uint32_t)k * 32u * j.lines_per_lane;  // the task's first line (same for all lanes)
  const uint32_t rounds = min(j.lines_per_lane, (lines - first + 31u) / 32u);
  uint32_t n = 0;
#pragma unroll 1
  for (uint32_t q = 0; q < rounds; q++) {
    const uint32_t c = c0 + 32u * q;
    const uint32_t ra = c % ea, rb = c / ea;
    const bool ok = c < lines && line_passes(j, s, W, alo + (int)ra, blo + (int)rb);
    const uint32_t vote = __ballot_sync(FULL, ok);
    if (ok) lines_smem[n + __popc(vote & lt)] = ra | (rb << 16);
    n += __popc(vote);
  }
  __syncwarp();
#pragma unroll 1
  for (uint32_t q = (uint32_t)lane; q < n; q += 32u) {
    const uint32_t r = lines_smem[q];
    vox_line<PASS>(j, s, (uint32_t)t, W, alo + (int)(r & 0xffffu), blo + (int)(r >> 16), wlo, whi, mono, dir, inv_dir);
  }
  __syncwarp();  // the list is free for the warp's next task
}

// Persistent warps pull 32-column tasks of large items from a global counter.
template <int PASS>
__global__ void __launch_bounds__(256, 4) k_vox_large(VoxJob j) {
  pdl_enter();
  extern __shared__ uint32_t lines_smem[];  // 32 x lines_per_lane per warp
  const int lane = threadIdx.x & 31;
  uint32_t* wl = lines_smem + (threadIdx.x >> 5) * 32u * j.lines_per_lane;
  const uint64_t total = j.task_off[j.n_items];
  if (total == 0) return;
  for (;;) {
    unsigned long long task = 0;
    if (lane == 0) task = atomicAdd(j.task_counter, 1ull);
    task = __shfl_sync(FULL, task, 0);
    if (task >= total) break;
    uint64_t lo_i = 0, hi_i = j.n_items;  // task_off[lo_i] <= task < task_off[hi_i]
    while (hi_i - lo_i > 1) {
      const uint64_t mid = (lo_i + hi_i) >> 1;
      if (j.task_off[mid] <= task) lo_i = mid;
      else hi_i = mid;
    }
    vox_large_task<PASS>(j, lo_i, task - j.task_off[lo_i], lane, wl);
  }
}

// ===========================================================================
// Occupancy pyramid: level l-1 bit i = (byte i of level l != 0); the byte is
// node i's 8-bit child mask.  Also the popcount of every 256-bit block.
// ===========================================================================
__device__ __forceinline__ uint32_t nonzero_bytes(uint32_t w) {
  const uint32_t t = (((w & 0x7f7f7f7fu) + 0x7f7f7f7fu) | w) & 0x80808080u;
  return ((t >> 7) & 1u) | ((t >> 14) & 2u) | ((t >> 21) & 4u) | ((t >> 28) & 8u);
}

// First word of level l (levels zl.. live in the buffer kept zero between builds).
__device__ __forceinline__ uint32_t* level_words(const Pyramid& p, int l) {
  return (l >= p.zl ? p.leaf : p.bits) + p.lv[l].off_w;
}

// Whether the leaf blocks under block b of level depth-1 (leaf blocks 8b..8b+7,
// one word of that block each) are all unmarked, so the block is zero.
// CG: the loads go to L2 (ld.global.cg), for data that other SMs wrote in the
// same launch (the persistent phase-A kernel); otherwise plain loads.
template <bool CG>
__device__ __forceinline__ uint4 ld4(const uint4* p) {
  if constexpr (CG) return __ldcg(p);
  else return *p;
}

template <bool CG = false>
__device__ __forceinline__ bool parent_block_empty(const Pyramid& p, uint64_t b) {
  const unsigned long long* t = reinterpret_cast<const unsigned long long*>(p.touch) + b;
  if constexpr (CG) return __ldcg(t) == 0ull;
  else return *t == 0ull;
}

// Block b of level l (not a marked leaf level): its popcount and parent word.
template <bool CG = false>
__device__ __forceinline__ void pyramid_block(const Pyramid& p, int l, uint64_t b) {
  const Level& L = p.lv[l];
  if (p.touch && l == p.depth - 1 && parent_block_empty<CG>(p, b)) {
    p.scan[L.off_b + b] = 0u;
    if (l > 0) level_words(p, l - 1)[b] = 0u;
    return;
  }
  const uint4* q = reinterpret_cast<const uint4*>(level_words(p, l) + 8 * b);
  const uint4 q0 = ld4<CG>(q), q1 = ld4<CG>(q + 1);
  const uint32_t w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
  uint32_t c = 0, pw = 0;
  uint64_t wo = 0;  // byte k: set bits in words 0..k-1 (at most 224)
#pragma unroll
  for (int k = 0; k < 8; k++) {
    wo |= (uint64_t)c << (8 * k);
    c += __popc(w[k]);
    pw |= nonzero_bytes(w[k]) << (4 * k);
  }
  p.scan[L.off_b + b] = c;
  if (l > 0) level_words(p, l - 1)[b] = pw;
  if (l == p.depth && p.woff) p.woff[b] = wo;
}

// Global node index of the first node of block blk of level l: the
// concatenated scan already counts every node of the shallower levels.
__device__ __forceinline__ uint64_t block_base(const Pyramid& p, int l, uint64_t blk) {
  if (l == p.depth && p.touch) return (uint64_t)p.scan[p.lv[l].off_b + blk / kLeafGroup] + p.local[blk];
  return p.scan[p.lv[l].off_b + blk];
}

// Global node index of bit `b` of level l.
__device__ __forceinline__ uint64_t node_index(const Pyramid& p, int l, uint64_t b) {
  const uint64_t blk = b >> 8;
  if (l == p.depth && p.woff) {  // the leaf level of a payload stripe: word offsets from the pyramid pass
    const uint32_t wi = (uint32_t)(b >> 5) & 7u;
    return block_base(p, l, blk) + ((p.woff[blk] >> (8 * wi)) & 0xffu) +
           __popc(level_words(p, l)[b >> 5] & ((1u << (b & 31)) - 1u));
  }
  return block_base(p, l, blk) + in_block_rank(level_words(p, l) + blk * 8, b);
}

// A marked leaf level, group q of kLeafGroup blocks: the parent words, the
// group's node count (its scan entry) and each marked block's offset in it.
template <bool CG = false>
__device__ __forceinline__ void leaf_group(const Pyramid& p, uint64_t q) {
  static_assert(kLeafGroup == 16, "one uint4 of marks per group");
  const Level& L = p.lv[p.depth];
  const uint4 m4 = ld4<CG>(reinterpret_cast<const uint4*>(p.touch) + q);
  uint4* parent = reinterpret_cast<uint4*>(level_words(p, p.depth - 1) + q * kLeafGroup);
  if (!(m4.x | m4.y | m4.z | m4.w)) {  // the parent words stay zero
    p.scan[L.off_b + q] = 0u;
    return;
  }
  const uint32_t mw[4] = {m4.x, m4.y, m4.z, m4.w};
  uint32_t pw[16];
  uint32_t total = 0;
#pragma unroll
  for (int k = 0; k < 16; k++) {
    pw[k] = 0u;
    if ((mw[k >> 2] >> (8 * (k & 3))) & 0xffu) {
      const uint64_t b = q * kLeafGroup + (uint64_t)k;
      const uint4* w4 = reinterpret_cast<const uint4*>(level_words(p, p.depth) + 8 * b);
      const uint4 q0 = ld4<CG>(w4), q1 = ld4<CG>(w4 + 1);
      const uint32_t w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
      uint32_t c = 0;
      uint64_t wo = 0;
#pragma unroll
      for (int i = 0; i < 8; i++) {
        wo |= (uint64_t)c << (8 * i);
        c += __popc(w[i]);
        pw[k] |= nonzero_bytes(w[i]) << (4 * i);
      }
      if (p.woff) p.woff[b] = wo;
      p.local[b] = (uint16_t)total;
      total += c;
    }
  }
  parent[0] = make_uint4(pw[0], pw[1], pw[2], pw[3]);
  parent[1] = make_uint4(pw[4], pw[5], pw[6], pw[7]);
  parent[2] = make_uint4(pw[8], pw[9], pw[10], pw[11]);
  parent[3] = make_uint4(pw[12], pw[13], pw[14], pw[15]);
  p.scan[L.off_b + q] = total;
}

__device__ __forceinline__ uint32_t child_mask(const Pyramid& p, int l, uint32_t k) {
  return (level_words(p, l)[k >> 2] >> ((k & 3) * 8)) & 0xffu;
}

// Keys of block lb of level l, from node index r on.
__device__ __forceinline__ void block_keys(const uint32_t* __restrict__ words, uint64_t lb, uint64_t r,
                                           uint32_t* __restrict__ keys) {
  const uint4* q = reinterpret_cast<const uint4*>(words + 8 * lb);
  const uint4 q0 = q[0], q1 = q[1];
  if (!(q0.x | q0.y | q0.z | q0.w | q1.x | q1.y | q1.z | q1.w)) return;
  const uint32_t w[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
  const uint64_t wl0 = lb * 8;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    uint32_t word = w[k];
    while (word) {
      const int bit = __ffs(word) - 1;
      keys[r++] = (uint32_t)(((wl0 + k) << 5) | (uint64_t)bit);
      word &= word - 1;
    }
  }
}

// Keys of all levels in one launch.  The elements of a stripe are the blocks
// of levels 0..depth-1 (blocks are 8 aligned words and never straddle two
// levels), padded to a multiple of 32, then the leaf level's scan entries,
// padded likewise, so every warp works on one region.  An unmarked leaf level
// has one element per block.  In a marked leaf level each lane takes a group
// of kLeafGroup blocks; the warp gathers the marked blocks of its 32 groups and
// hands them out one per lane.
__device__ __forceinline__ uint64_t compact_elems(const Pyramid& p) {
  const uint64_t upper = p.lv[p.depth].off_b - p.lv[0].off_b;
  return (upper + 31) / 32 * 32 + (p.lv[p.depth].nscan + 31) / 32 * 32;
}

__device__ __forceinline__ void compact_elem(const Pyramid& p, uint64_t e, uint32_t* __restrict__ keys) {
  const Level& L = p.lv[p.depth];
  const uint64_t first = p.lv[0].off_b, upper = L.off_b - first, up32 = (upper + 31) / 32 * 32;
  if (e >= compact_elems(p)) return;  // whole warps
  if (e < up32) {
    if (e >= upper) return;
    int l = p.depth - 1;  // most upper blocks are on the level above the leaves
    if (first + e < p.lv[l].off_b) {
      l = 0;
      while (p.lv[l + 1].off_b <= first + e) l++;
    }
    const uint64_t lb = first + e - p.lv[l].off_b;
    if (p.touch && l == p.depth - 1 && parent_block_empty(p, lb)) return;
    block_keys(level_words(p, l), lb, p.scan[first + e], keys);
    return;
  }
  const uint64_t q = e - up32;
  if (!p.touch) {
    if (q < L.nblocks) block_keys(level_words(p, p.depth), q, p.scan[L.off_b + q], keys);
    return;
  }
  // marked leaf level: all 32 lanes of the warp are here
  const int lane = threadIdx.x & 31;
  uint32_t marked = 0;  // bit k: block k of group q is marked
  if (q < L.nscan) {
    const uint4 m4 = reinterpret_cast<const uint4*>(p.touch)[q];
    marked = nonzero_bytes(m4.x) | (nonzero_bytes(m4.y) << 4) | (nonzero_bytes(m4.z) << 8) | (nonzero_bytes(m4.w) << 12);
  }
  const uint32_t cnt = __popc(marked);
  uint32_t incl = cnt;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, incl, o);
    if (lane >= o) incl += y;
  }
  const uint32_t total = __shfl_sync(FULL, incl, 31);
  const uint64_t q0 = q - (uint64_t)lane;
  for (uint32_t round = 0; round < total; round += 32) {
    const uint32_t j = round + (uint32_t)lane;  // this lane's marked block, in warp order
    uint32_t o = 0;                             // its owner lane: the first with incl > j
#pragma unroll
    for (uint32_t st = 16; st; st >>= 1) {
      const uint32_t t = __shfl_sync(FULL, incl, (int)(o + st - 1));
      if (t <= j) o += st;
    }
    uint32_t m = __shfl_sync(FULL, marked, (int)o);
    const uint32_t before = __shfl_sync(FULL, incl - cnt, (int)o);
    if (j < total) {
      for (uint32_t k = j - before; k; k--) m &= m - 1;
      const uint64_t qo = q0 + o;
      const uint64_t blk = qo * kLeafGroup + (uint64_t)(__ffs(m) - 1);
      block_keys(level_words(p, p.depth), blk, (uint64_t)p.scan[L.off_b + qo] + p.local[blk], keys);
    }
  }
}

// Mark bytes 16i .. 16i+15 of a stripe: zero their marked leaf blocks, the
// group's 16 parent words, then the marks.  A stripe without marks has its 16
// leaf blocks zeroed outright.
__device__ __forceinline__ void clean_touch16(const Pyramid& p, uint64_t i) {
  if (i * 16 >= touch_bytes(p.lv[p.depth])) return;
  if (!p.touch) {  // T threads zero the level's 2 x nblocks <= 32 T uint4, coalesced
    const uint64_t T = touch_bytes(p.lv[p.depth]) / 16, n4 = p.lv[p.depth].nwords / 4;
    uint4* leaf = reinterpret_cast<uint4*>(level_words(p, p.depth));
    for (uint64_t q = i; q < n4; q += T) leaf[q] = make_uint4(0u, 0u, 0u, 0u);
    return;
  }
  uint4* t4 = reinterpret_cast<uint4*>(p.touch) + i;
  const uint4 t = *t4;
  if (!(t.x | t.y | t.z | t.w)) return;
  const uint4 z = make_uint4(0u, 0u, 0u, 0u);
  *t4 = z;
  uint4* parent = reinterpret_cast<uint4*>(level_words(p, p.depth - 1) + i * 16);  // the group's 16 parent words
  parent[0] = z;
  parent[1] = z;
  parent[2] = z;
  parent[3] = z;
  uint4* leaf = reinterpret_cast<uint4*>(level_words(p, p.depth));
  const uint32_t tw[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const uint32_t nz = nonzero_bytes(tw[q]);  // bit k: mark byte k of this word is set
    for (uint32_t m = nz; m; m &= m - 1) {
      const uint64_t blk = i * 16 + (uint64_t)(4 * q + __ffs(m) - 1);
      leaf[2 * blk] = z;
      leaf[2 * blk + 1] = z;
    }
  }
}

// ===========================================================================
// Leaf payload (voxelizer.cpp:295-299, BarycentricCoords.h, main.cpp:373-382)
// ===========================================================================
__device__ void payload_color(const TriVerts& tv, const float n[3], int x, int y, int z, float unit_div,
                              const float* __restrict__ tr, float col[3]) {
  const float qx = __fdiv_rn((float)x, unit_div);
  const float qy = __fdiv_rn((float)y, unit_div);
  const float qz = __fdiv_rn((float)z, unit_div);
  const float coeffD = -dot3(tv.v[0][0], tv.v[0][1], tv.v[0][2], n[0], n[1], n[2]);
  const float nn = __fadd_rn(__fadd_rn(__fmul_rn(n[0], n[0]), __fmul_rn(n[1], n[1])), __fmul_rn(n[2], n[2]));
  const float k = __fdiv_rn(__fadd_rn(dot3(qx, qy, qz, n[0], n[1], n[2]), coeffD), nn);
  const float ptx = __fsub_rn(qx, __fmul_rn(k, n[0]));
  const float pty = __fsub_rn(qy, __fmul_rn(k, n[1]));
  const float ptz = __fsub_rn(qz, __fmul_rn(k, n[2]));
  // inverse(mat3(v0, v1, v2)) by adjugate over determinant
  const float a = tv.v[0][0], b = tv.v[1][0], c = tv.v[2][0];
  const float d = tv.v[0][1], e = tv.v[1][1], f = tv.v[2][1];
  const float g = tv.v[0][2], h = tv.v[1][2], i = tv.v[2][2];
  const float C00 = __fsub_rn(__fmul_rn(e, i), __fmul_rn(f, h));
  const float C01 = __fsub_rn(__fmul_rn(f, g), __fmul_rn(d, i));
  const float C02 = __fsub_rn(__fmul_rn(d, h), __fmul_rn(e, g));
  const float det = __fadd_rn(__fadd_rn(__fmul_rn(a, C00), __fmul_rn(b, C01)), __fmul_rn(c, C02));
  const float r = __fdiv_rn(1.0f, det);
  const float C10 = __fsub_rn(__fmul_rn(c, h), __fmul_rn(b, i));
  const float C11 = __fsub_rn(__fmul_rn(a, i), __fmul_rn(c, g));
  const float C12 = __fsub_rn(__fmul_rn(b, g), __fmul_rn(a, h));
  const float C20 = __fsub_rn(__fmul_rn(b, f), __fmul_rn(c, e));
  const float C21 = __fsub_rn(__fmul_rn(c, d), __fmul_rn(a, f));
  const float C22 = __fsub_rn(__fmul_rn(a, e), __fmul_rn(b, d));
  const float i00 = __fmul_rn(C00, r), i10 = __fmul_rn(C01, r), i20 = __fmul_rn(C02, r);
  const float i01 = __fmul_rn(C10, r), i11 = __fmul_rn(C11, r), i21 = __fmul_rn(C12, r);
  const float i02 = __fmul_rn(C20, r), i12 = __fmul_rn(C21, r), i22 = __fmul_rn(C22, r);
  const float bx = __fadd_rn(__fadd_rn(__fmul_rn(i00, ptx), __fmul_rn(i01, pty)), __fmul_rn(i02, ptz));
  const float by = __fadd_rn(__fadd_rn(__fmul_rn(i10, ptx), __fmul_rn(i11, pty)), __fmul_rn(i12, ptz));
  const float bz = __fadd_rn(__fadd_rn(__fmul_rn(i20, ptx), __fmul_rn(i21, pty)), __fmul_rn(i22, ptz));
#pragma unroll
  for (int q = 0; q < 3; q++) {
    const float c0 = __ldg(tr + 12 + q), c1 = __ldg(tr + 15 + q), c2 = __ldg(tr + 18 + q);
    col[q] = __fadd_rn(__fadd_rn(__fmul_rn(bx, c0), __fmul_rn(by, c1)), __fmul_rn(bz, c2));
  }
}

// Colour and normal of leaf `li` (its index within the leaf level), local key `key`.
// Returns false (and flags) if the leaf has no winning triangle.
__device__ bool leaf_value(const EmitJob& e, uint64_t li, uint32_t key, float out[6]) {
  uint32_t lx, ly, lz;
  morton_local_decode(key, lx, ly, lz);
  const int x = e.origin[0] + (int)lx, y = e.origin[1] + (int)ly, z = e.origin[2] + (int)lz;
  const uint64_t t = e.winners[li];
  if (t >= e.n_tris) {  // every set voxel has a passing triangle; anything else is a bug
    atomicOr(e.flag, 4u);
    return false;
  }
  const float* tr = e.tris + t * 21;
  const float nx = __ldg(tr + 9), ny = __ldg(tr + 10), nz = __ldg(tr + 11);
  if (e.color_mode == 1) {  // COLOR_FIXED
    out[0] = out[1] = out[2] = 1.0f;
  } else if (e.color_mode == 2) {  // COLOR_LINEAR: mortonToRGB (svo_builder_util.h:14-18)
    const float fn = (float)e.gridsize;
    out[0] = __fdiv_rn((float)z, fn);
    out[1] = __fdiv_rn((float)y, fn);
    out[2] = __fdiv_rn((float)x, fn);
  } else if (e.color_mode == 3) {  // COLOR_NORMAL
    float a = nx, b = ny, c = nz;
    normalize3(a, b, c);
    out[0] = __fdiv_rn(__fadd_rn(a, 1.0f), 2.0f);
    out[1] = __fdiv_rn(__fadd_rn(b, 1.0f), 2.0f);
    out[2] = __fdiv_rn(__fadd_rn(c, 1.0f), 2.0f);
  } else {  // COLOR_FROM_MODEL
    const TriVerts tv = load_verts(e.tris, t, 21);
    float n[3];
    tri_normal(tv, n);
    payload_color(tv, n, x, y, z, e.unit_div, tr, out);
  }
  out[3] = nx;
  out[4] = ny;
  out[5] = nz;
  return true;
}

__device__ __forceinline__ void store_data_record(const EmitJob& e, uint64_t idx, uint64_t morton, const float* v);

// Leaf payloads: with -levels into the per-node cache (the averages need them);
// without, straight into the data file, where leaf i of the stripe is data record
// data_base + i (its data records are its leaves in key order), so the data file
// is final before the node records are laid out.
__device__ __forceinline__ void leaf_payload(const Pyramid& p, const EmitJob& e, uint64_t i) {
  const Level& L = p.lv[p.depth];
  const uint32_t k = e.keys[L.koff + i];
  float v[6];
  if (!leaf_value(e, i, k, v)) return;
  if (e.levels) {
    float* out = e.cache + (L.koff + i) * 6;
#pragma unroll
    for (int q = 0; q < 6; q++) out[q] = v[q];
  } else {
    store_data_record(e, e.data_base + i, e.stripe_base + k, v);
  }
}

// ===========================================================================
// Octree layout.  Subtree sizes bottom-up, then top-down the index of the
// first node / data record written inside every subtree; the reference writes
// a node's 8-child group when the Morton cursor leaves the node's region, so
// the node file is the post-order of groups (OctreeBuilder.cpp:58-128).
// ===========================================================================
__device__ __forceinline__ void average_children(const EmitJob& e, uint32_t mask, uint64_t c0, bool child_leaf,
                                                 float out[6]) {
  // OctreeBuilder.cpp:81-99: sum over the 8 slots in child order (null slots
  // add zero), divide by the non-null count, normalise the normal.
  float acc[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  float notnull = 0.0f;
  uint64_t c = c0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    if ((mask >> k) & 1u) {
      notnull = __fadd_rn(notnull, 1.0f);
      if (child_leaf && e.binary) {
#pragma unroll
        for (int q = 0; q < 6; q++) acc[q] = __fadd_rn(acc[q], 0.0f);
      } else {
        const float* cc = e.cache + c * 6;
#pragma unroll
        for (int q = 0; q < 6; q++) acc[q] = __fadd_rn(acc[q], cc[q]);
      }
      c++;
    } else {
#pragma unroll
      for (int q = 0; q < 6; q++) acc[q] = __fadd_rn(acc[q], 0.0f);
    }
  }
  out[0] = __fdiv_rn(acc[0], notnull);
  out[1] = __fdiv_rn(acc[1], notnull);
  out[2] = __fdiv_rn(acc[2], notnull);
  float tx = __fdiv_rn(acc[3], notnull), ty = __fdiv_rn(acc[4], notnull), tz = __fdiv_rn(acc[5], notnull);
  normalize3(tx, ty, tz);
  out[3] = tx;
  out[4] = ty;
  out[5] = tz;
}

// Subtree node / data counts, first-child index and (-levels) averages of node i of level l.
__device__ __forceinline__ void bottom_up_node(const Pyramid& p, const EmitJob& e, int l, uint64_t i) {
  const Level& L = p.lv[l];
  const uint64_t gi = L.koff + i;
  const uint32_t k = e.keys[gi];
  const uint32_t mask = child_mask(p, l + 1, k);
  const int nch = __popc(mask);
  const uint64_t c0 = node_index(p, l + 1, (uint64_t)k << 3);
  const bool child_leaf = (l + 1 == p.depth);
  uint32_t sz, dsz;
  if (child_leaf) {
    sz = 1u + (uint32_t)nch;
    dsz = (uint32_t)e.levels + (e.binary ? 0u : (uint32_t)nch);
  } else {
    sz = 1u;
    dsz = (uint32_t)e.levels;
    for (int q = 0; q < nch; q++) {
      sz += e.size[c0 + q];
      dsz += e.dsize[c0 + q];
    }
  }
  e.size[gi] = sz;
  e.dsize[gi] = dsz;
  e.first_child[gi] = (uint32_t)c0;
  if (e.levels) average_children(e, mask, c0, child_leaf, e.cache + gi * 6);
}

__device__ __forceinline__ void store_data_record(const EmitJob& e, uint64_t idx, uint64_t morton, const float* v) {
  if (idx < e.data_win_base || idx - e.data_win_base >= e.data_win_len) {
    atomicOr(e.flag, 2u);
    return;
  }
  uint4* dst = reinterpret_cast<uint4*>(e.data_win + (idx - e.data_win_base) * 32);
  dst[0] = make_uint4((uint32_t)morton, (uint32_t)(morton >> 32), __float_as_uint(v[0]), __float_as_uint(v[1]));
  dst[1] = make_uint4(__float_as_uint(v[2]), __float_as_uint(v[3]), __float_as_uint(v[4]), __float_as_uint(v[5]));
}

__device__ __forceinline__ void store_node_record(const EmitJob& e, uint64_t pos, uint64_t r0, uint64_t r1,
                                                  uint64_t r2) {
  if (pos < e.node_win_base || pos - e.node_win_base >= e.node_win_len) {
    atomicOr(e.flag, 1u);
    return;
  }
  uint64_t* rec = e.node_win + (pos - e.node_win_base) * 3;
  rec[0] = r0;
  rec[1] = r1;
  rec[2] = r2;
}

__device__ __forceinline__ uint64_t child_offsets(uint32_t mask) {
  uint64_t off = 0;
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const uint64_t byte = ((mask >> k) & 1u) ? (uint64_t)(r++) : 0xffull;
    off |= byte << (8 * k);
  }
  return off;
}

// Node i of level l (internal) writes its children's records: they form one
// contiguous group at its children_base, in child order (groupNodes,
// OctreeBuilder.cpp:58-79), and each child's subtree starts where the
// previous sibling's subtree ended.
__device__ __forceinline__ void top_down_node(const Pyramid& p, const EmitJob& e, int l, uint64_t i) {
  const Level& L = p.lv[l];
  const uint64_t gi = L.koff + i;
  const uint32_t k = e.keys[gi];
  const uint32_t mask = child_mask(p, l + 1, k);
  const int nch = __popc(mask);
  const uint64_t st = e.node_base + e.start[gi];
  uint64_t run_d = e.data_base + e.dstart[gi];
  uint64_t run_s = st;
  const uint64_t cb = st + (uint64_t)e.size[gi] - 1 - (uint64_t)nch;
  const uint64_t c0 = e.first_child[gi];
  const bool child_leaf = (l + 1 == p.depth);
  if (!child_leaf) {
    // every child's loads first (they are independent), then the running sums and stores
    uint32_t kc[8], szc[8], dszc[8], mc[8];
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (j < nch) {
        kc[j] = e.keys[c0 + j];
        szc[j] = e.size[c0 + j];
        dszc[j] = e.dsize[c0 + j];
      }
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (j < nch) mc[j] = child_mask(p, l + 2, kc[j]);
#pragma unroll
    for (int j = 0; j < 8; j++)
      if (j < nch) {
        const uint64_t c = c0 + (uint64_t)j;
        e.start[c] = (uint32_t)(run_s - e.node_base);
        e.dstart[c] = (uint32_t)(run_d - e.data_base);
        const uint64_t di = run_d + dszc[j] - 1;
        store_node_record(e, cb + j, e.levels ? di : 0, run_s + szc[j] - 1 - (uint64_t)__popc(mc[j]),
                          child_offsets(mc[j]));
        if (e.levels) store_data_record(e, di, 0, e.cache + c * 6);
        run_s += szc[j] - 1;
        run_d += dszc[j];
      }
    return;
  }
  for (int j = 0; j < nch; j++) {
    const uint64_t c = c0 + (uint64_t)j;
    const uint32_t kc = e.keys[c];
    if (e.binary) {
      store_node_record(e, cb + j, 1, 0, ~0ull);
    } else {
      store_node_record(e, cb + j, run_d, 0, ~0ull);
      if (!e.leaf_inline) {  // (without -levels the leaf payload pass wrote the data record)
        float v[6];
#pragma unroll
        for (int q = 0; q < 6; q++) v[q] = e.cache[c * 6 + q];
        store_data_record(e, run_d, e.stripe_base + kc, v);
      }
      run_d += 1;
    }
  }
}

// Children of level l+1, one thread per child, two at once (i0 < i1; either may
// be past the level's end).  A child finds its parent's run starts and adds its
// earlier siblings' subtree sizes (siblings are consecutive in the key order), so
// the launch reads and writes the child level contiguously.  Every load of both
// children is issued before the first store, so their chains of dependent loads
// overlap.
__device__ __forceinline__ void top_down_children(const Pyramid& p, const EmitJob& e, int l, uint64_t i0, uint64_t i1) {
  const Level& C = p.lv[l + 1];
  if (i0 >= C.n) return;
  const bool v1 = i1 < C.n;
  const uint64_t c0 = C.koff + i0, c1 = C.koff + (v1 ? i1 : i0);
  const uint32_t kc0 = e.keys[c0], kc1 = e.keys[c1];
  const uint64_t p0 = node_index(p, l, kc0 >> 3), p1 = node_index(p, l, kc1 >> 3);
  const uint64_t f0 = e.first_child[p0], f1 = e.first_child[p1];
  const uint32_t pm0 = child_mask(p, l + 1, kc0 >> 3), pm1 = child_mask(p, l + 1, kc1 >> 3);
  uint64_t rs0 = e.node_base + e.start[p0], rd0 = e.data_base + e.dstart[p0];
  uint64_t rs1 = e.node_base + e.start[p1], rd1 = e.data_base + e.dstart[p1];
  const uint64_t cb0 = rs0 + (uint64_t)e.size[p0] - 1 - (uint64_t)__popc(pm0);
  const uint64_t cb1 = rs1 + (uint64_t)e.size[p1] - 1 - (uint64_t)__popc(pm1);
  const uint32_t mc0 = child_mask(p, l + 2, kc0), mc1 = child_mask(p, l + 2, kc1);
  const uint64_t sz0 = e.size[c0], dsz0 = e.dsize[c0], sz1 = e.size[c1], dsz1 = e.dsize[c1];
  for (uint64_t q = f0; q < c0; q++) {
    rs0 += (uint64_t)e.size[q] - 1;
    rd0 += e.dsize[q];
  }
  for (uint64_t q = f1; q < c1; q++) {
    rs1 += (uint64_t)e.size[q] - 1;
    rd1 += e.dsize[q];
  }
  e.start[c0] = (uint32_t)(rs0 - e.node_base);
  e.dstart[c0] = (uint32_t)(rd0 - e.data_base);
  const uint64_t di0 = rd0 + dsz0 - 1;
  store_node_record(e, cb0 + (c0 - f0), e.levels ? di0 : 0, rs0 + sz0 - 1 - (uint64_t)__popc(mc0), child_offsets(mc0));
  if (e.levels) store_data_record(e, di0, 0, e.cache + c0 * 6);
  if (!v1) return;
  e.start[c1] = (uint32_t)(rs1 - e.node_base);
  e.dstart[c1] = (uint32_t)(rd1 - e.data_base);
  const uint64_t di1 = rd1 + dsz1 - 1;
  store_node_record(e, cb1 + (c1 - f1), e.levels ? di1 : 0, rs1 + sz1 - 1 - (uint64_t)__popc(mc1), child_offsets(mc1));
  if (e.levels) store_data_record(e, di1, 0, e.cache + c1 * 6);
}

// Leaf records, one thread per leaf: the parent (level depth-1) already knows
// where its child group and data run start.
__device__ __forceinline__ void top_down_leaf(const Pyramid& p, const EmitJob& e, uint64_t i) {
  const Level& L = p.lv[p.depth];
  const uint64_t gi = L.koff + i;
  const uint32_t k = e.keys[gi];
  const uint32_t pk = k >> 3;
  const uint64_t pidx = node_index(p, p.depth - 1, pk);
  const uint64_t rank = gi - e.first_child[pidx];
  const uint32_t pmask = child_mask(p, p.depth, pk);
  const uint64_t pcb = e.node_base + e.start[pidx] + (uint64_t)e.size[pidx] - 1 - (uint64_t)__popc(pmask);
  if (e.binary) {
    store_node_record(e, pcb + rank, 1, 0, ~0ull);
    return;
  }
  const uint64_t di = e.data_base + e.dstart[pidx] + rank;
  store_node_record(e, pcb + rank, di, 0, ~0ull);
  if (e.leaf_inline) return;  // the leaf payload pass wrote the data record
  float v[6];
#pragma unroll
  for (int q = 0; q < 6; q++) v[q] = e.cache[gi * 6 + q];
  store_data_record(e, di, e.stripe_base + k, v);
}

// Stripe root: child mask and payload for the host, and (with -levels, or a
// one-voxel stripe in payload mode) the root's own data record.
__device__ void root_info(const Pyramid& p, const EmitJob& e, uint64_t data_base, uint32_t* out) {
  const uint64_t r0 = p.lv[0].koff;  // global node index of the stripe root
  float c[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
  if (p.depth >= 1) {
    if (e.levels)
      for (int q = 0; q < 6; q++) c[q] = e.cache[r0 * 6 + q];
  } else if (!e.binary) {
    if (e.cache) {
      for (int q = 0; q < 6; q++) c[q] = e.cache[r0 * 6 + q];
    } else {
      leaf_value(e, 0, 0, c);
    }
  }
  out[0] = p.depth >= 1 ? child_mask(p, 1, 0) : 0u;
  for (int q = 0; q < 6; q++) out[1 + q] = __float_as_uint(c[q]);
  if (p.depth >= 1) {
    if (e.levels) store_data_record(e, data_base + e.dsize[r0] - 1, 0, c);
  } else if (!e.binary) {
    store_data_record(e, data_base, e.stripe_base, c);
  }
}

// n words into `dst` (mapped pinned host memory): small results the host waits for
// travel as the kernel's stores, not as copies queued on the copy engine.
__global__ void k_copy_words(const uint32_t* __restrict__ src, uint64_t n, uint32_t* __restrict__ dst) {
  pdl_enter();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

__global__ void k_scatter_records(const uint64_t* __restrict__ src, uint64_t n, int words, uint64_t* __restrict__ dst) {
  pdl_enter();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t* s = src + i * (1 + words);
  uint64_t* d = dst + s[0] * words;
  for (int q = 0; q < words; q++) d[q] = s[1 + q];
}

// Records with their own destination: src[i] = {address, words...}.
__global__ void k_scatter_to(const uint64_t* __restrict__ src, uint64_t n, int words) {
  pdl_enter();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const uint64_t* s = src + i * (1 + words);
  uint64_t* d = reinterpret_cast<uint64_t*>(s[0]);
  for (int q = 0; q < words; q++) d[q] = s[1 + q];
}

// ===========================================================================
// Batched forms: every stripe of a batch in one launch.  A chunk table gives
// each CTA one stripe and a run of at most kChunk elements; the CTA copies that
// stripe's job into shared memory and runs the per-element bodies above.
// ===========================================================================
template <typename T>
__device__ __forceinline__ void stage(T& dst, const T& src) {
  static_assert(sizeof(T) % 4 == 0, "staged structs are word-sized");
  const uint32_t* s = reinterpret_cast<const uint32_t*>(&src);
  uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
  for (uint32_t q = threadIdx.x; q < sizeof(T) / 4; q += blockDim.x) d[q] = s[q];
}

// CTA b belongs to the stripe s with cta_beg[s] <= b < cta_beg[s+1]; it is
// the stripe's CTA b - cta_beg[s] and covers the elements per CTA of its
// launch from there (kChunk, or kChunk * ept for the per-block and per-node
// launches, each thread taking one element of every kChunk-wide chunk).
__device__ __forceinline__ uint32_t cta_stripe(const uint64_t* __restrict__ cta_beg, uint32_t n, uint64_t& cta) {
  __shared__ uint32_t s_stripe;
  if (threadIdx.x == 0) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (cta_beg[mid] <= blockIdx.x) lo = mid;
      else hi = mid;
    }
    s_stripe = lo;
  }
  __syncthreads();
  const uint32_t s = s_stripe;
  cta = (uint64_t)(blockIdx.x - cta_beg[s]);  // the CTA's index within its stripe
  return s;
}

// A one-stripe launch (SINGLE) takes the stripe's job as a kernel parameter
// and indexes elements directly; a batch launch finds its stripe first and
// stages the job in shared memory.
template <int PASS, bool SINGLE>
__global__ void __launch_bounds__(kChunk, 4) kb_vox_small(const VoxJob* __restrict__ jobs,
                                                       const uint64_t* __restrict__ cta_beg, uint32_t n, VoxJob j0) {
  pdl_enter();
  if constexpr (SINGLE) {
    const uint64_t i = (uint64_t)blockIdx.x * kChunk + threadIdx.x;
    if (i >= j0.n_items) return;
    if (PASS == 0) vox_small_occ_item(j0, i);
    else vox_small_win_item(j0, i);
  } else {
    __shared__ VoxJob sj;
    uint64_t cta;
    const uint32_t s = cta_stripe(cta_beg, n, cta);
    stage(sj, jobs[s]);
    __syncthreads();
    const uint64_t i = cta * kChunk + threadIdx.x;
    if (i >= sj.n_items) return;
    if (PASS == 0) vox_small_occ_item(sj, i);
    else vox_small_win_item(sj, i);
  }
}

// The item and stripe of every warp task: map[t] = item | stripe << 32, one thread
// per item writing its tasks' entries.  Written only when all tasks fit in `cap`.
__global__ void __launch_bounds__(kChunk) kb_task_map(const uint64_t* __restrict__ cta_beg, uint32_t n,
                                                      const uint64_t* __restrict__ item_beg,
                                                      const uint64_t* __restrict__ task_off, uint64_t total_items,
                                                      uint64_t* __restrict__ map, uint64_t cap) {
  pdl_enter();
  uint64_t cta;
  const uint32_t s = cta_stripe(cta_beg, n, cta);
  if (task_off[total_items] > cap) return;
  const uint64_t i = item_beg[s] + cta * kChunk + threadIdx.x;
  if (i >= item_beg[s + 1]) return;
  for (uint64_t t = task_off[i], e = task_off[i + 1]; t < e; t++) map[t] = i | ((uint64_t)s << 32);
}

template <int PASS>
__global__ void __launch_bounds__(256, 4) kb_vox_large(const VoxJob* __restrict__ jobs, const uint64_t* __restrict__ item_beg,
                                                    uint32_t n_stripes, const uint64_t* __restrict__ task_off,
                                                    uint64_t total_items, unsigned long long* counter,
                                                    uint32_t lines_per_lane, const uint64_t* __restrict__ map,
                                                    uint64_t cap) {
  pdl_enter();
  extern __shared__ uint32_t lines_smem[];  // 32 x lines_per_lane per warp (every job has this lines_per_lane)
  const int lane = threadIdx.x & 31;
  uint32_t* wl = lines_smem + (threadIdx.x >> 5) * 32u * lines_per_lane;
  const uint64_t total = task_off[total_items];
  if (total == 0) return;  // no large items in this launch: no counter traffic
  for (;;) {
    unsigned long long task = 0;
    if (lane == 0) task = atomicAdd(counter, 1ull);
    task = __shfl_sync(FULL, task, 0);
    if (task >= total) break;
    uint64_t lo_i = 0;
    uint32_t s0 = 0;
    if (total <= cap) {  // one load instead of two searches of dependent loads
      const uint64_t v = map[task];
      lo_i = (uint32_t)v;
      s0 = (uint32_t)(v >> 32);
    } else {
      uint64_t hi_i = total_items;  // task_off[lo_i] <= task < task_off[hi_i]
      while (hi_i - lo_i > 1) {
        const uint64_t mid = (lo_i + hi_i) >> 1;
        if (task_off[mid] <= task) lo_i = mid;
        else hi_i = mid;
      }
      uint32_t s1 = n_stripes;  // item_beg[s0] <= lo_i < item_beg[s1]
      while (s1 - s0 > 1) {
        const uint32_t mid = (s0 + s1) >> 1;
        if (item_beg[mid] <= lo_i) s0 = mid;
        else s1 = mid;
      }
    }
    vox_large_task<PASS>(jobs[s0], lo_i - item_beg[s0], task - task_off[lo_i], lane, wl);
  }
}

// Element e of level l: a block, or a group of blocks of a marked leaf level.
template <bool CG = false>
__device__ __forceinline__ void pyramid_elem(const Pyramid& p, int l, uint64_t e) {
  if (l == p.depth && p.touch) leaf_group<CG>(p, e);
  else pyramid_block<CG>(p, l, e);
}

// Level depth - r of every stripe that has CTAs in this launch.
template <bool SINGLE>
__global__ void __launch_bounds__(kChunk) kb_pyramid(const Pyramid* __restrict__ pyrs,
                                                     const uint64_t* __restrict__ cta_beg, uint32_t n, int r, uint32_t ept,
                                                     Pyramid p0) {
  pdl_enter();
  if constexpr (SINGLE) {
    const int l = p0.depth - r;
    for (uint32_t k = 0; k < ept; k++) {
      const uint64_t b = ((uint64_t)blockIdx.x * ept + k) * kChunk + threadIdx.x;
      if (b < p0.lv[l].nscan) pyramid_elem(p0, l, b);
    }
  } else {
    __shared__ Pyramid sp;
    uint64_t cta;
    const uint32_t s = cta_stripe(cta_beg, n, cta);
    stage(sp, pyrs[s]);
    __syncthreads();
    const int l = sp.depth - r;
    for (uint32_t k = 0; k < ept; k++) {
      const uint64_t b = (cta * ept + k) * kChunk + threadIdx.x;
      if (b < sp.lv[l].nscan) pyramid_elem(sp, l, b);
    }
  }
}

__global__ void kb_pyramid_top(const Pyramid* __restrict__ pyrs, int l_hi, uint32_t* __restrict__ scan_end) {
  pdl_enter();
  if (blockIdx.x == 0 && threadIdx.x == 0) *scan_end = 0u;  // the scan's total entry
  __shared__ Pyramid sp;
  stage(sp, pyrs[blockIdx.x]);
  __syncthreads();
  for (int l = l_hi < sp.depth ? l_hi : sp.depth; l >= 0; l--) {
    for (uint64_t b = threadIdx.x; b < sp.lv[l].nblocks; b += blockDim.x) pyramid_block(sp, l, b);
    // the padding words of level l-1 (levels 0..2 are padded to a whole block)
    if (l > 0)
      for (uint64_t w = sp.lv[l].nblocks + threadIdx.x; w < sp.lv[l - 1].nwords; w += blockDim.x)
        level_words(sp, l - 1)[w] = 0u;
    __syncthreads();
  }
}

// Zero the marked leaf blocks and the marks of every stripe.
template <bool SINGLE>
__global__ void __launch_bounds__(kChunk) kb_clean_leaves(const Pyramid* __restrict__ pyrs,
                                                          const uint64_t* __restrict__ cta_beg, uint32_t n, uint32_t ept,
                                                          Pyramid p0) {
  pdl_enter();
  if constexpr (SINGLE) {
    for (uint32_t k = 0; k < ept; k++) clean_touch16(p0, ((uint64_t)blockIdx.x * ept + k) * kChunk + threadIdx.x);
  } else {
    __shared__ Pyramid sp;
    uint64_t cta;
    const uint32_t s = cta_stripe(cta_beg, n, cta);
    stage(sp, pyrs[s]);
    __syncthreads();
    for (uint32_t k = 0; k < ept; k++) clean_touch16(sp, (cta * ept + k) * kChunk + threadIdx.x);
  }
}

// Every block of every level of the stripe.
template <bool SINGLE>
__global__ void __launch_bounds__(kChunk) kb_compact(const Pyramid* __restrict__ pyrs,
                                                     const uint64_t* __restrict__ cta_beg, uint32_t n,
                                                     uint32_t* __restrict__ keys, uint32_t ept, Pyramid p0) {
  pdl_enter();
  if constexpr (SINGLE) {
    for (uint32_t k = 0; k < ept; k++)
      compact_elem(p0, ((uint64_t)blockIdx.x * ept + k) * kChunk + threadIdx.x, keys);
  } else {
    __shared__ Pyramid sp;
    uint64_t cta;
    const uint32_t s = cta_stripe(cta_beg, n, cta);
    stage(sp, pyrs[s]);
    __syncthreads();
    for (uint32_t k = 0; k < ept; k++) compact_elem(sp, (cta * ept + k) * kChunk + threadIdx.x, keys);
  }
}

// Also copies *tasks to *tasks_out and, when `code` is set, *code to *code_out.
__global__ void kb_level_bases(const Pyramid* __restrict__ pyrs, uint32_t n_stripes, uint32_t* __restrict__ out,
                               const uint64_t* __restrict__ tasks, uint64_t* __restrict__ tasks_out,
                               uint32_t* __restrict__ flag, const uint64_t* __restrict__ code,
                               uint64_t* __restrict__ code_out) {
  pdl_enter();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) {
    *tasks_out = *tasks;
    if (code) *code_out = *code;
    *flag = 0u;  // the layout check flag of the sub-batch's record kernels
  }
  if (s >= n_stripes) return;
  const Pyramid& p = pyrs[s];
  uint32_t* o = out + (uint64_t)s * (kMaxLevels + 1);
  for (int l = 0; l <= p.depth; l++) o[l] = p.scan[p.lv[l].off_b];
  o[p.depth + 1] = p.scan[p.lv[p.depth].off_b + p.lv[p.depth].nscan];
}

// Kinds of per-node launches that take (Pyramid, EmitJob) pairs.
enum NodeOp { OP_LEAF_PAYLOAD = 0, OP_BOTTOM_UP = 1, OP_TOP_DOWN = 2, OP_LEAVES = 3 };

template <int OP>
__device__ __forceinline__ void node_op(const Pyramid& p, const EmitJob& e, int arg, uint64_t i) {
  if (OP == OP_LEAF_PAYLOAD) {
    if (i < p.lv[p.depth].n) leaf_payload(p, e, i);
  } else if (OP == OP_BOTTOM_UP) {
    const int l = p.depth - arg;  // arg = distance from the leaf level
    if (i < p.lv[l].n) bottom_up_node(p, e, l, i);
  } else if (OP == OP_TOP_DOWN) {
    top_down_children(p, e, arg, i, ~0ull);  // arg = absolute parent level
  } else {
    if (i < p.lv[p.depth].n) top_down_leaf(p, e, i);
  }
}

template <int OP, bool SINGLE>
__global__ void __launch_bounds__(kChunk) kb_nodes(const Pyramid* __restrict__ pyrs, const EmitJob* __restrict__ emits,
                                                   const uint64_t* __restrict__ cta_beg, uint32_t n, int arg, uint32_t ept,
                                                   Pyramid p0, EmitJob e0) {
  pdl_enter();
  if constexpr (SINGLE) {
    if constexpr (OP == OP_TOP_DOWN) {
      for (uint32_t k = 0; k < ept; k += 2) {
        const uint64_t i = ((uint64_t)blockIdx.x * ept + k) * kChunk + threadIdx.x;
        top_down_children(p0, e0, arg, i, k + 1 < ept ? i + kChunk : ~0ull);
      }
    } else {
      for (uint32_t k = 0; k < ept; k++) node_op<OP>(p0, e0, arg, ((uint64_t)blockIdx.x * ept + k) * kChunk + threadIdx.x);
    }
  } else {
    __shared__ Pyramid sp;
    __shared__ EmitJob se;
    uint64_t cta;
    const uint32_t s = cta_stripe(cta_beg, n, cta);
    stage(sp, pyrs[s]);
    stage(se, emits[s]);
    __syncthreads();
    if constexpr (OP == OP_TOP_DOWN) {
      for (uint32_t k = 0; k < ept; k += 2) {
        const uint64_t i = (cta * ept + k) * kChunk + threadIdx.x;
        top_down_children(sp, se, arg, i, k + 1 < ept ? i + kChunk : ~0ull);
      }
    } else {
      for (uint32_t k = 0; k < ept; k++) node_op<OP>(sp, se, arg, (cta * ept + k) * kChunk + threadIdx.x);
    }
  }
}

// One CTA per stripe: bottom-up of levels l_small .. 0.
__global__ void kb_bottom_up_top(const Pyramid* __restrict__ pyrs, const EmitJob* __restrict__ emits) {
  pdl_enter();
  __shared__ Pyramid sp;
  __shared__ EmitJob se;
  stage(sp, pyrs[blockIdx.x]);
  stage(se, emits[blockIdx.x]);
  __syncthreads();
  if (sp.depth < 1 || sp.lv[sp.depth].n == 0) return;
  for (int l = se.l_small; l >= 0; l--) {
    for (uint64_t i = threadIdx.x; i < sp.lv[l].n; i += blockDim.x) bottom_up_node(sp, se, l, i);
    __syncthreads();
  }
}

// One CTA per stripe: the root starts at the stripe's bases; parents of levels 0 .. min(l_small, depth-2).
__global__ void kb_top_down_top(const Pyramid* __restrict__ pyrs, const EmitJob* __restrict__ emits) {
  pdl_enter();
  __shared__ Pyramid sp;
  __shared__ EmitJob se;
  stage(sp, pyrs[blockIdx.x]);
  stage(se, emits[blockIdx.x]);
  __syncthreads();
  if (sp.depth < 1 || sp.lv[sp.depth].n == 0) return;
  if (threadIdx.x == 0) {
    se.start[sp.lv[0].koff] = 0u;  // the stripe root starts at the stripe's bases
    se.dstart[sp.lv[0].koff] = 0u;
  }
  __syncthreads();
  const int last = se.l_small < sp.depth - 2 ? se.l_small : sp.depth - 2;
  for (int l = 0; l <= last; l++) {
    for (uint64_t i = threadIdx.x; i < sp.lv[l].n; i += blockDim.x) top_down_node(sp, se, l, i);
    __syncthreads();
  }
}

// ===========================================================================
// Persistent phase A (ooc_tuning::persistent): the occupancy passes and the
// pyramid levels of every stripe of a sub-batch in one launch.  Each warp
// takes tickets from one counter and runs the unit its ticket names.  Tickets
// come in this order:
//   [0, C)          32-item chunks of the small pass, stripe by stripe;
//   [C, C + T)      warp tasks of large items, in the order the chunks queued
//                   them (T is final once every chunk is done);
//   [C + T, + U)    pyramid units, level by level from the leaf level up to the
//                   top levels: 32 x ept elements of one level of one stripe;
//   [.., + n)       the top levels of each stripe, one warp each.
// A unit waits only for units with smaller tickets (its stripe's occupancy, or
// its stripe's level below), which running warps hold already, so every wait
// ends whether or not the whole grid is resident.  Each wait is still bounded:
// past kPersistSpins polls it records its code in ctr[3] and every warp stops.
// ===========================================================================
// Counters, each on its own 128-byte line so the polls of waiting warps do not
// queue behind the ticket atomics.
constexpr int kCtrTicket = 0, kCtrChunksDone = 16, kCtrTasksQueued = kPersistTasksWord,
              kCtrTimeout = kPersistTimeoutWord;
static_assert(kPersistChunkItems == 32u * 8u, "a chunk is kPersistChunkRounds x 32 items");
constexpr uint64_t kPersistWaitNs = 4000000000ull;  // a wait gives up after four seconds
constexpr uint32_t kPersistChunkRounds = 8;          // a chunk is 8 x 32 items

__device__ __forceinline__ uint64_t ld_acquire(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Polling with a growing pause (64 ns to 4 us) and a bound in time.
struct Backoff {
  uint64_t t0 = 0;
  uint32_t ns = 64;
  // false once the bound has passed (recording `code`) or another warp has recorded one
  __device__ __forceinline__ bool pause(unsigned long long* ctr, uint32_t code) {
    if (ld_acquire(ctr + kCtrTimeout) != 0ull) return false;
    const uint64_t now = global_ns();
    if (t0 == 0) t0 = now;
    if (now - t0 > kPersistWaitNs) {
      atomicCAS(ctr + kCtrTimeout, 0ull, (unsigned long long)code);
      return false;
    }
    __nanosleep(ns);
    if (ns < 4096) ns <<= 1;
    return true;
  }
};

// Lane 0: wait until *p is zero; false on a timeout (here or in another warp).
__device__ __forceinline__ bool persist_wait_zero(const uint32_t* p, unsigned long long* ctr, uint32_t code) {
  Backoff b;
  while (ld_acquire(p) != 0u)
    if (!b.pause(ctr, code)) return false;
  return true;
}

// Every lane's writes of the unit reach the GPU scope before lane 0 counts it done.
__device__ __forceinline__ void persist_done(uint32_t* left, int lane) {
  __threadfence();
  __syncwarp();
  if (lane == 0) atomicSub(left, 1u);
}

__device__ __forceinline__ uint32_t find_stripe(const uint64_t* __restrict__ beg, uint32_t n, uint64_t x) {
  uint32_t lo = 0, hi = n;  // beg[lo] <= x < beg[hi]
  while (hi - lo > 1) {
    const uint32_t mid = (lo + hi) >> 1;
    if (beg[mid] <= x) lo = mid;
    else hi = mid;
  }
  return lo;
}

template <typename T>
__device__ __forceinline__ void stage_warp(T& dst, const T& src, int lane) {
  static_assert(sizeof(T) % 4 == 0, "staged structs are word-sized");
  const uint32_t* s = reinterpret_cast<const uint32_t*>(&src);
  uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
  for (uint32_t q = (uint32_t)lane; q < sizeof(T) / 4; q += 32u) d[q] = s[q];
  __syncwarp();
}

// 32 items of stripe s from item i0: the small pass, then their large items are
// queued as warp tasks (or, when the task map is full, walked by this warp).
__device__ __forceinline__ void persist_items(const PersistJob& pj, uint32_t s, uint64_t i0, int lane, const VoxJob& j,
                                              uint32_t* __restrict__ wl) {
  const uint64_t i = i0 + (uint64_t)lane;
  uint32_t cost = 0;
  if (i < j.n_items) cost = (uint32_t)vox_small_occ_item(j, i);
  // warp-aggregated reservation of the items' tasks in the map
  uint32_t excl = cost;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL, excl, o);
    if (lane >= o) excl += y;
  }
  const uint32_t total = __shfl_sync(FULL, excl, 31);
  excl -= cost;
  if (total == 0) return;
  // One atomicAdd per 32 items (a compare-and-swap loop on this one counter
  // stalled the whole grid).  Tasks reserved at or past `cap` have no entry:
  // this warp walks them, and the warps that draw their tickets skip them.
  unsigned long long base = 0;
  if (lane == 0) {
    base = atomicAdd(pj.ctr + kCtrTasksQueued, (unsigned long long)total);
    const uint64_t queued = base >= pj.cap ? 0 : (base + total <= pj.cap ? total : pj.cap - base);
    if (queued) {
      // counted before any entry is written, so no task can finish before it
      atomicAdd(pj.occ_left + s, (uint32_t)queued);
      __threadfence();
    }
  }
  base = __shfl_sync(FULL, base, 0);
  __syncwarp();
  const uint64_t ig = pj.item_beg[s] + i;  // the item's index in the sub-batch
  uint32_t todo = __ballot_sync(FULL, cost != 0);
  while (todo) {
    const int src = __ffs(todo) - 1;
    todo &= todo - 1;
    const uint32_t c = __shfl_sync(FULL, cost, src);
    const uint64_t item = __shfl_sync(FULL, ig, src);
    const uint64_t b = base + __shfl_sync(FULL, excl, src);
    for (uint32_t k = (uint32_t)lane; k < c && b + k < pj.cap; k += 32u) {
      volatile unsigned long long* e = reinterpret_cast<volatile unsigned long long*>(pj.map + b + k);
      *e = item | ((uint64_t)k << 32);
    }
    const uint32_t walked_from = b >= pj.cap ? 0u : (pj.cap - b < c ? (uint32_t)(pj.cap - b) : c);
    for (uint32_t k = walked_from; k < c; k++)
      vox_large_task<0>(j, item - pj.item_beg[s], k, lane, wl);
  }
}

__global__ void __launch_bounds__(256, 4) kb_persist(PersistJob pj) {
  pdl_enter();
  extern __shared__ uint32_t lines_smem[];  // 32 x lines_per_lane per warp
  __shared__ VoxJob s_job[8];
  __shared__ Pyramid s_pyr[8];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t* wl = lines_smem + (uint32_t)w * 32u * pj.lines_per_lane;
  const uint64_t C = pj.chunk_beg[pj.n];
  const uint64_t U = pj.levels ? pj.unit_beg[(uint64_t)pj.levels * (pj.n + 1) - 1] : 0;
  uint32_t job_s = ~0u, pyr_s = ~0u;  // the stripe staged in s_job[w] / s_pyr[w]
  for (;;) {
    unsigned long long t = 0;
    if (lane == 0)
      t = ld_acquire(pj.ctr + kCtrTimeout) != 0ull ? ~0ull : atomicAdd(pj.ctr + kCtrTicket, 1ull);
    t = __shfl_sync(FULL, t, 0);
    if (t == ~0ull) return;
    if (t < C) {  // a chunk of kPersistChunkRounds x 32 items
      const uint32_t s = find_stripe(pj.chunk_beg, pj.n, t);
      if (s != job_s) {
        stage_warp(s_job[w], pj.jobs[s], lane);
        job_s = s;
      }
      const uint64_t c0 = (t - pj.chunk_beg[s]) * (32u * kPersistChunkRounds);
      for (uint32_t q = 0; q < kPersistChunkRounds; q++) {
        const uint64_t i0 = c0 + 32u * q;
        if (i0 >= s_job[w].n_items) break;
        persist_items(pj, s, i0, lane, s_job[w], wl);
      }
      // this chunk's bits, marks and queued tasks are visible before it counts as done
      __threadfence();
      __syncwarp();
      if (lane == 0) {
        atomicSub(pj.occ_left + s, 1u);
        atomicAdd(pj.ctr + kCtrChunksDone, 1ull);
      }
      continue;
    }
    // a queued task, or (once every chunk is done and no task is left) a pyramid unit
    const uint64_t u = t - C;
    // kind 1: task, 2: after the tasks, 3: stop, 4: a task its chunk walks
    unsigned long long kind = 0, tail = 0, entry = 0;
    if (lane == 0) {
      Backoff b;
      for (;;) {
        if (u < ld_acquire(pj.ctr + kCtrTasksQueued)) {
          kind = 1;
          break;
        }
        if (ld_acquire(pj.ctr + kCtrChunksDone) == C) {
          tail = ld_acquire(pj.ctr + kCtrTasksQueued);
          kind = u < tail ? 1 : 2;
          break;
        }
        if (!b.pause(pj.ctr, 1u)) {
          kind = 3;
          break;
        }
      }
      if (kind == 1 && u >= pj.cap) kind = 4;  // a task past the map: its chunk walks it
      if (kind == 1) {  // the chunk that reserved entry u writes it right after
        Backoff b2;
        while ((entry = ld_acquire(pj.map + u)) == ~0ull)
          if (!b2.pause(pj.ctr, 2u)) {
            kind = 3;
            break;
          }
        if (kind == 1) *reinterpret_cast<volatile unsigned long long*>(pj.map + u) = ~0ull;  // empty for the next launch
      }
    }
    kind = __shfl_sync(FULL, kind, 0);
    if (kind == 3) return;
    if (kind == 4) continue;
    if (kind == 1) {
      entry = __shfl_sync(FULL, entry, 0);
      const uint64_t item = (uint32_t)entry;
      const uint32_t s = find_stripe(pj.item_beg, pj.n, item);
      if (s != job_s) {
        stage_warp(s_job[w], pj.jobs[s], lane);
        job_s = s;
      }
      vox_large_task<0>(s_job[w], item - pj.item_beg[s], entry >> 32, lane, wl);
      persist_done(pj.occ_left + s, lane);
      continue;
    }
    const uint64_t v = u - __shfl_sync(FULL, tail, 0);
    if (v < U) {  // pyramid unit: level r of stripe s
      uint32_t r = 0;
      while (v >= pj.unit_beg[(uint64_t)r * (pj.n + 1) + pj.n]) r++;
      const uint64_t* ub = pj.unit_beg + (uint64_t)r * (pj.n + 1);
      const uint32_t s = find_stripe(ub, pj.n, v);
      bool ok = true;
      if (lane == 0)
        ok = persist_wait_zero(r == 0 ? pj.occ_left + s : pj.pyr_left + (uint64_t)(r - 1) * pj.n + s, pj.ctr, 3u);
      if (!__shfl_sync(FULL, ok, 0)) return;
      __syncwarp();  // the lanes' loads below follow lane 0's acquire
      if (s != pyr_s) {
        stage_warp(s_pyr[w], pj.pyrs[s], lane);
        pyr_s = s;
      }
      const Pyramid& P = s_pyr[w];
      const int l = P.depth - (int)r;
      const uint64_t e0 = (v - ub[s]) * pj.ept * 32u;
      for (uint32_t k = 0; k < pj.ept; k++) {
        const uint64_t e = e0 + (uint64_t)k * 32u + (uint64_t)lane;
        if (e < P.lv[l].nscan) pyramid_elem<true>(P, l, e);
      }
      persist_done(pj.pyr_left + (uint64_t)r * pj.n + s, lane);
      continue;
    }
    if (v - U >= pj.n) return;  // past the last unit
    // the top levels of stripe s, after its last pyramid unit
    const uint32_t s = (uint32_t)(v - U);
    if (s != pyr_s) {
      stage_warp(s_pyr[w], pj.pyrs[s], lane);
      pyr_s = s;
    }
    const Pyramid& P = s_pyr[w];
    const int below = P.depth - pj.top_level;  // pyramid levels of the stripe under the top ones
    bool ok = true;
    if (lane == 0)
      ok = persist_wait_zero(below <= 0 ? pj.occ_left + s : pj.pyr_left + (uint64_t)(below - 1) * pj.n + s, pj.ctr,
                             4u);
    if (!__shfl_sync(FULL, ok, 0)) return;
    __syncwarp();
    if (s == 0 && lane == 0) *pj.scan_end = 0u;  // the scan's total entry
    for (int l = pj.top_level < P.depth ? pj.top_level : P.depth; l >= 0; l--) {
      for (uint64_t b = (uint64_t)lane; b < P.lv[l].nblocks; b += 32u) pyramid_block<true>(P, l, b);
      if (l > 0)
        for (uint64_t x = P.lv[l].nblocks + (uint64_t)lane; x < P.lv[l - 1].nwords; x += 32u)
          level_words(P, l - 1)[x] = 0u;
      __threadfence_block();
      __syncwarp();
    }
  }
}

// Root information of every stripe into `out` (16 words each), and the layout
// check flag after them (out[16 n]).
__global__ void kb_root_info(const Pyramid* __restrict__ pyrs, const EmitJob* __restrict__ emits, uint32_t n_stripes,
                             uint32_t* __restrict__ out, const uint32_t* __restrict__ flag) {
  pdl_enter();
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s == 0) out[(uint64_t)n_stripes * 16] = *flag;
  if (s >= n_stripes) return;
  if (pyrs[s].lv[pyrs[s].depth].n == 0) return;
  root_info(pyrs[s], emits[s], emits[s].data_base, out + (uint64_t)s * 16);
}

}  // namespace

// ===========================================================================
// Launch wrappers
// ===========================================================================
uint64_t scan_partials_needed(uint64_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE + 1; }

void scan_u32_exclusive(uint32_t* data, uint64_t n, uint32_t* partials, cudaStream_t st) {
  scan_exclusive<uint32_t>(data, n, partials, st);
}
void scan_u64_exclusive(uint64_t* data, uint64_t n, uint64_t* partials, cudaStream_t st, bool flag_last) {
  unsigned long long* d = reinterpret_cast<unsigned long long*>(data);
  scan_exclusive<unsigned long long>(d, n, reinterpret_cast<unsigned long long*>(partials), st,
                                     flag_last ? d + n - 1 : nullptr);
}

void launch_copy_words(const uint32_t* src, uint64_t n, uint32_t* dst, cudaStream_t st) {
  if (n == 0) return;
  KScope k("copy_words", st);
  const uint64_t g = std::min<uint64_t>((n + 255) / 256, 4096);
  launch_k(k_copy_words, dim3((unsigned)g), dim3(256), 0, st, src, n, dst);
}

void launch_part_count(const float* tris, int stride, uint64_t n_tris, const float* axis_lo, const float* axis_hi,
                       int pa_bits, uint64_t n_parts, uint32_t* hist, cudaStream_t st) {
  if (n_tris == 0) return;
  const int use_smem = n_parts <= 4096;
  const size_t smem = use_smem ? n_parts * sizeof(uint32_t) : 0;
  KScope k("part_count", st);
  launch_k(k_part_count, dim3(grid_for(n_tris, 256)), dim3(256), smem, st, tris, stride, n_tris, axis_lo, axis_hi,
           pa_bits, (uint32_t)n_parts, hist, use_smem);
}

void launch_part_emit(const float* tris, int stride, uint64_t n_tris, const float* axis_lo, const float* axis_hi,
                      int pa_bits, uint64_t n_parts, uint32_t* cursor, uint32_t* items, cudaStream_t st) {
  if (n_tris == 0) return;
  const int use_smem = n_parts <= 4096;
  const size_t smem = use_smem ? 2 * n_parts * sizeof(uint32_t) : 0;
  KScope k("part_emit", st);
  launch_k(k_part_emit, dim3(grid_for(n_tris, 256)), dim3(256), smem, st, tris, stride, n_tris, axis_lo, axis_hi,
           pa_bits, (uint32_t)n_parts, cursor, items, use_smem);
}

uint32_t stream_ctas(uint64_t n) { return (uint32_t)((n + kStreamCta - 1) / kStreamCta); }

void launch_stream_bases(const uint32_t* part_off, uint32_t p0, uint32_t gp, uint64_t* base, cudaStream_t st) {
  if (gp == 0) return;
  KScope k("stream_bases", st);
  launch_k(k_stream_bases, dim3(grid_for(gp, 256)), dim3(256), 0, st, part_off, p0, gp, base);
}

void launch_stream_group_chunk(const float* tris, int stride, uint64_t n, const float* axis_lo, const float* axis_hi,
                               int pa_bits, uint32_t p0, uint32_t gp, uint32_t* mat, uint32_t* mat_partials,
                               uint64_t* base, float* out, cudaStream_t st) {
  if (n == 0 || gp == 0) return;
  const uint32_t n_cta = stream_ctas(n);
  {
    KScope k("stream_count", st);
    launch_k(k_stream_count, dim3(n_cta), dim3(kStreamCta), gp * sizeof(uint32_t), st, tris, stride, n, axis_lo,
             axis_hi, pa_bits, p0, gp, mat, n_cta);
  }
  scan_exclusive<uint32_t>(mat, (uint64_t)gp * n_cta + 1, mat_partials, st);
  {
    KScope k("stream_emit", st);
    launch_k(k_stream_emit, dim3(n_cta), dim3(kStreamCta), 0, st, tris, stride, n, axis_lo, axis_hi, pa_bits, p0, gp,
             mat, n_cta, base, out);
  }
  KScope k("stream_advance", st);
  launch_k(k_stream_advance, dim3(grid_for(gp, 256)), dim3(256), 0, st, mat, n_cta, gp, base);
}

// One-stripe occupancy pass with the job as a kernel parameter (the
// allocation-free entry point uses these).  Launched with cudaLaunchKernel so
// that each returns the status of its own launch.
cudaError_t launch_vox_small_occupancy(const VoxJob& j, cudaStream_t st) {
  if (j.n_items == 0) return cudaSuccess;
  KScope k("vox_small_occupancy", st);
  VoxJob arg = j;
  void* args[] = {&arg};
  return cudaLaunchKernel(reinterpret_cast<const void*>(&k_vox_small_occ), dim3(grid_for(j.n_items, 256)), dim3(256),
                          args, 0, st);
}

cudaError_t launch_vox_large_occupancy(const VoxJob& j, cudaStream_t st, int num_sms) {
  if (j.n_items == 0) return cudaSuccess;
  const cudaError_t e = cudaMemsetAsync(j.task_counter, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return e;
  KScope k("vox_large_occupancy", st);
  VoxJob arg = j;
  void* args[] = {&arg};
  return cudaLaunchKernel(reinterpret_cast<const void*>(&k_vox_large<0>), dim3((unsigned)num_sms * 8), dim3(256), args,
                          (size_t)256 * j.lines_per_lane * 4, st);
}

// scan_exclusive<uint64_t> with the status of every launch returned.
cudaError_t scan_u64_exclusive_checked(uint64_t* data, uint64_t n, uint64_t* partials, cudaStream_t st) {
  if (n == 0) return cudaSuccess;
  const unsigned nb = (unsigned)((n + SCAN_TILE - 1) / SCAN_TILE);
  const uint64_t* none = nullptr;  // no partials (one tile) / no skip flag
  if (nb == 1) {
    KScope k("scan_down", st);
    void* args[] = {&data, &n, &none, &none};
    return cudaLaunchKernel(reinterpret_cast<const void*>(&k_scan_down<uint64_t>), dim3(1), dim3(SCAN_THREADS), args,
                            0, st);
  }
  cudaError_t e;
  {
    KScope k("scan_reduce", st);
    void* args[] = {&data, &n, &partials, &none};
    e = cudaLaunchKernel(reinterpret_cast<const void*>(&k_scan_reduce<uint64_t>), dim3(nb), dim3(SCAN_THREADS), args,
                         0, st);
  }
  if (e != cudaSuccess) return e;
  {
    KScope k("scan_partials", st);
    uint64_t np = nb;
    void* args[] = {&partials, &np, &none};
    e = cudaLaunchKernel(reinterpret_cast<const void*>(&k_scan_partials<uint64_t>), dim3(1), dim3(1024), args, 0, st);
  }
  if (e != cudaSuccess) return e;
  KScope k("scan_down", st);
  const uint64_t* cp = partials;
  void* args[] = {&data, &n, &cp, &none};
  return cudaLaunchKernel(reinterpret_cast<const void*>(&k_scan_down<uint64_t>), dim3(nb), dim3(SCAN_THREADS), args, 0,
                          st);
}

void launch_scatter_records(const uint64_t* src, uint64_t n, int words, uint64_t* dst, cudaStream_t st) {
  if (n == 0) return;
  KScope k("scatter_records", st);
  launch_k(k_scatter_records, dim3(grid_for(n, 128)), dim3(128), 0, st, src, n, words, dst);
}

void launch_scatter_to(const uint64_t* src, uint64_t n, int words, cudaStream_t st) {
  if (n == 0) return;
  KScope k("scatter_records", st);
  launch_k(k_scatter_to, dim3(grid_for(n, 128)), dim3(128), 0, st, src, n, words);
}

// ---- batched launch wrappers ----
void launch_b_vox_small(const VoxJob* jobs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, int pass,
                        const VoxJob* single, cudaStream_t st) {
  if (ctas == 0) return;
  KScope k(pass == 0 ? "vox_small_occupancy" : "vox_small_winner", st);
  VoxJob j0;
  std::memset(&j0, 0, sizeof(j0));
  if (single) j0 = *single;
  if (pass == 0) {
    if (single) launch_k(kb_vox_small<0, true>, dim3((unsigned)ctas), dim3(kChunk), 0, st, jobs, cta_beg, n, j0);
    else launch_k(kb_vox_small<0, false>, dim3((unsigned)ctas), dim3(kChunk), 0, st, jobs, cta_beg, n, j0);
  } else {
    if (single) launch_k(kb_vox_small<1, true>, dim3((unsigned)ctas), dim3(kChunk), 0, st, jobs, cta_beg, n, j0);
    else launch_k(kb_vox_small<1, false>, dim3((unsigned)ctas), dim3(kChunk), 0, st, jobs, cta_beg, n, j0);
  }
}

void launch_b_task_map(const uint64_t* cta_beg, uint32_t n, uint64_t ctas, const uint64_t* item_beg,
                       const uint64_t* task_off, uint64_t total_items, uint64_t* map, uint64_t cap, cudaStream_t st) {
  if (ctas == 0) return;
  KScope k("task_map", st);
  launch_k(kb_task_map, dim3((unsigned)ctas), dim3(kChunk), 0, st, cta_beg, n, item_beg, task_off, total_items, map,
           cap);
}

void launch_b_vox_large(const VoxJob* jobs, const uint64_t* item_beg, uint32_t n_stripes, const uint64_t* task_off,
                        uint64_t total_items, unsigned long long* counter, int pass, cudaStream_t st, int num_sms,
                        int block, int ctas_per_sm, uint32_t lines_per_lane, const uint64_t* map, uint64_t cap) {
  if (total_items == 0) return;
  cudaMemsetAsync(counter, 0, sizeof(unsigned long long), st);
  const unsigned grid = (unsigned)num_sms * (unsigned)ctas_per_sm;
  const size_t smem = (size_t)block * lines_per_lane * 4;  // each warp's list of passing lines
  if (smem > (48u << 10)) {  // beyond the default dynamic limit (at most 256 x 64 x 4 = 64 KiB)
    cudaFuncSetAttribute(kb_vox_large<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    cudaFuncSetAttribute(kb_vox_large<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  }
  KScope k(pass == 0 ? "vox_large_occupancy" : "vox_large_winner", st);
  if (pass == 0)
    launch_k(kb_vox_large<0>, dim3(grid), dim3(block), smem, st, jobs, item_beg, n_stripes, task_off, total_items,
             counter, lines_per_lane, map, cap);
  else
    launch_k(kb_vox_large<1>, dim3(grid), dim3(block), smem, st, jobs, item_beg, n_stripes, task_off, total_items,
             counter, lines_per_lane, map, cap);
}

void launch_b_pyramid(const Pyramid* pyrs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept, int r,
                      const Pyramid* single, cudaStream_t st) {
  if (ctas == 0) return;
  KScope k(r == 0 ? "pyramid_leaf" : "pyramid", st);
  Pyramid p0;
  std::memset(&p0, 0, sizeof(p0));
  if (single) p0 = *single;
  if (single) launch_k(kb_pyramid<true>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, cta_beg, n, r, ept, p0);
  else launch_k(kb_pyramid<false>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, cta_beg, n, r, ept, p0);
}

void launch_b_pyramid_top(const Pyramid* pyrs, uint32_t n_stripes, int l_hi, uint32_t* scan_end, cudaStream_t st) {
  if (n_stripes == 0) return;
  KScope k("pyramid_top", st);
  launch_k(kb_pyramid_top, dim3(n_stripes), dim3(512), 0, st, pyrs, l_hi, scan_end);
}

void launch_b_compact(const Pyramid* pyrs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept,
                      uint32_t* keys, const Pyramid* single, cudaStream_t st) {
  if (ctas == 0) return;
  KScope k("compact", st);
  Pyramid p0;
  std::memset(&p0, 0, sizeof(p0));
  if (single) p0 = *single;
  if (single) launch_k(kb_compact<true>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, cta_beg, n, keys, ept, p0);
  else launch_k(kb_compact<false>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, cta_beg, n, keys, ept, p0);
}

void launch_b_clean_leaves(const Pyramid* pyrs, const uint64_t* cta_beg, uint32_t n, uint64_t ctas, uint32_t ept,
                           const Pyramid* single, cudaStream_t st) {
  if (ctas == 0) return;
  KScope k("clean_leaves", st);
  Pyramid p0;
  std::memset(&p0, 0, sizeof(p0));
  if (single) p0 = *single;
  if (single) launch_k(kb_clean_leaves<true>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, cta_beg, n, ept, p0);
  else launch_k(kb_clean_leaves<false>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, cta_beg, n, ept, p0);
}

void launch_b_level_bases(const Pyramid* pyrs, uint32_t n_stripes, uint32_t* out, const uint64_t* tasks,
                          uint64_t* tasks_out, uint32_t* flag, const uint64_t* code, uint64_t* code_out,
                          cudaStream_t st) {
  if (n_stripes == 0) return;
  KScope k("level_bases", st);
  launch_k(kb_level_bases, dim3(grid_for(n_stripes, 128)), dim3(128), 0, st, pyrs, n_stripes, out, tasks, tasks_out,
           flag, code, code_out);
}

namespace {
template <int OP>
void launch_nodes(const char* name, const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n,
                  uint64_t ctas, uint32_t ept, int arg, const Pyramid* sp, const EmitJob* se, cudaStream_t st) {
  if (ctas == 0) return;
  KScope k(name, st);
  Pyramid p0;
  EmitJob e0;
  std::memset(&p0, 0, sizeof(p0));
  std::memset(&e0, 0, sizeof(e0));
  if (sp && se) {
    p0 = *sp;
    e0 = *se;
    launch_k(kb_nodes<OP, true>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, emits, cta_beg, n, arg, ept, p0, e0);
  } else {
    launch_k(kb_nodes<OP, false>, dim3((unsigned)ctas), dim3(kChunk), 0, st, pyrs, emits, cta_beg, n, arg, ept, p0, e0);
  }
}
}  // namespace

void launch_b_leaf_payload(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n,
                           uint64_t ctas, uint32_t ept, const Pyramid* sp, const EmitJob* se, cudaStream_t st) {
  launch_nodes<OP_LEAF_PAYLOAD>("leaf_payload", pyrs, emits, cta_beg, n, ctas, ept, 0, sp, se, st);
}

void launch_b_bottom_up(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n, uint64_t ctas,
                        uint32_t ept, int r, const Pyramid* sp, const EmitJob* se, cudaStream_t st) {
  launch_nodes<OP_BOTTOM_UP>(r == 1 ? "bottom_up_leaf_parents" : "bottom_up", pyrs, emits, cta_beg, n, ctas, ept, r,
                             sp, se, st);
}

void launch_b_bottom_up_top(const Pyramid* pyrs, const EmitJob* emits, uint32_t n_stripes, cudaStream_t st) {
  if (n_stripes == 0) return;
  KScope k("bottom_up_top", st);
  launch_k(kb_bottom_up_top, dim3(n_stripes), dim3(256), 0, st, pyrs, emits);
}

void launch_b_top_down_top(const Pyramid* pyrs, const EmitJob* emits, uint32_t n_stripes, cudaStream_t st) {
  if (n_stripes == 0) return;
  KScope k("top_down_top", st);
  launch_k(kb_top_down_top, dim3(n_stripes), dim3(256), 0, st, pyrs, emits);
}

void launch_b_top_down(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n, uint64_t ctas,
                       uint32_t ept, int l, const Pyramid* sp, const EmitJob* se, cudaStream_t st) {
  launch_nodes<OP_TOP_DOWN>("top_down", pyrs, emits, cta_beg, n, ctas, ept, l, sp, se, st);
}

void launch_b_top_down_leaves(const Pyramid* pyrs, const EmitJob* emits, const uint64_t* cta_beg, uint32_t n,
                              uint64_t ctas, uint32_t ept, const Pyramid* sp, const EmitJob* se, cudaStream_t st) {
  launch_nodes<OP_LEAVES>("top_down_leaves", pyrs, emits, cta_beg, n, ctas, ept, 0, sp, se, st);
}

int persist_ctas_per_sm(uint32_t lines_per_lane) {
  int per_sm = 0;
  const size_t smem = (size_t)256 * lines_per_lane * 4;
  if (smem > (48u << 10) &&
      cudaFuncSetAttribute(kb_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
    return 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kb_persist, 256, smem) != cudaSuccess) return 0;
  return per_sm;
}

void launch_b_persist(const PersistJob& pj, int num_sms, int ctas_per_sm, cudaStream_t st) {
  KScope k("persistent_phase_a", st);
  const size_t smem = (size_t)256 * pj.lines_per_lane * 4;
  launch_k(kb_persist, dim3((unsigned)(num_sms * ctas_per_sm)), dim3(256), smem, st, pj);
}

void launch_b_root_info(const Pyramid* pyrs, const EmitJob* emits, uint32_t n_stripes, uint32_t* out,
                        const uint32_t* flag, cudaStream_t st) {
  if (n_stripes == 0) return;
  KScope k("root_info", st);
  launch_k(kb_root_info, dim3(grid_for(n_stripes, 128)), dim3(128), 0, st, pyrs, emits, n_stripes, out, flag);
}

}  // namespace ooc
