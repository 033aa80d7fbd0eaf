// ooc_voxelize_occupancy_noalloc: the occupancy (voxelization) pass for callers
// that cannot allocate GPU memory.
//
// Some callers of this library may not call cudaMalloc (or anything that
// allocates) on the path where they voxelize: code that runs while a CUDA
// stream is being captured into a graph, plugins whose host engine owns and
// pre-reserves all device memory, and latency-critical loops where an
// allocation would synchronise the device.  This entry point takes the
// triangles and the output bitfield from the caller and keeps the pass's only
// scratch -- the per-triangle task offsets, their scan partials and the task
// counter of the large-triangle kernel -- in a fixed-size array that lives in
// this file as a static __device__ variable.  Every GPU that loads the library
// holds that array (about 8.4 MB) until the process exits.
#include <cuda_runtime.h>

#include <cstring>
#include <mutex>

#include "ooc_internal.h"
#include "ooc_svo_gpu.h"

namespace {

using namespace ooc;

constexpr uint64_t kMaxTris = OOC_NOALLOC_MAX_TRIANGLES;
constexpr uint64_t kTaskWords = kMaxTris + 1;  // exclusive prefix of warp tasks, one entry per triangle + total
constexpr uint64_t kPartialWords = (kTaskWords + 4095) / 4096 + 1;  // scan partials (4096-element tiles)
constexpr uint64_t kScratchWords = kTaskWords + kPartialWords + 2;  // + task counter

// The scratch.  In host code this name is only a stand-in for the device
// variable: its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned long long g_noalloc_scratch[kScratchWords];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
unsigned long long* g_scratch_dev[kMaxDevices] = {nullptr};
int g_num_sms[kMaxDevices] = {0};

// Once per device, with that device current: the scratch address and the SM count.
int device_setup(int dev, unsigned long long** scratch, int* sms) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return OOC_ERR_DEVICE;
    int n = 0;
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return OOC_ERR_DEVICE;
    g_num_sms[dev] = n;
    g_scratch_dev[dev] = static_cast<unsigned long long*>(p);
  }
  *scratch = g_scratch_dev[dev];
  *sms = g_num_sms[dev];
  return OOC_OK;
}

}  // namespace

extern "C" int ooc_voxelize_occupancy_noalloc(const ooc_build_params* params, const float* tris_device,
                                              uint64_t n_tris, uint32_t* occupancy_device,
                                              uint64_t occupancy_words, void* stream) {
  if (!params || !occupancy_device || (n_tris && !tris_device)) return OOC_ERR_INVALID;
  const uint64_t N = params->gridsize;
  if (N == 0 || (N & (N - 1)) != 0) return OOC_ERR_INVALID;
  if (params->geometry_only != 0 && params->geometry_only != 1) return OOC_ERR_INVALID;
  if (N > OOC_NOALLOC_MAX_GRIDSIZE || n_tris > kMaxTris) return OOC_ERR_LIMIT;
  if (ooc_estimate_partitions(N, params->memory_limit_mb) != 1) return OOC_ERR_LIMIT;
  const uint64_t voxels = N * N * N;
  const uint64_t words = voxels < 32 ? 1 : voxels / 32;
  if (occupancy_words < words) return OOC_ERR_INVALID;

  if (scan_partials_needed(n_tris + 1) > kPartialWords) return OOC_ERR_LIMIT;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return OOC_ERR_DEVICE;
  unsigned long long* scratch = nullptr;
  int sms = 0;
  const int rc = device_setup(dev, &scratch, &sms);
  if (rc != OOC_OK) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);

  // This call has no context: its launches report to a launch state of its own
  // with no timing hooks, installed on this thread for the call only.
  LaunchState own;
  LaunchScope scope(&own);

  const float u = (params->bbox_max[0] - params->bbox_min[0]) / (float)N;  // main.cpp:311
  VoxJob j;
  std::memset(&j, 0, sizeof(j));
  j.tris = tris_device;
  j.stride = params->geometry_only ? 9 : 21;
  j.item_tri = nullptr;
  j.ibeg = 0;
  j.n_items = n_tris;
  for (int a = 0; a < 3; a++) {
    j.pa[a] = 0;
    j.pb[a] = (int)(N - 1);
    j.sa[a] = 0;
    j.sb[a] = (int)(N - 1);
  }
  j.u = u;
  j.unit_div = 1.0f / u;  // voxelizer.cpp:164
  j.small_vol = 64;
  j.lines_per_lane = 16;
  j.leafbits = occupancy_device;
  j.task_off = reinterpret_cast<uint64_t*>(scratch);
  uint64_t* partials = reinterpret_cast<uint64_t*>(scratch + kTaskWords);
  j.task_counter = scratch + kTaskWords + kPartialWords;
  j.item_mask = nullptr;

  // What must start at zero: the output bits and the end of the task-offset
  // scan (the other scratch entries are fully written before they are read).
  // Every step's own status is checked; the first failure ends the call.
  if (cudaMemsetAsync(occupancy_device, 0, words * 4, st) != cudaSuccess) return OOC_ERR_DEVICE;
  if (cudaMemsetAsync(j.task_off + n_tris, 0, 8, st) != cudaSuccess) return OOC_ERR_DEVICE;
  if (launch_vox_small_occupancy(j, st) != cudaSuccess) return OOC_ERR_DEVICE;
  if (scan_u64_exclusive_checked(j.task_off, n_tris + 1, partials, st) != cudaSuccess) return OOC_ERR_DEVICE;
  if (launch_vox_large_occupancy(j, st, sms) != cudaSuccess) return OOC_ERR_DEVICE;
  return OOC_OK;
}
