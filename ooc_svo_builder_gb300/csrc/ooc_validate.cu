// Structural check of an octree in device memory: the invariants of the
// .octreenodes / .octreedata format (octree_io.h:48-83) that any correct
// build satisfies, checked at any size.
//
// * Children of a node form one group written before the node: their
//   children_offset values are 0, 1, 2, ... in slot order and children_base +
//   offset is below the node's own index (the post-order of groupNodes,
//   OctreeBuilder.cpp:58-79).
// * Every node but the root (the last record) is the child of exactly one node.
// * Leaves sit at depth log2(gridsize), inner nodes above it.
// * Data indices fall inside the data file; a geometry-only leaf points at
//   entry 1 (the white record, OctreeBuilder.cpp:22-28); a payload leaf's data
//   record carries the Morton code of the path from the root to the leaf.
#include <cuda_runtime.h>

#include <cstring>

#include "ooc_svo_gpu.h"

namespace {

struct NodeRec {
  unsigned long long data, cb, off;
};

struct Shared {
  unsigned int errors;
  unsigned long long first_bad;
  unsigned long long leaves, inner;
  unsigned int max_depth;
};

__device__ __forceinline__ void flag(Shared* sh, unsigned int bit, unsigned long long i) {
  atomicOr(&sh->errors, bit);
  atomicMin(&sh->first_bad, i);
}

__device__ __forceinline__ NodeRec load_node(const unsigned long long* nodes, unsigned long long i) {
  const unsigned long long* p = nodes + i * 3;
  return NodeRec{p[0], p[1], p[2]};
}

__global__ void k_init(unsigned int* refc, unsigned char* depth, unsigned long long n) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  refc[i] = 0;
  depth[i] = 0xff;
}

// Child groups: order, position before the parent, reference counts, data indices.
__global__ void k_groups(const unsigned long long* nodes, unsigned long long n, unsigned long long n_data,
                         int binary, unsigned int* refc, Shared* sh) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const NodeRec r = load_node(nodes, i);
  unsigned int next = 0;
  for (int k = 0; k < 8; k++) {
    const unsigned int o = (unsigned int)(r.off >> (8 * k)) & 0xffu;
    if (o == 0xffu) continue;
    if (o != next || r.cb + o >= i) {
      flag(sh, OOC_CHECK_CHILD_ORDER, i);
      return;
    }
    next++;
    atomicAdd(&refc[r.cb + o], 1u);
  }
  if (next == 0) {
    // a leaf (or the root of an empty octree, whose data is the null entry 0)
    const bool empty_root = (i + 1 == n) && r.data == 0;
    if (!empty_root && (binary ? r.data != 1 : (r.data == 0 || r.data >= n_data))) flag(sh, OOC_CHECK_DATA_INDEX, i);
  } else if (r.data >= n_data) {
    flag(sh, OOC_CHECK_DATA_INDEX, i);
  }
}

__global__ void k_refs(const unsigned int* refc, unsigned long long n, Shared* sh) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (refc[i] != (i + 1 == n ? 0u : 1u)) flag(sh, OOC_CHECK_REFCOUNT, i);
}

// One level of the walk from the root: depth and Morton path of the children of level-l nodes.
__global__ void k_descend(const unsigned long long* nodes, unsigned long long n, unsigned int l,
                          unsigned char* depth, unsigned long long* path) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || depth[i] != l) return;
  const NodeRec r = load_node(nodes, i);
  for (int k = 0; k < 8; k++) {
    const unsigned int o = (unsigned int)(r.off >> (8 * k)) & 0xffu;
    if (o == 0xffu || r.cb + o >= n) continue;
    depth[r.cb + o] = (unsigned char)(l + 1);
    path[r.cb + o] = (path[i] << 3) | (unsigned long long)k;
  }
}

// Depth of every node and the payload leaves' Morton codes; counts.
__global__ void k_final(const unsigned long long* nodes, unsigned long long n, const unsigned long long* data,
                        unsigned long long n_data, int binary, unsigned int levels_below_root,
                        const unsigned char* depth, const unsigned long long* path, Shared* sh) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const NodeRec r = load_node(nodes, i);
  const bool leaf = r.off == ~0ull;
  const unsigned int d = depth[i];
  if (d == 0xffu) {  // not reached from the root
    flag(sh, OOC_CHECK_REFCOUNT, i);
    return;
  }
  if (leaf) {
    const bool empty_root = (i + 1 == n) && r.data == 0;
    if (!empty_root) {
      if (d != levels_below_root) flag(sh, OOC_CHECK_DEPTH, i);
      if (!binary && r.data < n_data && data[r.data * 4] != path[i]) flag(sh, OOC_CHECK_MORTON, i);
      atomicAdd(&sh->leaves, 1ull);
    }
  } else {
    if (d >= levels_below_root) flag(sh, OOC_CHECK_DEPTH, i);
    atomicAdd(&sh->inner, 1ull);
  }
  atomicMax(&sh->max_depth, d);
}

unsigned int grid(unsigned long long n) { return (unsigned int)((n + 255) / 256); }

}  // namespace

extern "C" int ooc_check_octree_device(const void* nodes, uint64_t n_nodes, const void* data, uint64_t n_data,
                                       uint64_t gridsize, int32_t geometry_only, void* stream,
                                       ooc_octree_check* out) {
  if (!out || !nodes || n_nodes == 0 || (n_data && !data) || gridsize == 0 || (gridsize & (gridsize - 1)) ||
      (geometry_only != 0 && geometry_only != 1))
    return OOC_ERR_INVALID;
  if ((reinterpret_cast<uintptr_t>(nodes) | reinterpret_cast<uintptr_t>(data)) & 7) return OOC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  out->n_nodes = n_nodes;
  out->n_data = n_data;
  out->first_bad = ~0ull;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  unsigned int levels = 0;
  while ((1ull << levels) < gridsize) levels++;
  unsigned int* refc = nullptr;
  unsigned char* depth = nullptr;
  unsigned long long* path = nullptr;
  Shared* sh = nullptr;
  int rc = OOC_OK;
  if (cudaMallocAsync(&refc, n_nodes * 4, st) != cudaSuccess || cudaMallocAsync(&depth, n_nodes, st) != cudaSuccess ||
      cudaMallocAsync(&path, n_nodes * 8, st) != cudaSuccess || cudaMallocAsync(&sh, sizeof(Shared), st) != cudaSuccess) {
    rc = OOC_ERR_OOM;
  } else {
    Shared init;
    std::memset(&init, 0, sizeof(init));
    init.first_bad = ~0ull;
    const auto* nd = static_cast<const unsigned long long*>(nodes);
    const auto* dt = static_cast<const unsigned long long*>(data);
    const unsigned char root_depth = 0;
    const unsigned long long root_path = 0;
    cudaMemcpyAsync(sh, &init, sizeof(init), cudaMemcpyHostToDevice, st);
    k_init<<<grid(n_nodes), 256, 0, st>>>(refc, depth, n_nodes);
    cudaMemcpyAsync(depth + (n_nodes - 1), &root_depth, 1, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(path + (n_nodes - 1), &root_path, 8, cudaMemcpyHostToDevice, st);
    k_groups<<<grid(n_nodes), 256, 0, st>>>(nd, n_nodes, n_data, geometry_only, refc, sh);
    k_refs<<<grid(n_nodes), 256, 0, st>>>(refc, n_nodes, sh);
    for (unsigned int l = 0; l < levels; l++) k_descend<<<grid(n_nodes), 256, 0, st>>>(nd, n_nodes, l, depth, path);
    k_final<<<grid(n_nodes), 256, 0, st>>>(nd, n_nodes, dt, n_data, geometry_only, levels, depth, path, sh);
    Shared res;
    if (cudaMemcpyAsync(&res, sh, sizeof(res), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess) {
      rc = OOC_ERR_DEVICE;
    } else {
      out->errors = res.errors;
      out->first_bad = res.first_bad;
      out->n_leaves = res.leaves;
      out->n_inner = res.inner;
      out->max_depth = res.max_depth;
    }
  }
  if (refc) cudaFreeAsync(refc, st);
  if (depth) cudaFreeAsync(depth, st);
  if (path) cudaFreeAsync(path, st);
  if (sh) cudaFreeAsync(sh, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && rc == OOC_OK) rc = OOC_ERR_DEVICE;
  return rc;
}
