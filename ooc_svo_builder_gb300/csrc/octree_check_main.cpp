// octree_check: read <base>.octree (+ .octreenodes, .octreedata) the way
// parseOctreeHeader and readNode do (octree_io.h:69-110) and check the files'
// structure on the GPU (ooc_check_octree_device).
//
//   octree_check [-b] <file.octree>
//     -b   the octree was built by svo_builder_binary (geometry only)
//
// Prints the header, the counts and the verdict; exit status 0 when the
// octree is well formed, 1 when a check fails, 2 on a usage or I/O error.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "ooc_svo_gpu.h"

namespace {

struct Header {
  int version = 0;
  unsigned long long gridlength = 0, n_nodes = 0, n_data = 0;
};

bool parse_header(const std::string& path, Header& h) {
  std::ifstream f(path);
  if (!f) return false;
  std::string tok;
  f >> tok;
  if (tok != "#octreeheader") return false;
  f >> h.version;
  while (f >> tok && tok != "END") {
    if (tok == "gridlength") f >> h.gridlength;
    else if (tok == "n_nodes") f >> h.n_nodes;
    else if (tok == "n_data") f >> h.n_data;
  }
  return h.gridlength > 0;
}

bool read_file(const std::string& path, std::vector<unsigned char>& out, unsigned long long expect) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  out.resize(expect);
  const size_t got = expect ? std::fread(out.data(), 1, expect, f) : 0;
  const int extra = std::fgetc(f);
  std::fclose(f);
  return got == expect && extra == EOF;
}

}  // namespace

int main(int argc, char** argv) {
  int binary = 0;
  std::string file;
  for (int i = 1; i < argc; i++) {
    if (!std::strcmp(argv[i], "-b")) binary = 1;
    else file = argv[i];
  }
  if (file.size() < 8 || file.substr(file.size() - 7) != ".octree") {
    std::fprintf(stderr, "usage: octree_check [-b] <file.octree>\n");
    return 2;
  }
  const std::string base = file.substr(0, file.size() - 7);
  Header h;
  if (!parse_header(file, h)) {
    std::fprintf(stderr, "cannot read an octree header from %s\n", file.c_str());
    return 2;
  }
  std::vector<unsigned char> nodes, data;
  if (!read_file(base + ".octreenodes", nodes, h.n_nodes * 24) || !read_file(base + ".octreedata", data, h.n_data * 32)) {
    std::fprintf(stderr, "node or data file missing, or its size disagrees with the header\n");
    return 1;
  }
  std::printf("octree %s: gridlength %llu, %llu nodes, %llu data records\n", base.c_str(), h.gridlength, h.n_nodes,
              h.n_data);
  if (h.n_nodes == 0) {
    std::printf("no nodes: not a complete octree\n");
    return 1;
  }
  void* d_nodes = nullptr;
  void* d_data = nullptr;
  if (cudaMalloc(&d_nodes, nodes.size()) != cudaSuccess || cudaMalloc(&d_data, data.size() + 32) != cudaSuccess ||
      cudaMemcpy(d_nodes, nodes.data(), nodes.size(), cudaMemcpyHostToDevice) != cudaSuccess ||
      (data.size() && cudaMemcpy(d_data, data.data(), data.size(), cudaMemcpyHostToDevice) != cudaSuccess)) {
    std::fprintf(stderr, "no CUDA device or not enough device memory\n");
    return 2;
  }
  ooc_octree_check r;
  const int rc = ooc_check_octree_device(d_nodes, h.n_nodes, d_data, h.n_data, h.gridlength, binary, nullptr, &r);
  cudaFree(d_nodes);
  cudaFree(d_data);
  if (rc != OOC_OK) {
    std::fprintf(stderr, "check failed to run (status %d)\n", rc);
    return 2;
  }
  std::printf("%llu voxels (leaves), %llu inner nodes, depth %u\n", (unsigned long long)r.n_leaves,
              (unsigned long long)r.n_inner, r.max_depth);
  if (!r.errors) {
    std::printf("well formed\n");
    return 0;
  }
  static const char* names[] = {"child group order", "reference count", "depth", "data index", "payload Morton code"};
  std::printf("violations:");
  for (int b = 0; b < 5; b++)
    if (r.errors & (1u << b)) std::printf(" [%s]", names[b]);
  std::printf(" first at node %llu\n", (unsigned long long)r.first_bad);
  return 1;
}
