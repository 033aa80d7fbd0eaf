// File front end of libooc_svo_gpu.so: .tri/.tridata in, .octree/.octreenodes/
// .octreedata out, named and formatted as the reference does.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>

#include "ooc_svo_gpu.h"

namespace {

struct TriHeader {
  std::string base;
  int version = 0;
  int geo_only = 0;
  uint64_t n_triangles = 0;
  float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
};

// parseTriHeader (tri_tools.h:75-115), same tokenisation and float parsing.
bool parse_tri_header(const std::string& filename, TriHeader& t, std::string& err) {
  std::ifstream file(filename.c_str(), std::ios::in);
  if (!file) {
    err = "file " + filename + " does not exist";
    return false;
  }
  t.base = filename.substr(0, filename.find_last_of("."));
  std::string line;
  file >> line;
  if (line.compare("#tri") != 0) {
    err = "first line reads [" + line + "] instead of [#tri]";
    return false;
  }
  file >> t.version;
  bool done = false;
  t.geo_only = 0;
  while (file.good() && !done) {
    file >> line;
    if (line.compare("END") == 0) {
      done = true;
    } else if (line.compare("ntriangles") == 0) {
      file >> t.n_triangles;
    } else if (line.compare("geo_only") == 0) {
      file >> t.geo_only;
    } else if (line.compare("bbox") == 0) {
      file >> t.bmin[0] >> t.bmin[1] >> t.bmin[2] >> t.bmax[0] >> t.bmax[1] >> t.bmax[2];
    } else {
      char c;
      do {
        c = file.get();
      } while (file.good() && (c != '\n'));
    }
  }
  if (!done) {
    err = "error reading header";
    return false;
  }
  return true;
}

struct FileSink {
  FILE* nodes = nullptr;
  FILE* data = nullptr;
};

int file_sink(void* user, int32_t kind, const void* bytes, uint64_t n) {
  FileSink* s = static_cast<FileSink*>(user);
  FILE* f = kind == OOC_STREAM_NODES ? s->nodes : s->data;
  return fwrite(bytes, 1, (size_t)n, f) == (size_t)n ? 0 : 1;
}

}  // namespace

extern "C" int ooc_build_files(ooc_ctx* ctx, const char* tri_path, const ooc_build_params* params_in, char* out_base,
                               uint64_t out_base_len, ooc_build_info* info) {
  if (!ctx || !tri_path || !params_in) return OOC_ERR_INVALID;
  TriHeader h;
  std::string err;
  if (!parse_tri_header(tri_path, h, err)) return OOC_ERR_IO;
  ooc_build_params prm = *params_in;
  prm.geometry_only = h.geo_only ? 1 : 0;
  for (int a = 0; a < 3; a++) {
    prm.bbox_min[a] = h.bmin[a];
    prm.bbox_max[a] = h.bmax[a];
  }
  const int stride = prm.geometry_only ? 9 : 21;
  const size_t bytes = (size_t)h.n_triangles * stride * sizeof(float);
  void* tris = nullptr;
  if (bytes && cudaMallocHost(&tris, bytes) != cudaSuccess) return OOC_ERR_OOM;
  std::string data_path = h.base + ".tridata";
  FILE* f = fopen(data_path.c_str(), "rb");
  if (!f) {
    if (tris) cudaFreeHost(tris);
    return OOC_ERR_IO;
  }
  const size_t got = bytes ? fread(tris, 1, bytes, f) : 0;
  fclose(f);
  if (got != bytes) {
    if (tris) cudaFreeHost(tris);
    return OOC_ERR_IO;
  }
  const uint64_t P = ooc_estimate_partitions(prm.gridsize, prm.memory_limit_mb);
  // <base><gridsize>_<npartitions> (partitioner.cpp:90, 141; main.cpp:325)
  const std::string base = h.base + std::to_string(prm.gridsize) + "_" + std::to_string(P);
  FileSink sink;
  sink.nodes = fopen((base + ".octreenodes").c_str(), "wb");
  sink.data = fopen((base + ".octreedata").c_str(), "wb");
  int rc = OOC_OK;
  ooc_build_info local;
  std::memset(&local, 0, sizeof(local));
  if (!sink.nodes || !sink.data) {
    rc = OOC_ERR_IO;
  } else {
    rc = ooc_build(ctx, &prm, static_cast<const float*>(tris), h.n_triangles, file_sink, &sink, &local);
  }
  if (sink.nodes) fclose(sink.nodes);
  if (sink.data) fclose(sink.data);
  if (tris) cudaFreeHost(tris);
  if (rc != OOC_OK) return rc;
  // writeOctreeHeader (octree_io.h:74-83)
  std::ofstream out((base + ".octree").c_str(), std::ios::out);
  out << "#octreeheader 1" << std::endl;
  out << "gridlength " << prm.gridsize << std::endl;
  out << "n_nodes " << local.n_nodes << std::endl;
  out << "n_data " << local.n_data << std::endl;
  out << "END" << std::endl;
  out.close();
  if (!out) return OOC_ERR_IO;
  if (out_base && out_base_len) {
    std::strncpy(out_base, base.c_str(), (size_t)out_base_len - 1);
    out_base[out_base_len - 1] = 0;
  }
  if (info) *info = local;
  return OOC_OK;
}
