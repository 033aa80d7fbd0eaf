// File front end of libooc_svo_gpu.so: .tri/.tridata in, .octree/.octreenodes/
// .octreedata out, named and formatted as the reference does.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <fstream>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "ooc_internal.h"
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

// .tridata straight into device memory: fixed-size chunks are read into two
// pinned buffers in turn, and each chunk's upload overlaps the read of the
// next, so no pinned copy of the whole file is made.
bool read_to_device(const std::string& path, size_t bytes, void* dst, std::string& err) {
  constexpr size_t kChunk = 64ull << 20;
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) {
    err = "cannot open " + path;
    return false;
  }
  void* pin[2] = {nullptr, nullptr};
  cudaEvent_t done[2] = {nullptr, nullptr};
  cudaStream_t st = nullptr;
  bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
  for (int i = 0; i < 2 && ok; i++)
    ok = cudaMallocHost(&pin[i], std::min(kChunk, std::max<size_t>(bytes, 1))) == cudaSuccess &&
         cudaEventCreateWithFlags(&done[i], cudaEventDisableTiming) == cudaSuccess;
  size_t off = 0;
  for (int i = 0; ok && off < bytes; i ^= 1) {
    const size_t n = std::min(kChunk, bytes - off);
    ok = cudaEventSynchronize(done[i]) == cudaSuccess;  // the buffer's previous upload is done
    if (ok && std::fread(pin[i], 1, n, f) != n) {
      err = "short read of " + path;
      ok = false;
      break;
    }
    ok = ok && cudaMemcpyAsync(static_cast<char*>(dst) + off, pin[i], n, cudaMemcpyHostToDevice, st) == cudaSuccess &&
         cudaEventRecord(done[i], st) == cudaSuccess;
    off += n;
  }
  if (st && cudaStreamSynchronize(st) != cudaSuccess) ok = false;
  for (int i = 0; i < 2; i++) {
    if (pin[i]) cudaFreeHost(pin[i]);
    if (done[i]) cudaEventDestroy(done[i]);
  }
  if (st) cudaStreamDestroy(st);
  std::fclose(f);
  if (!ok && err.empty()) err = "device upload of " + path + " failed";
  return ok;
}

// One writer thread per output file: the sink copies each piece into the
// file's current 16 MiB buffer and hands full buffers to the thread, so the
// two files are written in parallel and neither stalls the build.  At most
// four buffers per file are in flight.
class FileWriter {
 public:
  explicit FileWriter(FILE* f) : f_(f), th_([this] { loop(); }) {}
  ~FileWriter() { finish(); }

  bool put(const void* bytes, size_t n) {
    const char* p = static_cast<const char*>(bytes);
    while (n) {
      if (cur_.size() == kBuf) flush_current();
      const size_t k = std::min(n, kBuf - cur_.size());
      cur_.insert(cur_.end(), p, p + k);
      p += k;
      n -= k;
    }
    return !failed_.load();
  }

  // Write what is left, stop the thread; true when every write succeeded.
  bool finish() {
    if (th_.joinable()) {
      if (!cur_.empty()) flush_current();
      {
        std::lock_guard<std::mutex> lk(mu_);
        stop_ = true;
      }
      cv_.notify_all();
      th_.join();
    }
    return !failed_.load();
  }

 private:
  static constexpr size_t kBuf = 16ull << 20;
  static constexpr size_t kInFlight = 4;

  void flush_current() {
    std::unique_lock<std::mutex> lk(mu_);
    cv_.wait(lk, [&] { return q_.size() < kInFlight; });
    q_.push_back(std::move(cur_));
    cur_ = std::vector<char>();
    cur_.reserve(kBuf);
    cv_.notify_all();
  }

  void loop() {
    for (;;) {
      std::vector<char> b;
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return stop_ || !q_.empty(); });
        if (q_.empty()) return;
        b = std::move(q_.front());
        q_.pop_front();
      }
      cv_.notify_all();
      if (!b.empty() && std::fwrite(b.data(), 1, b.size(), f_) != b.size()) failed_ = true;
    }
  }

  FILE* f_;
  std::vector<char> cur_;
  std::deque<std::vector<char>> q_;
  std::mutex mu_;
  std::condition_variable cv_;
  bool stop_ = false;
  std::atomic<bool> failed_{false};
  std::thread th_;
};

int writer_sink(void* user, int32_t kind, const void* bytes, uint64_t n) {
  FileWriter** w = static_cast<FileWriter**>(user);
  return w[kind == OOC_STREAM_NODES ? 0 : 1]->put(bytes, (size_t)n) ? 0 : 1;
}

}  // namespace

extern "C" int ooc_build_files(ooc_ctx* ctx, const char* tri_path, const ooc_build_params* params_in, char* out_base,
                               uint64_t out_base_len, ooc_build_info* info) {
  if (!ctx || !tri_path || !params_in) return OOC_ERR_INVALID;
  using clock = std::chrono::steady_clock;
  auto ms_since = [](clock::time_point t) {
    return (float)std::chrono::duration<double, std::milli>(clock::now() - t).count();
  };
  const clock::time_point t_read = clock::now();
  ooc::set_ctx_file_times(ctx, 0.0f, 0.0f);
  TriHeader h;
  std::string err;
  if (!parse_tri_header(tri_path, h, err)) {
    ooc::set_ctx_error(ctx, err);
    return OOC_ERR_IO;
  }
  ooc_build_params prm = *params_in;
  prm.geometry_only = h.geo_only ? 1 : 0;
  for (int a = 0; a < 3; a++) {
    prm.bbox_min[a] = h.bmin[a];
    prm.bbox_max[a] = h.bmax[a];
  }
  const int stride = prm.geometry_only ? 9 : 21;
  const size_t bytes = (size_t)h.n_triangles * stride * sizeof(float);
  // out of core: the .tridata is read group of partitions by group, never whole
  const bool streamed = ooc::file_wants_stream(ctx, &prm, h.n_triangles);
  void* tris = nullptr;
  if (streamed) {
    FILE* probe = std::fopen((h.base + ".tridata").c_str(), "rb");
    long size = -1;
    if (probe && std::fseek(probe, 0, SEEK_END) == 0) size = std::ftell(probe);
    if (probe) std::fclose(probe);
    if (!probe || size < 0 || (uint64_t)size < bytes) {
      ooc::set_ctx_error(ctx, probe ? "short read of " + h.base + ".tridata" : "cannot open " + h.base + ".tridata");
      return OOC_ERR_IO;
    }
  } else if (bytes && cudaMalloc(&tris, bytes) != cudaSuccess) {
    ooc::set_ctx_error(ctx, "cannot allocate " + std::to_string(bytes) + " bytes of device memory for the triangles");
    return OOC_ERR_OOM;
  }
  if (!streamed && bytes && !read_to_device(h.base + ".tridata", bytes, tris, err)) {
    cudaFree(tris);
    ooc::set_ctx_error(ctx, err);
    return OOC_ERR_IO;
  }
  const float read_ms = ms_since(t_read);
  const uint64_t P = ooc_estimate_partitions(prm.gridsize, prm.memory_limit_mb);
  // <base><gridsize>_<npartitions> (partitioner.cpp:90, 141; main.cpp:325)
  const std::string base = h.base + std::to_string(prm.gridsize) + "_" + std::to_string(P);
  FILE* fn = std::fopen((base + ".octreenodes").c_str(), "wb");
  FILE* fd = std::fopen((base + ".octreedata").c_str(), "wb");
  int rc = OOC_OK;
  clock::time_point t_write = clock::now();
  ooc_build_info local;
  std::memset(&local, 0, sizeof(local));
  if (!fn || !fd) {
    rc = OOC_ERR_IO;
    ooc::set_ctx_error(ctx, "cannot create " + base + (fn ? ".octreedata" : ".octreenodes"));
  } else {
    FileWriter wn(fn), wd(fd);
    FileWriter* w[2] = {&wn, &wd};
    rc = streamed ? ooc::build_from_file_stream(ctx, &prm, (h.base + ".tridata").c_str(), h.n_triangles, writer_sink,
                                                w, &local)
                  : ooc_build_from_device(ctx, &prm, static_cast<const float*>(tris), h.n_triangles, writer_sink, w,
                                          &local);
    t_write = clock::now();
    const bool ok_n = wn.finish(), ok_d = wd.finish();
    if (rc == OOC_OK && !(ok_n && ok_d)) {
      rc = OOC_ERR_IO;
      ooc::set_ctx_error(ctx, "cannot write " + base + (ok_n ? ".octreedata" : ".octreenodes"));
    }
  }
  if (fn) std::fclose(fn);
  if (fd) std::fclose(fd);
  if (tris) cudaFree(tris);
  if (rc != OOC_OK) return rc;
  // writeOctreeHeader (octree_io.h:74-83)
  std::ofstream out((base + ".octree").c_str(), std::ios::out);
  out << "#octreeheader 1" << std::endl;
  out << "gridlength " << prm.gridsize << std::endl;
  out << "n_nodes " << local.n_nodes << std::endl;
  out << "n_data " << local.n_data << std::endl;
  out << "END" << std::endl;
  out.close();
  if (!out) {
    ooc::set_ctx_error(ctx, "cannot write " + base + ".octree");
    return OOC_ERR_IO;
  }
  ooc::set_ctx_file_times(ctx, read_ms, ms_since(t_write));
  if (out_base && out_base_len) {
    std::strncpy(out_base, base.c_str(), (size_t)out_base_len - 1);
    out_base[out_base_len - 1] = 0;
  }
  if (info) *info = local;
  return OOC_OK;
}
