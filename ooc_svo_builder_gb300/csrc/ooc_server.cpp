// Serving loop: requests are admitted by their computed HBM footprint and
// run in continuously formed batches.
//
// Each engine is a library context with its own streams.  An engine that is
// free takes every queued request that fits the remaining memory budget (up to
// max_batch) and builds them with one batch call; requests that arrive
// meanwhile wait for the next free engine.  With two or more engines, one
// batch's device work overlaps the next batch's.  A request completes as soon
// as its own mesh does.  Every batch is built into device memory, allocated
// stream-ordered from the device's memory pool.  Resident results stay there
// until the caller releases them; host results are copied into pinned blocks of
// a pool the server keeps, on a stream of its own, and a delivery thread frees
// their device memory and publishes them once the copy has landed.  Apart from
// those allocations the server uses only the public C ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "ooc_extents.h"
#include "ooc_footprint.h"
#include "ooc_svo_gpu.h"

namespace {

using Clock = std::chrono::steady_clock;
using ooc::Extents;
using ooc::voxel_bound;

// Pinned host memory for host results.  With ooc_server_config::host_pool_mb
// the server pins that much once, at creation, and carves each result's blocks
// out of it (best fit, freed extents merged with their neighbours): pinning
// memory costs far more than copying into it, and it holds a lock of the CUDA
// driver that other threads' calls wait for.  A block the arena cannot hold, or
// every block without an arena, comes from a pool of separately pinned blocks
// kept for reuse: the smallest free block that holds the request, if it is at
// most four times its size, else a new block of the next power of two from
// 64 KiB.
//
// A reserve outlives its server: it goes back to a process-wide list and the
// next server that asks for that many bytes takes it, pinned already.
std::mutex g_reserves_mu;
std::multimap<size_t, void*> g_reserves;  // pinned reserves of destroyed servers, by size

class PinnedPool {
 public:
  ~PinnedPool() {
    for (auto& kv : free_) cudaFreeHost(kv.second);
    if (arena_) {
      std::lock_guard<std::mutex> lk(g_reserves_mu);
      g_reserves.emplace(arena_bytes_, arena_);
    }
  }
  // Pins the arena (or takes a kept one of that size); false when the host cannot pin that much.
  bool reserve(size_t bytes) {
    if (bytes == 0) return true;
    void* p = nullptr;
    {
      std::lock_guard<std::mutex> lk(g_reserves_mu);
      auto it = g_reserves.find(bytes);
      if (it != g_reserves.end()) {
        p = it->second;
        g_reserves.erase(it);
      }
    }
    if (!p) {
      if (cudaHostAlloc(&p, bytes, cudaHostAllocPortable) != cudaSuccess) return false;
      first_touch(p, bytes);
    }
    arena_ = static_cast<char*>(p);
    arena_bytes_ = bytes;
    extents_.reset(bytes, kGrain);
    return true;
  }
  // A block of at least n bytes: from the reserve, from the kept blocks, or newly pinned.
  // Blocks pinned while serving are bounded (the reserve's size, 8 GiB at least): at the
  // bound (or once the server is closing) this returns nullptr, and the caller retries
  // after results have been released (wait_put).
  void* try_get(size_t n, size_t& cap) {
    std::unique_lock<std::mutex> lk(mu_);
    if (void* p = take(n, cap)) return p;
    size_t c = 64 << 10;
    while (c < n) c <<= 1;
    if (closing_ || on_demand_bytes_ + c > on_demand_limit()) return nullptr;
    on_demand_bytes_ += c;
    on_demand_allocs_++;
    lk.unlock();
    void* p = nullptr;
    if (cudaMallocHost(&p, c) == cudaSuccess) {
      cap = c;
      return p;
    }
    lk.lock();
    on_demand_bytes_ -= c;
    on_demand_allocs_--;
    return nullptr;
  }
  // Waits until a block is returned (or the pool closes), at most `t`.
  void wait_put(std::chrono::microseconds t) {
    std::unique_lock<std::mutex> lk(mu_);
    if (!closing_) cv_.wait_for(lk, t);
  }
  // Copies from the device over all of a freshly pinned block, once.  The first copy
  // into a page of newly pinned memory is the slow one: 56 GB/s against 193 GB/s into
  // the same block afterwards, measured on a box that had been serving.  Done here, it
  // stays out of the deliveries.
  static void first_touch(void* p, size_t bytes) {
    constexpr size_t kPiece = 64ull << 20;
    void* d = nullptr;
    cudaStream_t st = nullptr;
    if (cudaMalloc(&d, kPiece) != cudaSuccess) return;  // only a warm-up: skipped without memory
    if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess) {
      for (size_t off = 0; off < bytes; off += kPiece)
        if (cudaMemcpyAsync(static_cast<char*>(p) + off, d, std::min(kPiece, bytes - off), cudaMemcpyDeviceToHost,
                            st) != cudaSuccess)
          break;
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
    cudaFree(d);
  }
  // Refuses new pins and wakes wait_put, for good (the server is being destroyed).
  void close() {
    std::lock_guard<std::mutex> lk(mu_);
    closing_ = true;
    cv_.notify_all();
  }
  // reserve bytes, of them free, pinned outside the reserve, and the pins that took
  void stats(uint64_t& reserve, uint64_t& reserve_free, uint64_t& on_demand, uint64_t& allocs) {
    std::lock_guard<std::mutex> lk(mu_);
    reserve = arena_bytes_;
    reserve_free = extents_.free_bytes();
    on_demand = on_demand_bytes_;
    allocs = on_demand_allocs_;
  }
  void put(void* p, size_t cap) {
    if (!p) return;
    std::lock_guard<std::mutex> lk(mu_);
    cv_.notify_all();  // a delivery waiting at the bound may fit now
    char* c = static_cast<char*>(p);
    if (arena_ && c >= arena_ && c < arena_ + arena_bytes_) {
      extents_.put((size_t)(c - arena_), cap);
      return;
    }
    free_.emplace(cap, p);
  }

 private:
  static constexpr size_t kGrain = 64 << 10;
  size_t on_demand_limit() const { return std::max<size_t>(arena_bytes_, 8ull << 30); }
  // From the reserve (best fit) or a kept block at most four times the size; mu_ held.
  void* take(size_t n, size_t& cap) {
    size_t off = 0;
    if (arena_ && extents_.take(n, off, cap)) return arena_ + off;
    auto it = free_.lower_bound(n);
    if (it != free_.end() && it->first / 4 <= n) {
      cap = it->first;
      void* p = it->second;
      free_.erase(it);
      return p;
    }
    return nullptr;
  }
  std::mutex mu_;
  std::condition_variable cv_;
  bool closing_ = false;
  uint64_t on_demand_bytes_ = 0, on_demand_allocs_ = 0;
  std::multimap<size_t, void*> free_;  // separately pinned blocks, by capacity
  char* arena_ = nullptr;
  size_t arena_bytes_ = 0;
  Extents extents_;  // the reserve's free blocks
};

struct Request {
  uint64_t id = 0;
  ooc_mesh mesh;
  uint64_t footprint = 0;
  bool sized = false;                         // footprint computed (by a sizing thread)
  void* h_nodes = nullptr;                    // host results (pinned pool blocks)
  void* h_data = nullptr;
  size_t h_nodes_cap = 0, h_data_cap = 0;
  uint64_t h_nodes_bytes = 0, h_data_bytes = 0;
  void* d_nodes = nullptr;                    // device results
  void* d_data = nullptr;
  uint64_t d_nodes_bytes = 0, d_data_bytes = 0;
  ooc_build_info info;
  int32_t status = OOC_OK;
  double t_submit = 0, t_start = 0, t_built = 0, t_done = 0;
  uint64_t batch_size = 0;
};

// The per-mesh checks ooc_build makes on its parameters, so that a request
// that would fail is refused at submission and never shares a batch.
bool valid(const ooc_mesh& m) {
  const ooc_build_params& p = m.params;
  const uint64_t N = p.gridsize;
  if (N == 0 || (N & (N - 1)) != 0 || N > 65536) return false;
  if (p.memory_limit_mb < 1 || (p.geometry_only != 0 && p.geometry_only != 1)) return false;
  if (p.color_mode < 0 || p.color_mode > 3 || p.reserved != 0) return false;
  if (m.n_tris >= (1ull << 32) || (m.n_tris && !m.tris)) return false;
  return ooc_estimate_partitions(N, p.memory_limit_mb) <= (1ull << 21);
}

// HBM a request may hold while it is in flight: its triangles, the occupancy
// pyramids of its stripes, and per-node arrays plus output records for an upper
// bound on its nodes.  A tree with L leaves at depth D has at most min(8^l, L)
// nodes at level l.  The leaves are at most the summed per-triangle bounds on the
// voxels a triangle can set: the voxels of its grid box (voxelizer.cpp:189-204
// tests no other), and, for a triangle with a finite plane, the voxels that
// overlap it (the Schwarz-Seidel test is the triangle-box overlap test): their
// centres lie within the triangle grown by a cube of side u, so the voxels
// themselves lie within the triangle grown by a ball of radius sqrt(3) u, whose
// volume is 2 r A + (pi / 2) r^2 L + (4 / 3) pi r^3 for area A and perimeter L
// (Steiner's formula for a flat convex body).  A node costs at most kNodeBytes:
// its 24-byte record and 32-byte data record, its key, subtree sizes and
// starts, first child and winner (7 x 4 bytes) and its -levels cache (24
// bytes), with room for the batch's job tables.
constexpr uint64_t kNodeBytes = 120;
constexpr uint64_t kDeliverPiece = 16ull << 20;  // bytes per copy of a host result's copy back
constexpr std::chrono::seconds kPinWait{10};     // a host result waits this long for pinned memory
constexpr int kSizers = 4;  // threads that compute the footprints of submitted requests

uint64_t footprint(const ooc_mesh& m) {
  const ooc_build_params& p = m.params;
  const uint64_t N = p.gridsize;
  const uint64_t stride = p.geometry_only ? 9 : 21;
  uint64_t bytes = m.n_tris * stride * 4;
  int D = 0;
  while ((1ull << D) < N) D++;
  const uint64_t P = ooc_estimate_partitions(N, p.memory_limit_mb);
  int kP = 0;
  while ((1ull << (3 * kP)) < P) kP++;
  const int Ds = std::min(D - kP, 10);
  uint64_t words = 0;
  for (int l = 0; l <= Ds; l++) words += (((1ull << (3 * l)) + 31) / 32 + 7) / 8 * 8;
  const uint64_t stripes = (N * N * N) >> (3 * Ds);
  bytes += words * 4 * stripes;
  const float unit_div = 1.0f / ((p.bbox_max[0] - p.bbox_min[0]) / (float)N);
  const double cells = (double)N * (double)N * (double)N;
  double leaves = 0.0;
  for (uint64_t t = 0; t < m.n_tris && leaves < cells; t++) leaves += voxel_bound(m.tris + t * stride, unit_div, N);
  leaves = std::min(leaves, cells);
  double nodes = 0.0;
  for (int l = 0; l <= D; l++) nodes += std::min(std::ldexp(1.0, 3 * l), leaves);
  bytes += (uint64_t)std::min(nodes * (double)kNodeBytes, 1.8e19);
  return bytes;
}

}  // namespace

struct ooc_server {
  ooc_server_config cfg;
  std::vector<ooc_ctx*> engines;
  std::vector<std::thread> threads;
  cudaStream_t release_stream = nullptr;  // device results are freed on it
  cudaStream_t d2h_stream = nullptr;      // host results are copied back on it
  PinnedPool pinned;
  // host results: complete on the device, waiting for the delivery thread to queue their
  // copy back; and those whose copy back is queued, in order, with the event after it
  std::deque<Request*> to_copy;
  std::deque<std::pair<Request*, cudaEvent_t>> deliveries;
  std::vector<cudaEvent_t> spare_events;
  std::condition_variable cv_deliver;
  std::thread deliverer;
  bool stop_delivery = false;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request*> queue;                   // submission order
  std::deque<Request*> unsized;                 // footprints not yet computed, oldest first
  std::condition_variable cv_size;
  std::vector<std::thread> sizers;
  std::deque<Request*> done;
  std::unordered_map<uint64_t, Request*> held;  // polled, not yet released
  uint64_t next_id = 1;
  uint64_t in_flight = 0;  // admitted footprints, plus device results not yet released
  std::atomic<bool> injected{false};  // the fault injection of cfg.fail_batch_at_mesh has fired
  bool stop = false;
  Clock::time_point t0 = Clock::now();

  double now_us() const { return std::chrono::duration<double, std::micro>(Clock::now() - t0).count(); }

  // A request is admitted in submission order, once its footprint is known and
  // fits.  Every sized request left in the queue is within the budget (larger ones
  // are refused by the sizing threads), so it fits once nothing else holds memory.
  bool fits(const Request* r) const { return r->sized && in_flight + r->footprint <= cfg.memory_budget; }

  // Footprints are computed off the submitting thread: one pass over a request's
  // triangles costs up to milliseconds for large meshes.
  void sizing_loop() {
    for (;;) {
      Request* r = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_size.wait(lk, [&] { return stop || !unsized.empty(); });
        if (stop) return;
        r = unsized.front();
        unsized.pop_front();
      }
      const uint64_t fp = footprint(r->mesh);
      bool refused = false;
      {
        std::lock_guard<std::mutex> lk(mu);
        if (stop) return;  // the server is shutting down; `r` is dropped with the queue
        r->footprint = fp;
        r->sized = true;
        if (fp > cfg.memory_budget) {
          auto it = std::find(queue.begin(), queue.end(), r);
          if (it != queue.end()) queue.erase(it);
          refused = true;
        }
      }
      if (refused) publish(r, OOC_ERR_LIMIT);
      cv_work.notify_all();
    }
  }

  // A request is complete (and can be polled, then released by the caller)
  // as soon as its mesh is; the engine does not touch it afterwards.
  void publish(Request* r, int32_t status) {
    {
      std::lock_guard<std::mutex> lk(mu);
      r->status = status;
      r->t_done = now_us();
      if (status == OOC_OK) in_flight += r->d_nodes_bytes + r->d_data_bytes;  // held until released
      done.push_back(r);
    }
    cv_done.notify_all();
  }

  struct Call {
    ooc_server* s;
    std::vector<Request*> reqs;
    std::vector<ooc_build_info> infos;
    std::vector<char>* published;  // by index into the engine's batch
    std::vector<size_t> index;
    bool inject = false;  // fault injection armed for this call
  };

  // ooc_server_config::fail_batch_at_mesh: whether this batch's mesh `mesh` is the one to fail
  static bool injected_failure(Call& call, uint64_t mesh) {
    if (!call.inject || mesh + 1 != call.s->cfg.fail_batch_at_mesh) return false;
    return !call.s->injected.exchange(true);  // once per server
  }

  static void mark(Call& call, uint64_t mesh) {
    Request* r = call.reqs[mesh];
    r->t_built = call.s->now_us();
    r->info = call.infos[mesh];
    (*call.published)[call.index[mesh]] = 1;
    call.s->publish(r, OOC_OK);
  }

  static int alloc(void* user, uint64_t mesh, uint64_t nodes_bytes, uint64_t data_bytes, void* stream, void** nodes,
                   void** data) {
    Call& call = *static_cast<Call*>(user);
    Request* r = call.reqs[mesh];
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (injected_failure(call, mesh)) return 1;
    if (cudaMallocAsync(&r->d_nodes, nodes_bytes, st) != cudaSuccess) return 1;
    if (cudaMallocAsync(&r->d_data, data_bytes, st) != cudaSuccess) return 1;
    r->d_nodes_bytes = nodes_bytes;
    r->d_data_bytes = data_bytes;
    *nodes = r->d_nodes;
    *data = r->d_data;
    return 0;
  }

  static int ready(void* user, uint64_t mesh) {
    Call& call = *static_cast<Call*>(user);
    if (call.s->cfg.result_location == OOC_RESULT_DEVICE) {
      mark(call, mesh);
      return 0;
    }
    // host results: the mesh is complete in this batch (never rerun); the delivery
    // thread copies it into pinned memory and publishes it once the copy has landed.
    // Its device memory counts against the budget until then, so deliveries that fall
    // behind hold back admission instead of filling HBM.
    Request* r = call.reqs[mesh];
    r->t_built = call.s->now_us();
    r->info = call.infos[mesh];
    (*call.published)[call.index[mesh]] = 1;
    {
      std::lock_guard<std::mutex> lk(call.s->mu);
      call.s->in_flight += r->d_nodes_bytes + r->d_data_bytes;
      call.s->to_copy.push_back(r);
    }
    call.s->cv_deliver.notify_one();
    return 0;
  }

  // Queue a host result's copy back into pinned pool blocks on d2h_stream (delivery thread):
  // kQueued, kNoMemory (pinned memory at its bound: retry once results are released; a
  // block already taken stays with the request), or kFailed (published with an error).
  enum { kQueued = 0, kNoMemory = 1, kFailed = 2 };
  int deliver(Request* r) {
    r->h_nodes_bytes = r->d_nodes_bytes;
    r->h_data_bytes = r->d_data_bytes;
    if (r->h_nodes_bytes && !r->h_nodes && !(r->h_nodes = pinned.try_get(r->h_nodes_bytes, r->h_nodes_cap)))
      return kNoMemory;
    if (r->h_data_bytes && !r->h_data && !(r->h_data = pinned.try_get(r->h_data_bytes, r->h_data_cap)))
      return kNoMemory;
    bool ok = true;
    cudaEvent_t ev = nullptr;
    {
      std::lock_guard<std::mutex> lk(mu);
      if (!spare_events.empty()) {
        ev = spare_events.back();
        spare_events.pop_back();
      }
    }
    if (!ev) ok = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) == cudaSuccess;
    // in pieces, so that the engines' own small reads back (their level counts) do not
    // wait behind a whole result of hundreds of megabytes on the copy engine
    auto copy = [&](void* dst, const void* src, uint64_t bytes) {
      for (uint64_t off = 0; ok && off < bytes; off += kDeliverPiece)
        ok = cudaMemcpyAsync(static_cast<char*>(dst) + off, static_cast<const char*>(src) + off,
                             std::min<uint64_t>(kDeliverPiece, bytes - off), cudaMemcpyDeviceToHost,
                             d2h_stream) == cudaSuccess;
    };
    if (ok && r->h_nodes_bytes) copy(r->h_nodes, r->d_nodes, r->h_nodes_bytes);
    if (ok && r->h_data_bytes) copy(r->h_data, r->d_data, r->h_data_bytes);
    if (ok) ok = cudaEventRecord(ev, d2h_stream) == cudaSuccess;
    if (!ok) {
      if (ev) cudaEventDestroy(ev);
      cudaStreamSynchronize(d2h_stream);  // nothing of this request stays queued
      release_delivered(r);
      publish(r, OOC_ERR_OOM);
      return kFailed;
    }
    deliveries.push_back({r, ev});
    return kQueued;
  }

  // The delivery thread: queues the copy back of every host result the engines hand
  // over, in order (pinning pool blocks as needed, off the engines' threads), and
  // publishes the results in that order once each copy has landed.  When pinned memory
  // is at its bound, the waiting results stay queued while landed copies are published
  // (so the caller can release them); with nothing in flight either, the oldest waiting
  // result fails with OOC_ERR_OOM after kPinWait, or at once when the server is closing.
  void delivery_loop() {
    cudaSetDevice(cfg.device);
    std::deque<Request*> waiting;  // this thread's: handed over, copy not yet queued
    Clock::time_point starved_since{};
    for (;;) {
      bool closing = false;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_deliver.wait(lk, [&] { return stop_delivery || !to_copy.empty() || !deliveries.empty() || !waiting.empty(); });
        waiting.insert(waiting.end(), to_copy.begin(), to_copy.end());
        to_copy.clear();
        closing = stop_delivery;
        if (waiting.empty() && deliveries.empty()) return;
      }
      bool starved = false;
      while (!waiting.empty()) {
        if (deliver(waiting.front()) == kNoMemory) {
          starved = true;
          break;
        }
        waiting.pop_front();
      }
      if (!starved) starved_since = Clock::time_point{};
      else if (starved_since == Clock::time_point{}) starved_since = Clock::now();
      if (!deliveries.empty()) {
        const std::pair<Request*, cudaEvent_t> d = deliveries.front();
        // with results waiting (to be queued, or for memory), only take the oldest copy if it has landed
        bool more = starved;
        {
          std::lock_guard<std::mutex> lk(mu);
          more = more || !to_copy.empty();
        }
        const cudaError_t e = more ? cudaEventQuery(d.second) : cudaEventSynchronize(d.second);
        if (e == cudaErrorNotReady) {
          if (starved) pinned.wait_put(std::chrono::microseconds(200));
          continue;
        }
        deliveries.pop_front();
        Request* r = d.first;
        release_delivered(r);
        {
          std::lock_guard<std::mutex> lk(mu);
          spare_events.push_back(d.second);
        }
        publish(r, e == cudaSuccess ? OOC_OK : OOC_ERR_DEVICE);
        continue;
      }
      if (starved) {  // nothing in flight: only the caller's releases free pinned memory
        if (closing || Clock::now() - starved_since > kPinWait) {
          Request* r = waiting.front();
          waiting.pop_front();
          release_delivered(r);
          publish(r, OOC_ERR_OOM);
          starved_since = Clock::time_point{};
        } else {
          pinned.wait_put(std::chrono::milliseconds(10));
        }
      }
    }
  }

  // A host result's device memory, once its copy back is done or failed: freed and
  // taken off the budget.
  void release_delivered(Request* r) {
    free_device(r);
    {
      std::lock_guard<std::mutex> lk(mu);
      in_flight -= r->d_nodes_bytes + r->d_data_bytes;
    }
    r->d_nodes_bytes = r->d_data_bytes = 0;
    cv_work.notify_all();
  }

  void free_device(Request* r) {
    if (r->d_nodes) cudaFreeAsync(r->d_nodes, release_stream);
    if (r->d_data) cudaFreeAsync(r->d_data, release_stream);
    r->d_nodes = r->d_data = nullptr;
  }

  // One batch call over batch[index...]; each request is published when its mesh completes.
  int run(ooc_ctx* ctx, const std::vector<Request*>& batch, const std::vector<size_t>& index,
          std::vector<char>& published) {
    Call call{this, {}, std::vector<ooc_build_info>(index.size()), &published, index};
    call.inject = cfg.fail_batch_at_mesh != 0 && !injected.load() && index.size() > 1;
    std::vector<ooc_mesh> meshes(index.size());
    for (size_t i = 0; i < index.size(); i++) {
      Request* r = batch[index[i]];
      call.reqs.push_back(r);
      meshes[i] = r->mesh;
    }
    const int rc = ooc_build_batch_device(ctx, meshes.data(), meshes.size(), &ooc_server::alloc, &ooc_server::ready,
                                          &call, call.infos.data());
    if (rc != OOC_OK) {
      // the failed call may have left writes queued into the destinations
      cudaSetDevice(cfg.device);
      cudaDeviceSynchronize();
      for (size_t i = 0; i < index.size(); i++)
        if (!published[index[i]]) {
          free_device(call.reqs[i]);
          call.reqs[i]->d_nodes_bytes = call.reqs[i]->d_data_bytes = 0;
        }
    }
    return rc;
  }

  void engine_loop(ooc_ctx* ctx) {
    cudaSetDevice(cfg.device);
    for (;;) {
      std::vector<Request*> batch;
      uint64_t taken = 0;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_work.wait(lk, [&] { return stop || (!queue.empty() && fits(queue.front())); });
        if (stop && queue.empty()) return;
        while (!queue.empty() && batch.size() < cfg.max_batch && fits(queue.front())) {
          Request* r = queue.front();
          queue.pop_front();
          in_flight += r->footprint;
          taken += r->footprint;
          batch.push_back(r);
        }
      }
      if (batch.empty()) {  // shutting down while another engine still holds the budget
        std::this_thread::sleep_for(std::chrono::microseconds(100));
        continue;
      }
      const double ts = now_us();
      for (Request* r : batch) {
        r->t_start = ts;
        r->batch_size = batch.size();
      }
      std::vector<char> published(batch.size(), 0);
      std::vector<size_t> all(batch.size());
      for (size_t i = 0; i < batch.size(); i++) all[i] = i;
      const int rc = run(ctx, batch, all, published);
      if (rc != OOC_OK) {
        // A failure (out of memory, too many triangle/partition pairs) belongs
        // to one request: the ones not yet complete run again alone, so that
        // only the failing one reports it.
        for (size_t i = 0; i < batch.size(); i++) {
          if (published[i]) continue;
          int rc1 = rc;
          if (batch.size() > 1) {
            batch[i]->batch_size = 1;
            rc1 = run(ctx, batch, std::vector<size_t>(1, i), published);
          }
          if (!published[i]) publish(batch[i], rc1 != OOC_OK ? rc1 : OOC_ERR_DEVICE);
        }
      }
      {
        std::lock_guard<std::mutex> lk(mu);
        in_flight -= taken;
      }
      cv_work.notify_all();
    }
  }
};

extern "C" {

int ooc_server_create(const ooc_server_config* cfg, ooc_server** out) {
  if (!cfg || !out || cfg->engines < 1 || cfg->max_batch < 1 || cfg->memory_budget == 0) return OOC_ERR_INVALID;
  if (cfg->result_location != OOC_RESULT_HOST && cfg->result_location != OOC_RESULT_DEVICE) return OOC_ERR_INVALID;
  *out = nullptr;
  ooc_server* s = new (std::nothrow) ooc_server();
  if (!s) return OOC_ERR_OOM;
  s->cfg = *cfg;
  for (int i = 0; i < cfg->engines; i++) {
    ooc_ctx* c = nullptr;
    const int rc = ooc_ctx_create(cfg->device, &c);
    if (rc != OOC_OK) {
      for (ooc_ctx* e : s->engines) ooc_ctx_destroy(e);
      delete s;
      return rc;
    }
    s->engines.push_back(c);
  }
  {
    // keep freed result memory in the pool instead of returning it to the driver at every synchronisation
    cudaMemPool_t pool;
    uint64_t keep = ~0ull;
    if (cudaSetDevice(cfg->device) != cudaSuccess || cudaDeviceGetDefaultMemPool(&pool, cfg->device) != cudaSuccess ||
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->release_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&s->d2h_stream, cudaStreamNonBlocking) != cudaSuccess) {
      if (s->release_stream) cudaStreamDestroy(s->release_stream);
      for (ooc_ctx* e : s->engines) ooc_ctx_destroy(e);
      delete s;
      return OOC_ERR_DEVICE;
    }
  }
  if (cfg->result_location == OOC_RESULT_HOST && !s->pinned.reserve((size_t)cfg->host_pool_mb << 20)) {
    cudaStreamDestroy(s->release_stream);
    cudaStreamDestroy(s->d2h_stream);
    for (ooc_ctx* e : s->engines) ooc_ctx_destroy(e);
    delete s;
    return OOC_ERR_OOM;
  }
  if (cfg->result_location == OOC_RESULT_HOST) s->deliverer = std::thread([s] { s->delivery_loop(); });
  for (int i = 0; i < kSizers; i++) s->sizers.emplace_back([s] { s->sizing_loop(); });
  for (ooc_ctx* c : s->engines) s->threads.emplace_back([s, c] { s->engine_loop(c); });
  *out = s;
  return OOC_OK;
}

int ooc_server_submit(ooc_server* s, const ooc_mesh* mesh, uint64_t* id) {
  if (!s || !mesh || !valid(*mesh)) return OOC_ERR_INVALID;
  const double t = s->now_us();
  Request* r = new (std::nothrow) Request();
  if (!r) return OOC_ERR_OOM;
  r->mesh = *mesh;
  r->t_submit = t;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    r->id = s->next_id++;
    s->queue.push_back(r);
    s->unsized.push_back(r);
  }
  if (id) *id = r->id;
  s->cv_size.notify_one();
  return OOC_OK;
}

int ooc_server_poll(ooc_server* s, int32_t timeout_ms, ooc_result* out) {
  if (!s || !out) return OOC_ERR_INVALID;
  Request* r = nullptr;
  {
    std::unique_lock<std::mutex> lk(s->mu);
    if (!s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms < 0 ? 0 : timeout_ms),
                             [&] { return !s->done.empty(); }))
      return OOC_ERR_TIMEOUT;
    r = s->done.front();
    s->done.pop_front();
    s->held[r->id] = r;
  }
  std::memset(out, 0, sizeof(*out));
  out->id = r->id;
  out->status = r->status;
  out->location = s->cfg.result_location;
  if (s->cfg.result_location == OOC_RESULT_DEVICE) {
    out->nodes = r->d_nodes;
    out->nodes_bytes = r->status == OOC_OK ? r->d_nodes_bytes : 0;
    out->data = r->d_data;
    out->data_bytes = r->status == OOC_OK ? r->d_data_bytes : 0;
  } else {
    out->nodes = r->h_nodes;
    out->nodes_bytes = r->status == OOC_OK ? r->h_nodes_bytes : 0;
    out->data = r->h_data;
    out->data_bytes = r->status == OOC_OK ? r->h_data_bytes : 0;
  }
  out->info = r->info;
  out->t_submit_us = r->t_submit;
  out->t_start_us = r->t_start;
  out->t_built_us = r->t_built;
  out->t_done_us = r->t_done;
  out->batch_size = r->batch_size;
  return OOC_OK;
}

int ooc_server_stats(ooc_server* s, ooc_server_state* out) {
  if (!s || !out) return OOC_ERR_INVALID;
  std::memset(out, 0, sizeof(*out));
  {
    std::lock_guard<std::mutex> lk(s->mu);
    out->queued = s->queue.size();
    out->in_flight_bytes = s->in_flight;
    out->completed_unpolled = s->done.size();
    out->held = s->held.size();
    out->deliveries = s->to_copy.size();
  }
  s->pinned.stats(out->pinned_reserve_bytes, out->pinned_reserve_free_bytes, out->pinned_on_demand_bytes,
                  out->pinned_on_demand_allocs);
  return OOC_OK;
}

int ooc_server_read(ooc_server* s, uint64_t id, void* nodes_host, void* data_host) {
  if (!s) return OOC_ERR_INVALID;
  Request* r = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->held.find(id);
    if (it == s->held.end()) return OOC_ERR_INVALID;
    r = it->second;
  }
  if (r->status != OOC_OK) return r->status;
  if (s->cfg.result_location == OOC_RESULT_DEVICE) {
    if (cudaSetDevice(s->cfg.device) != cudaSuccess) return OOC_ERR_DEVICE;
    if (nodes_host && cudaMemcpy(nodes_host, r->d_nodes, r->d_nodes_bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      return OOC_ERR_DEVICE;
    if (data_host && cudaMemcpy(data_host, r->d_data, r->d_data_bytes, cudaMemcpyDeviceToHost) != cudaSuccess)
      return OOC_ERR_DEVICE;
  } else {
    if (nodes_host && r->h_nodes_bytes) std::memcpy(nodes_host, r->h_nodes, r->h_nodes_bytes);
    if (data_host && r->h_data_bytes) std::memcpy(data_host, r->h_data, r->h_data_bytes);
  }
  return OOC_OK;
}

int ooc_server_release(ooc_server* s, uint64_t id) {
  if (!s) return OOC_ERR_INVALID;
  Request* r = nullptr;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->held.find(id);
    if (it == s->held.end()) return OOC_ERR_INVALID;
    r = it->second;
    s->held.erase(it);
    if (r->status == OOC_OK) s->in_flight -= r->d_nodes_bytes + r->d_data_bytes;
  }
  if (r->d_nodes || r->d_data) {
    cudaSetDevice(s->cfg.device);
    s->free_device(r);
  }
  s->pinned.put(r->h_nodes, r->h_nodes_cap);
  s->pinned.put(r->h_data, r->h_data_cap);
  delete r;
  s->cv_work.notify_all();
  return OOC_OK;
}

void ooc_server_destroy(ooc_server* s) {
  if (!s) return;
  std::deque<Request*> dropped;  // never started
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
    dropped.swap(s->queue);
    s->unsized.clear();
  }
  s->cv_size.notify_all();
  for (std::thread& t : s->sizers) t.join();  // a sizing thread may still hold one of `dropped`
  for (Request* r : dropped) delete r;
  s->cv_work.notify_all();
  for (std::thread& t : s->threads) t.join();
  {  // the engines are done: deliver what they queued, then stop
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop_delivery = true;
  }
  s->pinned.close();  // a delivery waiting for pinned memory gives up rather than wait for releases
  s->cv_deliver.notify_all();
  if (s->deliverer.joinable()) s->deliverer.join();
  for (ooc_ctx* c : s->engines) ooc_ctx_destroy(c);
  cudaSetDevice(s->cfg.device);
  auto drop = [s](Request* r) {
    s->free_device(r);
    s->pinned.put(r->h_nodes, r->h_nodes_cap);
    s->pinned.put(r->h_data, r->h_data_cap);
    delete r;
  };
  for (Request* r : s->done) drop(r);
  for (auto& kv : s->held) drop(kv.second);
  for (cudaEvent_t e : s->spare_events) cudaEventDestroy(e);
  if (s->release_stream) {
    cudaStreamSynchronize(s->release_stream);
    cudaStreamDestroy(s->release_stream);
  }
  if (s->d2h_stream) cudaStreamDestroy(s->d2h_stream);
  delete s;
}

}  // extern "C"
