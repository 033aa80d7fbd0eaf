/*
 * ooc_svo_gpu.h -- C ABI of the GB300 partition -> voxelize -> SVO-build path.
 *
 * Library: ooc_svo_builder_gb300/libooc_svo_gpu.so (CUDA sm_103a).
 *
 * The reference (ooc_svo_builder v1.6.4) has no plugin or FFI layer; its
 * boundary is the svo_builder / svo_builder_binary command line and the
 * .tri/.tridata -> .octree/.octreenodes/.octreedata file formats.  The calls
 * below replace the reference's internal C++ seams that main.cpp drives:
 *
 *   ooc_estimate_partitions   estimate_partitions      partitioner.cpp:12-28
 *   ooc_build / ooc_build_device
 *                             partition                partitioner.cpp:101-149
 *                             + voxelize_schwarz_method voxelizer.cpp:139-307
 *                             + std::sort + colour modes main.cpp:354-385
 *                             + OctreeBuilder::addVoxel / finalizeTree
 *                                                      OctreeBuilder.cpp:34-167
 *                             (the whole loop of main.cpp:294-392)
 *
 * Output bytes are those of the reference's files: the node file is n_nodes
 * records of 24 bytes {u64 data, u64 children_base, i8 children_offset[8]}
 * (octree_io.h:62-66), the data file n_data records of 32 bytes
 * {u64 morton, f32 color[3], f32 normal[3]} (octree_io.h:49-53).
 *
 * Conventions: every call returns OOC_OK (0) or an OOC_ERR_* code and never
 * throws; ooc_last_error() describes the last failure of a context.  One host
 * thread per context; any number of contexts.  All device memory and streams
 * belong to the library.
 */
#ifndef OOC_SVO_GPU_H_
#define OOC_SVO_GPU_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OOC_OK 0
#define OOC_ERR_INVALID 1  /* bad argument (gridsize not a power of two, ...)    */
#define OOC_ERR_OOM 2      /* device or pinned-host allocation failed            */
#define OOC_ERR_DEVICE 3   /* a CUDA call or kernel failed                       */
#define OOC_ERR_IO 4       /* file could not be read or written                  */
#define OOC_ERR_SINK 5     /* the caller's sink returned non-zero                */
#define OOC_ERR_LIMIT 6    /* input beyond the fixed limits of ooc_voxelize_occupancy_noalloc */
#define OOC_ERR_TIMEOUT 7  /* ooc_server_poll: nothing completed within the timeout                */

/* Colour modes of svo_builder's -c flag (main.cpp:23, 154-179). */
#define OOC_COLOR_MODEL 0
#define OOC_COLOR_FIXED 1
#define OOC_COLOR_LINEAR 2
#define OOC_COLOR_NORMAL 3

/* Which file a sink call carries. */
#define OOC_STREAM_NODES 0
#define OOC_STREAM_DATA 1
#define OOC_STREAM_END 2   /* ooc_batch_sink_fn only: the mesh is complete (bytes NULL, nbytes 0) */

typedef struct ooc_ctx ooc_ctx;

/* Build parameters: the flags of main.cpp:100-196 plus the .tri header. */
typedef struct {
  uint64_t gridsize;        /* -s: power of two, 1 .. 65536                   */
  uint64_t memory_limit_mb; /* -l: sets the partition count like the reference */
  int32_t geometry_only;    /* 1: svo_builder_binary (9 floats / triangle);
                               0: svo_builder with payload (21 floats)         */
  int32_t color_mode;       /* OOC_COLOR_*; ignored when geometry_only == 1    */
  int32_t generate_levels;  /* -levels                                         */
  int32_t reserved;         /* must be 0                                       */
  float bbox_min[3];        /* .tri header bbox (only max.x - min.x is used,   */
  float bbox_max[3];        /*  as in main.cpp:311)                            */
} ooc_build_params;

typedef struct {
  uint64_t n_nodes;      /* octree header n_nodes                         */
  uint64_t n_data;       /* octree header n_data                          */
  uint64_t n_filled;     /* "Total amount of voxels" (main.cpp:391)       */
  uint64_t n_partitions; /* estimate_partitions result                    */
  uint64_t n_stripes;    /* device work units the grid was processed in   */
  uint64_t n_items;      /* (triangle, partition) pairs after binning     */
} ooc_build_info;

/* Receives the node file (kind OOC_STREAM_NODES) and the data file
 * (OOC_STREAM_DATA) in file order, in pieces.  `bytes` is valid only during
 * the call.  Return 0 to continue, non-zero to abort with OOC_ERR_SINK. */
typedef int (*ooc_sink_fn)(void* user, int32_t kind, const void* bytes, uint64_t nbytes);

/* Create a context on CUDA device `device`. */
int ooc_ctx_create(int32_t device, ooc_ctx** out);
void ooc_ctx_destroy(ooc_ctx* ctx);
/* Text of the last error of `ctx` (never NULL; "" after success). */
const char* ooc_last_error(const ooc_ctx* ctx);

/* estimate_partitions (partitioner.cpp:12-28): 1 if gridsize^3 bytes fit in
 * memory_limit_mb, otherwise the smallest 8^k that brings a partition under
 * the limit, dividing the megabyte count by 8 with integer division. */
uint64_t ooc_estimate_partitions(uint64_t gridsize, uint64_t memory_limit_mb);

/* Whole path from host triangles (n_tris records of 9 or 21 FP32 values,
 * pinned or pageable) to the octree, streamed to `sink` in file order.
 * Replaces main.cpp:294-392. */
int ooc_build(ooc_ctx* ctx, const ooc_build_params* params, const float* tris_host, uint64_t n_tris,
              ooc_sink_fn sink, void* user, ooc_build_info* info);

/* One mesh of a batch: host triangles (pinned or pageable) and its flags. */
typedef struct {
  const float* tris;
  uint64_t n_tris;
  ooc_build_params params;
} ooc_mesh;

/* Like ooc_sink_fn, with the index of the mesh whose file the bytes belong to.
 * Each mesh's files arrive in file order; meshes may interleave.  Meshes
 * complete in index order, each as soon as its last stripe is built: after a
 * mesh's last piece the sink is called once with kind OOC_STREAM_END (bytes
 * NULL, nbytes 0), and that mesh's ooc_build_info is final at that moment. */
typedef int (*ooc_batch_sink_fn)(void* user, uint64_t mesh, int32_t kind, const void* bytes, uint64_t nbytes);

/* Many meshes with their own gridsize, mode and flags in one call: every stripe
 * of every mesh goes through one launch sequence (split into sub-batches only
 * when the occupancy pyramids exceed the context's memory budget).  Each
 * mesh's output is byte-identical to ooc_build on that mesh.  `infos` (may be
 * NULL) receives one ooc_build_info per mesh.  No counterpart in the
 * reference, which builds one mesh per process. */
int ooc_build_batch(ooc_ctx* ctx, const ooc_mesh* meshes, uint64_t n_meshes, ooc_batch_sink_fn sink, void* user,
                    ooc_build_info* infos);

/* Triangles already in device memory (n_tris * 9 or 21 floats), octree files
 * delivered to the sink in host memory: the path of ooc_build without its
 * upload (the file front end reads .tridata straight to the device). */
int ooc_build_from_device(ooc_ctx* ctx, const ooc_build_params* params, const float* tris_device, uint64_t n_tris,
                          ooc_sink_fn sink, void* user, ooc_build_info* info);

/* ---- Batched build into device memory (no counterpart in the reference) ----
 * Like ooc_build_batch (host triangles in), but every mesh's node and data
 * files are written straight into device memory that the caller provides:
 * `alloc` is called once per mesh, in mesh order, as soon as the mesh's sizes
 * are known and before any of its records are written.  It returns two device
 * pointers (8-byte aligned) through `nodes` and `data`; `stream` is the
 * cudaStream_t the library writes them on, so memory allocated stream-ordered
 * on it (cudaMallocAsync) may be used.  `ready` (may be NULL) is called once
 * per mesh, in mesh order, when every byte of its files has been written.  The
 * files are byte-identical to what ooc_build writes for that mesh alone.
 * Both callbacks return 0, or non-zero to abort the call. */
typedef int (*ooc_alloc_fn)(void* user, uint64_t mesh, uint64_t nodes_bytes, uint64_t data_bytes, void* stream,
                            void** nodes, void** data);
typedef int (*ooc_ready_fn)(void* user, uint64_t mesh);
int ooc_build_batch_device(ooc_ctx* ctx, const ooc_mesh* meshes, uint64_t n_meshes, ooc_alloc_fn alloc,
                           ooc_ready_fn ready, void* user, ooc_build_info* infos);

/* A bump allocator over one caller-owned device buffer, usable as `alloc`
 * with `user` = the arena: each file starts on a 256-byte boundary; a full
 * arena fails the call with OOC_ERR_OOM. */
typedef struct {
  void* base;
  uint64_t capacity;
  uint64_t used;
} ooc_device_arena;
int ooc_arena_alloc(void* arena, uint64_t mesh, uint64_t nodes_bytes, uint64_t data_bytes, void* stream,
                    void** nodes, void** data);

/* ---- Tuning and the autotuner (no counterpart in the reference) ----
 * Launch choices of the voxelizer and the batch engine.  Every value gives the
 * same output; they only change speed. */
typedef struct {
  uint32_t small_vol;         /* triangles whose box has at most this many voxels run one per thread (1..64) */
  uint32_t lines_per_lane;    /* lines of a large triangle each lane of a warp task walks (1..64);
                                 the work-queue chunk is 32 x this many lines */
  uint32_t large_block;       /* threads per CTA of the large-triangle kernel: 64, 128 or 256 */
  uint32_t large_ctas_per_sm; /* persistent CTAs per SM of the large-triangle kernel (1..16) */
  uint64_t batch_budget;      /* occupancy-pyramid bytes per sub-batch (>= 4096), as ooc_set_batch_budget */
  uint32_t graphs;            /* 1: replay each sub-batch's two launch sequences as CUDA graphs; 0: launch directly */
  uint32_t light_per_thread;  /* elements each thread of the per-block and per-node kernels takes (1..16) */
  uint32_t pdl;               /* 1: each kernel of a launch sequence may start while its predecessor drains
                                 (programmatic dependent launch; it waits for the predecessor's results
                                 before touching memory); 0: it starts when the predecessor has finished */
  uint32_t persistent;        /* 1: the occupancy passes and the pyramid levels of a sub-batch run as one
                                 persistent launch whose warps take (stripe, chunk), large-triangle task
                                 and (stripe, level, block range) units from a device work queue; 0: one
                                 launch per pass and level */
} ooc_tuning;

int ooc_get_tuning(const ooc_ctx* ctx, ooc_tuning* out);
/* OOC_ERR_INVALID for a value out of range. */
int ooc_set_tuning(ooc_ctx* ctx, const ooc_tuning* tuning);
/* Time builds of `sample` (host triangles, results resident in a scratch
 * arena) over a coordinate search of the tuning values, keep the fastest in
 * the context and return it in `best` (may be NULL). */
int ooc_autotune(ooc_ctx* ctx, const ooc_mesh* sample, uint64_t n_meshes, ooc_tuning* best);

/* Bytes of occupancy pyramids one sub-batch may hold (default 4 GiB, at least
 * 4096): the stripes of a batch call run in sub-batches of at most this much
 * pyramid (a single stripe larger than it runs alone).  Output is the same for
 * every budget. */
int ooc_set_batch_budget(ooc_ctx* ctx, uint64_t bytes);
uint64_t ooc_batch_budget(const ooc_ctx* ctx);

/* Same path from triangles already in device memory; the octree stays in
 * device memory (see ooc_result_device).  `stream` is a cudaStream_t (NULL:
 * the context's own stream); all work is ordered on it and the call returns
 * after the stream has drained. */
int ooc_build_device(ooc_ctx* ctx, const ooc_build_params* params, const float* tris_device, uint64_t n_tris,
                     void* stream, ooc_build_info* info);

/* Device pointers to the node and data files produced by the last
 * ooc_build_device call of `ctx`; valid until the next build on `ctx`. */
int ooc_result_device(ooc_ctx* ctx, const void** nodes_device, const void** data_device);
/* Copy the last ooc_build_device result to host memory: n_nodes * 24 bytes to
 * `nodes_host` and n_data * 32 bytes to `data_host` (either may be NULL). */
int ooc_result_copy(ooc_ctx* ctx, void* nodes_host, void* data_host);

/* Device time in milliseconds of each phase of the last build of `ctx`
 * (CUDA events on the build stream): [0] partition binning, [1] voxelization
 * (both passes), [2] occupancy pyramid + scans, [3] octree layout and record
 * emission, [4] host<->device copies, [5] whole build.  `n` entries are
 * written (at most 6).  Phase timing is recorded only after
 * ooc_set_phase_timing(ctx, 1). */
int ooc_set_phase_timing(ooc_ctx* ctx, int32_t enable);
int ooc_phase_times(const ooc_ctx* ctx, float* ms, int32_t n);

/* Launch count of this library's kernels in the last build of `ctx`. */
uint64_t ooc_kernel_launches(const ooc_ctx* ctx);

/* Per-partition counts of the last build of `ctx` (its first mesh), for the
 * progress lines of the reference's driver: for partitions first ..
 * first + n - 1, the triangles binned to it (TripInfo::part_tricounts,
 * partitioner.cpp:80-98 and :101-149; with one partition every triangle) and
 * the voxels it filled ("found N new voxels", main.cpp:346-348).  Either
 * array may be NULL; entries past the last partition are left alone.
 * Returns the build's partition count (0 before the first build, or after a
 * failed one). */
uint64_t ooc_partition_counts(const ooc_ctx* ctx, uint64_t first, uint64_t n, uint64_t* triangles,
                              uint64_t* filled);

/* ---- Out-of-core builds (main.cpp:294-392: partitions streamed from disk) ----
 * A one-mesh build (ooc_build, ooc_build_batch of one mesh, ooc_build_files)
 * of more than one partition whose triangle records exceed the device
 * triangle budget never holds the mesh in device memory.  A first pass over
 * the triangles (host memory, or the .tridata file) counts each partition's
 * records with the reference's box test (partitioner.cpp:101-149); the
 * partitions are cut into consecutive groups whose records fit half the
 * budget; before a group's partitions are voxelized, another pass gathers
 * their records into device memory, each partition's in stream order, as the
 * reference's .tripdata files hold them.  The output is the in-core build's,
 * byte for byte.  One partition's records must fit half the budget
 * (OOC_ERR_LIMIT otherwise).  `bytes` = 0 (the default) makes the budget half
 * of the device memory free at the start of each build. */
int ooc_set_stream_budget(ooc_ctx* ctx, uint64_t bytes);
uint64_t ooc_stream_budget(const ooc_ctx* ctx);
/* Passes over the triangles of the last build of `ctx` (0: not built out of core). */
uint64_t ooc_stream_passes(const ooc_ctx* ctx);

/* Host wall-clock milliseconds of the file work of the last ooc_build_files
 * call of `ctx`: [0] reading the .tri header and the .tridata into device
 * memory, [1] writing the octree files after the build (waiting for the
 * writer threads, and the header).  They stand in for the reference's
 * IO IN / IO OUT timers (main.cpp:219-241).  `n` entries are written (at
 * most 2). */
int ooc_file_times(const ooc_ctx* ctx, float* ms, int32_t n);

/* Per-kernel CUDA-event timing of later builds on `ctx`: `kernel` names one
 * kernel (e.g. "vox_small_occupancy"), "*" selects all, NULL or "" turns it
 * off.  Each timed launch is bracketed by two events on the build stream. */
int ooc_set_kernel_timing(ooc_ctx* ctx, const char* kernel);
/* Entry `index` (0-based) of the last build's per-kernel timing: kernel name
 * (valid until the next build), summed device milliseconds, launch count.
 * Returns OOC_ERR_INVALID past the last entry. */
int ooc_kernel_time(const ooc_ctx* ctx, int32_t index, const char** name, float* total_ms, uint64_t* launches);

/* Occupancy pass without any allocation -- no counterpart in the reference.
 *
 * For callers that must not allocate GPU memory where they voxelize: code
 * running while its stream is captured into a CUDA graph, plugins whose host
 * engine owns and pre-reserves all device memory, and latency-critical loops
 * in which a cudaMalloc would synchronise the device.  The caller passes the
 * triangles (device memory, 9 or 21 FP32 values each as geometry_only says)
 * and the output; the only scratch is a fixed array compiled into the library
 * (about 8.4 MB held on every GPU that loads it, until the process exits).
 * Nothing is allocated: no cudaMalloc, no cudaFree, no allocating library call.
 *
 * Output: the grid's occupancy bitfield in Morton order, bit (m % 32) of word
 * m / 32 set when the voxel with Morton code m is set, exactly the voxels of
 * the reference's voxelize_schwarz_method (voxelizer.cpp:139-307) for a
 * single partition.  `occupancy_words` must be at least gridsize^3 / 32 (at
 * least 1); the words are cleared first.  Work is queued on `stream` (a
 * cudaStream_t on the current device; NULL = default stream) and the call
 * returns without waiting for it.
 *
 * Limits: n_tris <= OOC_NOALLOC_MAX_TRIANGLES, gridsize <= OOC_NOALLOC_MAX_GRIDSIZE
 * and memory_limit_mb large enough for one partition; beyond them the call
 * returns OOC_ERR_LIMIT before touching the GPU.
 * The first call on each device looks up the scratch array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture.  All calls on a device share the one scratch
 * array, which keeps the last call's contents: calls that may overlap on the
 * GPU (different streams without ordering between them) race. */
#define OOC_NOALLOC_MAX_TRIANGLES 1048576
#define OOC_NOALLOC_MAX_GRIDSIZE 1024
int ooc_voxelize_occupancy_noalloc(const ooc_build_params* params, const float* tris_device, uint64_t n_tris,
                                   uint32_t* occupancy_device, uint64_t occupancy_words, void* stream);

/* ---- Serving loop (no counterpart in the reference) ----
 * Requests (meshes) are admitted by their computed HBM footprint against
 * `memory_budget`: their triangles, the occupancy pyramids of their stripes,
 * and per-node arrays plus output records for an upper bound on their nodes
 * (a tree whose L leaves are at depth D has at most min(8^l, L) nodes at level
 * l, and L is at most the summed grid boxes of the triangles, clamped to the
 * grid).  Footprints are computed by sizing threads of the server, so a
 * submission returns at once; a request whose footprint exceeds the whole
 * budget completes, without running, with status OOC_ERR_LIMIT.  Requests are
 * admitted in submission order.  Requests run in
 * continuously formed batches: each of `engines` contexts (own streams and
 * scratch) takes, whenever it is free, every queued request that fits (at
 * most max_batch) and builds them in one ooc_build_batch_device call, into
 * device memory from the device's memory pool.  Host results are then copied
 * into pinned blocks the server keeps for reuse, on a stream of its own, and
 * their device memory is freed once the copy has landed.  A request
 * completes as soon as its mesh does, not when its batch does.  Each result is
 * byte-identical to ooc_build on that mesh alone.  Device-resident results
 * hold their HBM until released, and count against `memory_budget` until
 * then. */
typedef struct ooc_server ooc_server;

#define OOC_RESULT_HOST 0    /* results are copied back into host memory            */
#define OOC_RESULT_DEVICE 1  /* results stay resident in device memory (HBM)         */

typedef struct {
  int32_t device;
  int32_t engines;         /* batches in flight at once, >= 1                       */
  uint32_t max_batch;      /* requests per batch, >= 1 (1: every request alone)     */
  int32_t result_location; /* OOC_RESULT_HOST or OOC_RESULT_DEVICE                  */
  uint64_t memory_budget;  /* bytes of HBM the requests in flight may hold          */
  /* Fault injection for tests, 0 in normal use: the first batch of two or more
   * requests fails when it reaches its mesh number `fail_batch_at_mesh`
   * (1-based): that mesh's device allocation fails as if out of memory.  The
   * batch's requests not yet complete then run again alone, as after any failed
   * batch. */
  uint32_t fail_batch_at_mesh;
  /* Host results: MiB of pinned host memory to reserve at creation for them
   * (0: pin blocks on demand).  Pinning takes a lock of the CUDA driver for as
   * long as it runs, so a block pinned while serving delays every engine; a
   * reserve that covers the results in flight keeps pinning out of the serving
   * loop.  A result the reserve cannot hold gets a block pinned on demand; such
   * blocks total at most the reserve's size (8 GiB at least).  At that bound a
   * delivery waits for the caller to release results, and after 10 s its
   * request completes with OOC_ERR_OOM.  Ignored for device results;
   * OOC_ERR_OOM from ooc_server_create when the host cannot pin the reserve. */
  uint32_t host_pool_mb;
} ooc_server_config;

typedef struct {
  uint64_t id;
  int32_t status;         /* OOC_OK or the build's error code                      */
  int32_t location;       /* OOC_RESULT_HOST or OOC_RESULT_DEVICE: where the bytes are */
  const void* nodes;      /* node file bytes (valid until ooc_server_release)      */
  uint64_t nodes_bytes;
  const void* data;       /* data file bytes                                       */
  uint64_t data_bytes;
  ooc_build_info info;
  double t_submit_us;     /* times in microseconds since the server started:       */
  double t_start_us;      /*   its batch started                                   */
  double t_built_us;      /*   its octree was complete in device memory            */
  double t_done_us;       /*   it completed (host results: after the copy back)    */
  uint64_t batch_size;    /* requests in the batch this one ran in                 */
} ooc_result;

int ooc_server_create(const ooc_server_config* cfg, ooc_server** out);
/* Queue one mesh; its triangles (host memory) must stay valid until its result
 * is polled.  OOC_ERR_INVALID for parameters ooc_build would refuse. */
int ooc_server_submit(ooc_server* server, const ooc_mesh* mesh, uint64_t* id);
/* Next completed request (OOC_OK), or OOC_ERR_TIMEOUT after `timeout_ms`. */
int ooc_server_poll(ooc_server* server, int32_t timeout_ms, ooc_result* out);
/* The serving loop's state, for monitoring. */
typedef struct {
  uint64_t queued;                   /* submitted, not yet started                         */
  uint64_t in_flight_bytes;          /* HBM held: admitted footprints, results not released
                                        (resident) or not yet copied back (host)           */
  uint64_t completed_unpolled;       /* complete, not yet polled                           */
  uint64_t held;                     /* polled, not yet released                           */
  uint64_t deliveries;               /* host results waiting for their copy back to start  */
  uint64_t pinned_reserve_bytes;     /* host_pool_mb, pinned at creation                   */
  uint64_t pinned_reserve_free_bytes;
  uint64_t pinned_on_demand_bytes;   /* pinned while serving (kept for reuse)              */
  uint64_t pinned_on_demand_allocs;  /* pins made while serving                            */
} ooc_server_state;
int ooc_server_stats(ooc_server* server, ooc_server_state* out);
/* Copy a polled result's files into host memory (either location). */
int ooc_server_read(ooc_server* server, uint64_t id, void* nodes_host, void* data_host);
/* Free a polled result's buffers.  A device-resident result is freed stream-
 * ordered on a stream of the server's own, so work the caller queued on the
 * result must have completed before this call. */
int ooc_server_release(ooc_server* server, uint64_t id);
/* Drop the requests not yet started, let running batches finish, then stop
 * the engines and free everything (results not yet released included). */
void ooc_server_destroy(ooc_server* server);

/* ---- Octree check (replaces the reference's external viewer for checks) ----
 * The invariants of the .octreenodes/.octreedata format (octree_io.h:48-83)
 * that every correct build satisfies, checked on the GPU at any size: child
 * groups written as consecutive slots before their parent (OctreeBuilder.cpp:
 * 58-79), every node but the root (the last record) the child of exactly one
 * node, leaves at depth log2(gridsize), data indices inside the data file
 * (geometry-only leaves at the white entry 1), and each payload leaf's data
 * record carrying the Morton code of its path from the root. */
#define OOC_CHECK_CHILD_ORDER 1  /* a child group out of slot order, or not before its parent */
#define OOC_CHECK_REFCOUNT 2     /* a node that is not the child of exactly one node          */
#define OOC_CHECK_DEPTH 4        /* a leaf not at depth log2(gridsize), or an inner node there */
#define OOC_CHECK_DATA_INDEX 8   /* a data index outside the data file                        */
#define OOC_CHECK_MORTON 16      /* a payload leaf whose data Morton code is not its path     */

typedef struct {
  uint64_t n_nodes, n_data;
  uint64_t n_leaves;   /* voxels (the root of an empty octree is not counted) */
  uint64_t n_inner;
  uint64_t first_bad;  /* lowest node index with a violation, ~0 when none */
  uint32_t errors;     /* OOC_CHECK_* bits; 0 for a well-formed octree */
  uint32_t max_depth;
} ooc_octree_check;

/* `nodes` and `data` are device pointers to the two files' bytes (8-byte
 * aligned); `stream` is a cudaStream_t (NULL: the default stream).  Returns
 * OOC_OK when the check ran; the verdict is `out->errors`. */
int ooc_check_octree_device(const void* nodes, uint64_t n_nodes, const void* data, uint64_t n_data,
                            uint64_t gridsize, int32_t geometry_only, void* stream, ooc_octree_check* out);

/* File front end used by the svo_builder CLIs: reads <base>.tri/.tridata and
 * writes <base><gridsize>_<npartitions>.octree/.octreenodes/.octreedata
 * (main.cpp:296-398).  `out_base` receives the output base name (may be NULL).
 * The header's geo_only and bbox override those fields of `params`.  A header
 * that does not parse, a .tridata shorter than its triangle count, or an
 * output file that cannot be written returns OOC_ERR_IO, and ooc_last_error
 * names the file. */
int ooc_build_files(ooc_ctx* ctx, const char* tri_path, const ooc_build_params* params, char* out_base,
                    uint64_t out_base_len, ooc_build_info* info);

#ifdef __cplusplus
}
#endif
#endif /* OOC_SVO_GPU_H_ */
