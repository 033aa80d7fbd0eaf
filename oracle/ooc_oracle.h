/*
 * CPU oracle for the partition -> voxelize -> SVO-build path of ooc_svo_builder.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference's
 * single-threaded algorithm, used by the test suite and by the benchmark's CPU
 * baseline as the checker.  The product (libooc_svo_gpu.so) never links,
 * loads or calls it.
 *
 * Pinning: tests/test_oracle_pin.py compares this restatement byte for byte
 * with the reference's own sources built by oracle/Makefile (target `ref`,
 * output oracle/_ref/), and tests/golden/ holds fixtures produced by that
 * reference build.
 */
#ifndef OOC_ORACLE_H_
#define OOC_ORACLE_H_

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Colour modes of svo_builder's -c flag (main.cpp:23). */
enum { ORACLE_COLOR_MODEL = 0, ORACLE_COLOR_FIXED = 1, ORACLE_COLOR_LINEAR = 2, ORACLE_COLOR_NORMAL = 3 };

typedef struct {
  uint64_t gridsize;        /* -s, power of two */
  uint64_t memory_limit_mb; /* -l */
  int geometry_only;        /* 1: svo_builder_binary semantics, 0: svo_builder (payload) */
  int color_mode;           /* ORACLE_COLOR_* (payload build only) */
  int generate_levels;      /* -levels */
  float bbox_min[3];        /* .tri header bbox */
  float bbox_max[3];
} oracle_params;

typedef struct {
  unsigned char* nodes; /* n_nodes records of 24 bytes (octree_io.h:62-66) */
  uint64_t n_nodes;
  unsigned char* data;  /* n_data records of 32 bytes (octree_io.h:49-53) */
  uint64_t n_data;
  uint64_t n_filled;     /* "Total amount of voxels" (main.cpp:391) */
  uint64_t n_partitions; /* estimate_partitions result */
  uint64_t* part_tricounts; /* triangles binned per partition (n_partitions entries) */
} oracle_result;

/* partitioner.cpp:12-28 */
uint64_t oracle_estimate_partitions(uint64_t gridsize, uint64_t memory_limit_mb);

/* Whole path on an in-memory triangle array (9 or 21 floats per triangle,
 * chosen by params->geometry_only).  Returns 0 on success. */
int oracle_build(const oracle_params* params, const float* tris, uint64_t n_tris, oracle_result* out);

void oracle_free(oracle_result* r);

/* libmorton 3D 64-bit encode/decode: x -> bit 0, y -> bit 1, z -> bit 2. */
uint64_t oracle_morton_encode(uint32_t x, uint32_t y, uint32_t z);
void oracle_morton_decode(uint64_t m, uint32_t* x, uint32_t* y, uint32_t* z);

#ifdef __cplusplus
}
#endif
#endif
