/*
 * Command-line front end of the CPU oracle (test infrastructure only).
 *
 * Reads <base>.tri + <base>.tridata, runs oracle_build() and writes
 * <base><gridsize>_<npartitions>.octree / .octreenodes / .octreedata the way
 * svo_builder does (main.cpp:294-398, octree_io.h:48-83).  Built twice by
 * oracle/Makefile: with -DORACLE_BINARY (svo_builder_binary semantics) and
 * without (svo_builder).  Flags: -f -s -l -levels -c -d -v -h (main.cpp:100-196).
 */
#define _POSIX_C_SOURCE 199309L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "ooc_oracle.h"

static int is_pow2(unsigned int x) { return x != 0 && (x & (x - 1)) == 0; }

static int parse_tri_header(const char* path, uint64_t* ntri, int* geo, float bmin[3], float bmax[3]) {
  FILE* f = fopen(path, "r");
  if (!f) { printf("  Error: file %s does not exist.\n", path); return 0; }
  char tok[256];
  int version = 0, done = 0;
  *geo = 0;
  if (fscanf(f, "%255s", tok) != 1 || strcmp(tok, "#tri") != 0) { fclose(f); return 0; }
  if (fscanf(f, "%d", &version) != 1) { fclose(f); return 0; }
  while (!done && fscanf(f, "%255s", tok) == 1) {
    if (!strcmp(tok, "END")) done = 1;
    else if (!strcmp(tok, "ntriangles")) { unsigned long long v; if (fscanf(f, "%llu", &v) == 1) *ntri = v; }
    else if (!strcmp(tok, "geo_only")) { if (fscanf(f, "%d", geo) != 1) break; }
    else if (!strcmp(tok, "bbox")) {
      if (fscanf(f, "%f %f %f %f %f %f", &bmin[0], &bmin[1], &bmin[2], &bmax[0], &bmax[1], &bmax[2]) != 6) break;
    } else {
      int c;
      do { c = fgetc(f); } while (c != EOF && c != '\n');
    }
  }
  fclose(f);
  return done;
}

int main(int argc, char** argv) {
  const char* filename = NULL;
  uint64_t gridsize = 1024, limit = 2048;
  int levels = 0, color = ORACLE_COLOR_MODEL;
  if (argc < 3) { printf("Not enough or invalid arguments, please try again.\n"); return 0; }
  for (int i = 1; i < argc; i++) {
    if (!strcmp(argv[i], "-f") && i + 1 < argc) {
      filename = argv[++i];
      if (!strstr(filename, ".tri")) { printf("Data filename does not end in .tri - I only support that file format\n"); return 0; }
    } else if (!strcmp(argv[i], "-s") && i + 1 < argc) {
      gridsize = (uint64_t)atoi(argv[++i]);
      if (!is_pow2((unsigned int)gridsize)) { printf("Requested gridsize is not a power of 2\n"); return 0; }
    } else if (!strcmp(argv[i], "-l") && i + 1 < argc) {
      long v = atoi(argv[++i]);
      if (v <= 1) { printf("Requested memory limit is nonsensical. Use a value >= 1\n"); return 0; }
      limit = (uint64_t)v;
    } else if (!strcmp(argv[i], "-d") && i + 1 < argc) {
      i++; /* sizes a side buffer in the reference; never changes the output */
    } else if (!strcmp(argv[i], "-v")) {
    } else if (!strcmp(argv[i], "-levels")) {
      levels = 1;
    } else if (!strcmp(argv[i], "-c") && i + 1 < argc) {
      const char* c = argv[++i];
#ifndef ORACLE_BINARY
      if (!strcmp(c, "model")) color = ORACLE_COLOR_MODEL;
      else if (!strcmp(c, "linear")) color = ORACLE_COLOR_LINEAR;
      else if (!strcmp(c, "normal")) color = ORACLE_COLOR_NORMAL;
      else if (!strcmp(c, "fixed")) color = ORACLE_COLOR_FIXED;
#else
      (void)c;
#endif
    } else if (!strcmp(argv[i], "-h")) {
      return 0;
    } else {
      printf("Not enough or invalid arguments, please try again.\n");
      return 0;
    }
  }
  if (!filename) return 0;
  uint64_t ntri = 0;
  int geo = 0;
  float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};
  if (!parse_tri_header(filename, &ntri, &geo, bmin, bmax)) return 0;
#ifdef ORACLE_BINARY
  if (!geo) { printf("You're using a .tri file which contains more than just geometry with a geometry-only SVO Builder!\n"); return 0; }
  const int stride = 9;
#else
  if (geo) { printf("You're using a .tri file which contains only geometry with the regular SVO Builder!\n"); return 0; }
  const int stride = 21;
#endif
  char base[4096];
  snprintf(base, sizeof(base), "%s", filename);
  char* dot = strrchr(base, '.');
  if (dot) *dot = 0;
  char path[4400];
  snprintf(path, sizeof(path), "%s.tridata", base);
  FILE* f = fopen(path, "rb");
  if (!f) { printf("Not all required .tri or .tridata files exist.\n"); return 0; }
  float* tris = (float*)malloc((size_t)(ntri ? ntri : 1) * stride * sizeof(float));
  if (!tris || fread(tris, sizeof(float) * stride, (size_t)ntri, f) != (size_t)ntri) {
    fclose(f);
    printf("short .tridata\n");
    return 1;
  }
  fclose(f);

  oracle_params prm;
  memset(&prm, 0, sizeof(prm));
  prm.gridsize = gridsize;
  prm.memory_limit_mb = limit;
#ifdef ORACLE_BINARY
  prm.geometry_only = 1;
#else
  prm.geometry_only = 0;
#endif
  prm.color_mode = color;
  prm.generate_levels = levels;
  memcpy(prm.bbox_min, bmin, sizeof(bmin));
  memcpy(prm.bbox_max, bmax, sizeof(bmax));

  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  oracle_result res;
  if (oracle_build(&prm, tris, ntri, &res) != 0) { printf("oracle_build failed\n"); return 1; }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  printf("Partitioning data into %llu partitions ... done.\n", (unsigned long long)res.n_partitions);
  printf("Total amount of voxels: %llu\n", (unsigned long long)res.n_filled);
  printf("oracle build time: %.3f ms\n", (t1.tv_sec - t0.tv_sec) * 1e3 + (t1.tv_nsec - t0.tv_nsec) * 1e-6);

  char outbase[4300];
  snprintf(outbase, sizeof(outbase), "%s%llu_%llu", base, (unsigned long long)gridsize,
           (unsigned long long)res.n_partitions);
  snprintf(path, sizeof(path), "%s.octreenodes", outbase);
  f = fopen(path, "wb");
  if (!f) return 1;
  fwrite(res.nodes, 24, (size_t)res.n_nodes, f);
  fclose(f);
  snprintf(path, sizeof(path), "%s.octreedata", outbase);
  f = fopen(path, "wb");
  if (!f) return 1;
  fwrite(res.data, 32, (size_t)res.n_data, f);
  fclose(f);
  snprintf(path, sizeof(path), "%s.octree", outbase);
  f = fopen(path, "w");
  if (!f) return 1;
  fprintf(f, "#octreeheader 1\ngridlength %llu\nn_nodes %llu\nn_data %llu\nEND\n", (unsigned long long)gridsize,
          (unsigned long long)res.n_nodes, (unsigned long long)res.n_data);
  fclose(f);
  oracle_free(&res);
  free(tris);
  return 0;
}
