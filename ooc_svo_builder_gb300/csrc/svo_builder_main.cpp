// svo_builder / svo_builder_binary: drop-in command lines for the reference's
// executables (src/svo_builder/main.cpp), running the path on the GPU through
// libooc_svo_gpu.so.  Built twice; -DOOC_CLI_BINARY gives svo_builder_binary.
//
// Flags, messages, output file names and exit codes follow main.cpp:100-398:
// every error prints a message and exits with status 0, as the reference does.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "ooc_svo_gpu.h"

namespace {

const char* kVersion = "1.6.4";

std::string filename;
uint64_t gridsize = 1024;      // main.cpp:30
uint64_t memory_limit = 2048;  // main.cpp:31
float sparseness_limit = 0.10f;  // main.cpp:32; printed by -v, no effect on the output
int color = OOC_COLOR_MODEL;
const char* color_name = "Color from model (fallback to fixed color if model has no color)";
bool generate_levels = false;
bool verbose = false;

// the .tri header (check_tri)
std::string base;  // the file name without its extension
int version = 0;
uint64_t n_triangles = 0;
float bmin[3] = {0, 0, 0}, bmax[3] = {0, 0, 0};

void print_info() {
  std::cout << "--------------------------------------------------------------------" << std::endl;
#ifdef OOC_CLI_BINARY
  std::cout << "Out-Of-Core SVO Builder " << kVersion << " - Geometry only version (GB300)" << std::endl;
#else
  std::cout << "Out-Of-Core SVO Builder " << kVersion << " (GB300)" << std::endl;
#endif
  std::cout << "--------------------------------------------------------------------" << std::endl << std::endl;
}

void print_help() {
  std::cout << "Example: svo_builder -f /home/user/bunny.tri" << std::endl << std::endl;
  std::cout << "All available program options:" << std::endl << std::endl;
  std::cout << "-f <filename.tri>     Path to a .tri input file." << std::endl;
  std::cout << "-s <gridsize>         Voxel gridsize, should be a power of 2. Default 1024." << std::endl;
  std::cout << "-l <memory_limit>     Memory limit for process, in Mb. Default 2048." << std::endl;
  std::cout << "-levels               Generate intermediary voxel levels by averaging voxel data" << std::endl;
  std::cout << "-c <option>           Coloring of voxels (Options: model (default), fixed, linear, normal)" << std::endl;
  std::cout << "-d <percentage>       Accepted for compatibility; does not change the output" << std::endl;
  std::cout << "-v                    Be very verbose." << std::endl;
  std::cout << "-h                    Print help and exit." << std::endl;
}

void print_invalid() {
  std::cout << "Not enough or invalid arguments, please try again." << std::endl;
  std::cout << "At the bare minimum, I need a path to a .TRI file" << std::endl << std::endl;
  print_help();
}

bool is_pow2(unsigned int x) { return x != 0 && !(x & (x - 1)); }

// parseProgramParameters (main.cpp:100-196).  Values are parsed with atoi into
// the reference's unsigned types, so "-l -5" passes the ">= 1" check as a huge
// limit (one partition) exactly as it does there.  One deliberate difference: a
// flag that takes a value but ends the command line reads past argv there and
// crashes; here it is an invalid argument.
void parse(int argc, char** argv) {
  std::cout << "Reading program parameters ..." << std::endl;
  if (argc < 3) {
    print_invalid();
    std::exit(0);
  }
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    const bool has_next = i + 1 < argc;
    if (a == "-f" && has_next) {
      filename = argv[i + 1];
      if (filename.find(".tri") == std::string::npos) {
        std::cout << "Data filename does not end in .tri - I only support that file format" << std::endl;
        print_invalid();
        std::exit(0);
      }
      i++;
    } else if (a == "-s" && has_next) {
      gridsize = (uint64_t)(int64_t)std::atoi(argv[i + 1]);
      if (!is_pow2((unsigned int)gridsize)) {
        std::cout << "Requested gridsize is not a power of 2" << std::endl;
        print_invalid();
        std::exit(0);
      }
      i++;
    } else if (a == "-l" && has_next) {
      memory_limit = (uint64_t)(int64_t)std::atoi(argv[i + 1]);
      if (memory_limit <= 1) {
        std::cout << "Requested memory limit is nonsensical. Use a value >= 1" << std::endl;
        print_invalid();
        std::exit(0);
      }
      i++;
    } else if (a == "-d" && has_next) {
      sparseness_limit = std::atoi(argv[i + 1]) / 100.0f;
      if (sparseness_limit < 0) {
        std::cout << "Requested data memory limit is nonsensical. Use a value > 0" << std::endl;
        print_invalid();
        std::exit(0);
      }
      i++;
    } else if (a == "-v") {
      verbose = true;
    } else if (a == "-levels") {
      generate_levels = true;
    } else if (a == "-c" && has_next) {
      const std::string c = argv[i + 1];
#ifdef OOC_CLI_BINARY
      (void)c;
      std::cout << "You asked to generate colors, but we're only doing binary voxelisation." << std::endl;
#else
      if (c == "model") {
        color = OOC_COLOR_MODEL;
      } else if (c == "linear") {
        color = OOC_COLOR_LINEAR;
        color_name = "Linear";
      } else if (c == "normal") {
        color = OOC_COLOR_NORMAL;
        color_name = "Normal";
      } else if (c == "fixed") {
        color = OOC_COLOR_FIXED;
        color_name = "Fixed";
      } else {
        std::cout << "Unrecognized color switch: " << c << ", so reverting to colors from model." << std::endl;
      }
#endif
      i++;
    } else if (a == "-h") {
      print_help();
      std::exit(0);
    } else {
      print_invalid();
      std::exit(0);
    }
  }
  if (verbose) {
    std::cout << "  filename: " << filename << std::endl;
    std::cout << "  gridsize: " << gridsize << std::endl;
    std::cout << "  memory limit: " << memory_limit << std::endl;
    std::cout << "  sparseness optimization limit: " << sparseness_limit << " resulting in "
              << sparseness_limit * (float)memory_limit << " memory limit." << std::endl;
    std::cout << "  color type: " << color_name << std::endl;
    std::cout << "  generate levels: " << generate_levels << std::endl;
    std::cout << "  verbosity: " << verbose << std::endl;
  }
}

bool file_exists(const std::string& name) {
  std::FILE* f = std::fopen(name.c_str(), "r");
  if (!f) return false;
  std::fclose(f);
  return true;
}

// readTriHeader (main.cpp:244-267) over parseTriHeader (tri_tools.h:75-115):
// the same token loop and the same messages, each followed by exit status 0.
// The loop keeps the last keyword when a read fails at the end of the file, so a
// header without END reports a trailing unknown keyword twice, as there.
void check_tri(const std::string& fn) {
  std::cout << "Parsing tri header " << fn << " ..." << std::endl;
  std::ifstream f(fn.c_str(), std::ios::in);
  if (!f) {
    std::cout << "  Error: file " << fn << " does not exist." << std::endl;
    std::exit(0);
  }
  base = fn.substr(0, fn.find_last_of("."));
  std::string word;
  f >> word;
  if (word != "#tri") {
    std::cout << "  Error: first line reads [" << word << "] instead of [#tri]" << std::endl;
    std::exit(0);
  }
  int geo = 0;
  f >> version;
  bool seen_end = false;
  while (f.good() && !seen_end) {
    f >> word;
    if (word == "END") {
      seen_end = true;
    } else if (word == "ntriangles") {
      f >> n_triangles;
    } else if (word == "geo_only") {
      f >> geo;
    } else if (word == "bbox") {
      f >> bmin[0] >> bmin[1] >> bmin[2] >> bmax[0] >> bmax[1] >> bmax[2];
    } else {
      std::cout << "  unrecognized keyword [" << word << "], skipping" << std::endl;
      char c;
      do {
        c = (char)f.get();
      } while (f.good() && c != '\n');
    }
  }
  if (!seen_end) {
    std::cout << "  error reading header" << std::endl;
    std::exit(0);
  }
  if (!file_exists(base + ".tri") || !file_exists(base + ".tridata")) {
    std::cout << "Not all required .tri or .tridata files exist. Please regenerate using tri_convert." << std::endl;
    std::exit(0);
  }
  if (verbose) {
    std::cout << "  base_filename: " << base << std::endl;
    std::cout << "  tri version: " << version << std::endl;
    std::cout << "  geometry only: " << geo << std::endl;
    std::cout << "  n_triangles: " << n_triangles << std::endl;
    std::cout << "  bbox min: " << bmin[0] << " " << bmin[1] << " " << bmin[2] << std::endl;
    std::cout << "  bbox max: " << bmax[0] << " " << bmax[1] << " " << bmax[2] << std::endl;
  }
#ifdef OOC_CLI_BINARY
  if (!geo) {
    std::cout << "You're using a .tri file which contains more than just geometry with a geometry-only SVO Builder! "
                 "Regenerate that .tri file using tri_convert_binary."
              << std::endl;
    std::exit(0);
  }
#else
  if (geo) {
    std::cout << "You're using a .tri file which contains only geometry with the regular SVO Builder! Regenerate "
                 "that .tri file using tri_convert."
              << std::endl;
    std::exit(0);
  }
#endif
}

// estimate_partitions' report (partitioner.cpp:12-28); the count is the library's.
// Dividing the in-core size by 8 once per factor of 8 partitions floors to the
// same value as dividing it by the partition count.
uint64_t report_partitions() {
  std::cout << "Estimating best partition count ..." << std::endl;
  const uint64_t required = gridsize * gridsize * gridsize / 1024 / 1024;
  std::cout << "  to do this in-core I would need " << required << " Mb of system memory" << std::endl;
  const uint64_t P = ooc_estimate_partitions(gridsize, memory_limit);
  if (P == 1)
    std::cout << "  memory limit of " << memory_limit << " Mb allows that" << std::endl;
  else
    std::cout << "  going to do it in " << P << " partitions of " << required / P << " Mb each." << std::endl;
  return P;
}

// createBuffers' verbose report of the partition boxes (partitioner.cpp:43-77):
// Morton range, grid box and world box of every partition, with the world box
// as the reference forms it, grid coordinate times the unit length in float.
void report_partition_boxes(uint64_t P, float unitlength) {
  const uint64_t part = gridsize * gridsize * gridsize / P;
  auto decode = [](uint64_t m, unsigned int v[3]) {
    for (int a = 0; a < 3; a++) {
      unsigned int c = 0;
      for (int b = 0; b < 21; b++) c |= (unsigned int)((m >> (3 * b + a)) & 1u) << b;
      v[a] = c;
    }
  };
  for (uint64_t i = 0; i < P; i++) {
    unsigned int lo[3], hi[3];
    decode(part * i, lo);
    decode(part * (i + 1) - 1, hi);
    float wlo[3], whi[3];
    for (int a = 0; a < 3; a++) {
      wlo[a] = lo[a] * unitlength;
      whi[a] = (hi[a] + 1) * unitlength;
    }
    std::cout << "Partitioning partition #" << i + 1 << " / " << P << " id: " << i << " ..." << std::endl;
    std::cout << "  morton from " << part * i << " to " << part * (i + 1) << std::endl;
    std::cout << "  grid coordinates from (" << lo[0] << "," << lo[1] << "," << lo[2] << ") to (" << hi[0] << ","
              << hi[1] << "," << hi[2] << ")" << std::endl;
    std::cout << "  worldspace coordinates from (" << wlo[0] << "," << wlo[1] << "," << wlo[2] << ") to (" << whi[0]
              << "," << whi[1] << "," << whi[2] << ")" << std::endl;
  }
}

// The reference's timers count whole milliseconds (timer.h:59).
double whole_ms(double ms) { return (double)(long long)ms; }

}  // namespace

int main(int argc, char** argv) {
  const auto t0 = std::chrono::steady_clock::now();
  print_info();
  parse(argc, argv);
  check_tri(filename);
  const uint64_t P = report_partitions();
  std::cout << "Partitioning data into " << P << " partitions ... ";
  std::cout.flush();

  ooc_ctx* ctx = nullptr;
  if (ooc_ctx_create(0, &ctx) != OOC_OK) {
    std::cout << std::endl << "No CUDA device available." << std::endl;
    return 0;
  }
  ooc_set_phase_timing(ctx, 1);
  ooc_build_params prm = {};
  prm.gridsize = gridsize;
  prm.memory_limit_mb = memory_limit;
#ifdef OOC_CLI_BINARY
  prm.geometry_only = 1;
#else
  prm.geometry_only = 0;
#endif
  prm.color_mode = color;
  prm.generate_levels = generate_levels ? 1 : 0;
  ooc_build_info info = {};
  char out_base[4096];
  const int rc = ooc_build_files(ctx, filename.c_str(), &prm, out_base, sizeof(out_base), &info);
  if (verbose && P > 1) report_partition_boxes(P, (bmax[0] - bmin[0]) / (float)gridsize);
  std::cout << "done." << std::endl;
  if (rc != OOC_OK) {
    std::cout << "Build failed (" << rc << "): " << ooc_last_error(ctx) << std::endl;
    ooc_ctx_destroy(ctx);
    return 0;
  }
  // per-partition progress (main.cpp:329-355); the partitions were built together,
  // so their lines come after the build, in partition order
  std::vector<uint64_t> tris(P, 0), filled(P, 0);
  ooc_partition_counts(ctx, 0, P, tris.data(), filled.data());
  const std::string trip_base = base + std::to_string(gridsize) + "_" + std::to_string(P);
  if (verbose) {  // readTripHeader's TripInfo::print (main.cpp:271-279, trip_tools.h:28-40)
    std::cout << "  base_filename: " << trip_base << std::endl;
    std::cout << "  trip version: " << version << std::endl;
#ifdef OOC_CLI_BINARY
    std::cout << "  geometry only: 1" << std::endl;
#else
    std::cout << "  geometry only: 0" << std::endl;
#endif
    std::cout << "  gridsize: " << gridsize << std::endl;
    std::cout << "  bbox min: " << bmin[0] << " " << bmin[1] << " " << bmin[2] << std::endl;
    std::cout << "  bbox max: " << bmax[0] << " " << bmax[1] << " " << bmax[2] << std::endl;
    std::cout << "  n_triangles: " << n_triangles << std::endl;
    std::cout << "  n_partitions: " << P << std::endl;
    for (uint64_t i = 0; i < P; i++) std::cout << "  partition " << i << " - tri_count: " << tris[i] << std::endl;
  }
  for (uint64_t i = 0; i < P; i++) {
    if (tris[i] == 0) continue;  // main.cpp:330
    std::cout << "Voxelizing partition " << i << " ..." << std::endl;
    if (verbose) {
      std::cout << "  reading " << tris[i] << " triangles from " << trip_base << "_" << i << ".tripdata" << std::endl;
      std::cout << "  found " << filled[i] << " new voxels." << std::endl;
    }
    std::cout << "Building SVO for partition " << i << " ..." << std::endl;
  }
  std::cout << "done" << std::endl;
  std::cout << "Total amount of voxels: " << info.n_filled << std::endl;
  float ms[6] = {0, 0, 0, 0, 0, 0}, fms[2] = {0, 0};
  ooc_phase_times(ctx, ms, 6);
  ooc_file_times(ctx, fms, 2);
  ooc_ctx_destroy(ctx);
  const double main_ms =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  // printTimerInfo (main.cpp:219-241), filled from the GPU phases and the file times
  const double part_in = whole_ms(fms[0]), part_algo = whole_ms(ms[0]), part_total = whole_ms(fms[0] + ms[0]);
  const double vox_algo = whole_ms(ms[1] + ms[2]), vox_total = vox_algo;
  const double svo_out = whole_ms(fms[1]), svo_algo = whole_ms(ms[3]), svo_total = whole_ms(fms[1] + ms[3] + ms[4]);
  std::cout << "Total MAIN time      : " << whole_ms(main_ms) << " ms." << std::endl;
  std::cout << "PARTITIONING" << std::endl;
  std::cout << "  Total time\t\t: " << part_total << " ms." << std::endl;
  std::cout << "  IO IN time\t\t: " << part_in << " ms." << std::endl;
  std::cout << "  algorithm time\t: " << part_algo << " ms." << std::endl;
  std::cout << "  IO OUT time\t\t: " << 0.0 << " ms." << std::endl;
  std::cout << "  misc time\t\t: " << part_total - part_in - part_algo << " s." << std::endl;
  std::cout << "VOXELIZING" << std::endl;
  std::cout << "  Total time\t\t: " << vox_total << " ms." << std::endl;
  std::cout << "  IO IN time\t\t: " << 0.0 << " ms." << std::endl;
  std::cout << "  algorithm time\t: " << vox_algo << " ms." << std::endl;
  std::cout << "  misc time\t\t: " << vox_total - vox_algo << " s." << std::endl;
  std::cout << "SVO BUILDING" << std::endl;
  std::cout << "  Total time\t\t: " << svo_total << " ms." << std::endl;
  std::cout << "  IO OUT time\t\t: " << svo_out << " ms." << std::endl;
  std::cout << "  algorithm time\t: " << svo_algo << " ms." << std::endl;
  std::cout << "  misc time\t\t: " << svo_total - svo_out - svo_algo << " s." << std::endl;
  if (std::getenv("OOC_GPU_PHASES")) {  // device-time detail, off unless asked for
    std::cout << "GPU PHASES (device time)" << std::endl;
    std::cout << "  partitioning        : " << ms[0] << " ms." << std::endl;
    std::cout << "  voxelizing          : " << ms[1] << " ms." << std::endl;
    std::cout << "  occupancy pyramid   : " << ms[2] << " ms." << std::endl;
    std::cout << "  octree layout       : " << ms[3] << " ms." << std::endl;
    std::cout << "  host<->device copies: " << ms[4] << " ms." << std::endl;
    std::cout << "  whole build         : " << ms[5] << " ms." << std::endl;
    std::cout << "Output: " << out_base << ".octree" << std::endl;
  }
  return 0;
}
