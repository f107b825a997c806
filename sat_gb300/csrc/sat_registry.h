// sat_registry.h -- table of compiled kernel variants (host side).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace satgb {

struct SatParams;

using LaunchFn = cudaError_t (*)(const SatParams& p, int grid, cudaStream_t s);

// One compiled instantiation of sat_tile_kernel.
struct Variant {
  int in_t, out_t; // satgb_dtype codes
  int mode;        // satgb_mode
  int dir;         // satgb_direction
  int cfg;         // tile configuration index (see kConfigs)
  LaunchFn launch;
  const void* kernel; // for occupancy queries
  int TH, TW, K, threads;
};

// Tile configurations: rows per warp; every configuration has 8 warps.
struct TileConfig {
  int rows_per_warp;
  const char* name;
};
constexpr int kNumConfigs = 3;
extern const TileConfig kConfigs[kNumConfigs];

// Lists of variants, one per instantiation translation unit.
const Variant* variants_u8(int* n);
const Variant* variants_i8(int* n);
const Variant* variants_int32(int* n);
const Variant* variants_f32(int* n);
const Variant* variants_f64(int* n);

const Variant* find_variant(int in_t, int out_t, int mode, int dir, int cfg);

}  // namespace satgb
