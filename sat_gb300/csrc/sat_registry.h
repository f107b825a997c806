// sat_registry.h -- table of compiled kernel variants and host helpers shared
// by the entry-point translation units.
#pragma once
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace satgb {

struct SatParams;
struct ImageDesc;

using LaunchFn = cudaError_t (*)(const SatParams& p, int grid, cudaStream_t s);
using PrepareFn = cudaError_t (*)();

// One compiled instantiation of sat_tile_kernel.
struct Variant {
  int in_t, out_t; // satgb_dtype codes
  int mode;        // satgb_mode
  int dir;         // satgb_direction
  int cfg;         // tile configuration index (see kConfigs)
  LaunchFn launch;
  PrepareFn prepare;  // sets the dynamic shared-memory limit on the current device
  const void* kernel; // for occupancy queries
  int TH, TW, K, threads, dyn_smem;
};

// Tile configurations (rows per warp, warps per CTA).
struct TileConfig {
  int rows_per_warp;
  int warps;
  const char* name;
};
constexpr int kNumConfigs = 7;
extern const TileConfig kConfigs[kNumConfigs];

// Lists of variants, one per instantiation translation unit.
const Variant* variants_u8(int* n);
const Variant* variants_i8(int* n);
const Variant* variants_int32(int* n);
const Variant* variants_f32(int* n);
const Variant* variants_f64(int* n);

const Variant* find_variant(int in_t, int out_t, int mode, int dir, int cfg);

// Fills `d` for one image or a stack of `planes` images at the given plane
// strides (pointers, sizes, tile grid, alignment flags) and, where TMA can
// address the rows, its tensor maps.
void fill_image_desc(ImageDesc& d, const Variant* v, int in_t, int out_t, const void* in, void* out,
                     int64_t in_pitch, int64_t out_pitch, int64_t width, int64_t height, int64_t tile_base,
                     int64_t planes, int64_t in_plane, int64_t out_plane);

}  // namespace satgb
