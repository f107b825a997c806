// sat_inst.cuh -- helpers for the instantiation translation units.
#pragma once
#include "sat_kernel.cuh"
#include "sat_registry.h"

namespace satgb {

template <class TIn, class TOut, class A, bool REV, int RPW>
cudaError_t launch_impl(const SatParams& p, int grid, cudaStream_t s) {
  sat_tile_kernel<TIn, TOut, A, REV, RPW, 8><<<grid, 256, 0, s>>>(p);
  return cudaGetLastError();
}

template <class TIn, class TOut, class A, bool REV, int RPW>
constexpr Variant make_variant(int in_t, int out_t, int mode, int cfg) {
  return Variant{in_t, out_t, mode, REV ? 1 : 0, cfg,
                 &launch_impl<TIn, TOut, A, REV, RPW>,
                 (const void*)&sat_tile_kernel<TIn, TOut, A, REV, RPW, 8>,
                 8 * RPW, 32 * (16 / (int)sizeof(TOut)), Ar<A>::K, 256};
}

}  // namespace satgb

// dtype codes (satgb_dtype)
#define SG_U8 0
#define SG_I8 1
#define SG_U32 4
#define SG_I32 5
#define SG_F32 6
#define SG_F64 7

// all three tile configurations, both directions
#define SG_ALL(TIN, TOUT, A, IT, OT, MODE)                                  \
  satgb::make_variant<TIN, TOUT, A, false, 8>(IT, OT, MODE, 0),             \
      satgb::make_variant<TIN, TOUT, A, false, 16>(IT, OT, MODE, 1),        \
      satgb::make_variant<TIN, TOUT, A, false, 4>(IT, OT, MODE, 2),         \
      satgb::make_variant<TIN, TOUT, A, true, 8>(IT, OT, MODE, 0),          \
      satgb::make_variant<TIN, TOUT, A, true, 16>(IT, OT, MODE, 1),         \
      satgb::make_variant<TIN, TOUT, A, true, 4>(IT, OT, MODE, 2)

#define SG_TABLE(NAME, ...)                                   \
  namespace satgb {                                           \
  static const Variant k_##NAME[] = {__VA_ARGS__};            \
  const Variant* variants_##NAME(int* n) {                    \
    *n = (int)(sizeof(k_##NAME) / sizeof(k_##NAME[0]));       \
    return k_##NAME;                                          \
  }                                                           \
  }
