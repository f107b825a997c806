// sat_inst.cuh -- helpers for the instantiation translation units.
#pragma once
#include <atomic>

#include "sat_kernel.cuh"
#include "sat_kernel_r.cuh"
#include "sat_kernel_ws.cuh"
#include "sat_kernel_rm.cuh"
#include "sat_registry.h"

namespace satgb {

// Raises the kernel's dynamic shared-memory limit on the current device (once
// per device); must precede occupancy queries and launches.
template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB, int KIND = kKindSat,
          bool DIRECT = false>
cudaError_t prepare_impl() {
  using SH = TileShape<TIn, TOut, A, RPW, NW, MINB, DIRECT>;
  constexpr int kMaxDev = 64;
  static std::atomic<int> done[kMaxDev];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxDev && done[dev].load(std::memory_order_acquire)) return cudaSuccess;
  e = cudaFuncSetAttribute(&sat_tile_kernel<TIn, TOut, A, REV, RPW, NW, MINB, KIND, DIRECT>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, SH::DYN_SMEM);
  if (e == cudaSuccess && dev >= 0 && dev < kMaxDev) done[dev].store(1, std::memory_order_release);
  return e;
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB, int KIND = kKindSat,
          bool DIRECT = false>
cudaError_t launch_impl(const SatParams& p, int grid, cudaStream_t s) {
  using SH = TileShape<TIn, TOut, A, RPW, NW, MINB, DIRECT>;
  cudaError_t e = prepare_impl<TIn, TOut, A, REV, RPW, NW, MINB, KIND, DIRECT>();
  if (e != cudaSuccess) return e;
  sat_tile_kernel<TIn, TOut, A, REV, RPW, NW, MINB, KIND, DIRECT><<<grid, SH::THREADS, SH::DYN_SMEM, s>>>(p);
  return cudaGetLastError();
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB, int KIND = kKindSat,
          bool DIRECT = false>
Variant make_variant(int in_t, int out_t, int mode, int cfg) {
  using SH = TileShape<TIn, TOut, A, RPW, NW, MINB, DIRECT>;
  return Variant{in_t, out_t, mode, REV ? 1 : 0, cfg,
                 &launch_impl<TIn, TOut, A, REV, RPW, NW, MINB, KIND, DIRECT>,
                 &prepare_impl<TIn, TOut, A, REV, RPW, NW, MINB, KIND, DIRECT>,
                 (const void*)&sat_tile_kernel<TIn, TOut, A, REV, RPW, NW, MINB, KIND, DIRECT>,
                 SH::TH, SH::TW, Ar<A>::K, SH::THREADS, SH::DYN_SMEM};
}

// The same three for sat_tile_kernel_r (inputs held in registers, several
// CTAs per SM).
template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB>
cudaError_t prepare_impl_r() {
  using SH = TileShapeR<TIn, TOut, A, RPW, NW, MINB>;
  constexpr int kMaxDev = 64;
  static std::atomic<int> done[kMaxDev];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxDev && done[dev].load(std::memory_order_acquire)) return cudaSuccess;
  e = cudaFuncSetAttribute(&sat_tile_kernel_r<TIn, TOut, A, REV, RPW, NW, MINB>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, SH::DYN_SMEM);
  if (e == cudaSuccess && dev >= 0 && dev < kMaxDev) done[dev].store(1, std::memory_order_release);
  return e;
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB>
cudaError_t launch_impl_r(const SatParams& p, int grid, cudaStream_t s) {
  using SH = TileShapeR<TIn, TOut, A, RPW, NW, MINB>;
  cudaError_t e = prepare_impl_r<TIn, TOut, A, REV, RPW, NW, MINB>();
  if (e != cudaSuccess) return e;
  sat_tile_kernel_r<TIn, TOut, A, REV, RPW, NW, MINB><<<grid, SH::THREADS, SH::DYN_SMEM, s>>>(p);
  return cudaGetLastError();
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NW, int MINB>
Variant make_variant_r(int in_t, int out_t, int mode, int cfg) {
  using SH = TileShapeR<TIn, TOut, A, RPW, NW, MINB>;
  return Variant{in_t, out_t, mode, REV ? 1 : 0, cfg,
                 &launch_impl_r<TIn, TOut, A, REV, RPW, NW, MINB>,
                 &prepare_impl_r<TIn, TOut, A, REV, RPW, NW, MINB>,
                 (const void*)&sat_tile_kernel_r<TIn, TOut, A, REV, RPW, NW, MINB>,
                 SH::TH, SH::TW, Ar<A>::K, SH::THREADS, SH::DYN_SMEM};
}

// The same three for sat_tile_kernel_ws (warp-specialized; NWC compute warps
// plus three role warps, one CTA per SM).
template <class TIn, class TOut, class A, bool REV, int RPW, int NWC, bool DIRECT = false, int CTAS = 1>
cudaError_t prepare_impl_ws() {
  using SH = TileShapeWS<TIn, TOut, A, RPW, NWC, DIRECT, CTAS>;
  constexpr int kMaxDev = 64;
  static std::atomic<int> done[kMaxDev];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxDev && done[dev].load(std::memory_order_acquire)) return cudaSuccess;
  e = cudaFuncSetAttribute(&sat_tile_kernel_ws<TIn, TOut, A, REV, RPW, NWC, DIRECT, CTAS>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, SH::DYN_SMEM);
  if (e == cudaSuccess && dev >= 0 && dev < kMaxDev) done[dev].store(1, std::memory_order_release);
  return e;
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC, bool DIRECT = false, int CTAS = 1>
cudaError_t launch_impl_ws(const SatParams& p, int grid, cudaStream_t s) {
  using SH = TileShapeWS<TIn, TOut, A, RPW, NWC, DIRECT, CTAS>;
  cudaError_t e = prepare_impl_ws<TIn, TOut, A, REV, RPW, NWC, DIRECT, CTAS>();
  if (e != cudaSuccess) return e;
  sat_tile_kernel_ws<TIn, TOut, A, REV, RPW, NWC, DIRECT, CTAS><<<grid, SH::THREADS, SH::DYN_SMEM, s>>>(p);
  return cudaGetLastError();
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC, bool DIRECT = false, int CTAS = 1>
Variant make_variant_ws(int in_t, int out_t, int mode, int cfg) {
  using SH = TileShapeWS<TIn, TOut, A, RPW, NWC, DIRECT, CTAS>;
  return Variant{in_t, out_t, mode, REV ? 1 : 0, cfg,
                 &launch_impl_ws<TIn, TOut, A, REV, RPW, NWC, DIRECT, CTAS>,
                 &prepare_impl_ws<TIn, TOut, A, REV, RPW, NWC, DIRECT, CTAS>,
                 (const void*)&sat_tile_kernel_ws<TIn, TOut, A, REV, RPW, NWC, DIRECT, CTAS>,
                 SH::TH, SH::TW, Ar<A>::K, SH::THREADS, SH::DYN_SMEM};
}

// The same three for sat_tile_kernel_rm (row-major tile order, direct stores).
template <class TIn, class TOut, class A, bool REV, int RPW, int NWC>
cudaError_t prepare_impl_rm() {
  using SH = TileShapeRM<TIn, TOut, A, RPW, NWC>;
  constexpr int kMaxDev = 64;
  static std::atomic<int> done[kMaxDev];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev >= 0 && dev < kMaxDev && done[dev].load(std::memory_order_acquire)) return cudaSuccess;
  e = cudaFuncSetAttribute(&sat_tile_kernel_rm<TIn, TOut, A, REV, RPW, NWC>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, SH::DYN_SMEM);
  if (e == cudaSuccess && dev >= 0 && dev < kMaxDev) done[dev].store(1, std::memory_order_release);
  return e;
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC>
cudaError_t launch_impl_rm(const SatParams& p, int grid, cudaStream_t s) {
  using SH = TileShapeRM<TIn, TOut, A, RPW, NWC>;
  cudaError_t e = prepare_impl_rm<TIn, TOut, A, REV, RPW, NWC>();
  if (e != cudaSuccess) return e;
  sat_tile_kernel_rm<TIn, TOut, A, REV, RPW, NWC><<<grid, SH::THREADS, SH::DYN_SMEM, s>>>(p);
  return cudaGetLastError();
}

template <class TIn, class TOut, class A, bool REV, int RPW, int NWC>
Variant make_variant_rm(int in_t, int out_t, int mode, int cfg) {
  using SH = TileShapeRM<TIn, TOut, A, RPW, NWC>;
  return Variant{in_t, out_t, mode, REV ? 1 : 0, cfg,
                 &launch_impl_rm<TIn, TOut, A, REV, RPW, NWC>,
                 &prepare_impl_rm<TIn, TOut, A, REV, RPW, NWC>,
                 (const void*)&sat_tile_kernel_rm<TIn, TOut, A, REV, RPW, NWC>,
                 SH::TH, SH::TW, Ar<A>::K, SH::THREADS, SH::DYN_SMEM};
}

}  // namespace satgb

// dtype codes (satgb_dtype)
#define SG_U8 0
#define SG_I8 1
#define SG_U32 4
#define SG_I32 5
#define SG_F32 6
#define SG_F64 7

// every tile configuration, both directions (kernel, rows per warp, warps,
// CTAs per SM):
//   0: warp-specialized, 64-row tiles, 16 compute warps (8 for 8-byte
//      accumulators) + column, row and store warps
//   1: pipelined, 128-row tiles (64 for 8-byte accumulators), 16 warps, 1 CTA
//   2: pipelined, 64-row tiles (32 for 8-byte accumulators), 8 warps, 2 CTAs
//   3: registers, 128-row tiles, 16 warps, 1 CTA (for 8-byte accumulators too:
//      the compensated f32 SAT measured 0.284 ms with 64-row and 0.217 ms with
//      128-row tiles at 8192^2)
//   4: (1-byte inputs, 4-byte sums only, SG_TALL) pipelined, 256-row tiles, direct stores
//   5: warp-specialized with direct stores, 8 rows a compute warp: 128-row
//      tiles and 16 compute warps for 4-byte accumulators (64-row tiles and 8
//      compute warps for 8-byte ones)
//   6: as 5, with the tiles in row-major order: rowleft is the sum of every
//      row aggregate to the left, the look-back is vertical only (no corner)
#define SG_CFG1_RPW(A) (sizeof(A) == 8 ? 4 : 8)
#define SG_R0_RPW(A) (sizeof(A) == 8 ? 4 : 8)
#define SG_WS_RPW(A) (sizeof(A) == 8 ? 8 : 4)  /* 64-row tiles either way: */
#define SG_WS_NWC(A) (sizeof(A) == 8 ? 8 : 16) /* 8-byte accumulators need the registers of fewer warps */
#define SG_DIR(TIN, TOUT, A, IT, OT, MODE, REV)                                         \
  satgb::make_variant_ws<TIN, TOUT, A, REV, SG_WS_RPW(A), SG_WS_NWC(A)>(IT, OT, MODE, 0), \
      satgb::make_variant<TIN, TOUT, A, REV, SG_CFG1_RPW(A), 16, 1>(IT, OT, MODE, 1),    \
      satgb::make_variant<TIN, TOUT, A, REV, SG_R0_RPW(A), 8, 2>(IT, OT, MODE, 2),       \
      satgb::make_variant_r<TIN, TOUT, A, REV, 8, 16, 1>(IT, OT, MODE, 3),               \
      satgb::make_variant_ws<TIN, TOUT, A, REV, 8, SG_WS_NWC(A), true>(IT, OT, MODE, 5),   \
      satgb::make_variant_rm<TIN, TOUT, A, REV, 8, SG_WS_NWC(A)>(IT, OT, MODE, 6)
#define SG_ALL(TIN, TOUT, A, IT, OT, MODE) \
  SG_DIR(TIN, TOUT, A, IT, OT, MODE, false), SG_DIR(TIN, TOUT, A, IT, OT, MODE, true)

// column-only scans (mode SG_MODE_COLS): the pipelined 128-row tiles, forward
// (the row-only scan has its own kernel, scan_rows_t.cu)
#define SG_MODE_COLS 3
#define SG_SCANS(TIN, TOUT, A, IT, OT) \
  satgb::make_variant<TIN, TOUT, A, false, SG_CFG1_RPW(A), 16, 1, satgb::kKindCols>(IT, OT, SG_MODE_COLS, 1)

// configuration 4, for 1-byte inputs with 4-byte sums: the pipelined kernel
// with 256-row tiles (16 warps x 16 rows) and direct stores, both directions
#define SG_TALL(TIN, TOUT, A, IT, OT)                                                      \
  satgb::make_variant<TIN, TOUT, A, false, 16, 16, 1, satgb::kKindSat, true>(IT, OT, 0, 4), \
      satgb::make_variant<TIN, TOUT, A, true, 16, 16, 1, satgb::kKindSat, true>(IT, OT, 0, 4)

#define SG_TABLE(NAME, ...)                                   \
  namespace satgb {                                           \
  static const Variant k_##NAME[] = {__VA_ARGS__};            \
  const Variant* variants_##NAME(int* n) {                    \
    *n = (int)(sizeof(k_##NAME) / sizeof(k_##NAME[0]));       \
    return k_##NAME;                                          \
  }                                                           \
  }
