// scan_rows_t.cu -- row scan with transposed output:
//
//   out(x, y) = sum_{i <= x} in(y, i)      in: W x H (row y, column x), out: H x W
//
// the reference's SerielScan::TestX (integralImage/BRLT-Scan.cu:128-190), whose
// serielScan launch reads rows and stores the scanned rows transposed
// (compared there with IntegralImageAllRow + Transpose).  Rows are
// independent, so there is no look-back: a CTA owns a strip of 32 rows and
// walks it left to right in tiles of 128 columns.  Warp w (of 16) owns strip rows
// [2w, 2w+2) and keeps their running sums (the carry) in registers from tile to
// tile; lane l owns columns [4l, 4l+4) of the tile.  Per tile: in-thread prefix,
// Kogge-Stone warp scan of the lane totals, plus the carry; the 32 x 128 block
// of results is transposed through shared memory (row stride 33) and leaves as
// 128 output rows of 32 consecutive elements, one coalesced store per warp and
// row.  The next tile's inputs are loaded before the current one is scanned.
// Accumulators: u32 for integer outputs (mod-2^32 wrap, i32 results are the
// two's-complement bits), f32 for f32, f64 for f64.
#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "../../include/satgb.h"

namespace satgb {
satgb_status api_fail(satgb_status st, const char* msg);
satgb_status api_cuda_fail(cudaError_t e, const char* what);
void api_count_launch();
}  // namespace satgb

namespace {

constexpr int kWarps = 16;
constexpr int kRPW = 2;                 // strip rows per warp
constexpr int kStrip = kWarps * kRPW;   // 32 rows per CTA
constexpr int kCPT = 4;                 // tile columns per lane
constexpr int kTileW = 32 * kCPT;       // 128 columns per tile

template <class A, class TIn>
__device__ __forceinline__ A to_acc(TIn v) {
  if constexpr (std::is_same<A, uint32_t>::value) {
    if constexpr (std::is_signed<TIn>::value) return (uint32_t)(int32_t)v;
    else return (uint32_t)v;
  } else {
    return (A)v;
  }
}

template <class TOut, class A>
__device__ __forceinline__ TOut from_acc(A v) {
  return (TOut)v; // u32 -> i32 keeps the bits
}

// one vector access for N elements of up to 16 bytes in all
template <class TIn, int N>
struct Vec {
  static_assert(sizeof(TIn) * N <= 16, "at most one 16-byte access");
  using T = typename std::conditional<sizeof(TIn) * N == 4, uint32_t,
            typename std::conditional<sizeof(TIn) * N == 8, uint2, uint4>::type>::type;
};

// this warp's kRPW rows x kCPT columns of the tile at column x0; zero outside the image
template <class TIn>
__device__ __forceinline__ void load_tile(const TIn* in, long long pitch, int W, int H, int y, int x, bool vec,
                                          TIn (&v)[kRPW][kCPT]) {
#pragma unroll
  for (int r = 0; r < kRPW; ++r) {
    const TIn* row = in + (long long)(y + r) * pitch;
    const bool yin = y + r < H;
    bool done = false;
    if constexpr (sizeof(TIn) * kCPT <= 16) { // 8-byte inputs: two 16-byte halves, element by element below
      if (vec && yin && x + kCPT <= W) {
        union {
          typename Vec<TIn, kCPT>::T u;
          TIn e[kCPT];
        } s;
        s.u = __ldcs(reinterpret_cast<const typename Vec<TIn, kCPT>::T*>(row + x));
#pragma unroll
        for (int c = 0; c < kCPT; ++c) v[r][c] = s.e[c];
        done = true;
      }
    }
    if (!done) {
#pragma unroll
      for (int c = 0; c < kCPT; ++c) v[r][c] = (yin && x + c < W) ? __ldcs(row + x + c) : TIn(0);
    }
  }
}

template <class TIn, class TOut, class A>
__global__ void __launch_bounds__(kWarps * 32) scan_rows_t_kernel(const TIn* __restrict__ in, long long in_pitch,
                                                                  TOut* __restrict__ out, long long out_pitch, int W,
                                                                  int H, bool vec) {
  __shared__ A tr[kTileW][kStrip + 1];
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int y0 = blockIdx.x * kStrip;
  const int yw = y0 + warp * kRPW;
  A carry[kRPW];
#pragma unroll
  for (int r = 0; r < kRPW; ++r) carry[r] = A(0);
  TIn nxt[kRPW][kCPT];
  load_tile<TIn>(in, in_pitch, W, H, yw, lane * kCPT, vec, nxt);
  for (int x0 = 0; x0 < W; x0 += kTileW) {
    TIn cur[kRPW][kCPT];
#pragma unroll
    for (int r = 0; r < kRPW; ++r)
#pragma unroll
      for (int c = 0; c < kCPT; ++c) cur[r][c] = nxt[r][c];
    if (x0 + kTileW < W) load_tile<TIn>(in, in_pitch, W, H, yw, x0 + kTileW + lane * kCPT, vec, nxt);
    A v[kRPW][kCPT];
    A incl[kRPW];
#pragma unroll
    for (int r = 0; r < kRPW; ++r) {
#pragma unroll
      for (int c = 0; c < kCPT; ++c) v[r][c] = c ? v[r][c - 1] + to_acc<A>(cur[r][c]) : to_acc<A>(cur[r][c]);
      incl[r] = v[r][kCPT - 1];
    }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
#pragma unroll
      for (int r = 0; r < kRPW; ++r) {
        const A o = __shfl_up_sync(0xffffffffu, incl[r], d);
        if (lane >= d) incl[r] = o + incl[r];
      }
    }
#pragma unroll
    for (int r = 0; r < kRPW; ++r) {
      A ex = __shfl_up_sync(0xffffffffu, incl[r], 1);
      if (lane == 0) ex = A(0);
      const A total = __shfl_sync(0xffffffffu, incl[r], 31);
      const A base = carry[r] + ex;
#pragma unroll
      for (int c = 0; c < kCPT; ++c) v[r][c] = base + v[r][c];
      carry[r] = carry[r] + total;
    }
    __syncthreads(); // the previous tile's transposed reads are done
#pragma unroll
    for (int r = 0; r < kRPW; ++r)
#pragma unroll
      for (int c = 0; c < kCPT; ++c) tr[lane * kCPT + c][warp * kRPW + r] = v[r][c];
    __syncthreads();
    const int y = y0 + lane;
#pragma unroll 4
    for (int xr = warp; xr < kTileW; xr += kWarps) {
      const int x = x0 + xr;
      if (x < W && y < H) __stcs(out + (long long)x * out_pitch + y, from_acc<TOut, A>(tr[xr][lane]));
    }
  }
}

template <class TIn, class TOut, class A>
cudaError_t launch(const void* in, long long in_pitch, void* out, long long out_pitch, int W, int H, cudaStream_t s) {
  const bool vec = ((uintptr_t)in % (kCPT * sizeof(TIn))) == 0 && ((size_t)in_pitch * sizeof(TIn)) % (kCPT * sizeof(TIn)) == 0;
  const unsigned grid = (unsigned)((H + kStrip - 1) / kStrip);
  scan_rows_t_kernel<TIn, TOut, A><<<grid, kWarps * 32, 0, s>>>(static_cast<const TIn*>(in), in_pitch,
                                                                 static_cast<TOut*>(out), out_pitch, W, H, vec);
  return cudaGetLastError();
}

size_t elem_size(int t) {
  switch (t) {
    case SATGB_U8:
    case SATGB_I8: return 1;
    case SATGB_U16:
    case SATGB_I16: return 2; // listed in the reference's DataType, never dispatched
    case SATGB_U32:
    case SATGB_I32:
    case SATGB_F32: return 4;
    case SATGB_F64: return 8;
    default: return 0;
  }
}

}  // namespace

extern "C" satgb_status satgb_scan_rows_transposed(satgb_dtype in_t, satgb_dtype out_t, const void* d_in,
                                                   int64_t in_pitch, void* d_out, int64_t out_pitch, int64_t width,
                                                   int64_t height, satgb_stream stream) {
  const size_t si = elem_size(in_t), so = elem_size(out_t);
  if (!si || !so) return satgb::api_fail(SATGB_ERR_INVALID_ARG, "scan_rows_transposed: unknown dtype code");
  if (width < 0 || height < 0) return satgb::api_fail(SATGB_ERR_INVALID_ARG, "scan_rows_transposed: negative size");
  if (width == 0 || height == 0) return SATGB_OK;
  if (!d_in || !d_out) return satgb::api_fail(SATGB_ERR_INVALID_ARG, "scan_rows_transposed: null buffer");
  if (in_pitch < width || out_pitch < height)
    return satgb::api_fail(SATGB_ERR_INVALID_ARG,
                           "scan_rows_transposed: in pitch below the width or out pitch below the height");
  // column and row indices are ints in the kernel, and the tile loop steps past the last column
  if (width > (1LL << 31) - 2 * kTileW || height > (1LL << 31) - 2 * kStrip || height - 1 > INT64_MAX / 16 / in_pitch ||
      width - 1 > INT64_MAX / 16 / out_pitch)
    return satgb::api_fail(SATGB_ERR_OVERFLOW, "scan_rows_transposed: image too large");
  if (((uintptr_t)d_in % si) != 0 || ((uintptr_t)d_out % so) != 0)
    return satgb::api_fail(SATGB_ERR_MISALIGNED, "scan_rows_transposed: buffer not aligned to its element size");
  const char* ib = static_cast<const char*>(d_in);
  const char* ie = ib + ((height - 1) * in_pitch + width) * (int64_t)si;
  const char* ob = static_cast<const char*>(d_out);
  const char* oe = ob + ((width - 1) * out_pitch + height) * (int64_t)so;
  if (ib < oe && ob < ie) return satgb::api_fail(SATGB_ERR_INVALID_ARG, "scan_rows_transposed: input and output overlap");
  cudaStream_t s = (cudaStream_t)stream;
  const int W = (int)width, H = (int)height;
  cudaError_t e = cudaSuccess;
#define SG_T(IT, OT, TIN, TOUT, A) \
  if (in_t == IT && out_t == OT) e = launch<TIN, TOUT, A>(d_in, in_pitch, d_out, out_pitch, W, H, s); else
  SG_T(SATGB_U8, SATGB_U32, uint8_t, uint32_t, uint32_t)
  SG_T(SATGB_U8, SATGB_F32, uint8_t, float, float)
  SG_T(SATGB_U8, SATGB_F64, uint8_t, double, double)
  SG_T(SATGB_I8, SATGB_I32, int8_t, int32_t, uint32_t)
  SG_T(SATGB_I8, SATGB_F32, int8_t, float, float)
  SG_T(SATGB_I8, SATGB_F64, int8_t, double, double)
  SG_T(SATGB_I32, SATGB_I32, int32_t, int32_t, uint32_t)
  SG_T(SATGB_I32, SATGB_F64, int32_t, double, double)
  SG_T(SATGB_U32, SATGB_U32, uint32_t, uint32_t, uint32_t)
  SG_T(SATGB_F32, SATGB_F32, float, float, float)
  SG_T(SATGB_F32, SATGB_F64, float, double, double)
  SG_T(SATGB_F64, SATGB_F64, double, double, double)
  return satgb::api_fail(SATGB_ERR_UNSUPPORTED_TYPES, "scan_rows_transposed: type pair not offered");
#undef SG_T
  if (e != cudaSuccess) return satgb::api_cuda_fail(e, "scan_rows_t_kernel launch");
  satgb::api_count_launch();
  return SATGB_OK;
}
