// scan_rows_t.cu -- the row scans, which need no look-back: the row scan with
// transposed output (satgb_scan_rows_transposed) and, further down, the plain
// row scan (satgb_scan_rows).
//
//   transposed: out(x, y) = sum_{i <= x} in(y, i)   in: W x H (row y, column x), out: H x W
//
// is the reference's SerielScan::TestX (integralImage/BRLT-Scan.cu:128-190), whose
// serielScan launch reads rows and stores the scanned rows transposed
// (compared there with IntegralImageAllRow + Transpose).  Rows are
// independent, so there is no look-back: a CTA owns a strip of 32 rows and
// walks it left to right in tiles of 32 x CPT columns, CPT = 16 / sizeof(in),
// so that every thread reads one 16-byte vector per row and tile whatever the
// input type (a tile is 16 KB of input).  Warp w (of 16) owns strip rows
// [2w, 2w+2) and keeps their running sums (the carry) in registers from tile
// to tile; lane l owns columns [l CPT, (l+1) CPT) of the tile.  The next two
// tiles' vectors are in flight while a tile is scanned (32 KB a CTA), which
// is what keeps HBM busy with one CTA per 32 rows.  Per tile: in-thread
// prefix, Kogge-Stone warp scan of the lane totals, plus the carry; the
// 32-row block of results is transposed through shared memory and leaves as
// output rows of 32 consecutive elements, each written as 16-byte vectors (8
// lanes a row for 4-byte sums, 16 for 8-byte).  The transpose buffer has rows
// of 32 entries held as 16 pairs (strip rows 2k, 2k+1: one thread's two rows)
// with pair k of row x in slot k ^ ((x / CPT) mod 16): a warp's pair stores
// (one slot per lane, 16 different slots per half-warp) and its 16-byte reads
// (whole rows) both take the fewest shared-memory wavefronts.
// Accumulators: u32 for integer outputs (mod-2^32 wrap, i32 results are the
// two's-complement bits), f32 for f32, f64 for f64.
#include <cuda_runtime.h>

#include <atomic>
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
constexpr int kMaxTileW = 32 * 16;      // the widest tile (1-byte inputs)

template <class TIn>
struct Shape {
  static constexpr int CPT = 16 / (int)sizeof(TIn); // tile columns per lane
  static constexpr int TW = 32 * CPT;               // tile columns
};

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
  static_assert(sizeof(TOut) == sizeof(A), "sums are stored with their own bits");
  return (TOut)v; // u32 -> i32 keeps the bits
}

template <class A>
__device__ __forceinline__ uint32_t bits32(A v) {
  if constexpr (std::is_same<A, float>::value) return __float_as_uint(v);
  else return (uint32_t)v;
}
__device__ __forceinline__ unsigned long long bits64(double v) { return (unsigned long long)__double_as_longlong(v); }

template <class TIn>
union Seg {
  uint4 u;
  TIn e[Shape<TIn>::CPT];
};

// this warp's kRPW rows x CPT columns of the tile at column x (raw 16-byte
// vectors); zero outside the image
template <class TIn>
__device__ __forceinline__ void load_tile(const TIn* in, long long pitch, int W, int H, int y, int x, bool vec,
                                          uint4 (&v)[kRPW]) {
  constexpr int CPT = Shape<TIn>::CPT;
#pragma unroll
  for (int r = 0; r < kRPW; ++r) {
    const TIn* row = in + (long long)(y + r) * pitch;
    const bool yin = y + r < H;
    if (vec && yin && x + CPT <= W) {
      v[r] = __ldcs(reinterpret_cast<const uint4*>(row + x));
    } else {
      Seg<TIn> s;
#pragma unroll
      for (int c = 0; c < CPT; ++c) s.e[c] = (yin && x + c < W) ? __ldcs(row + x + c) : TIn(0);
      v[r] = s.u;
    }
  }
}

template <class TIn, class TOut, class A>
__global__ void __launch_bounds__(kWarps * 32) scan_rows_t_kernel(const TIn* __restrict__ in, long long in_pitch,
                                                                  TOut* __restrict__ out, long long out_pitch, int W,
                                                                  int H, bool vec, bool ovec) {
  constexpr int CPT = Shape<TIn>::CPT, TW = Shape<TIn>::TW;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  A* tr = reinterpret_cast<A*>(smem_raw); // TW rows of 32 (swizzled)
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int y0 = blockIdx.x * kStrip;
  const int yw = y0 + warp * kRPW;
  A carry[kRPW];
#pragma unroll
  for (int r = 0; r < kRPW; ++r) carry[r] = A(0);
  uint4 n0[kRPW], n1[kRPW];
  load_tile<TIn>(in, in_pitch, W, H, yw, lane * CPT, vec, n0);
  if (TW < W) load_tile<TIn>(in, in_pitch, W, H, yw, TW + lane * CPT, vec, n1);
  for (int x0 = 0; x0 < W; x0 += TW) {
    Seg<TIn> cur[kRPW];
#pragma unroll
    for (int r = 0; r < kRPW; ++r) {
      cur[r].u = n0[r];
      n0[r] = n1[r];
    }
    if (x0 + 2 * TW < W) load_tile<TIn>(in, in_pitch, W, H, yw, x0 + 2 * TW + lane * CPT, vec, n1);
    A v[kRPW][CPT];
    A incl[kRPW];
#pragma unroll
    for (int r = 0; r < kRPW; ++r) {
#pragma unroll
      for (int c = 0; c < CPT; ++c) v[r][c] = c ? v[r][c - 1] + to_acc<A>(cur[r].e[c]) : to_acc<A>(cur[r].e[c]);
      incl[r] = v[r][CPT - 1];
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
      for (int c = 0; c < CPT; ++c) v[r][c] = base + v[r][c];
      carry[r] = carry[r] + total;
    }
    __syncthreads(); // the previous tile's transposed reads are done
    // column x = lane CPT + c: the thread's two rows (2 warp, 2 warp + 1) as
    // one pair, in pair slot warp ^ (lane mod 16) of transpose row x
#pragma unroll
    for (int c = 0; c < CPT; ++c) {
      A* slot = tr + (lane * CPT + c) * 32 + 2 * (warp ^ (lane & 15));
      if constexpr (sizeof(A) == 4) *reinterpret_cast<uint2*>(slot) = make_uint2(bits32(v[0][c]), bits32(v[1][c]));
      else *reinterpret_cast<ulonglong2*>(slot) = make_ulonglong2(bits64(v[0][c]), bits64(v[1][c]));
    }
    __syncthreads();
    // output rows of 32 elements as 16-byte vectors: LPR lanes a row, RPI rows
    // a warp instruction
    constexpr int EPV = 16 / (int)sizeof(A), LPR = 32 / EPV, RPI = 32 / LPR;
    const int j = lane % LPR;
#pragma unroll 2
    for (int xr = warp * RPI + lane / LPR; xr < TW; xr += kWarps * RPI) {
      const int h = (xr / CPT) & 15; // the swizzle of transpose row xr
      union {
        uint4 u;
        A e[EPV];
      } q;
      if constexpr (sizeof(A) == 4) {
        // rows 4j .. 4j+3 are pairs 2j and 2j+1: slots (2j)^h and its neighbour,
        // one aligned 16 bytes, in swapped order when h is odd
        q.u = *reinterpret_cast<const uint4*>(tr + xr * 32 + 4 * (j ^ (h >> 1)));
        if (h & 1) q.u = make_uint4(q.u.z, q.u.w, q.u.x, q.u.y);
      } else {
        q.u = *reinterpret_cast<const uint4*>(tr + xr * 32 + 2 * (j ^ h)); // rows 2j, 2j+1
      }
      const int x = x0 + xr, y = y0 + j * EPV;
      if (x < W) {
        TOut* o = out + (long long)x * out_pitch + y;
        if (ovec && y + EPV <= H) {
          __stcs(reinterpret_cast<uint4*>(o), q.u); // TOut and A have the same bits
        } else {
#pragma unroll
          for (int e = 0; e < EPV; ++e)
            if (y + e < H) __stcs(o + e, from_acc<TOut, A>(q.e[e]));
        }
      }
    }
  }
}

template <class TIn, class TOut, class A>
cudaError_t launch(const void* in, long long in_pitch, void* out, long long out_pitch, int W, int H, cudaStream_t s) {
  constexpr int smem = Shape<TIn>::TW * 32 * (int)sizeof(A);
  // the dynamic shared-memory limit, raised once per device (up to 128 KB, for 1-byte inputs and f64 sums)
  static std::atomic<int> raised[64];
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64 || !raised[dev].load(std::memory_order_acquire)) {
    e = cudaFuncSetAttribute(&scan_rows_t_kernel<TIn, TOut, A>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < 64) raised[dev].store(1, std::memory_order_release);
  }
  const bool vec = ((uintptr_t)in % 16) == 0 && ((size_t)in_pitch * sizeof(TIn)) % 16 == 0;
  const bool ovec = ((uintptr_t)out % 16) == 0 && ((size_t)out_pitch * sizeof(TOut)) % 16 == 0;
  const unsigned grid = (unsigned)((H + kStrip - 1) / kStrip);
  scan_rows_t_kernel<TIn, TOut, A><<<grid, kWarps * 32, smem, s>>>(static_cast<const TIn*>(in), in_pitch,
                                                                   static_cast<TOut*>(out), out_pitch, W, H, vec, ovec);
  return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// Row scan, untransposed (satgb_scan_rows): out(y, x) = sum_{i <= x} in(y, i)
// in the input's own layout.  Rows are independent and the output needs no
// transpose, so every warp works alone: it owns R rows, walks them left to
// right in the same tiles as above (one 16-byte input vector per lane and
// row, two tiles in flight, the running sums in registers) and stores each
// lane's CPT results of a row straight from registers as 16-byte vectors.
// No shared memory, no barrier.  Two rows a warp in CTAs of 4 warps for tall
// images; one row a warp in CTAs of 8 for shorter ones, which would otherwise
// leave most warp slots empty (f32 4096^2: 4630 -> 5390 GB/s; at 8192^2 the
// two shapes are within 2 %).
template <class TIn, int R>
__device__ __forceinline__ void load_rows(const TIn* in, long long pitch, int W, int H, int y, int x, bool vec,
                                          uint4 (&v)[R]) {
  constexpr int CPT = Shape<TIn>::CPT;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const TIn* row = in + (long long)(y + r) * pitch;
    const bool yin = y + r < H;
    if (vec && yin && x + CPT <= W) {
      v[r] = __ldcs(reinterpret_cast<const uint4*>(row + x));
    } else {
      Seg<TIn> s;
#pragma unroll
      for (int c = 0; c < CPT; ++c) s.e[c] = (yin && x + c < W) ? __ldcs(row + x + c) : TIn(0);
      v[r] = s.u;
    }
  }
}

template <class TIn, class TOut, class A, int R, int NWARPS>
__global__ void __launch_bounds__(NWARPS * 32) scan_rows_strip_kernel(const TIn* __restrict__ in, long long in_pitch,
                                                                      long long in_plane, TOut* __restrict__ out,
                                                                      long long out_pitch, long long out_plane, int W,
                                                                      int H, bool vec, bool ovec) {
  constexpr int CPT = Shape<TIn>::CPT, TW = Shape<TIn>::TW;
  constexpr int OV = CPT * (int)sizeof(TOut) / 16; // 16-byte output vectors per lane and row
  static_assert(CPT * sizeof(TOut) % 16 == 0, "whole output vectors");
  const int lane = threadIdx.x & 31;
  const int yw = (blockIdx.x * NWARPS + (threadIdx.x >> 5)) * R;
  if (yw >= H) return;
  in += blockIdx.y * in_plane;
  out += blockIdx.y * out_plane;
  A carry[R];
#pragma unroll
  for (int r = 0; r < R; ++r) carry[r] = A(0);
  uint4 n0[R], n1[R];
  load_rows<TIn, R>(in, in_pitch, W, H, yw, lane * CPT, vec, n0);
  if (TW < W) load_rows<TIn, R>(in, in_pitch, W, H, yw, TW + lane * CPT, vec, n1);
  for (int x0 = 0; x0 < W; x0 += TW) {
    Seg<TIn> cur[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      cur[r].u = n0[r];
      n0[r] = n1[r];
    }
    if (x0 + 2 * TW < W) load_rows<TIn, R>(in, in_pitch, W, H, yw, x0 + 2 * TW + lane * CPT, vec, n1);
    const int x = x0 + lane * CPT;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      union {
        uint4 u[OV];
        TOut e[CPT];
      } o;
      A v = A(0); // the lane's total
#pragma unroll
      for (int c = 0; c < CPT; ++c) v = v + to_acc<A>(cur[r].e[c]);
      A incl = v;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const A t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl = t + incl;
      }
      A ex = __shfl_up_sync(0xffffffffu, incl, 1);
      if (lane == 0) ex = A(0);
      const A base = carry[r] + ex;
      carry[r] = carry[r] + __shfl_sync(0xffffffffu, incl, 31);
      A run = base;
#pragma unroll
      for (int c = 0; c < CPT; ++c) {
        run = run + to_acc<A>(cur[r].e[c]);
        o.e[c] = from_acc<TOut, A>(run);
      }
      const int y = yw + r;
      if (y < H && x < W) {
        TOut* orow = out + (long long)y * out_pitch + x;
        if (ovec && x + CPT <= W) {
#pragma unroll
          for (int q = 0; q < OV; ++q) __stcs(reinterpret_cast<uint4*>(orow) + q, o.u[q]);
        } else {
#pragma unroll
          for (int c = 0; c < CPT; ++c)
            if (x + c < W) __stcs(orow + c, o.e[c]);
        }
      }
    }
  }
}

// SMs of the current device (once per device)
int device_sms() {
  static std::atomic<int> sms[64];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int n = sms[dev].load(std::memory_order_relaxed);
  if (n == 0) {
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
    sms[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}

template <class TIn, class TOut, class A>
cudaError_t launch_rows(const void* in, long long in_pitch, long long in_plane, void* out, long long out_pitch,
                        long long out_plane, int W, int H, int planes, cudaStream_t s) {
  const bool vec = ((uintptr_t)in % 16) == 0 && ((size_t)in_pitch * sizeof(TIn)) % 16 == 0 &&
                   (planes == 1 || ((size_t)in_plane * sizeof(TIn)) % 16 == 0);
  const bool ovec = ((uintptr_t)out % 16) == 0 && ((size_t)out_pitch * sizeof(TOut)) % 16 == 0 &&
                    (planes == 1 || ((size_t)out_plane * sizeof(TOut)) % 16 == 0);
  const TIn* ip = static_cast<const TIn*>(in);
  TOut* op = static_cast<TOut*>(out);
  // two rows a warp once there are at least 48 rows (24 warps) an SM
  if ((long long)H * planes >= 48LL * device_sms()) {
    const dim3 grid((unsigned)((H + 7) / 8), (unsigned)planes);
    scan_rows_strip_kernel<TIn, TOut, A, 2, 4><<<grid, 128, 0, s>>>(ip, in_pitch, in_plane, op, out_pitch, out_plane,
                                                                      W, H, vec, ovec);
  } else {
    const dim3 grid((unsigned)((H + 7) / 8), (unsigned)planes);
    scan_rows_strip_kernel<TIn, TOut, A, 1, 8><<<grid, 256, 0, s>>>(ip, in_pitch, in_plane, op, out_pitch, out_plane,
                                                                      W, H, vec, ovec);
  }
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
  if (width > (1LL << 31) - 3 * kMaxTileW || height > (1LL << 31) - 2 * kStrip || height - 1 > INT64_MAX / 16 / in_pitch ||
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

namespace satgb {
// satgb_scan_rows' kernel, for arguments the caller has validated (sizes,
// pitches, overlap, type pair): planes of width x height at the given strides.
satgb_status scan_rows_strips(int in_t, int out_t, const void* d_in, int64_t in_pitch, int64_t in_plane, void* d_out,
                              int64_t out_pitch, int64_t out_plane, int64_t width, int64_t height, int64_t planes,
                              cudaStream_t s) {
  if (width > (1LL << 31) - 3 * kMaxTileW || height > (1LL << 31) - 2 * kStrip || planes > 65535)
    return api_fail(SATGB_ERR_OVERFLOW, "scan_rows: image too large");
  const int W = (int)width, H = (int)height, NP = (int)planes;
  cudaError_t e = cudaSuccess;
#define SG_R(IT, OT, TIN, TOUT, A) \
  if (in_t == IT && out_t == OT) e = launch_rows<TIN, TOUT, A>(d_in, in_pitch, in_plane, d_out, out_pitch, out_plane, W, H, NP, s); else
  SG_R(SATGB_U8, SATGB_U32, uint8_t, uint32_t, uint32_t)
  SG_R(SATGB_U8, SATGB_F32, uint8_t, float, float)
  SG_R(SATGB_U8, SATGB_F64, uint8_t, double, double)
  SG_R(SATGB_I8, SATGB_I32, int8_t, int32_t, uint32_t)
  SG_R(SATGB_I8, SATGB_F32, int8_t, float, float)
  SG_R(SATGB_I8, SATGB_F64, int8_t, double, double)
  SG_R(SATGB_I32, SATGB_I32, int32_t, int32_t, uint32_t)
  SG_R(SATGB_I32, SATGB_F64, int32_t, double, double)
  SG_R(SATGB_U32, SATGB_U32, uint32_t, uint32_t, uint32_t)
  SG_R(SATGB_F32, SATGB_F32, float, float, float)
  SG_R(SATGB_F32, SATGB_F64, float, double, double)
  SG_R(SATGB_F64, SATGB_F64, double, double, double)
  return api_fail(SATGB_ERR_UNSUPPORTED_TYPES, "scan_rows: type pair not offered");
#undef SG_R
  if (e != cudaSuccess) return api_cuda_fail(e, "scan_rows_strip_kernel launch");
  api_count_launch();
  return SATGB_OK;
}
}  // namespace satgb
