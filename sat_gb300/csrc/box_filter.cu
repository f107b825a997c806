// box_filter.cu -- box-filter means read from a summed-area table, and their
// adjoint, for n_planes f32 planes and up to four radii in one pass.
//
// Forward, radius r, output (y,x): the window is rows [ya, yb] =
// [max(0, y-r), min(H-1, y+r)] and columns [xa, xb] likewise, and
//   mean = (S(yb,xb) - S(ya-1,xb) - S(yb,xa-1) + S(ya-1,xa-1)) / area,
// with S(-1, .) = S(., -1) = 0 and area = (yb-ya+1)(xb-xa+1).
//
// Backward: with h = g / area (g the incoming gradient of the mean), the
// gradient of S at (p,q) collects +-h from every output whose window has a
// corner there.  The index sets separate: rows y with yb(y) = p enter with +1
// (y = p - r, or for p = H-1 every y >= H-1-r), rows with ya(y) - 1 = p with
// -1 (y = p + 1 + r); the same for columns.  So
//   dS(p,q) = sum_{y in Y(p)} sum_{x in X(q)} sy * sx * h(y,x),
// a gather of at most four terms except on the last row and column, which
// collect up to r+1 terms each.  A gather rather than a scatter keeps the
// result deterministic.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/satgb.h"

namespace satgb {
satgb_status api_fail(satgb_status st, const char* msg);
satgb_status api_cuda_fail(cudaError_t e, const char* what);
void api_count_launch();
}  // namespace satgb

namespace {

struct BoxArgs {
  int64_t w, h, planes;
  float* sat;
  int64_t sat_pitch, sat_plane;
  int nr;
  int rmax; // the largest radius
  int r[SATGB_MAX_RADII];
  float inv_full[SATGB_MAX_RADII]; // 1 / (2r + 1): the reciprocal window length away from the edges
  float* box[SATGB_MAX_RADII];
  int64_t box_pitch, box_plane;
  int idx32; // every in-plane element offset fits in 32 bits: only then the interior paths run (int offsets)
};

// A block covers 32 columns x 64 rows of one plane: blockDim (32, 8), each
// thread 8 rows 8 apart, so a warp touches 32 consecutive columns of a row.
constexpr int kBX = 32, kBY = 8, kRows = 8;
// The backward blocks are 32 rows tall (4 rows a thread): the blocks that
// touch the 2r-wide border band, which take the general path, are fewer.
constexpr int kBRows = 4;

// Window [lo, hi] of radius r around i, clipped to [0, n-1], and 1 / its length.
struct Win {
  int lo, hi;
  float inv;
};
__device__ __forceinline__ Win win(int i, int r, int n, float inv_full) {
  Win w;
  w.lo = max(0, i - r);
  w.hi = min(n - 1, i + r);
  if (i - r >= 0 && i + r <= n - 1) {
    w.inv = inv_full; // the whole window fits: the common case, no division
  } else {
    w.inv = __frcp_rn((float)(w.hi - w.lo + 1)); // the correctly rounded 1/len, as 1.0f / len
  }
  return w;
}

// A block is interior for the forward pass when every output in it has its
// whole window and the row and column before it inside the image, for the
// largest radius and so for all: then the four corners sit at fixed offsets and
// a thread issues all its rows' corner loads before it needs them.
__device__ __forceinline__ bool fwd_block_interior(const BoxArgs& a, int x0, int y0) {
  const long long W = a.w, H = a.h, r = a.rmax;
  return x0 - r - 1 >= 0 && x0 + kBX - 1 + r <= W - 1 && y0 - r - 1 >= 0 && y0 + kBY * kRows - 1 + r <= H - 1;
}

template <int NR>
__global__ void __launch_bounds__(kBX * kBY) box_fwd_kernel(const __grid_constant__ BoxArgs a) {
  const int W = (int)a.w, H = (int)a.h;
  const int x = blockIdx.x * kBX + threadIdx.x;
  if (x >= W) return;
  const long long pl = blockIdx.z;
  const float* S = a.sat + pl * a.sat_plane;
  const int ybase = blockIdx.y * (kBY * kRows) + threadIdx.y;
  if (a.idx32 && fwd_block_interior(a, blockIdx.x * kBX, blockIdx.y * (kBY * kRows))) {
    const int sp = (int)a.sat_pitch, bp = (int)a.box_pitch;
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      const int r = a.r[i];
      const float inv2 = a.inv_full[i] * a.inv_full[i];
      const int hi = (ybase + r) * sp + x; // in-plane element offsets
      const int lo = hi - (2 * r + 1) * sp;
      float* B = a.box[i] + pl * a.box_plane;
      const int bo = ybase * bp + x;
      float out[kRows];
#pragma unroll
      for (int k = 0; k < kRows; ++k) {
        const int o = k * kBY * sp;
        out[k] = ((__ldg(S + (hi + o + r)) - __ldg(S + (hi + o - r - 1))) -
                  (__ldg(S + (lo + o + r)) - __ldg(S + (lo + o - r - 1)))) *
                 inv2;
      }
#pragma unroll
      for (int k = 0; k < kRows; ++k) __stcs(B + (bo + k * kBY * bp), out[k]);
    }
    return;
  }
#pragma unroll 1
  for (int i = 0; i < NR; ++i) {
    const int r = a.r[i];
    const float inv_full = a.inv_full[i];
    const float inv2 = inv_full * inv_full;
    const Win wx = win(x, r, W, inv_full);
    // columns whose window and the column before it lie inside the image
    const bool xin = x - r - 1 >= 0 && x + r <= W - 1;
    float* B = a.box[i] + pl * a.box_plane;
#pragma unroll 4
    for (int k = 0; k < kRows; ++k) {
      const int y = ybase + k * kBY;
      if (y >= H) break;
      float out;
      if (xin && y - r - 1 >= 0 && y + r <= H - 1) {
        // interior: four corners at fixed offsets, full window area
        const float* hi = S + (long long)(y + r) * a.sat_pitch + x;
        const float* lo = S + (long long)(y - r - 1) * a.sat_pitch + x;
        out = ((__ldg(hi + r) - __ldg(hi - r - 1)) - (__ldg(lo + r) - __ldg(lo - r - 1))) * inv2;
      } else {
        const Win wy = win(y, r, H, inv_full);
        const float* lo = S + (long long)(wy.lo - 1) * a.sat_pitch; // row ya-1 (unused when ya == 0)
        const float* hi = S + (long long)wy.hi * a.sat_pitch;
        float sum = __ldg(hi + wx.hi);
        if (wx.lo > 0) sum -= __ldg(hi + wx.lo - 1);
        if (wy.lo > 0) {
          float t = __ldg(lo + wx.hi);
          if (wx.lo > 0) t -= __ldg(lo + wx.lo - 1);
          sum -= t;
        }
        out = sum * (wy.inv * wx.inv);
      }
      __stcs(B + (long long)y * a.box_pitch + x, out);
    }
  }
}

// h(y,x) = g(y,x) / area(y,x) for radius r
__device__ __forceinline__ float h_at(const float* g, long long pitch, int y, int x, int r, int H, int W) {
  return __ldg(g + (long long)y * pitch + x) / (float)((min(H - 1, y + r) - max(0, y - r) + 1) *
                                                        (min(W - 1, x + r) - max(0, x - r) + 1));
}

// dS(p,q) for radius r on the last row or column, where the +1 index set is
// a range: the general gather.
__device__ __noinline__ float adjoint_edge(const float* g, long long pitch, int pr, int q, int r, int H, int W) {
  int y0, y1, x0, x1;
  if (pr < H - 1) {
    y0 = y1 = pr - r;
  } else {
    y0 = max(0, H - 1 - r);
    y1 = H - 1;
  }
  const int y2 = pr + 1 + r;
  if (q < W - 1) {
    x0 = x1 = q - r;
  } else {
    x0 = max(0, W - 1 - r);
    x1 = W - 1;
  }
  const int x2 = q + 1 + r;
  float t = 0.f;
  for (int y = max(0, y0); y <= y1; ++y) {
    float row = 0.f;
    for (int x = max(0, x0); x <= x1; ++x) row += h_at(g, pitch, y, x, r, H, W);
    if (x2 <= W - 1) row -= h_at(g, pitch, y, x2, r, H, W);
    t += row;
  }
  if (y2 <= H - 1) {
    float row = 0.f;
    for (int x = max(0, x0); x <= x1; ++x) row += h_at(g, pitch, y2, x, r, H, W);
    if (x2 <= W - 1) row -= h_at(g, pitch, y2, x2, r, H, W);
    t -= row;
  }
  return t;
}

// adjoint_edge for one element, summed by the 32 lanes of a warp together:
// lane l takes taps l, l + 32, ... of the (rows x columns) tap set, and a
// butterfly sum gives every lane the same total.  Used for the corner
// (H-1, W-1), whose (r + 1)^2 taps would otherwise fall to a single lane.
__device__ __noinline__ float adjoint_edge_warp(const float* g, long long pitch, int pr, int q, int r, int H, int W,
                                                int lane) {
  const int ylo = pr < H - 1 ? pr - r : max(0, H - 1 - r);
  const int yhi = pr < H - 1 ? pr - r : H - 1;
  const int xlo = q < W - 1 ? q - r : max(0, W - 1 - r);
  const int xhi = q < W - 1 ? q - r : W - 1;
  const int y2 = pr + 1 + r, x2 = q + 1 + r;
  const int y0 = max(0, ylo), x0 = max(0, xlo);
  const int npy = yhi >= y0 ? yhi - y0 + 1 : 0, npx = xhi >= x0 ? xhi - x0 + 1 : 0;
  const int ny = npy + (y2 <= H - 1 ? 1 : 0), nx = npx + (x2 <= W - 1 ? 1 : 0);
  float s = 0.f;
  for (int t = lane; t < ny * nx; t += 32) {
    const int iy = t / nx, ix = t - iy * nx;
    const int y = iy < npy ? y0 + iy : y2;
    const int x = ix < npx ? x0 + ix : x2;
    const float v = h_at(g, pitch, y, x, r, H, W);
    s += (iy < npy) == (ix < npx) ? v : -v;
  }
#pragma unroll
  for (int m = 16; m >= 1; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
  return s;
}

// A block is interior for the backward pass when the four outputs with a
// corner at each of its positions have whole windows, for every radius: then
// the taps sit at fixed offsets (and the block misses the last row and column).
__device__ __forceinline__ bool bwd_block_interior(const BoxArgs& a, int x0, int y0) {
  const long long W = a.w, H = a.h, r2 = 2LL * a.rmax;
  return x0 >= r2 && x0 + kBX - 1 <= W - 2 - r2 && y0 >= r2 && y0 + kBY * kBRows - 1 <= H - 2 - r2;
}

template <int NR>
__global__ void __launch_bounds__(kBX * kBY, 3) box_bwd_kernel(const __grid_constant__ BoxArgs a) {
  const int W = (int)a.w, H = (int)a.h;
  const int q = blockIdx.x * kBX + threadIdx.x;
  const long long pl = blockIdx.z;
  const int ybase = blockIdx.y * (kBY * kBRows) + threadIdx.y;
  if (a.idx32 && bwd_block_interior(a, blockIdx.x * kBX, blockIdx.y * (kBY * kBRows))) {
    // dS(p,q) = sum_i c_i ((g(p-r,q-r) - g(p-r,q+1+r)) - (g(p+1+r,q-r) - g(p+1+r,q+1+r))),
    // with in-plane element offsets in ints
    const int gp = (int)a.box_pitch;
    float acc[kBRows];
#pragma unroll
    for (int k = 0; k < kBRows; ++k) acc[k] = 0.f;
#pragma unroll
    for (int i = 0; i < NR; ++i) {
      const int r = a.r[i];
      const int d = 2 * r + 1;
      const float c = a.inv_full[i] * a.inv_full[i];
      const float* g = a.box[i] + pl * a.box_plane;
      const int t = (ybase - r) * gp + (q - r);
      const int b = t + d * gp;
#pragma unroll
      for (int k = 0; k < kBRows; ++k) {
        const int o = k * kBY * gp;
        acc[k] += ((__ldg(g + (t + o)) - __ldg(g + (t + o + d))) - (__ldg(g + (b + o)) - __ldg(g + (b + o + d)))) * c;
      }
    }
    float* dS = a.sat + pl * a.sat_plane;
    const int so = ybase * (int)a.sat_pitch + q;
#pragma unroll
    for (int k = 0; k < kBRows; ++k) __stcs(dS + (so + k * kBY * (int)a.sat_pitch), acc[k]);
    return;
  }
  const bool live = q < W;
  // per radius: +h at column q - r, -h at column q + 1 + r (when inside),
  // each with its reciprocal window width (0 marks a column outside)
  float ixp[NR], ixm[NR];
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    const int r = a.r[i];
    ixp[i] = live && q - r >= 0 ? win(q - r, r, W, a.inv_full[i]).inv : 0.f;
    ixm[i] = live && q + 1 + r <= W - 1 ? win(q + 1 + r, r, W, a.inv_full[i]).inv : 0.f;
  }
  // Every row at once and without branches: a tap outside the image reads
  // nothing and counts 0; 1/(window length) of a tap row is inv_full unless the
  // window is clipped.  The last row and column are summed apart below.
  const long long gp = a.box_pitch;
  float acc[kBRows];
#pragma unroll
  for (int k = 0; k < kBRows; ++k) acc[k] = 0.f;
#pragma unroll
  for (int i = 0; i < NR; ++i) {
    const int r = a.r[i];
    const float* g = a.box[i] + pl * a.box_plane;
    const int xp = q - r, xm = q + 1 + r;
    const bool okp = live && xp >= 0, okm = live && xm <= W - 1;
#pragma unroll
    for (int k = 0; k < kBRows; ++k) {
      const int pr = ybase + k * kBY;
      const int yp = pr - r, ym = pr + 1 + r;
      const bool oyp = yp >= 0 && pr < H, oym = ym <= H - 1;
      const float iyp = !oyp ? 0.f : (yp >= r && yp + r <= H - 1 ? a.inv_full[i] : win(yp, r, H, a.inv_full[i]).inv);
      const float iym = !oym ? 0.f : (ym >= r && ym + r <= H - 1 ? a.inv_full[i] : win(ym, r, H, a.inv_full[i]).inv);
      const float* rp = g + (long long)yp * gp;
      const float* rm = g + (long long)ym * gp;
      const float a0 = oyp && okp ? __ldg(rp + xp) : 0.f;
      const float a1 = oyp && okm ? __ldg(rp + xm) : 0.f;
      const float b0 = oym && okp ? __ldg(rm + xp) : 0.f;
      const float b1 = oym && okm ? __ldg(rm + xm) : 0.f;
      acc[k] += (a0 * ixp[i] - a1 * ixm[i]) * iyp - (b0 * ixp[i] - b1 * ixm[i]) * iym;
    }
  }
  // the last row and column belong to box_bwd_edge_kernel
  float* dS = a.sat + pl * a.sat_plane;
#pragma unroll
  for (int k = 0; k < kBRows; ++k) {
    const int pr = ybase + k * kBY;
    if (pr < H - 1 && q < W - 1) __stcs(dS + (long long)pr * a.sat_pitch + q, acc[k]);
  }
}

// The last row and the last column of dS, where the +1 index set of the
// gather is a range of r + 1 rows or columns: one thread per element, and the
// corner (H-1, W-1), with (r + 1)^2 taps per radius, summed by one warp.
constexpr int kEdgeThreads = 256;

template <int NR>
__global__ void __launch_bounds__(kEdgeThreads) box_bwd_edge_kernel(const __grid_constant__ BoxArgs a) {
  const int W = (int)a.w, H = (int)a.h;
  const long long pl = blockIdx.z;
  float* dS = a.sat + pl * a.sat_plane;
  const long long e = (long long)blockIdx.x * kEdgeThreads + threadIdx.x;
  const long long n_edge = (long long)(W - 1) + (H - 1); // the last row and column without the corner
  if (blockIdx.x == gridDim.x - 1) {
    if (threadIdx.x < 32) { // the corner
      float v = 0.f;
      for (int i = 0; i < NR; ++i)
        v += adjoint_edge_warp(a.box[i] + pl * a.box_plane, a.box_pitch, H - 1, W - 1, a.r[i], H, W, threadIdx.x);
      if (threadIdx.x == 0) dS[(long long)(H - 1) * a.sat_pitch + (W - 1)] = v;
    }
    return;
  }
  if (e >= n_edge) return;
  const int pr = e < W - 1 ? H - 1 : (int)(e - (W - 1));
  const int q = e < W - 1 ? (int)e : W - 1;
  float v = 0.f;
  for (int i = 0; i < NR; ++i) v += adjoint_edge(a.box[i] + pl * a.box_plane, a.box_pitch, pr, q, a.r[i], H, W);
  dS[(long long)pr * a.sat_pitch + q] = v;
}

satgb_status check_desc_(const satgb_box_desc* d, BoxArgs& a);

satgb_status check_desc(const satgb_box_desc* d, BoxArgs& a) {
  const satgb_status st = check_desc_(d, a);
  if (st == SATGB_ERR_MISALIGNED) return satgb::api_fail(st, "box filter: f32 pointer not 4-byte aligned");
  if (st != SATGB_OK) return satgb::api_fail(st, "box filter: invalid descriptor (sizes, pitches, radii or pointers)");
  return st;
}

satgb_status check_desc_(const satgb_box_desc* d, BoxArgs& a) {
  if (!d) return SATGB_ERR_INVALID_ARG;
  if (d->width < 0 || d->height < 0 || d->n_planes < 0) return SATGB_ERR_INVALID_ARG;
  if (d->n_radii < 1 || d->n_radii > SATGB_MAX_RADII) return SATGB_ERR_INVALID_ARG;
  if (d->width == 0 || d->height == 0 || d->n_planes == 0) return SATGB_OK;
  if (!d->d_sat || d->sat_pitch < d->width || d->box_pitch < d->width) return SATGB_ERR_INVALID_ARG;
  // in-plane coordinates are 32-bit; grid.y (32-row blocks of the backward) and grid.z limits
  if (d->width > (1LL << 30) || d->height > 65535LL * kBY * kBRows || d->n_planes > 65535) return SATGB_ERR_INVALID_ARG;
  if (d->n_planes > 1 && (d->sat_plane_stride < (d->height - 1) * d->sat_pitch + d->width ||
                          d->box_plane_stride < (d->height - 1) * d->box_pitch + d->width))
    return SATGB_ERR_INVALID_ARG;
  if (((uintptr_t)d->d_sat % 4) != 0) return SATGB_ERR_MISALIGNED;
  a.w = d->width;
  a.h = d->height;
  a.planes = d->n_planes;
  a.sat = static_cast<float*>(d->d_sat);
  a.sat_pitch = d->sat_pitch;
  a.sat_plane = d->sat_plane_stride;
  a.nr = d->n_radii;
  a.rmax = 0;
  a.idx32 = (d->height - 1) * d->sat_pitch + d->width < (1LL << 31) &&
            (d->height - 1) * d->box_pitch + d->width < (1LL << 31);
  a.box_pitch = d->box_pitch;
  a.box_plane = d->box_plane_stride;
  for (int i = 0; i < SATGB_MAX_RADII; ++i) {
    a.r[i] = 0;
    a.inv_full[i] = 1.0f;
    a.box[i] = nullptr;
  }
  // A window of radius max(W, H) - 1 around any pixel already covers the whole
  // image, so larger radii give the same means: they are clamped there, which
  // keeps every index expression of the kernels (x + r, 2r + 1, ...) in int.
  const int64_t rcap = (d->width > d->height ? d->width : d->height) - 1;
  for (int i = 0; i < d->n_radii; ++i) {
    if (d->radius[i] < 0 || !d->d_box[i]) return SATGB_ERR_INVALID_ARG;
    if (((uintptr_t)d->d_box[i] % 4) != 0) return SATGB_ERR_MISALIGNED;
    a.r[i] = (int)((int64_t)d->radius[i] < rcap ? (int64_t)d->radius[i] : rcap);
    a.rmax = a.r[i] > a.rmax ? a.r[i] : a.rmax;
    a.inv_full[i] = 1.0f / (float)(2 * (double)a.r[i] + 1);
    a.box[i] = static_cast<float*>(d->d_box[i]);
  }
  return SATGB_OK;
}

}  // namespace

extern "C" satgb_status satgb_box_filter_fwd(const satgb_box_desc* d, satgb_stream stream) {
  BoxArgs a;
  satgb_status st = check_desc(d, a);
  if (st != SATGB_OK || d->width == 0 || d->height == 0 || d->n_planes == 0) return st;
  dim3 grid((unsigned)((d->width + kBX - 1) / kBX), (unsigned)((d->height + kBY * kRows - 1) / (kBY * kRows)),
            (unsigned)d->n_planes);
  const dim3 block(kBX, kBY);
  cudaStream_t s = (cudaStream_t)stream;
  switch (a.nr) {
    case 1: box_fwd_kernel<1><<<grid, block, 0, s>>>(a); break;
    case 2: box_fwd_kernel<2><<<grid, block, 0, s>>>(a); break;
    case 3: box_fwd_kernel<3><<<grid, block, 0, s>>>(a); break;
    default: box_fwd_kernel<4><<<grid, block, 0, s>>>(a); break;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return satgb::api_cuda_fail(e, "box_fwd_kernel launch");
  satgb::api_count_launch();
  return SATGB_OK;
}

extern "C" satgb_status satgb_box_filter_bwd(const satgb_box_desc* d, satgb_stream stream) {
  BoxArgs a;
  satgb_status st = check_desc(d, a);
  if (st != SATGB_OK || d->width == 0 || d->height == 0 || d->n_planes == 0) return st;
  dim3 grid((unsigned)((d->width + kBX - 1) / kBX), (unsigned)((d->height + kBY * kBRows - 1) / (kBY * kBRows)),
            (unsigned)d->n_planes);
  const dim3 block(kBX, kBY);
  cudaStream_t s = (cudaStream_t)stream;
  switch (a.nr) {
    case 1: box_bwd_kernel<1><<<grid, block, 0, s>>>(a); break;
    case 2: box_bwd_kernel<2><<<grid, block, 0, s>>>(a); break;
    case 3: box_bwd_kernel<3><<<grid, block, 0, s>>>(a); break;
    default: box_bwd_kernel<4><<<grid, block, 0, s>>>(a); break;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return satgb::api_cuda_fail(e, "box_bwd_kernel launch");
  satgb::api_count_launch();
  // the last row and column: (W - 1) + (H - 1) elements a plane, then one block for the corner
  const dim3 egrid((unsigned)((d->width + d->height - 2 + kEdgeThreads - 1) / kEdgeThreads + 1), 1,
                   (unsigned)d->n_planes);
  switch (a.nr) {
    case 1: box_bwd_edge_kernel<1><<<egrid, kEdgeThreads, 0, s>>>(a); break;
    case 2: box_bwd_edge_kernel<2><<<egrid, kEdgeThreads, 0, s>>>(a); break;
    case 3: box_bwd_edge_kernel<3><<<egrid, kEdgeThreads, 0, s>>>(a); break;
    default: box_bwd_edge_kernel<4><<<egrid, kEdgeThreads, 0, s>>>(a); break;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return satgb::api_cuda_fail(e, "box_bwd_edge_kernel launch");
  satgb::api_count_launch();
  return SATGB_OK;
}
