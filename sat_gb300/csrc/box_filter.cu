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
  int r[SATGB_MAX_RADII];
  float inv_full[SATGB_MAX_RADII]; // 1 / (2r + 1): the reciprocal window length away from the edges
  float* box[SATGB_MAX_RADII];
  int64_t box_pitch, box_plane;
};

// A block covers 32 columns x 64 rows of one plane: blockDim (32, 8), each
// thread 8 rows 8 apart, so a warp touches 32 consecutive columns of a row.
constexpr int kBX = 32, kBY = 8, kRows = 8;

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
    w.inv = 1.0f / (float)(w.hi - w.lo + 1);
  }
  return w;
}

__global__ void __launch_bounds__(kBX * kBY) box_fwd_kernel(const __grid_constant__ BoxArgs a) {
  const int W = (int)a.w, H = (int)a.h;
  const int x = blockIdx.x * kBX + threadIdx.x;
  if (x >= W) return;
  const long long pl = blockIdx.z;
  const float* S = a.sat + pl * a.sat_plane;
  const int ybase = blockIdx.y * (kBY * kRows) + threadIdx.y;
#pragma unroll 1
  for (int i = 0; i < a.nr; ++i) {
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

__global__ void __launch_bounds__(kBX * kBY, 4) box_bwd_kernel(const __grid_constant__ BoxArgs a) {
  const int W = (int)a.w, H = (int)a.h;
  const int q = blockIdx.x * kBX + threadIdx.x;
  if (q >= W) return;
  const long long pl = blockIdx.z;
  const int ybase = blockIdx.y * (kBY * kRows) + threadIdx.y;
  const bool col_edge = q == W - 1;
  // per radius: +h at column q - r, -h at column q + 1 + r (when inside),
  // each with its reciprocal window width (0 marks a column outside)
  float ixp[SATGB_MAX_RADII], ixm[SATGB_MAX_RADII];
#pragma unroll
  for (int i = 0; i < SATGB_MAX_RADII; ++i) {
    ixp[i] = ixm[i] = 0.f;
    if (i < a.nr) {
      const int r = a.r[i];
      if (q - r >= 0) ixp[i] = win(q - r, r, W, a.inv_full[i]).inv;
      if (q + 1 + r <= W - 1) ixm[i] = win(q + 1 + r, r, W, a.inv_full[i]).inv;
    }
  }
  float* dS = a.sat + pl * a.sat_plane;
#pragma unroll 2
  for (int k = 0; k < kRows; ++k) {
    const int pr = ybase + k * kBY;
    if (pr >= H) break;
    float acc = 0.f;
    if (col_edge || pr == H - 1) {
      for (int i = 0; i < a.nr; ++i)
        acc += adjoint_edge(a.box[i] + pl * a.box_plane, a.box_pitch, pr, q, a.r[i], H, W);
      __stcs(dS + (long long)pr * a.sat_pitch + q, acc);
      continue;
    }
#pragma unroll
    for (int i = 0; i < SATGB_MAX_RADII; ++i) {
      if (i >= a.nr) break;
      const int r = a.r[i];
      const float* g = a.box[i] + pl * a.box_plane;
      const int xp = q - r, xm = q + 1 + r, yp = pr - r, ym = pr + 1 + r;
      if (pr >= 2 * r && pr <= H - 2 - 2 * r && q >= 2 * r && q <= W - 2 - 2 * r) {
        // interior: the four outputs with a corner here have whole windows
        const float* rp = g + (long long)yp * a.box_pitch;
        const float* rm = g + (long long)ym * a.box_pitch;
        acc += ((__ldg(rp + xp) - __ldg(rp + xm)) - (__ldg(rm + xp) - __ldg(rm + xm))) *
               (a.inv_full[i] * a.inv_full[i]);
        continue;
      }
      float t = 0.f;
      if (yp >= 0) {
        const float* row = g + (long long)yp * a.box_pitch;
        float u = ixp[i] != 0.f ? __ldg(row + xp) * ixp[i] : 0.f;
        if (ixm[i] != 0.f) u -= __ldg(row + xm) * ixm[i];
        t = u * win(yp, r, H, a.inv_full[i]).inv;
      }
      if (ym <= H - 1) {
        const float* row = g + (long long)ym * a.box_pitch;
        float u = ixp[i] != 0.f ? __ldg(row + xp) * ixp[i] : 0.f;
        if (ixm[i] != 0.f) u -= __ldg(row + xm) * ixm[i];
        t -= u * win(ym, r, H, a.inv_full[i]).inv;
      }
      acc += t;
    }
    __stcs(dS + (long long)pr * a.sat_pitch + q, acc);
  }
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
  // in-plane coordinates are 32-bit; grid.y and grid.z limits
  if (d->width > (1LL << 30) || d->height > (1LL << 22) || d->n_planes > 65535) return SATGB_ERR_INVALID_ARG;
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
  a.box_pitch = d->box_pitch;
  a.box_plane = d->box_plane_stride;
  for (int i = 0; i < SATGB_MAX_RADII; ++i) {
    a.r[i] = 0;
    a.inv_full[i] = 1.0f;
    a.box[i] = nullptr;
  }
  for (int i = 0; i < d->n_radii; ++i) {
    if (d->radius[i] < 0 || !d->d_box[i]) return SATGB_ERR_INVALID_ARG;
    if (((uintptr_t)d->d_box[i] % 4) != 0) return SATGB_ERR_MISALIGNED;
    a.r[i] = d->radius[i];
    a.inv_full[i] = 1.0f / (float)(2 * (double)d->radius[i] + 1);
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
  box_fwd_kernel<<<grid, dim3(kBX, kBY), 0, (cudaStream_t)stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return satgb::api_cuda_fail(e, "box_fwd_kernel launch");
  satgb::api_count_launch();
  return SATGB_OK;
}

extern "C" satgb_status satgb_box_filter_bwd(const satgb_box_desc* d, satgb_stream stream) {
  BoxArgs a;
  satgb_status st = check_desc(d, a);
  if (st != SATGB_OK || d->width == 0 || d->height == 0 || d->n_planes == 0) return st;
  dim3 grid((unsigned)((d->width + kBX - 1) / kBX), (unsigned)((d->height + kBY * kRows - 1) / (kBY * kRows)),
            (unsigned)d->n_planes);
  box_bwd_kernel<<<grid, dim3(kBX, kBY), 0, (cudaStream_t)stream>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return satgb::api_cuda_fail(e, "box_bwd_kernel launch");
  satgb::api_count_launch();
  return SATGB_OK;
}
