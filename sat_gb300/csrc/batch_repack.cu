// batch_repack.cu -- staging of inputs whose rows TMA cannot address.
//
// A tensor map needs a 16-byte aligned base and a row pitch of whole 16-byte
// chunks.  Images packed row after row (a pitch of width elements, e.g. u8
// images of odd widths) have neither, and the tile kernels would read them
// with plain loads on their compute warps.  A batch plan instead copies such
// inputs, at each execution and inside the same graph, into rows padded to 16
// bytes in a staging buffer of its own, and runs the tile kernels on the
// copies through TMA; a single large image with 1-byte inputs is staged the
// same way in its call's workspace (repack_launch_one).
//
// One warp per row, rows of all the staged images in one launch (a job per
// image, found by binary search over the jobs' first rows).  A lane writes
// 16-byte chunks of the padded row; each is assembled from the five aligned
// 4-byte words that cover the 16 unaligned source bytes (a funnel shift by
// the source's misalignment).  Only words holding at least one byte of the
// row are read: an aligned word never straddles a page, so no read leaves the
// caller's buffer's pages, and the words past the row's end count as zeros
// (they land in the padding, which no kernel reads).
#include <cuda_runtime.h>

#include <cstdint>

#include "batch_repack.h"

namespace satgb {
satgb_status api_cuda_fail(cudaError_t e, const char* what);
void api_count_launch();

namespace {

constexpr int kRepackWarps = 8;

// one row of a job, by a whole warp
__device__ __forceinline__ void repack_row(const RepackJob& J, long long y, int lane) {
  const unsigned char* src = J.src + y * J.src_pitch;
  const unsigned char* end = src + J.row_bytes;
  uint4* dst = reinterpret_cast<uint4*>(J.dst + y * J.dst_pitch);
  const long long nchunks = (J.row_bytes + 15) / 16;
  for (long long c = lane; c < nchunks; c += 32) {
    const unsigned char* p = src + 16 * c;
    const uintptr_t a = (uintptr_t)p & ~(uintptr_t)3;
    const unsigned sh = (unsigned)((uintptr_t)p & 3) * 8;
    uint32_t w[5];
#pragma unroll
    for (int i = 0; i < 5; ++i) {
      const unsigned char* q = reinterpret_cast<const unsigned char*>(a + 4 * i);
      w[i] = q < end ? __ldcs(reinterpret_cast<const unsigned int*>(q)) : 0u;
    }
    uint4 o;
    o.x = __funnelshift_r(w[0], w[1], sh);
    o.y = __funnelshift_r(w[1], w[2], sh);
    o.z = __funnelshift_r(w[2], w[3], sh);
    o.w = __funnelshift_r(w[3], w[4], sh);
    dst[c] = o;
  }
}

__global__ void __launch_bounds__(kRepackWarps * 32) repack_kernel(const RepackJob* __restrict__ jobs, int n_jobs,
                                                                   long long n_rows) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * kRepackWarps;
  for (long long rr = (long long)blockIdx.x * kRepackWarps + (threadIdx.x >> 5); rr < n_rows; rr += nwarps) {
    int lo = 0, hi = n_jobs - 1; // the last job whose first row is <= rr
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].row_base <= rr) lo = mid;
      else hi = mid - 1;
    }
    repack_row(jobs[lo], rr - jobs[lo].row_base, lane);
  }
}

// a single image's rows, the job passed by value
__global__ void __launch_bounds__(kRepackWarps * 32) repack_one_kernel(const __grid_constant__ RepackJob J,
                                                                       long long n_rows) {
  const int lane = threadIdx.x & 31;
  const long long nwarps = (long long)gridDim.x * kRepackWarps;
  for (long long y = (long long)blockIdx.x * kRepackWarps + (threadIdx.x >> 5); y < n_rows; y += nwarps)
    repack_row(J, y, lane);
}

}  // namespace

namespace {
unsigned repack_grid(long long n_rows, int sms) {
  const long long want = (n_rows + kRepackWarps - 1) / kRepackWarps;
  const long long cap = 8LL * (sms > 0 ? sms : 1);
  return (unsigned)(want < cap ? want : cap);
}
}  // namespace

satgb_status repack_launch(const RepackJob* jobs_dev, int n_jobs, long long n_rows, int sms, cudaStream_t s) {
  if (n_jobs <= 0 || n_rows <= 0) return SATGB_OK;
  repack_kernel<<<repack_grid(n_rows, sms), kRepackWarps * 32, 0, s>>>(jobs_dev, n_jobs, n_rows);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_cuda_fail(e, "repack_kernel launch");
  api_count_launch();
  return SATGB_OK;
}

satgb_status repack_launch_one(const RepackJob& job, long long n_rows, int sms, cudaStream_t s) {
  if (n_rows <= 0) return SATGB_OK;
  repack_one_kernel<<<repack_grid(n_rows, sms), kRepackWarps * 32, 0, s>>>(job, n_rows);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return api_cuda_fail(e, "repack_one_kernel launch");
  api_count_launch();
  return SATGB_OK;
}

}  // namespace satgb
