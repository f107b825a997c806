// satgb_noalloc.cu -- satgb_sat_noalloc(): the single-image SAT for callers
// that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not an option -- inside a
// custom allocator or memory-pool callback (allocating would re-enter it), in
// a process whose device memory is fully reserved up front by a framework
// that forbids other allocations, or in a latency-critical loop where an
// allocation (and the device-wide synchronisation cudaFree implies) is not
// acceptable.  The other entry points allocate their look-back workspace on
// first use; this one never does.
//
// How: the look-back scratch (a 64-byte header with the tile ticket, the
// finished-CTA count, the launch epoch and an error word, followed by the
// status words of the tiles) lives in the file-scope array below.  Every GPU
// that loads libsatgb.so holds these kSatgbNoallocBytes bytes until the
// process exits.  Host code cannot use the array's name as a device address
// (in host code it names a host-side shadow), so the first call on each
// device, with that device current, asks the runtime for the device address
// with cudaGetSymbolAddress and caches it; that first call should therefore
// come before any stream capture.
//
// All calls share the one array: calls whose kernels overlap on the GPU (on
// different streams, or from different host threads) race on it and give
// wrong results.  The array keeps the last call's contents; before each launch
// the ticket, CTA count and the running launch's error word are cleared with
// cudaMemsetAsync (not an allocation), while the epoch and status words are
// kept on purpose: the kernel tags every status word with the launch epoch,
// so old contents never read as valid.
//
// Argument and CUDA failures are reported like those of every other entry
// point (a status, and the message in satgb_last_error_string), and each
// launch is counted by satgb_launch_count.  A look-back wait that gives up
// records an error in the array's header, but this entry point cannot report
// it without a synchronising read; callers that need device-side error
// reporting use satgb_sat_ex with satgb_stream_check.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/satgb.h"
#include "sat_kernel.cuh"
#include "sat_registry.h"

namespace satgb {
satgb_status api_fail(satgb_status st, const char* msg);
void api_count_launch();
}  // namespace satgb

namespace {

constexpr size_t kSatgbNoallocBytes = 16u << 20; // 16 MiB
constexpr int kNoallocConfig = 1;                // the largest tiles: least scratch per pixel
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kSatgbNoallocBytes];

std::mutex g_noalloc_mu;
void* g_noalloc_ptr[kMaxDevices] = {};
int g_noalloc_grid_sms[kMaxDevices] = {};

// Failures go to the library's error channel (satgb_last_error_string), like
// those of every other entry point.
satgb_status noalloc_fail(satgb_status st, const std::string& msg) {
  return satgb::api_fail(st, ("satgb_sat_noalloc: " + msg).c_str());
}

size_t elem_size(int t) {
  switch (t) {
    case SATGB_U8:
    case SATGB_I8: return 1;
    case SATGB_U32:
    case SATGB_I32:
    case SATGB_F32: return 4;
    case SATGB_F64: return 8;
    default: return 0;
  }
}

}  // namespace

extern "C" satgb_status satgb_sat_noalloc(const satgb_sat_desc* d, satgb_stream stream) {
  using namespace satgb;
  if (!d) return noalloc_fail(SATGB_ERR_INVALID_ARG, "null descriptor");
  const size_t in_sz = elem_size(d->in_t), out_sz = elem_size(d->out_t);
  if (!in_sz || !out_sz) return noalloc_fail(SATGB_ERR_UNSUPPORTED_TYPES, "dtype pair not offered");
  if (d->direction != SATGB_FORWARD && d->direction != SATGB_REVERSE)
    return noalloc_fail(SATGB_ERR_INVALID_ARG, "unknown direction");
  if (d->mode != SATGB_MODE_PLAIN && d->mode != SATGB_MODE_COMPENSATED)
    return noalloc_fail(SATGB_ERR_INVALID_ARG, "unknown mode");
  const Variant* v = find_variant(d->in_t, d->out_t, d->mode, d->direction, kNoallocConfig);
  if (!v) return noalloc_fail(SATGB_ERR_UNSUPPORTED_TYPES, "dtype pair / mode not offered");
  if (d->width < 0 || d->height < 0) return noalloc_fail(SATGB_ERR_INVALID_ARG, "negative width/height");
  if (d->width == 0 || d->height == 0) return SATGB_OK;
  if (!d->d_in || !d->d_out) return noalloc_fail(SATGB_ERR_INVALID_ARG, "null buffer");
  if (d->in_pitch < d->width || d->out_pitch < d->width)
    return noalloc_fail(SATGB_ERR_INVALID_ARG, "pitch smaller than width");
  if (((uintptr_t)d->d_in % in_sz) != 0 || ((uintptr_t)d->d_out % out_sz) != 0)
    return noalloc_fail(SATGB_ERR_MISALIGNED, "buffer not aligned to its element size");
  const long long lim = INT64_MAX / 16;
  if (d->height > lim / d->in_pitch || d->height > lim / d->out_pitch)
    return noalloc_fail(SATGB_ERR_OVERFLOW, "image extent overflows 64-bit byte offsets");
  {
    // same buffer (in place) or disjoint, as for the other entry points
    const char* ib = (const char*)d->d_in;
    const char* ie = ib + ((d->height - 1) * d->in_pitch + d->width) * (long long)in_sz;
    const char* ob = (const char*)d->d_out;
    const char* oe = ob + ((d->height - 1) * d->out_pitch + d->width) * (long long)out_sz;
    const bool same = ib == ob && in_sz == out_sz && d->in_pitch == d->out_pitch;
    if (!same && ib < oe && ob < ie) return noalloc_fail(SATGB_ERR_INVALID_ARG, "input and output overlap");
  }

  // the scratch this image needs, against the array's fixed size
  const long long ntx = (d->width + v->TW - 1) / v->TW;
  const long long nty = (d->height + v->TH - 1) / v->TH;
  const long long n_tiles = ntx * nty;
  const size_t w8 = sizeof(unsigned long long);
  const size_t row_off = sizeof(WsHeader);
  const size_t col_off = row_off + (size_t)n_tiles * v->TH * v->K * w8;
  const size_t corner_off = col_off + (size_t)n_tiles * v->TW * v->K * w8;
  const size_t need = corner_off + (size_t)n_tiles * v->K * w8;
  if (ntx > INT32_MAX || nty > INT32_MAX || need > kSatgbNoallocBytes) {
    char buf[256];
    std::snprintf(buf, sizeof buf,
                  "a %lld x %lld image needs %zu bytes of look-back scratch; the fixed scratch array holds %zu",
                  (long long)d->width, (long long)d->height, need, kSatgbNoallocBytes);
    return noalloc_fail(SATGB_ERR_INVALID_ARG, buf);
  }

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return noalloc_fail(SATGB_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return noalloc_fail(SATGB_ERR_CUDA, "device ordinal " + std::to_string(dev) + " is beyond the " +
                                            std::to_string(kMaxDevices) + " devices this entry point keeps scratch addresses for");
  void* base = nullptr;
  int sms = 0;
  {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
      // set-up, once per device, with that device current
      void* p = nullptr;
      e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p)
        return noalloc_fail(SATGB_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      e = cudaDeviceGetAttribute(&g_noalloc_grid_sms[dev], cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess)
        return noalloc_fail(SATGB_ERR_CUDA, std::string("cudaDeviceGetAttribute: ") + cudaGetErrorString(e));
      g_noalloc_ptr[dev] = p;
    }
    base = g_noalloc_ptr[dev];
    sms = g_noalloc_grid_sms[dev];
  }
  int occ = 1;
  e = v->prepare();
  if (e != cudaSuccess) return noalloc_fail(SATGB_ERR_CUDA, std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e));
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, v->kernel, v->threads, v->dyn_smem);
  if (e != cudaSuccess) return noalloc_fail(SATGB_ERR_CUDA, std::string("occupancy query: ") + cudaGetErrorString(e));
  if (occ < 1) occ = 1;
  const int grid = (int)std::max(1LL, std::min((long long)sms * occ, n_tiles));

  cudaStream_t s = (cudaStream_t)stream;
  // ticket, finished-CTA count and error word start at zero (the epoch stays)
  e = cudaMemsetAsync(base, 0, offsetof(WsHeader, epoch), s);
  if (e == cudaSuccess) e = cudaMemsetAsync((char*)base + offsetof(WsHeader, error), 0, 2 * sizeof(uint32_t), s);
  if (e != cudaSuccess) return noalloc_fail(SATGB_ERR_CUDA, std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));

  ImageDesc img;
  fill_image_desc(img, v, d->in_t, d->out_t, d->d_in, d->d_out, d->in_pitch, d->out_pitch, d->width, d->height, 0, 1, 0, 0);

  SatParams P;
  std::memset(&P, 0, sizeof P);
  P.images = nullptr;
  P.img0 = img;
  P.n_images = 1;
  P.n_tiles = n_tiles;
  char* b = (char*)base;
  P.ws = (WsHeader*)b;
  P.row_words = (unsigned long long*)(b + row_off);
  P.col_words = (unsigned long long*)(b + col_off);
  P.corner_words = (unsigned long long*)(b + corner_off);
  P.wait_limit_ns = 2000000000LL;
  P.stall_tile = -1;
  e = v->launch(P, grid, s);
  if (e != cudaSuccess) return noalloc_fail(SATGB_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  satgb::api_count_launch();
  return SATGB_OK;
}
