// satgb_api.cu -- host side of libsatgb.so: the C ABI declared in
// include/satgb.h.  Argument validation, the per-stream look-back workspace,
// kernel-variant dispatch, the autotuner, batch plans (one persistent launch
// captured in a CUDA graph) and device-error reporting.
//
// No CPU fallback exists: every SAT is computed by sat_tile_kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/satgb.h"
#include "batch_repack.h"
#include "sat_kernel.cuh"
#include "sat_registry.h"

namespace satgb {

const TileConfig kConfigs[kNumConfigs] = {
    {4, 16, "warp-specialized: 64-row tiles, one look-back thread per row and column"},
    {8, 16, "pipelined: 128-row tiles (64 for 8-byte accumulators), 16 warps"},
    {8, 8, "pipelined: 64-row tiles (32 for 8-byte accumulators), 8 warps, 2 CTAs per SM"},
    {8, 16, "registers: 128-row tiles, 16 warps"},
    {16, 16, "pipelined, 256-row tiles, direct stores (1-byte inputs, 4-byte sums)"},
    {8, 16, "warp-specialized, direct stores: 128-row tiles (64 for 8-byte accumulators)"},
    {8, 16, "warp-specialized, direct stores, row-major tile order: 128-row tiles (64 for 8-byte accumulators)"},
};

namespace {
PFN_cuTensorMapEncodeTiled_v12000 tmap_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }();
  return fn;
}

size_t elem_bytes(int t) {
  switch (t) {
    case 0: case 1: return 1;
    case 2: case 3: return 2;
    case 4: case 5: case 6: return 4;
    case 7: return 8;
    default: return 0;
  }
}
}  // namespace

namespace {
// Rank-3 tiled map (x, y, plane) with a TW x TH x 1 box; false when the
// driver rejects it (the image then uses plain loads or stores).
bool encode_map(CUtensorMap* m, int t, const void* base, int64_t width, int64_t height, int64_t pitch,
                int64_t planes, int64_t plane, int tw, int th) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tmap_encoder();
  if (!enc) return false;
  const int64_t sz = (int64_t)elem_bytes(t);
  CUtensorMapDataType dt = sz == 1 ? CU_TENSOR_MAP_DATA_TYPE_UINT8
                           : t == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32
                           : t == 5 ? CU_TENSOR_MAP_DATA_TYPE_INT32
                           : t == 6 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                    : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  cuuint64_t dims[3] = {(cuuint64_t)width, (cuuint64_t)height, (cuuint64_t)planes};
  cuuint64_t strides[2] = {(cuuint64_t)(pitch * sz), (cuuint64_t)(plane * sz)};
  cuuint32_t box[3] = {(cuuint32_t)tw, (cuuint32_t)th, 1u};
  cuuint32_t estr[3] = {1, 1, 1};
  return enc(m, dt, 3, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
             CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
             CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// TMA needs the base, the row pitch and the plane stride in multiples of 16
// bytes.  It moves whole 16-byte chunks of a row, so the map covers only the
// row's whole chunks (tma_columns); the kernel moves the rest of each row,
// fewer than 16 bytes, with plain accesses.  Other images use plain loads and
// stores throughout.
bool tma_ok(const void* base, int64_t width, int64_t height, int64_t pitch, int64_t planes, int64_t plane,
            size_t sz) {
  return ((uintptr_t)base % 16) == 0 && ((size_t)pitch * sz) % 16 == 0 && ((size_t)plane * sz) % 16 == 0 &&
         (size_t)width * sz >= 16 && width < (1LL << 32) && height < (1LL << 32) && planes < (1LL << 31);
}

int64_t tma_columns(int64_t width, size_t sz) { return (int64_t)(((size_t)width * sz / 16) * 16 / sz); }
}  // namespace

void fill_image_desc(ImageDesc& d, const Variant* v, int in_t, int out_t, const void* in, void* out,
                     int64_t in_pitch, int64_t out_pitch, int64_t width, int64_t height, int64_t tile_base,
                     int64_t planes, int64_t in_plane, int64_t out_plane) {
  std::memset(&d, 0, sizeof d);
  const size_t in_sz = elem_bytes(in_t), out_sz = elem_bytes(out_t);
  if (planes < 1) planes = 1;
  if (planes == 1) {
    // one image: any plane stride past its last element will do
    in_plane = in_pitch * height;
    out_plane = out_pitch * height;
    in_plane += (16 - (in_plane * (int64_t)in_sz) % 16) % 16 / (int64_t)in_sz;
    out_plane += (16 - (out_plane * (int64_t)out_sz) % 16) % 16 / (int64_t)out_sz;
  }
  d.in = in;
  d.out = out;
  d.in_pitch = in_pitch;
  d.out_pitch = out_pitch;
  d.width = width;
  d.height = height;
  d.planes = planes;
  d.in_plane = in_plane;
  d.out_plane = out_plane;
  d.tile_base = tile_base;
  d.ntx = (int32_t)((width + v->TW - 1) / v->TW);
  d.nty = (int32_t)((height + v->TH - 1) / v->TH);
  d.tiles_per_plane = (int64_t)d.ntx * d.nty;
  const int cpt = v->TW / 32;
  const size_t seg_in = (size_t)cpt * in_sz;
  uint32_t flags = 0;
  if (((uintptr_t)in % seg_in) == 0 && ((size_t)in_pitch * in_sz) % seg_in == 0 &&
      ((size_t)in_plane * in_sz) % seg_in == 0)
    flags |= kInVec;
  if (((uintptr_t)out % 16) == 0 && ((size_t)out_pitch * out_sz) % 16 == 0 && ((size_t)out_plane * out_sz) % 16 == 0)
    flags |= kOutVec;
  d.tma_in_w = tma_columns(width, in_sz);
  d.tma_out_w = tma_columns(width, out_sz);
  if (tma_ok(in, width, height, in_pitch, planes, in_plane, in_sz) &&
      encode_map(&d.tmap_in, in_t, in, d.tma_in_w, height, in_pitch, planes, in_plane, v->TW, v->TH))
    flags |= kInTma;
  if (tma_ok(out, width, height, out_pitch, planes, out_plane, out_sz) &&
      encode_map(&d.tmap_out, out_t, out, d.tma_out_w, height, out_pitch, planes, out_plane, v->TW, v->TH))
    flags |= kOutTma;
  d.flags = flags;
}

const Variant* find_variant(int in_t, int out_t, int mode, int dir, int cfg) {
  using ListFn = const Variant* (*)(int*);
  static const ListFn lists[] = {variants_u8, variants_i8, variants_int32, variants_f32, variants_f64};
  for (ListFn f : lists) {
    int n = 0;
    const Variant* v = f(&n);
    for (int i = 0; i < n; ++i)
      if (v[i].in_t == in_t && v[i].out_t == out_t && v[i].mode == mode && v[i].dir == dir && v[i].cfg == cfg)
        return &v[i];
  }
  return nullptr;
}

}  // namespace satgb

using namespace satgb;

namespace {

thread_local std::string g_last_error;
std::mutex g_mu;                      // guards every map below
std::atomic<long long> g_launches{0}; // kernel launches issued
std::atomic<long long> g_wait_limit_ns{2000000000LL};
std::atomic<long long> g_stall_tile{-1};
int g_forced_config = -1;
satgb_alloc_fn g_alloc = nullptr;
satgb_free_fn g_free = nullptr;
void* g_alloc_ctx = nullptr;

satgb_status fail(satgb_status st, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return st;
}

satgb_status cuda_fail(cudaError_t e, const char* what) {
  return fail(SATGB_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

void* ws_alloc(size_t bytes) {
  if (g_alloc) return g_alloc(bytes, g_alloc_ctx);
  void* p = nullptr;
  if (cudaMalloc(&p, bytes) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return p;
}

void ws_free(void* p) {
  if (!p) return;
  if (g_free) g_free(p, g_alloc_ctx);
  else cudaFree(p);
}

size_t dtype_size(int t) {
  switch (t) {
    case SATGB_U8:
    case SATGB_I8: return 1;
    case SATGB_U16:
    case SATGB_I16: return 2;
    case SATGB_U32:
    case SATGB_I32:
    case SATGB_F32: return 4;
    case SATGB_F64: return 8;
    default: return 0;
  }
}

const char* dtype_name(int t) {
  static const char* names[] = {"u8", "i8", "u16", "i16", "u32", "i32", "f32", "f64"};
  return (t >= 0 && t < 8) ? names[t] : "?";
}

// One look-back workspace: a header block followed by the three status arrays.
struct Workspace {
  void* base = nullptr;
  size_t bytes = 0;
};

struct Layout {
  size_t row_off, col_off, corner_off, total;
};

Layout layout_for(long long n_tiles, const Variant* v) {
  Layout L;
  const size_t w = sizeof(unsigned long long);
  L.row_off = sizeof(WsHeader);
  L.col_off = L.row_off + (size_t)n_tiles * v->TH * v->K * w;
  L.corner_off = L.col_off + (size_t)n_tiles * v->TW * v->K * w;
  L.total = L.corner_off + (size_t)n_tiles * v->K * w;
  return L;
}

// Single-image calls stage 1-byte inputs that TMA cannot address from this
// many pixels up (u8 -> u32 1023^2: 18.7 us read in place, 15 us for the
// aligned SAT alone, so the extra launch would not pay).
constexpr long long kStageMinPixels = 1LL << 22;

// Workspaces of single-image calls, one per (device, stream).
std::map<std::pair<int, void*>, Workspace> g_ws;

satgb_status get_device(int* dev) {
  cudaError_t e = cudaGetDevice(dev);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return cuda_fail(e, "cudaGetDevice");
  }
  return SATGB_OK;
}

// Makes sure ws holds at least `bytes`; called with g_mu held.
satgb_status ensure_ws(Workspace& ws, size_t bytes, cudaStream_t s) {
  if (ws.bytes >= bytes) return SATGB_OK;
  bytes = std::max(bytes, ws.bytes + ws.bytes / 2);
  bytes = (bytes + 4095) & ~(size_t)4095;
  if (ws.base) {
    cudaError_t e = cudaStreamSynchronize(s); // earlier calls may still use it
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    ws_free(ws.base);
    ws.base = nullptr;
    ws.bytes = 0;
  }
  void* p = ws_alloc(bytes);
  if (!p) return fail(SATGB_ERR_ALLOC, "workspace allocation of %zu bytes failed", bytes);
  cudaError_t e = cudaMemsetAsync(p, 0, bytes, s);
  if (e != cudaSuccess) {
    ws_free(p);
    return cuda_fail(e, "cudaMemsetAsync");
  }
  ws.base = p;
  ws.bytes = bytes;
  return SATGB_OK;
}

struct DevInfo {
  int sms = 0;
};

// descriptor cache of sat_single (guarded by g_mu)
struct DescKey {
  const Variant* v;
  int in_t, out_t;
  const void* in;
  const void* out;
  long long in_pitch, out_pitch, width, height, planes, in_plane, out_plane;
  bool operator<(const DescKey& o) const {
    return std::tie(v, in_t, out_t, in, out, in_pitch, out_pitch, width, height, planes, in_plane, out_plane) <
           std::tie(o.v, o.in_t, o.out_t, o.in, o.out, o.in_pitch, o.out_pitch, o.width, o.height, o.planes,
                    o.in_plane, o.out_plane);
  }
};
std::map<DescKey, ImageDesc> g_desc_cache;
std::map<int, DevInfo> g_dev;
std::map<std::pair<int, const void*>, int> g_occ; // (device, kernel) -> CTAs per SM

satgb_status grid_for(int dev, const Variant* v, long long n_tiles, int* grid) {
  auto it = g_dev.find(dev);
  if (it == g_dev.end()) {
    DevInfo d;
    cudaError_t e = cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
    it = g_dev.emplace(dev, d).first;
  }
  auto key = std::make_pair(dev, v->kernel);
  auto jt = g_occ.find(key);
  if (jt == g_occ.end()) {
    int occ = 0;
    cudaError_t e = v->prepare();
    if (e != cudaSuccess) return cuda_fail(e, "cudaFuncSetAttribute");
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, v->kernel, v->threads, v->dyn_smem);
    if (e != cudaSuccess) return cuda_fail(e, "cudaOccupancyMaxActiveBlocksPerMultiprocessor");
    if (occ < 1) occ = 1;
    jt = g_occ.emplace(key, occ).first;
  }
  long long g = (long long)it->second.sms * jt->second;
  *grid = (int)std::max(1LL, std::min(g, n_tiles));
  return SATGB_OK;
}

bool pair_offered(int in_t, int out_t, int mode) {
  // satgb_scanrow_brlt & co. offer the reference's dispatched pairs.
  for (int cfg = 0; cfg < kNumConfigs; ++cfg)
    if (find_variant(in_t, out_t, mode, 0, cfg)) return true;
  return false;
}

struct ImgCheck {
  const void* in;
  void* out;
  long long in_pitch, out_pitch, width, height;
};

satgb_status validate_image(const ImgCheck& c, size_t in_sz, size_t out_sz) {
  if (c.width < 0 || c.height < 0) return fail(SATGB_ERR_INVALID_ARG, "negative width/height (%lld x %lld)", c.width, c.height);
  if (c.width == 0 || c.height == 0) return SATGB_OK; // empty image: nothing to do
  if (!c.in || !c.out) return fail(SATGB_ERR_INVALID_ARG, "null buffer");
  if (c.in_pitch < c.width || c.out_pitch < c.width)
    return fail(SATGB_ERR_INVALID_ARG, "pitch (%lld in, %lld out elements) smaller than width %lld", c.in_pitch, c.out_pitch, c.width);
  if (((uintptr_t)c.in % in_sz) != 0 || ((uintptr_t)c.out % out_sz) != 0)
    return fail(SATGB_ERR_MISALIGNED, "buffer not aligned to its element size");
  // (height-1)*pitch + width elements must fit in int64 bytes
  const long long lim = INT64_MAX / 16;
  if (c.height > lim / std::max(1LL, c.in_pitch) || c.height > lim / std::max(1LL, c.out_pitch))
    return fail(SATGB_ERR_OVERFLOW, "image extent overflows 64-bit byte offsets");
  // the input and output must be the same buffer or disjoint
  const char* ib = (const char*)c.in;
  const char* ie = ib + ((c.height - 1) * c.in_pitch + c.width) * (long long)in_sz;
  const char* ob = (const char*)c.out;
  const char* oe = ob + ((c.height - 1) * c.out_pitch + c.width) * (long long)out_sz;
  const bool same = ib == ob && in_sz == out_sz && c.in_pitch == c.out_pitch;
  if (!same && ib < oe && ob < ie) return fail(SATGB_ERR_INVALID_ARG, "input and output overlap without being the same buffer");
  return SATGB_OK;
}

// The images of one batch run concurrently in one launch, so no image may
// write memory another image reads or writes.  Inputs may be shared (they are
// only read); an image computed in place is one output range.  Ranges are the
// byte extents from the first to the last element; two ranges of images with
// the same row pitch whose rows fall into disjoint columns of that pitch (side
// by side in one pitched buffer) do not touch each other and pass.  Sorting by
// start and keeping the open ranges makes the check O(n log n) unless many
// ranges overlap (then it compares each new range with every open one).
struct ByteRange {
  uintptr_t b, e; // [b, e)
  uint64_t pitch, row;
  size_t img;
  bool out;
};

bool ranges_touch(const ByteRange& x, const ByteRange& y) {
  if (x.e <= y.b || y.e <= x.b) return false;
  if (x.pitch != y.pitch || x.pitch == 0) return true;
  // same pitch: the columns of each modulo the pitch, on a circle of length pitch
  const uint64_t P = x.pitch;
  const uint64_t a = ((uint64_t)(y.b % P) + P - (uint64_t)(x.b % P)) % P; // y's start relative to x's
  return a < x.row || a + y.row > P;
}

satgb_status check_batch_disjoint(const std::vector<ImgCheck>& imgs, size_t in_sz, size_t out_sz) {
  std::vector<ByteRange> r;
  r.reserve(2 * imgs.size());
  for (size_t i = 0; i < imgs.size(); ++i) {
    const ImgCheck& c = imgs[i];
    const uintptr_t ib = (uintptr_t)c.in, ob = (uintptr_t)c.out;
    const uintptr_t ie = ib + (uintptr_t)(((c.height - 1) * c.in_pitch + c.width) * (long long)in_sz);
    const uintptr_t oe = ob + (uintptr_t)(((c.height - 1) * c.out_pitch + c.width) * (long long)out_sz);
    const bool same = ib == ob && in_sz == out_sz && c.in_pitch == c.out_pitch;
    const uint64_t ip = c.height > 1 ? (uint64_t)c.in_pitch * in_sz : 0, op = c.height > 1 ? (uint64_t)c.out_pitch * out_sz : 0;
    if (!same) r.push_back({ib, ie, ip, (uint64_t)c.width * in_sz, i, false});
    r.push_back({ob, oe, op, (uint64_t)c.width * out_sz, i, true});
  }
  std::sort(r.begin(), r.end(), [](const ByteRange& x, const ByteRange& y) { return x.b < y.b; });
  std::vector<const ByteRange*> open;
  for (const ByteRange& x : r) {
    size_t k = 0;
    for (size_t j = 0; j < open.size(); ++j)
      if (open[j]->e > x.b) open[k++] = open[j];
    open.resize(k);
    for (const ByteRange* y : open)
      if ((x.out || y->out) && x.img != y->img && ranges_touch(*y, x))
        return fail(SATGB_ERR_INVALID_ARG, "images %zu and %zu of the batch overlap (one writes memory the other uses)",
                    std::min(x.img, y->img), std::max(x.img, y->img));
    open.push_back(&x);
  }
  return SATGB_OK;
}

// ----------------------------------------------------------------------------
// tuning table: (in, out, mode, dir, log2 w bucket, log2 h bucket, SMs) -> cfg
// ----------------------------------------------------------------------------
using TuneKey = std::tuple<int, int, int, int, int, int, int>;
std::map<TuneKey, int> g_tune;
// batch plans: (in, out, mode, dir, size class, log2 pixels, log2 images, all rows TMA-able, SMs) -> cfg
using BatchKey = std::tuple<int, int, int, int, int, int, int, int, int>;
std::map<BatchKey, int> g_batch_tune;
bool g_tune_loaded = false;

int log2_bucket(long long x) {
  int b = 0;
  while ((1LL << b) < x && b < 62) ++b;
  return b;
}

void tune_load_locked() {
  if (g_tune_loaded) return;
  g_tune_loaded = true;
  const char* path = getenv("SATGB_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "r");
  if (!f) return;
  // one entry per line: {"in":0,"out":4,"mode":0,"dir":0,"wb":13,"hb":13,"sms":152,"cfg":1}
  char line[512];
  while (fgets(line, sizeof line, f)) {
    int a[8];
    int b[10];
    if (sscanf(line, " {\"in\":%d,\"out\":%d,\"mode\":%d,\"dir\":%d,\"wb\":%d,\"hb\":%d,\"sms\":%d,\"cfg\":%d}",
               &a[0], &a[1], &a[2], &a[3], &a[4], &a[5], &a[6], &a[7]) == 8)
      g_tune[TuneKey(a[0], a[1], a[2], a[3], a[4], a[5], a[6])] = a[7];
    else if (sscanf(line,
                    " {\"batch_in\":%d,\"out\":%d,\"mode\":%d,\"dir\":%d,\"class\":%d,\"pxb\":%d,\"nb\":%d,"
                    "\"tma\":%d,\"sms\":%d,\"cfg\":%d}",
                    &b[0], &b[1], &b[2], &b[3], &b[4], &b[5], &b[6], &b[7], &b[8], &b[9]) == 10)
      g_batch_tune[BatchKey(b[0], b[1], b[2], b[3], b[4], b[5], b[6], b[7], b[8])] = b[9];
  }
  fclose(f);
}

void tune_save_locked() {
  const char* path = getenv("SATGB_TUNE_CACHE");
  if (!path) return;
  FILE* f = fopen(path, "w");
  if (!f) return;
  for (auto& kv : g_tune) {
    const TuneKey& k = kv.first;
    fprintf(f, "{\"in\":%d,\"out\":%d,\"mode\":%d,\"dir\":%d,\"wb\":%d,\"hb\":%d,\"sms\":%d,\"cfg\":%d}\n",
            std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), std::get<4>(k), std::get<5>(k),
            std::get<6>(k), kv.second);
  }
  for (auto& kv : g_batch_tune) {
    const BatchKey& k = kv.first;
    fprintf(f,
            "{\"batch_in\":%d,\"out\":%d,\"mode\":%d,\"dir\":%d,\"class\":%d,\"pxb\":%d,\"nb\":%d,"
            "\"tma\":%d,\"sms\":%d,\"cfg\":%d}\n",
            std::get<0>(k), std::get<1>(k), std::get<2>(k), std::get<3>(k), std::get<4>(k), std::get<5>(k),
            std::get<6>(k), std::get<7>(k), std::get<8>(k), kv.second);
  }
  fclose(f);
}

int sms_of(int dev) {
  auto it = g_dev.find(dev);
  if (it != g_dev.end()) return it->second.sms;
  DevInfo d;
  if (cudaDeviceGetAttribute(&d.sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  g_dev.emplace(dev, d);
  return d.sms;
}

// Heuristic default when no tuning entry exists, from measurements on GB300
// (CUDA events, square images 1024^2 .. 32768^2):
// 4-byte accumulators: the warp-specialized direct-store tiles (configuration
// 5) once there are at least 4 tiles of 128 x 128 per SM (f32: 2959 vs 2851
// GB/s at 4096^2, 4521 vs 3893 at 8192^2, 5510 vs 4370 at 16384^2), else the
// 128-row pipelined tiles (1494 vs 1369 GB/s at 2048^2).
// 1-byte inputs with 4-byte sums: configuration 5 from 16 tiles per SM (3185
// vs 3093 GB/s at 8192^2, 4022 vs 3518 at 16384^2, 4358 vs 3621 at 32768^2),
// the 256-row direct-store tiles below that (2159 vs 2051 at 4096^2).
// Compensated f32: the 128-row register tiles (2474 vs 1570 GB/s for
// configuration 5 at 8192^2, 1096 vs 911 for the 64-row tiles at 2048^2).
// f64 outputs (slow FP64 adds on GB300): the warp-specialized tiles, whose
// compute warps never wait at a CTA barrier.
// Stacks of planes count all their tiles for the size classes, but
// configuration 5 needs its tile count in one plane: its gain is in long
// look-back chains, and stacks of small planes (64 x 3 planes of 1024^2, the
// box-filter layer) ran 15 % slower with it than with the pipelined tiles.
int default_config(long long width, long long height, int sms, int in_sz, int out_sz, bool compensated,
                   long long planes = 1) {
  const int cpt = 16 / out_sz;
  const long long tw = 32LL * cpt;
  const long long ntx = (width + tw - 1) / tw;
  const long long plane_tiles = ntx * ((height + 127) / 128);
  const long long tiles128 = plane_tiles * std::max(1LL, planes);
  sms = std::max(1, sms);
  if (out_sz == 8) return tiles128 >= 8LL * sms ? 0 : 2;
  if (compensated) return tiles128 >= sms ? 3 : 2;
  // Small single images: the row-major kernel (configuration 6), whose short
  // tile rows make its sums over the row aggregates cheap (f32 1536^2 17.8 ->
  // 14.9 us, 2048^2 21.2 -> 19.1, 3072^2 29.3 -> 27.7; u8 -> u32 1024^2 15.2 ->
  // 12.9); stacks of small planes stay on configuration 1.
  const bool single = planes <= 1;
  if (in_sz == 1) {
    if (plane_tiles >= 16LL * sms) return 5;
    if (single && plane_tiles < 3LL * sms) return 6;
    if (ntx * ((height + 255) / 256) * std::max(1LL, planes) >= 64) return 4;
    return single ? 6 : 1;
  }
  if (plane_tiles >= 4LL * sms) return 5;
  return single ? 6 : 1;
}

int choose_config_locked(int in_t, int out_t, int mode, int dir, long long w, long long h, int dev,
                         long long planes = 1) {
  if (g_forced_config >= 0) return g_forced_config;
  tune_load_locked();
  const int sms = sms_of(dev);
  auto it = g_tune.find(TuneKey(in_t, out_t, mode, dir, log2_bucket(w), log2_bucket(h * std::max(1LL, planes)), sms));
  if (it != g_tune.end()) return it->second;
  return default_config(w, h, sms, (int)dtype_size(in_t), (int)dtype_size(out_t), mode == SATGB_MODE_COMPENSATED,
                        planes);
}

satgb_status launch_locked(const Variant* v, const ImageDesc* table_dev, const ImageDesc& img0,
                           long long n_images, long long n_tiles, Workspace& ws, int dev,
                           cudaStream_t s, const unsigned long long* order = nullptr) {
  const Layout L = layout_for(n_tiles, v);
  satgb_status st = ensure_ws(ws, L.total, s);
  if (st != SATGB_OK) return st;
  int grid = 0;
  st = grid_for(dev, v, n_tiles, &grid);
  if (st != SATGB_OK) return st;
  SatParams P;
  std::memset(&P, 0, sizeof P);
  P.images = table_dev;
  P.img0 = img0;
  P.n_images = n_images;
  P.n_tiles = n_tiles;
  char* b = (char*)ws.base;
  P.ws = (WsHeader*)b;
  P.row_words = (unsigned long long*)(b + L.row_off);
  P.col_words = (unsigned long long*)(b + L.col_off);
  P.corner_words = (unsigned long long*)(b + L.corner_off);
  P.wait_limit_ns = g_wait_limit_ns.load();
  P.stall_tile = g_stall_tile.load();
  P.order = order;

  cudaError_t e = v->launch(P, grid, s);
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  g_launches.fetch_add(1);
  return SATGB_OK;
}

// internal modes of the variant table: the row-only and column-only scans
constexpr int kModeRows = 2;
}  // namespace
namespace satgb {
satgb_status scan_rows_strips(int in_t, int out_t, const void* d_in, int64_t in_pitch, int64_t in_plane, void* d_out,
                              int64_t out_pitch, int64_t out_plane, int64_t width, int64_t height, int64_t planes,
                              cudaStream_t s);
}  // namespace satgb
namespace {
constexpr int kModeCols = 3;

satgb_status sat_single(int in_t, int out_t, int mode, int dir, const void* d_in, long long in_pitch,
                        void* d_out, long long out_pitch, long long width, long long height,
                        cudaStream_t s, int force_cfg, long long planes = 1, long long in_plane = 0,
                        long long out_plane = 0) {
  const size_t in_sz = dtype_size(in_t), out_sz = dtype_size(out_t);
  if (!in_sz || !out_sz) return fail(SATGB_ERR_INVALID_ARG, "unknown dtype code (%d, %d)", in_t, out_t);
  if (mode != SATGB_MODE_PLAIN && mode != SATGB_MODE_COMPENSATED && mode != kModeRows && mode != kModeCols)
    return fail(SATGB_ERR_INVALID_ARG, "unknown mode %d", mode);
  if (dir != SATGB_FORWARD && dir != SATGB_REVERSE) return fail(SATGB_ERR_INVALID_ARG, "unknown direction %d", dir);
  // the row-only scan (its own kernel) offers the plain SAT's pairs
  if (!pair_offered(in_t, out_t, mode == kModeRows ? (int)SATGB_MODE_PLAIN : mode))
    return fail(SATGB_ERR_UNSUPPORTED_TYPES, "type pair %s -> %s%s not offered", dtype_name(in_t), dtype_name(out_t),
                mode == SATGB_MODE_COMPENSATED ? " (compensated)" : "");
  if (planes < 0) return fail(SATGB_ERR_INVALID_ARG, "negative plane count");
  if (planes == 0) return SATGB_OK;
  ImgCheck c{d_in, d_out, in_pitch, out_pitch, width, height};
  satgb_status st = validate_image(c, in_sz, out_sz);
  if (st != SATGB_OK) return st;
  if (width == 0 || height == 0) return SATGB_OK;
  if (planes > 1) {
    // planes may not overlap each other; the whole stacks are the same buffer or disjoint
    const long long in_span = (height - 1) * in_pitch + width, out_span = (height - 1) * out_pitch + width;
    if (in_plane < in_span || out_plane < out_span)
      return fail(SATGB_ERR_INVALID_ARG, "plane stride smaller than a plane (%lld in, %lld out)", in_plane, out_plane);
    const long long lim = INT64_MAX / 16;
    if (planes > lim / in_plane || planes > lim / out_plane) return fail(SATGB_ERR_OVERFLOW, "plane stack overflows");
    const char* ib = (const char*)d_in;
    const char* ie = ib + ((planes - 1) * in_plane + in_span) * (long long)in_sz;
    const char* ob = (const char*)d_out;
    const char* oe = ob + ((planes - 1) * out_plane + out_span) * (long long)out_sz;
    const bool same = ib == ob && in_sz == out_sz && in_pitch == out_pitch && in_plane == out_plane;
    if (!same && ib < oe && ob < ie) return fail(SATGB_ERR_INVALID_ARG, "input and output stacks overlap");
  }

  // the row-only scan has no look-back: its own kernel (scan_rows_t.cu), no workspace
  if (mode == kModeRows && dir == SATGB_FORWARD)
    return scan_rows_strips(in_t, out_t, d_in, in_pitch, planes > 1 ? in_plane : 0, d_out, out_pitch,
                            planes > 1 ? out_plane : 0, width, height, planes, s);

  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  st = get_device(&dev);
  if (st != SATGB_OK) return st;
  int cfg = force_cfg >= 0 ? force_cfg
            : (mode >= kModeRows) ? 1
                                  : choose_config_locked(in_t, out_t, mode, dir, width, height, dev, planes);
  const Variant* v = find_variant(in_t, out_t, mode, dir, cfg);
  if (!v && mode < kModeRows) // a configuration this pair does not have: the untuned choice
    v = find_variant(in_t, out_t, mode, dir,
                     default_config(width, height, sms_of(dev), (int)in_sz, (int)out_sz,
                                    mode == SATGB_MODE_COMPENSATED, planes));
  if (!v) v = find_variant(in_t, out_t, mode, dir, 0);
  if (!v) return fail(SATGB_ERR_UNSUPPORTED_TYPES, "no kernel for %s -> %s mode %d dir %d", dtype_name(in_t), dtype_name(out_t), mode, dir);
  Workspace& ws = g_ws[std::make_pair(dev, (void*)s)];
  // A large image of 1-byte inputs whose rows TMA cannot address (packed rows
  // of odd widths) is first copied into 16-byte rows behind the look-back words
  // in the workspace, and the tile kernel reads the copy through TMA: u8 -> u32
  // 8191^2 239 -> 158 us, 4095^2 68 -> 59 us.  For wider inputs the copy costs
  // more than it saves (f32 8191^2: 197 us in place against ~220 staged).
  const void* src = d_in;
  long long src_pitch = in_pitch;
  satgb::RepackJob job{};
  bool staged = false;
  if (planes == 1 && in_sz == 1 && width * height >= kStageMinPixels && width >= 16 &&
      !tma_ok(d_in, width, height, in_pitch, 1, 0, in_sz)) {
    const long long tiles = ((width + v->TW - 1) / v->TW) * ((height + v->TH - 1) / v->TH);
    const size_t look = (layout_for(tiles, v).total + 255) & ~(size_t)255;
    const size_t pitch = ((size_t)width + 15) & ~(size_t)15;
    st = ensure_ws(ws, look + pitch * (size_t)height, s);
    if (st != SATGB_OK) return st;
    job.src = static_cast<const unsigned char*>(d_in);
    job.dst = static_cast<unsigned char*>(ws.base) + look;
    job.src_pitch = in_pitch;
    job.dst_pitch = (int64_t)pitch;
    job.row_bytes = width;
    job.row_base = 0;
    src = job.dst;
    src_pitch = (long long)pitch;
    staged = true;
  }
  ImageDesc d;
  {
    // Encoding the two tensor maps costs host time comparable to a small
    // image's kernel; repeated calls on the same buffers (benchmarks, serving
    // loops) reuse the descriptor.  A map holds the buffer's address, so the key
    // is every argument of fill_image_desc.
    const DescKey key{v, in_t, out_t, src, d_out, src_pitch, out_pitch, width, height, planes, in_plane, out_plane};
    auto it = g_desc_cache.find(key);
    if (it != g_desc_cache.end()) {
      d = it->second;
    } else {
      fill_image_desc(d, v, in_t, out_t, src, d_out, src_pitch, out_pitch, width, height, 0, planes, in_plane,
                      out_plane);
      if (g_desc_cache.size() >= 64) g_desc_cache.clear();
      g_desc_cache.emplace(key, d);
    }
  }
  const long long n_tiles = (long long)d.ntx * d.nty * d.planes;
  if ((long long)d.ntx * v->TW < width || n_tiles > (1LL << 40))
    return fail(SATGB_ERR_OVERFLOW, "image too large (%lld x %lld)", width, height);
  if (staged) {
    st = repack_launch_one(job, height, sms_of(dev), s);
    if (st != SATGB_OK) return st;
  }
  return launch_locked(v, nullptr, d, 1, n_tiles, ws, dev, s);
}

}  // namespace

// ============================================================================
// Batch plans
// ============================================================================
// The images of a plan fall into two size classes, each run by its own
// persistent launch with its own tile configuration (both launches follow one
// another in the plan's CUDA graph, sharing one workspace): large images,
// whose long look-back chains favour the big warp-specialized tiles, and small
// ones, where smaller tiles or the row-major order waste less.
constexpr int kBatchClasses = 2;
constexpr long long kLargeTiles = 64; // an image of at least 64 tiles of 128 x 128 is large

struct BatchSeg {
  const Variant* v = nullptr;
  std::vector<ImgCheck> imgs;
  long long n_images = 0, n_tiles = 0;
  double pixels = 0;
  ImageDesc img0;
  ImageDesc* table = nullptr;          // device: the descriptors, then the tile order
  unsigned long long* order = nullptr; // inside the same allocation (nullptr: images one after the other)
};

struct satgb_batch_plan_s {
  int in_t = 0, out_t = 0, mode = 0, dir = 0;
  int dev = 0;
  bool all_tma = true; // every image's rows can go through TMA (16-byte aligned bases and pitches)
  // Inputs whose rows TMA cannot address are copied at each execution into
  // padded rows of `stage` (batch_repack.cu); `jobs` (device) lists them.
  void* stage = nullptr;
  satgb::RepackJob* jobs = nullptr;
  int n_jobs = 0;
  long long stage_rows = 0;
  BatchSeg seg[kBatchClasses];
  long long n_tiles = 0;
  Workspace ws;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace satgb {
// Shared with the other translation units of the library (box filters).
satgb_status api_fail(satgb_status st, const char* msg) { return fail(st, "%s", msg); }
satgb_status api_cuda_fail(cudaError_t e, const char* what) { return cuda_fail(e, what); }
void api_count_launch() { g_launches.fetch_add(1); }
}  // namespace satgb

extern "C" {

int satgb_version(void) { return SATGB_VERSION; }

const char* satgb_last_error_string(void) { return g_last_error.c_str(); }

int64_t satgb_launch_count(void) { return g_launches.load(); }

satgb_status satgb_set_wait_limit_us(int64_t us) {
  if (us <= 0) return fail(SATGB_ERR_INVALID_ARG, "wait limit must be positive");
  g_wait_limit_ns.store(us * 1000LL);
  return SATGB_OK;
}

satgb_status satgb_debug_stall_tile(int64_t tile) {
  g_stall_tile.store(tile < 0 ? -1 : tile);
  return SATGB_OK;
}

satgb_status satgb_set_allocator(satgb_alloc_fn alloc_fn, satgb_free_fn free_fn, void* ctx) {
  std::lock_guard<std::mutex> lk(g_mu);
  if ((alloc_fn == nullptr) != (free_fn == nullptr)) return fail(SATGB_ERR_INVALID_ARG, "allocator needs both functions");
  g_alloc = alloc_fn;
  g_free = free_fn;
  g_alloc_ctx = ctx;
  return SATGB_OK;
}

int satgb_num_configs(void) { return kNumConfigs; }

const char* satgb_config_name(int config) {
  return (config >= 0 && config < kNumConfigs) ? kConfigs[config].name : "";
}

satgb_status satgb_set_config(int config) {
  if (config < -1 || config >= kNumConfigs) return fail(SATGB_ERR_INVALID_ARG, "no configuration %d", config);
  std::lock_guard<std::mutex> lk(g_mu);
  g_forced_config = config;
  return SATGB_OK;
}

satgb_status satgb_scanrow_brlt(satgb_dtype in_t, satgb_dtype out_t, int scan_type, const void* d_in,
                                int64_t in_pitch, void* d_out, int64_t out_pitch, int64_t width,
                                int64_t height, satgb_stream stream) {
  if (scan_type != SATGB_SCAN_KOGGE_STONE && scan_type != SATGB_SCAN_LF)
    return fail(SATGB_ERR_INVALID_ARG, "scan_type %d is neither KoggeStone_SCAN (0) nor LF_SCAN (1)", scan_type);
  return sat_single(in_t, out_t, SATGB_MODE_PLAIN, SATGB_FORWARD, d_in, in_pitch, d_out, out_pitch, width,
                    height, (cudaStream_t)stream, -1);
}

satgb_status satgb_brlt_scanrow(satgb_dtype in_t, satgb_dtype out_t, int scan_type, const void* d_in,
                                int64_t in_pitch, void* d_out, int64_t out_pitch, int64_t width,
                                int64_t height, satgb_stream stream) {
  if (scan_type != SATGB_SCAN_KOGGE_STONE && scan_type != SATGB_SCAN_LF)
    return fail(SATGB_ERR_INVALID_ARG, "scan_type %d is neither KoggeStone_SCAN (0) nor LF_SCAN (1)", scan_type);
  return sat_single(in_t, out_t, SATGB_MODE_PLAIN, SATGB_FORWARD, d_in, in_pitch, d_out, out_pitch, width,
                    height, (cudaStream_t)stream, -1);
}

satgb_status satgb_scanrowcolumn(satgb_dtype in_t, satgb_dtype out_t, int scan_type, const void* d_in,
                                 int64_t in_pitch, void* d_out, int64_t out_pitch, int64_t width,
                                 int64_t height, satgb_stream stream) {
  if (scan_type != SATGB_SCAN_KOGGE_STONE && scan_type != SATGB_SCAN_LF)
    return fail(SATGB_ERR_INVALID_ARG, "scan_type %d is neither KoggeStone_SCAN (0) nor LF_SCAN (1)", scan_type);
  return sat_single(in_t, out_t, SATGB_MODE_PLAIN, SATGB_FORWARD, d_in, in_pitch, d_out, out_pitch, width,
                    height, (cudaStream_t)stream, -1);
}

satgb_status satgb_scan_rows(satgb_dtype in_t, satgb_dtype out_t, const void* d_in, int64_t in_pitch, void* d_out,
                             int64_t out_pitch, int64_t width, int64_t height, satgb_stream stream) {
  return sat_single(in_t, out_t, kModeRows, SATGB_FORWARD, d_in, in_pitch, d_out, out_pitch, width, height,
                    (cudaStream_t)stream, -1);
}

satgb_status satgb_scan_cols(satgb_dtype in_t, satgb_dtype out_t, const void* d_in, int64_t in_pitch, void* d_out,
                             int64_t out_pitch, int64_t width, int64_t height, satgb_stream stream) {
  return sat_single(in_t, out_t, kModeCols, SATGB_FORWARD, d_in, in_pitch, d_out, out_pitch, width, height,
                    (cudaStream_t)stream, -1);
}

satgb_status satgb_sat_ex(const satgb_sat_desc* d, satgb_stream stream) {
  if (!d) return fail(SATGB_ERR_INVALID_ARG, "null descriptor");
  if (d->mode != SATGB_MODE_PLAIN && d->mode != SATGB_MODE_COMPENSATED)
    return fail(SATGB_ERR_INVALID_ARG, "unknown mode %d", d->mode);
  return sat_single(d->in_t, d->out_t, d->mode, d->direction, d->d_in, d->in_pitch, d->d_out, d->out_pitch,
                    d->width, d->height, (cudaStream_t)stream, -1);
}

satgb_status satgb_sat_planes(const satgb_sat_desc* d, int64_t n_planes, int64_t in_plane_stride,
                              int64_t out_plane_stride, satgb_stream stream) {
  if (!d) return fail(SATGB_ERR_INVALID_ARG, "null descriptor");
  if (d->mode != SATGB_MODE_PLAIN && d->mode != SATGB_MODE_COMPENSATED)
    return fail(SATGB_ERR_INVALID_ARG, "unknown mode %d", d->mode);
  return sat_single(d->in_t, d->out_t, d->mode, d->direction, d->d_in, d->in_pitch, d->d_out, d->out_pitch,
                    d->width, d->height, (cudaStream_t)stream, -1, n_planes, in_plane_stride, out_plane_stride);
}

satgb_status satgb_reserve(int64_t width, int64_t height, satgb_stream stream) {
  if (width <= 0 || height <= 0) return fail(SATGB_ERR_INVALID_ARG, "reserve needs positive sizes");
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  satgb_status st = get_device(&dev);
  if (st != SATGB_OK) return st;
  // the largest layout over every variant, with the staging rows of a 1-byte
  // input behind it where a call would stage one (sat_single)
  size_t need = 0;
  const size_t stage = width * height >= kStageMinPixels ? (((size_t)width + 15) & ~(size_t)15) * (size_t)height : 0;
  using ListFn = const Variant* (*)(int*);
  static const ListFn lists[] = {variants_u8, variants_i8, variants_int32, variants_f32, variants_f64};
  for (ListFn f : lists) {
    int n = 0;
    const Variant* v = f(&n);
    for (int i = 0; i < n; ++i) {
      long long nt = ((width + v[i].TW - 1) / v[i].TW) * ((height + v[i].TH - 1) / v[i].TH);
      const size_t look = layout_for(nt, &v[i]).total;
      need = std::max(need, dtype_size(v[i].in_t) == 1 && stage ? ((look + 255) & ~(size_t)255) + stage : look);
    }
  }
  Workspace& ws = g_ws[std::make_pair(dev, (void*)stream)];
  return ensure_ws(ws, need, (cudaStream_t)stream);
}

satgb_status satgb_stream_check(satgb_stream stream) {
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  satgb_status st = get_device(&dev);
  if (st != SATGB_OK) return st;
  satgb_status result = SATGB_OK;
  auto check = [&](Workspace& ws) {
    if (!ws.base) return;
    WsHeader h;
    if (cudaMemcpy(&h, ws.base, sizeof h, cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaGetLastError();
      return;
    }
    if (h.sticky != 0) {
      result = fail(SATGB_ERR_TIMEOUT, "a look-back wait timed out (tile %u)", h.sticky_tile);
      const uint32_t zero[2] = {0u, 0u};
      cudaMemcpy((char*)ws.base + offsetof(WsHeader, sticky), zero, sizeof zero, cudaMemcpyHostToDevice);
    }
  };
  for (auto& kv : g_ws)
    if (kv.first.first == dev) check(kv.second);
  return result;
}

satgb_status satgb_release(void) {
  std::lock_guard<std::mutex> lk(g_mu);
  cudaDeviceSynchronize();
  for (auto& kv : g_ws) ws_free(kv.second.base);
  g_ws.clear();
  g_desc_cache.clear();
  return SATGB_OK;
}

satgb_status satgb_autotune(satgb_dtype in_t, satgb_dtype out_t, int mode, const void* d_in,
                            int64_t in_pitch, void* d_out, int64_t out_pitch, int64_t width,
                            int64_t height, satgb_stream stream, int* best_config) {
  cudaStream_t s = (cudaStream_t)stream;
  if (!pair_offered(in_t, out_t, mode)) return fail(SATGB_ERR_UNSUPPORTED_TYPES, "type pair not offered");
  if (width <= 0 || height <= 0) return fail(SATGB_ERR_INVALID_ARG, "autotune needs a non-empty image");
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return cuda_fail(cudaGetLastError(), "cudaEventCreate");
  int best = -1;
  float best_ms = 1e30f;
  for (int cfg = 0; cfg < kNumConfigs; ++cfg) {
    if (!find_variant(in_t, out_t, mode, 0, cfg)) continue;
    satgb_status st = SATGB_OK;
    for (int i = 0; i < 3 && st == SATGB_OK; ++i)
      st = sat_single(in_t, out_t, mode, 0, d_in, in_pitch, d_out, out_pitch, width, height, s, cfg);
    if (st != SATGB_OK) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      return st;
    }
    const int reps = 10;
    cudaEventRecord(e0, s);
    for (int i = 0; i < reps; ++i)
      sat_single(in_t, out_t, mode, 0, d_in, in_pitch, d_out, out_pitch, width, height, s, cfg);
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_ms) {
      best_ms = ms;
      best = cfg;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  satgb_status st = satgb_stream_check(stream);
  if (st != SATGB_OK) return st;
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  st = get_device(&dev);
  if (st != SATGB_OK) return st;
  tune_load_locked();
  const int sms = sms_of(dev);
  for (int dir = 0; dir < 2; ++dir)
    g_tune[TuneKey(in_t, out_t, mode, dir, log2_bucket(width), log2_bucket(height), sms)] = best;
  tune_save_locked();
  if (best_config) *best_config = best;
  return SATGB_OK;
}

// ---------------------------------------------------------------------------
// box-filter backward to the image
// ---------------------------------------------------------------------------
satgb_status satgb_box_filter_bwd_x(const satgb_box_desc* desc, void* d_dx, int64_t dx_pitch,
                                    int64_t dx_plane_stride, satgb_stream stream) {
  if (!desc) return fail(SATGB_ERR_INVALID_ARG, "box filter backward: null descriptor");
  const long long w = desc->width, h = desc->height, planes = desc->n_planes;
  if (w < 0 || h < 0 || planes < 0 || desc->n_radii < 1 || desc->n_radii > SATGB_MAX_RADII)
    return fail(SATGB_ERR_INVALID_ARG, "box filter backward: invalid sizes or radius count");
  if (w == 0 || h == 0 || planes == 0) return SATGB_OK;
  if (!d_dx) return fail(SATGB_ERR_INVALID_ARG, "box filter backward: null gradient output");
  if (((uintptr_t)d_dx % 4) != 0) return fail(SATGB_ERR_MISALIGNED, "box filter backward: f32 pointer not 4-byte aligned");
  const long long span = (h - 1) * dx_pitch + w;
  if (dx_pitch < w || (planes > 1 && dx_plane_stride < span))
    return fail(SATGB_ERR_INVALID_ARG, "box filter backward: gradient output pitch or plane stride too small");
  // the output may not overlap any gradient plane it is computed from
  if (desc->box_pitch >= w && (planes == 1 || desc->box_plane_stride > 0)) {
    const long long gspan = ((h - 1) * desc->box_pitch + w) + (planes - 1) * (planes > 1 ? desc->box_plane_stride : 0);
    const long long xspan = span + (planes - 1) * (planes > 1 ? dx_plane_stride : 0);
    const char* xb = (const char*)d_dx;
    for (int i = 0; i < desc->n_radii; ++i) {
      const char* gb = (const char*)desc->d_box[i];
      if (gb && xb < gb + gspan * 4 && gb < xb + xspan * 4)
        return fail(SATGB_ERR_INVALID_ARG, "box filter backward: the gradient output overlaps the gradients of the means");
    }
  }
  // dL/dSAT into the output, then its reverse SAT in place
  satgb_box_desc d = *desc;
  d.d_sat = d_dx;
  d.sat_pitch = dx_pitch;
  d.sat_plane_stride = planes > 1 ? dx_plane_stride : 0;
  satgb_status st = satgb_box_filter_bwd(&d, stream);
  if (st != SATGB_OK) return st;
  return sat_single(SATGB_F32, SATGB_F32, SATGB_MODE_PLAIN, SATGB_REVERSE, d_dx, dx_pitch, d_dx, dx_pitch, w, h,
                    (cudaStream_t)stream, -1, planes, d.sat_plane_stride, d.sat_plane_stride);
}

// ---------------------------------------------------------------------------
// batch plans
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {

BatchKey batch_key(const satgb_batch_plan_s* p, int cls, int sms) {
  const BatchSeg& g = p->seg[cls];
  return BatchKey(p->in_t, p->out_t, p->mode, p->dir, cls, log2_bucket((long long)std::max(1.0, g.pixels)),
                  log2_bucket(std::max(1LL, g.n_images)), p->all_tma ? 1 : 0, sms);
}

// Untuned choice for a class (GB300, the 512-image u8 batch): large images the
// warp-specialized direct-store tiles; small images the 64-row two-CTA tiles
// when rows go through TMA, the row-major tiles when they cannot (packed rows:
// 1401 vs 1015 GB/s); f64 outputs and the compensated mode as for one image.
int batch_default_config(const satgb_batch_plan_s* p, int cls) {
  if (dtype_size(p->out_t) == 8) return 0;
  if (p->mode == SATGB_MODE_COMPENSATED) return 3;
  if (cls == 0) return 5;
  return p->all_tma ? 2 : 6;
}

void seg_free(BatchSeg& g) {
  if (g.table) cudaFree(g.table);
  g.table = nullptr;
  g.order = nullptr;
}

// The tile order of a class: every tile of every image by anti-diagonal
// (tx + ty) first, then by image, then by row.  A tile's left and upper
// neighbours lie on the previous diagonal of the same image, so they come
// earlier (the persistent grid cannot deadlock), and the look-back wavefronts
// of all the images advance together instead of one image after another,
// whose chains of dependent tiles would otherwise leave most SMs waiting.
// Empty when a tile coordinate or an image index does not fit the encoding.
std::vector<unsigned long long> diagonal_order(const std::vector<ImageDesc>& table) {
  std::vector<unsigned long long> order;
  if (table.size() >= (1ULL << 24)) return order;
  long long maxd = 0, n = 0;
  for (auto& d : table) {
    if (d.ntx >= (1 << 20) || d.nty >= (1 << 20)) return order;
    maxd = std::max(maxd, (long long)d.ntx + d.nty - 1);
    n += (long long)d.ntx * d.nty;
  }
  // counting sort by diagonal, images and rows in order within a diagonal
  std::vector<long long> count(maxd + 1, 0);
  for (auto& d : table)
    for (long long dd = 0; dd < (long long)d.ntx + d.nty - 1; ++dd) {
      const long long lo = std::max(0LL, dd - (d.ntx - 1)), hi = std::min<long long>(dd, d.nty - 1);
      count[dd] += hi - lo + 1;
    }
  std::vector<long long> start(maxd + 1, 0);
  for (long long dd = 1; dd <= maxd; ++dd) start[dd] = start[dd - 1] + count[dd - 1];
  order.assign(n, 0ull);
  for (size_t i = 0; i < table.size(); ++i) {
    const ImageDesc& d = table[i];
    for (long long dd = 0; dd < (long long)d.ntx + d.nty - 1; ++dd) {
      const long long lo = std::max(0LL, dd - (d.ntx - 1)), hi = std::min<long long>(dd, d.nty - 1);
      for (long long ty = lo; ty <= hi; ++ty)
        order[start[dd]++] = ((unsigned long long)i << 40) | ((unsigned long long)ty << 20) | (unsigned long long)(dd - ty);
    }
  }
  return order;
}

// (Re)builds a class's descriptor table for the configuration `cfg`; called
// with g_mu held.
satgb_status seg_build(satgb_batch_plan_s* p, int cls, int cfg, cudaStream_t s) {
  BatchSeg& g = p->seg[cls];
  const Variant* v = find_variant(p->in_t, p->out_t, p->mode, p->dir, cfg);
  if (!v) v = find_variant(p->in_t, p->out_t, p->mode, p->dir, batch_default_config(p, cls));
  if (!v) v = find_variant(p->in_t, p->out_t, p->mode, p->dir, 0);
  if (!v) return fail(SATGB_ERR_UNSUPPORTED_TYPES, "no kernel for this batch");
  std::vector<ImageDesc> table;
  long long base = 0;
  for (auto& c : g.imgs) {
    ImageDesc d;
    fill_image_desc(d, v, p->in_t, p->out_t, c.in, c.out, c.in_pitch, c.out_pitch, c.width, c.height, base, 1, 0, 0);
    base += (long long)d.ntx * d.nty;
    table.push_back(d);
  }
  seg_free(g);
  g.v = v;
  g.n_tiles = base;
  if (table.empty()) return SATGB_OK;
  g.img0 = table[0];
  const std::vector<unsigned long long> order = table.size() > 1 ? diagonal_order(table) : std::vector<unsigned long long>();
  const size_t tbytes = (table.size() * sizeof(ImageDesc) + 255) & ~(size_t)255;
  if (cudaMalloc(&g.table, tbytes + order.size() * sizeof(unsigned long long)) != cudaSuccess) {
    cudaGetLastError();
    g.table = nullptr;
    return fail(SATGB_ERR_ALLOC, "image table allocation failed");
  }
  cudaError_t e = cudaMemcpyAsync(g.table, table.data(), table.size() * sizeof(ImageDesc), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess && !order.empty()) {
    g.order = reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(g.table) + tbytes);
    e = cudaMemcpyAsync(g.order, order.data(), order.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice, s);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "image table upload");
  return SATGB_OK;
}

satgb_status plan_ws(satgb_batch_plan_s* p, cudaStream_t s) {
  size_t need = 0;
  p->n_tiles = 0;
  for (auto& g : p->seg)
    if (g.n_tiles) {
      need = std::max(need, layout_for(g.n_tiles, g.v).total);
      p->n_tiles += g.n_tiles;
    }
  satgb_status st = ensure_ws(p->ws, need, s);
  if (st != SATGB_OK) return st;
  cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? SATGB_OK : cuda_fail(e, "cudaStreamSynchronize");
}

satgb_status plan_repack(satgb_batch_plan_s* p, cudaStream_t s) {
  return repack_launch(p->jobs, p->n_jobs, p->stage_rows, sms_of(p->dev), s);
}

satgb_status plan_launch_locked(satgb_batch_plan_s* p, cudaStream_t s) {
  satgb_status st0 = plan_repack(p, s);
  if (st0 != SATGB_OK) return st0;
  for (auto& g : p->seg) {
    if (!g.n_tiles) continue;
    satgb_status st = launch_locked(g.v, g.table, g.img0, g.n_images, g.n_tiles, p->ws, p->dev, s, g.order);
    if (st != SATGB_OK) return st;
  }
  return SATGB_OK;
}

// Captures the classes' launches, one after the other, in the plan's graph.
satgb_status plan_capture(satgb_batch_plan_s* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  p->exec = nullptr;
  p->graph = nullptr;
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
  satgb_status st = SATGB_OK;
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    const long long before = g_launches.load();
    st = plan_launch_locked(p, cs);
    g_launches.store(before); // the capture itself launches nothing
    cudaError_t e2 = cudaStreamEndCapture(cs, &p->graph);
    if (st == SATGB_OK && e2 != cudaSuccess) st = cuda_fail(e2, "cudaStreamEndCapture");
    if (st == SATGB_OK) {
      e2 = cudaGraphInstantiate(&p->exec, p->graph, 0);
      if (e2 != cudaSuccess) st = cuda_fail(e2, "cudaGraphInstantiate");
    }
  } else {
    st = cuda_fail(e, "cudaStreamBeginCapture");
  }
  cudaStreamDestroy(cs);
  return st;
}

void plan_free(satgb_batch_plan_s* p) {
  if (p->exec) cudaGraphExecDestroy(p->exec);
  if (p->graph) cudaGraphDestroy(p->graph);
  ws_free(p->ws.base);
  ws_free(p->stage);
  if (p->jobs) cudaFree(p->jobs);
  for (auto& g : p->seg) seg_free(g);
  delete p;
}

// Inputs that TMA cannot address (base or row pitch not 16-byte aligned, at
// least 16 bytes a row) get a copy in padded rows: the plan's staging buffer,
// one region per image (256-byte aligned, rows of the width rounded up to 16
// bytes), and the tile kernels read the copies.  Rewrites the images' input
// pointers and pitches in `imgs`.
satgb_status plan_stage_inputs(satgb_batch_plan_s* p, std::vector<ImgCheck>& imgs, size_t in_sz, cudaStream_t s) {
  std::vector<satgb::RepackJob> jobs;
  std::vector<size_t> offs, which;
  size_t total = 0;
  long long rows = 0;
  for (size_t i = 0; i < imgs.size(); ++i) {
    const ImgCheck& c = imgs[i];
    const size_t row_bytes = (size_t)c.width * in_sz;
    if (row_bytes < 16 || tma_ok(c.in, c.width, c.height, c.in_pitch, 1, 0, in_sz)) continue;
    const size_t pitch = (row_bytes + 15) & ~(size_t)15;
    satgb::RepackJob j;
    j.src = static_cast<const unsigned char*>(c.in);
    j.dst = nullptr;
    j.src_pitch = c.in_pitch * (int64_t)in_sz;
    j.dst_pitch = (int64_t)pitch;
    j.row_bytes = (int64_t)row_bytes;
    j.row_base = rows;
    jobs.push_back(j);
    which.push_back(i);
    offs.push_back(total);
    total += ((pitch * (size_t)c.height) + 255) & ~(size_t)255;
    rows += c.height;
  }
  if (jobs.empty()) return SATGB_OK;
  p->stage = ws_alloc(total);
  if (!p->stage) return fail(SATGB_ERR_ALLOC, "batch staging allocation of %zu bytes failed", total);
  for (size_t k = 0; k < jobs.size(); ++k) {
    ImgCheck& c = imgs[which[k]];
    jobs[k].dst = static_cast<unsigned char*>(p->stage) + offs[k];
    c.in = jobs[k].dst;
    c.in_pitch = jobs[k].dst_pitch / (int64_t)in_sz;
  }
  if (cudaMalloc(&p->jobs, jobs.size() * sizeof(satgb::RepackJob)) != cudaSuccess) {
    cudaGetLastError();
    p->jobs = nullptr;
    return fail(SATGB_ERR_ALLOC, "batch staging table allocation failed");
  }
  cudaError_t e = cudaMemcpyAsync(p->jobs, jobs.data(), jobs.size() * sizeof(satgb::RepackJob), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "batch staging table upload");
  p->n_jobs = (int)jobs.size();
  p->stage_rows = rows;
  return SATGB_OK;
}

}  // namespace

extern "C" {

satgb_status satgb_batch_plan_create(satgb_batch_plan** plan, satgb_dtype in_t, satgb_dtype out_t, int mode,
                                     int direction, const satgb_image* images, int64_t n_images,
                                     satgb_stream stream) {
  if (!plan) return fail(SATGB_ERR_INVALID_ARG, "null plan pointer");
  *plan = nullptr;
  const size_t in_sz = dtype_size(in_t), out_sz = dtype_size(out_t);
  if (!in_sz || !out_sz) return fail(SATGB_ERR_INVALID_ARG, "unknown dtype code");
  if (direction != SATGB_FORWARD && direction != SATGB_REVERSE) return fail(SATGB_ERR_INVALID_ARG, "unknown direction");
  if (mode != SATGB_MODE_PLAIN && mode != SATGB_MODE_COMPENSATED) return fail(SATGB_ERR_INVALID_ARG, "unknown mode %d", mode);
  if (!pair_offered(in_t, out_t, mode)) return fail(SATGB_ERR_UNSUPPORTED_TYPES, "type pair not offered");
  if (n_images <= 0 || !images) return fail(SATGB_ERR_INVALID_ARG, "empty image list");
  cudaStream_t s = (cudaStream_t)stream;
  // Validate every image; empty images are dropped from the table.
  std::vector<ImgCheck> keep;
  for (int64_t i = 0; i < n_images; ++i) {
    ImgCheck c{images[i].d_in, images[i].d_out, images[i].in_pitch, images[i].out_pitch, images[i].width, images[i].height};
    satgb_status st = validate_image(c, in_sz, out_sz);
    if (st != SATGB_OK) return fail(st, "image %lld: %s", (long long)i, g_last_error.c_str());
    if (c.width > 0 && c.height > 0) keep.push_back(c);
  }
  {
    satgb_status st = check_batch_disjoint(keep, in_sz, out_sz);
    if (st != SATGB_OK) return st;
  }
  std::lock_guard<std::mutex> lk(g_mu);
  int dev = 0;
  satgb_status st = get_device(&dev);
  if (st != SATGB_OK) return st;
  auto* p = new satgb_batch_plan_s();
  p->in_t = in_t;
  p->out_t = out_t;
  p->mode = mode;
  p->dir = direction;
  p->dev = dev;
  st = plan_stage_inputs(p, keep, in_sz, s);
  if (st != SATGB_OK) {
    plan_free(p);
    return st;
  }
  const int cpt = (int)(16 / out_sz);
  for (auto& c : keep) {
    const long long tiles = ((c.width + 32LL * cpt - 1) / (32LL * cpt)) * ((c.height + 127) / 128);
    BatchSeg& g = p->seg[tiles >= kLargeTiles ? 0 : 1];
    g.imgs.push_back(c);
    g.n_images += 1;
    g.pixels += (double)c.width * (double)c.height;
    p->all_tma = p->all_tma && ((uintptr_t)c.in % 16) == 0 && ((uintptr_t)c.out % 16) == 0 &&
                 ((size_t)c.in_pitch * in_sz) % 16 == 0 && ((size_t)c.out_pitch * out_sz) % 16 == 0;
  }
  tune_load_locked();
  const int sms = sms_of(dev);
  for (int cls = 0; cls < kBatchClasses && st == SATGB_OK; ++cls) {
    if (!p->seg[cls].n_images) continue;
    int cfg = g_forced_config;
    if (cfg < 0) {
      auto it = g_batch_tune.find(batch_key(p, cls, sms));
      cfg = it != g_batch_tune.end() ? it->second : batch_default_config(p, cls);
    }
    st = seg_build(p, cls, cfg, s);
  }
  if (st == SATGB_OK) st = plan_ws(p, s);
  if (st == SATGB_OK && p->n_tiles > 0) st = plan_capture(p);
  if (st != SATGB_OK) {
    plan_free(p);
    return st;
  }
  *plan = p;
  return SATGB_OK;
}

satgb_status satgb_batch_plan_autotune(satgb_batch_plan* p, satgb_stream stream, int* configs) {
  if (!p) return fail(SATGB_ERR_INVALID_ARG, "null plan");
  cudaStream_t s = (cudaStream_t)stream;
  std::lock_guard<std::mutex> lk(g_mu);
  tune_load_locked();
  const int sms = sms_of(p->dev);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return cuda_fail(cudaGetLastError(), "cudaEventCreate");
  satgb_status st = plan_repack(p, s); // the staged inputs the timed launches read
  for (int cls = 0; cls < kBatchClasses && st == SATGB_OK; ++cls) {
    BatchSeg& g = p->seg[cls];
    if (configs) configs[cls] = -1;
    if (!g.n_images) continue;
    int best = -1;
    float best_ms = 1e30f;
    for (int cfg = 0; cfg < kNumConfigs && st == SATGB_OK; ++cfg) {
      const Variant* v = find_variant(p->in_t, p->out_t, p->mode, p->dir, cfg);
      if (!v || v->cfg != cfg) continue;
      st = seg_build(p, cls, cfg, s);
      if (st == SATGB_OK) st = plan_ws(p, s);
      if (st != SATGB_OK) break;
      for (int i = 0; i < 2 && st == SATGB_OK; ++i)
        st = launch_locked(g.v, g.table, g.img0, g.n_images, g.n_tiles, p->ws, p->dev, s, g.order);
      const int reps = 5;
      cudaEventRecord(e0, s);
      for (int i = 0; i < reps && st == SATGB_OK; ++i)
        st = launch_locked(g.v, g.table, g.img0, g.n_images, g.n_tiles, p->ws, p->dev, s, g.order);
      cudaEventRecord(e1, s);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) st = cuda_fail(e, "cudaEventSynchronize");
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (st == SATGB_OK && ms < best_ms) {
        best_ms = ms;
        best = cfg;
      }
    }
    if (st != SATGB_OK) break;
    st = seg_build(p, cls, best, s);
    g_batch_tune[batch_key(p, cls, sms)] = best;
    if (configs) configs[cls] = best;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st == SATGB_OK) st = plan_ws(p, s);
  if (st == SATGB_OK) {
    WsHeader h;
    cudaError_t e = cudaMemcpy(&h, p->ws.base, sizeof h, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) st = cuda_fail(e, "cudaMemcpy");
    else if (h.sticky) st = fail(SATGB_ERR_TIMEOUT, "a look-back wait timed out while tuning (tile %u)", h.sticky_tile);
  }
  if (st == SATGB_OK) tune_save_locked();
  if (st == SATGB_OK && p->n_tiles > 0) st = plan_capture(p);
  return st;
}

satgb_status satgb_batch_plan_exec(satgb_batch_plan* p, satgb_stream stream) {
  if (!p) return fail(SATGB_ERR_INVALID_ARG, "null plan");
  if (p->n_tiles == 0) return SATGB_OK;
  cudaError_t e = cudaGraphLaunch(p->exec, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
  for (auto& g : p->seg)
    if (g.n_tiles) g_launches.fetch_add(1);
  return SATGB_OK;
}

satgb_status satgb_batch_plan_launch(satgb_batch_plan* p, satgb_stream stream) {
  if (!p) return fail(SATGB_ERR_INVALID_ARG, "null plan");
  if (p->n_tiles == 0) return SATGB_OK;
  std::lock_guard<std::mutex> lk(g_mu);
  return plan_launch_locked(p, (cudaStream_t)stream);
}

satgb_status satgb_batch_plan_info(const satgb_batch_plan* p, int64_t* n_tiles, int* config) {
  if (!p) return fail(SATGB_ERR_INVALID_ARG, "null plan");
  if (n_tiles) *n_tiles = p->n_tiles;
  if (config) {
    // the configuration of the large class, or of the small one if it is alone
    *config = p->seg[0].n_images ? p->seg[0].v->cfg : (p->seg[1].n_images ? p->seg[1].v->cfg : -1);
  }
  return SATGB_OK;
}

satgb_status satgb_batch_plan_classes(const satgb_batch_plan* p, int64_t* n_images, int64_t* n_tiles, int* configs) {
  if (!p) return fail(SATGB_ERR_INVALID_ARG, "null plan");
  for (int cls = 0; cls < kBatchClasses; ++cls) {
    const BatchSeg& g = p->seg[cls];
    if (n_images) n_images[cls] = g.n_images;
    if (n_tiles) n_tiles[cls] = g.n_tiles;
    if (configs) configs[cls] = g.n_images ? g.v->cfg : -1;
  }
  return SATGB_OK;
}

satgb_status satgb_batch_plan_check(satgb_batch_plan* p, satgb_stream stream) {
  if (!p) return fail(SATGB_ERR_INVALID_ARG, "null plan");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
  if (!p->ws.base) return SATGB_OK;
  WsHeader h;
  e = cudaMemcpy(&h, p->ws.base, sizeof h, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemcpy");
  if (h.sticky) {
    const uint32_t zero[2] = {0u, 0u};
    cudaMemcpy((char*)p->ws.base + offsetof(WsHeader, sticky), zero, sizeof zero, cudaMemcpyHostToDevice);
    return fail(SATGB_ERR_TIMEOUT, "a look-back wait timed out (tile %u)", h.sticky_tile);
  }
  return SATGB_OK;
}

satgb_status satgb_batch_plan_destroy(satgb_batch_plan* p) {
  if (!p) return SATGB_OK;
  cudaDeviceSynchronize();
  plan_free(p);
  return SATGB_OK;
}

}  // extern "C"
