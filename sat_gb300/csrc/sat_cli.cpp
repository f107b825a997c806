// sat_cli.cpp -- the reference's benchmark command line over libsatgb.so.
//
//   sat A S D0 D1 R [--reps N]
//
// mirrors `sat <algo> <scan> <dtIn> <dtOut> <repeat>` (pengdada/SAT
// integralImage/main.cpp:8-44, GetArgs integralImage.h:56-63): A selects the
// algorithm (0 ScanRow-BRLT, 1 BRLT-ScanRow, 2 ScanRowColumn, 3 the
// column-only scan, 4 the row-only scan), S the warp scan (0
// Kogge-Stone, 1 Ladner-Fischer), D0/D1 the input and output DataType codes
// (integralImage.h:22-32), and R the sizes: square images of i*1024 for
// i = 1..R, as the reference's drivers loop (ScanRow-BRLT.cu:272-273).
// Inputs are 0/1 values like the reference's (`rand() % 2`,
// ScanRow-BRLT.cu:207) in pitched device buffers (cudaMallocPitch, as its
// GpuData allocates with cudaMalloc3D).  For each size one CSV line:
//   width, height, total time = <host ms>, <gpu ms>, <GB/s>
// where the times are per launch, averaged over --reps launches (default 1,
// the reference's REPEAT_COUNT), GB/s counts input + output bytes.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "satgb.h"

namespace {

const char* type_name(int t) {
  switch (t) {
    case SATGB_U8: return "uchar";
    case SATGB_I8: return "char";
    case SATGB_U32: return "uint";
    case SATGB_I32: return "int";
    case SATGB_F32: return "float";
    case SATGB_F64: return "double";
    default: return "?";
  }
}

size_t type_size(int t) {
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

// fills `n` host elements of type t with 0/1 values
void fill01(std::vector<unsigned char>& buf, int t, size_t n, unsigned seed) {
  std::mt19937 rng(seed);
  const size_t sz = type_size(t);
  buf.assign(n * sz, 0);
  for (size_t i = 0; i < n; ++i) {
    const int v = (int)(rng() & 1u);
    unsigned char* p = buf.data() + i * sz;
    switch (t) {
      case SATGB_U8:
      case SATGB_I8: *p = (unsigned char)v; break;
      case SATGB_U32:
      case SATGB_I32: { const int32_t x = v; std::memcpy(p, &x, 4); break; }
      case SATGB_F32: { const float x = (float)v; std::memcpy(p, &x, 4); break; }
      case SATGB_F64: { const double x = (double)v; std::memcpy(p, &x, 8); break; }
    }
  }
}

int usage() {
  std::fprintf(stderr,
               "usage: sat A S D0 D1 R [--reps N]\n"
               "  A   0 ScanRow-BRLT, 1 BRLT-ScanRow, 2 ScanRowColumn, 3 column-only, 4 row-only\n"
               "  S   0 Kogge-Stone, 1 Ladner-Fischer\n"
               "  D0  input type, D1 output type: 0 u8, 1 i8, 4 u32, 5 i32, 6 f32, 7 f64\n"
               "  R   sizes i*1024 x i*1024 for i = 1..R\n");
  return 2;
}

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  std::fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
  return false;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 6) return usage();
  const int algo = std::atoi(argv[1]);
  const int scan = std::atoi(argv[2]);
  const int d0 = std::atoi(argv[3]);
  const int d1 = std::atoi(argv[4]);
  const int repeat = std::atoi(argv[5]);
  int reps = 1;
  for (int i = 6; i + 1 < argc; ++i)
    if (std::strcmp(argv[i], "--reps") == 0) reps = std::max(1, std::atoi(argv[i + 1]));
  if (algo < 0 || algo > 4 || repeat < 1 || type_size(d0) == 0 || type_size(d1) == 0) return usage();
  using Fn = satgb_status (*)(satgb_dtype, satgb_dtype, int, const void*, int64_t, void*, int64_t, int64_t,
                              int64_t, satgb_stream);
  // the single-direction scans take no scan type
  struct Scans {
    static satgb_status cols(satgb_dtype a, satgb_dtype b, int, const void* i, int64_t ip, void* o, int64_t op,
                             int64_t w, int64_t h, satgb_stream s) {
      return satgb_scan_cols(a, b, i, ip, o, op, w, h, s);
    }
    static satgb_status rows(satgb_dtype a, satgb_dtype b, int, const void* i, int64_t ip, void* o, int64_t op,
                             int64_t w, int64_t h, satgb_stream s) {
      return satgb_scan_rows(a, b, i, ip, o, op, w, h, s);
    }
  };
  const Fn fns[5] = {&satgb_scanrow_brlt, &satgb_brlt_scanrow, &satgb_scanrowcolumn, &Scans::cols, &Scans::rows};
  const char* names[5] = {"ScanRow-BRLT", "BRLT-ScanRow", "ScanRowColumn", "ScanY (column only)", "ScanX (row only)"};
  std::printf("%s-->%s, %s, %s\n", type_name(d0), type_name(d1), names[algo],
              scan == 0 ? "KoggeStone_SCAN" : "LF_SCAN");
  cudaStream_t stream;
  if (!cuda_ok(cudaStreamCreate(&stream), "cudaStreamCreate")) return 1;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int rc = 0;
  for (int i = 1; i <= repeat && rc == 0; ++i) {
    const int64_t w = 1024LL * i, h = 1024LL * i;
    const size_t si = type_size(d0), so = type_size(d1);
    void* din = nullptr;
    void* dout = nullptr;
    size_t pin = 0, pout = 0;
    if (!cuda_ok(cudaMallocPitch(&din, &pin, (size_t)w * si, (size_t)h), "cudaMallocPitch") ||
        !cuda_ok(cudaMallocPitch(&dout, &pout, (size_t)w * so, (size_t)h), "cudaMallocPitch")) {
      rc = 1;
      break;
    }
    std::vector<unsigned char> host;
    fill01(host, d0, (size_t)(w * h), 1234u + (unsigned)i);
    cuda_ok(cudaMemcpy2D(din, pin, host.data(), (size_t)w * si, (size_t)w * si, (size_t)h, cudaMemcpyHostToDevice),
            "cudaMemcpy2D");
    // one untimed call (workspace, first-use setup), then the timed ones
    satgb_status st = fns[algo]((satgb_dtype)d0, (satgb_dtype)d1, scan, din, (int64_t)(pin / si), dout,
                                (int64_t)(pout / so), w, h, stream);
    if (st != SATGB_OK) {
      std::fprintf(stderr, "error: %s\n", satgb_last_error_string());
      rc = 1;
    } else {
      cudaStreamSynchronize(stream);
      const auto t0 = std::chrono::steady_clock::now();
      cudaEventRecord(e0, stream);
      for (int k = 0; k < reps && st == SATGB_OK; ++k)
        st = fns[algo]((satgb_dtype)d0, (satgb_dtype)d1, scan, din, (int64_t)(pin / si), dout, (int64_t)(pout / so),
                       w, h, stream);
      cudaEventRecord(e1, stream);
      if (satgb_stream_check(stream) != SATGB_OK || st != SATGB_OK) {
        std::fprintf(stderr, "error: %s\n", satgb_last_error_string());
        rc = 1;
      }
      const double host_ms =
          std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count() / reps;
      float gpu_ms = 0.f;
      cudaEventElapsedTime(&gpu_ms, e0, e1);
      gpu_ms /= reps;
      const double gbs = (double)w * h * (si + so) / (gpu_ms * 1e-3) / 1e9;
      if (rc == 0) std::printf("%lld, %lld, total time = %f, %f, %.1f\n", (long long)w, (long long)h, host_ms, gpu_ms, gbs);
    }
    cudaFree(din);
    cudaFree(dout);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(stream);
  satgb_release();
  return rc;
}
