// ref_gpu_bench.cu -- times the reference's own GPU kernels (pengdada/SAT:
// BlockScan::blockScan x2, integralImage/ScanRow-BRLT.cu:224-227;
// SerielScan::serielScan x2, BRLT-Scan.cu:236-239; IncrementScan::ScanX +
// ScanY, ScanRowColumn.cu:474-477) on this GPU, from the cubins that
// baseline/build_ref_gpu.sh compiles from the reference's sources, with the
// reference's own launch shapes (blocks of 1024 threads, one CTA per 32-row
// strip; ScanX 32 x 32 threads per 32 rows, ScanY 32 x 32 threads per 32
// columns) on square images, the only shape its kernels support.
//
// Test infrastructure for the measured reference-GPU baseline: it is not
// part of libsatgb.so.  Every result is checked on the host against a serial
// SAT of the same input (the reference's own Compare returns true without
// comparing, integralImage.h:268): bit for bit for u8 -> u32, within 1e-5 of
// SAT(|a|) in double for f32.  Output: one JSON line per algorithm and pair,
// with the SAT's algorithmic bytes W x H x (sizeof(in) + sizeof(out)) over
// the time of both launches (CUDA events, median of the repetitions).
//
// Usage: ref_gpu_bench <cubin dir> [size=8192] [reps=20]
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#define CK(x)                                                                                   \
  do {                                                                                          \
    CUresult r_ = (x);                                                                          \
    if (r_ != CUDA_SUCCESS) {                                                                   \
      const char* s_ = nullptr;                                                                 \
      cuGetErrorString(r_, &s_);                                                                \
      std::fprintf(stderr, "%s failed: %s\n", #x, s_ ? s_ : "?");                               \
      std::exit(1);                                                                             \
    }                                                                                           \
  } while (0)
#define CR(x)                                                                                   \
  do {                                                                                          \
    cudaError_t e_ = (x);                                                                       \
    if (e_ != cudaSuccess) {                                                                    \
      std::fprintf(stderr, "%s failed: %s\n", #x, cudaGetErrorString(e_));                      \
      std::exit(1);                                                                             \
    }                                                                                           \
  } while (0)

struct Algo {
  const char* name;   // the reference's algorithm name
  const char* cubin;  // file the kernels are in
  const char* k1[2];  // first launch, per pair (u8 -> u32, f32 -> f32)
  const char* k2[2];  // second launch
  int kind;           // 0: two transposing row scans; 1: ScanX then ScanY
};

// Kernel names as the compiler mangles the reference's template instances
// (LF_SCAN where the kernel takes a scan type, as its command line does by default).
static const Algo kAlgos[] = {
    {"ScanRow-BRLT", "ScanRow-BRLT.cubin",
     {"_ZN9BlockScan9blockScanIhjLi1ELj32ELj8EEEvPKT_PT0_jjjj", "_ZN9BlockScan9blockScanIffLi1ELj32ELj8EEEvPKT_PT0_jjjj"},
     {"_ZN9BlockScan9blockScanIjjLi1ELj32ELj8EEEvPKT_PT0_jjjj", "_ZN9BlockScan9blockScanIffLi1ELj32ELj8EEEvPKT_PT0_jjjj"},
     0},
    {"BRLT-ScanRow", "BRLT-Scan.cubin",
     {"_ZN10SerielScan10serielScanIhjLj32ELj8ELj1024EEEvPKT_PT0_jjjj",
      "_ZN10SerielScan10serielScanIffLj32ELj8ELj1024EEEvPKT_PT0_jjjj"},
     {"_ZN10SerielScan10serielScanIjjLj32ELj8ELj1024EEEvPKT_PT0_jjjj",
      "_ZN10SerielScan10serielScanIffLj32ELj8ELj1024EEEvPKT_PT0_jjjj"},
     0},
    {"ScanRowColumn", "ScanRowColumn.cubin",
     {"_ZN13IncrementScan5ScanXIhjLi1ELi32ELi32ELi32EEEvPKT_PT0_jjj",
      "_ZN13IncrementScan5ScanXIffLi1ELi32ELi32ELi32EEEvPKT_PT0_jjj"},
     {"_ZN13IncrementScan5ScanYIjjLj1ELj32ELj32EEEvPKT_PT0_jjj", "_ZN13IncrementScan5ScanYIffLj1ELj32ELj32EEEvPKT_PT0_jjj"},
     1},
};

static uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s <cubin dir> [size=8192] [reps=20]\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  const unsigned N = argc > 2 ? (unsigned)std::atoi(argv[2]) : 8192u;
  const int reps = argc > 3 ? std::atoi(argv[3]) : 20;
  if (N == 0 || N % 1024 != 0) {
    std::fprintf(stderr, "the reference's kernels need square sizes that are multiples of 1024\n");
    return 2;
  }
  CR(cudaFree(nullptr)); // the runtime's primary context, current for the driver calls below
  const size_t n = (size_t)N * N;
  std::vector<uint8_t> a8(n);
  std::vector<float> af(n);
  for (size_t i = 0; i < n; ++i) {
    const uint64_t z = mix(0x5A7A5A7A5A7A5A7AULL + (i + 1) * 0x9E3779B97F4A7C15ULL);
    a8[i] = (uint8_t)(z >> 56);
    af[i] = (float)(z >> 40) * (1.0f / 16777216.0f);
  }
  // host references: the serial SAT of each input
  std::vector<uint32_t> ref8(n);
  std::vector<double> reff(n), refabs(n);
  for (unsigned y = 0; y < N; ++y) {
    uint32_t r8 = 0;
    double rf = 0;
    for (unsigned x = 0; x < N; ++x) {
      const size_t i = (size_t)y * N + x;
      r8 += a8[i];
      rf += af[i];
      ref8[i] = r8 + (y ? ref8[i - N] : 0u);
      reff[i] = rf + (y ? reff[i - N] : 0.0);
    }
  }
  refabs = reff; // U[0,1) inputs: SAT(|a|) == SAT(a)

  void *d_in = nullptr, *d_tmp = nullptr, *d_out = nullptr;
  CR(cudaMalloc(&d_in, n * 4));
  CR(cudaMalloc(&d_tmp, n * 4));
  CR(cudaMalloc(&d_out, n * 4));
  cudaEvent_t e0, e1;
  CR(cudaEventCreate(&e0));
  CR(cudaEventCreate(&e1));

  for (const Algo& al : kAlgos) {
    CUmodule mod;
    CK(cuModuleLoad(&mod, (dir + "/" + al.cubin).c_str()));
    for (int pair = 0; pair < 2; ++pair) {
      const size_t in_sz = pair == 0 ? 1 : 4;
      CUfunction f1, f2;
      CK(cuModuleGetFunction(&f1, mod, al.k1[pair]));
      CK(cuModuleGetFunction(&f2, mod, al.k2[pair]));
      if (pair == 0) CR(cudaMemcpy(d_in, a8.data(), n, cudaMemcpyHostToDevice));
      else CR(cudaMemcpy(d_in, af.data(), n * 4, cudaMemcpyHostToDevice));
      CR(cudaMemset(d_out, 0, n * 4));
      unsigned w = N, h = N, p = N; // square: every pitch is N elements
      void* a1[6] = {&d_in, &d_tmp, &w, &p, &h, &p};
      void* a2[6] = {&d_tmp, &d_out, &h, &p, &w, &p};
      auto launch = [&]() {
        if (al.kind == 0) {
          CK(cuLaunchKernel(f1, 1, N / 32, 1, 1024, 1, 1, 0, nullptr, a1, nullptr));
          CK(cuLaunchKernel(f2, 1, N / 32, 1, 1024, 1, 1, 0, nullptr, a2, nullptr));
        } else {
          void* x1[5] = {&d_in, &d_tmp, &w, &p, &h};
          void* x2[5] = {&d_tmp, &d_out, &w, &p, &h};
          CK(cuLaunchKernel(f1, 1, N / 32, 1, 32, 32, 1, 0, nullptr, x1, nullptr));
          CK(cuLaunchKernel(f2, N / 32, 1, 1, 32, 32, 1, 0, nullptr, x2, nullptr));
        }
      };
      for (int i = 0; i < 3; ++i) launch();
      CR(cudaDeviceSynchronize());
      std::vector<float> ms(reps);
      for (int i = 0; i < reps; ++i) {
        CR(cudaEventRecord(e0, nullptr));
        launch();
        CR(cudaEventRecord(e1, nullptr));
        CR(cudaEventSynchronize(e1));
        CR(cudaEventElapsedTime(&ms[i], e0, e1));
      }
      CR(cudaGetLastError());
      std::sort(ms.begin(), ms.end());
      const double med = ms[reps / 2];
      // check the result of the last launch
      bool ok = true;
      double worst = 0;
      if (pair == 0) {
        std::vector<uint32_t> got(n);
        CR(cudaMemcpy(got.data(), d_out, n * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i)
          if (got[i] != ref8[i]) {
            ok = false;
            break;
          }
      } else {
        std::vector<float> got(n);
        CR(cudaMemcpy(got.data(), d_out, n * 4, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) worst = std::max(worst, std::fabs((double)got[i] - reff[i]) / std::max(refabs[i], 1e-30));
        ok = worst <= 1e-5;
      }
      const double bytes = (double)n * (in_sz + 4);
      std::printf("{\"algorithm\": \"%s\", \"pair\": \"%s\", \"size\": %u, \"launches\": 2, \"ms_median\": %.5f, "
                  "\"gbs\": %.1f, \"correct\": %s, \"max_rel_abs\": %.3g}\n",
                  al.name, pair == 0 ? "u8->u32" : "f32->f32", N, med, bytes / (med * 1e-3) / 1e9,
                  ok ? "true" : "false", worst);
      std::fflush(stdout);
    }
    CK(cuModuleUnload(mod));
  }
  return 0;
}
