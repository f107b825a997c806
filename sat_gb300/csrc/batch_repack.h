// batch_repack.h -- a batch plan's staged copy of one image's input rows
// (batch_repack.cu): rows of row_bytes at src_pitch bytes into rows at
// dst_pitch bytes (a multiple of 16, dst 16-byte aligned); row_base is the
// image's first row in the launch's flat row index.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/satgb.h"

namespace satgb {

struct RepackJob {
  const unsigned char* src;
  unsigned char* dst;
  int64_t src_pitch, dst_pitch, row_bytes, row_base;
};

// One launch for every staged row of n_jobs images (jobs sorted by row_base,
// in device memory), on up to 8 CTAs of 8 warps per SM.
satgb_status repack_launch(const RepackJob* jobs_dev, int n_jobs, long long n_rows, int sms, cudaStream_t s);
// One image's n_rows rows (row_base 0), the job passed by value.
satgb_status repack_launch_one(const RepackJob& job, long long n_rows, int sms, cudaStream_t s);

}  // namespace satgb
