// launch.h -- per-scalar-type kernel launchers (one translation unit each,
// compiled in parallel).
#pragma once

#include <cuda_runtime.h>

#include "job.h"

namespace zg {

struct LaunchArgs {
  Job one;                // the job when njobs == 1
  const Job* jobs;        // device array when njobs > 1
  int njobs;
  LaunchScratch sc;
  uint32_t total_tiles;
  int use_ticket;
  uint32_t img_words;     // staging words per tile
  uint64_t* gimg;         // global staging (grid * img_words words) when shared memory is too small
  int grid;
};

// type: zfp_type numbering (1 int32, 2 int64, 3 float, 4 double)
cudaError_t launch_encode(int type, int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode(int type, int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_parse(int type, int dims, const Job& job, cudaStream_t st);

cudaError_t launch_encode_i32(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_encode_i64(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_encode_f32(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_encode_f64(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode_i32(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode_i64(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode_f32(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode_f64(int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_parse_i32(int dims, const Job& job, cudaStream_t st);
cudaError_t launch_parse_i64(int dims, const Job& job, cudaStream_t st);
cudaError_t launch_parse_f32(int dims, const Job& job, cudaStream_t st);
cudaError_t launch_parse_f64(int dims, const Job& job, cudaStream_t st);

// largest dynamic shared memory a tile may use before staging moves to global memory
constexpr size_t kMaxTileSmem = 160 * 1024;

}  // namespace zg
