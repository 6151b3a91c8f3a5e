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

// Launchers, one explicit instantiation per (scalar type, dimensionality) in
// kern_<type>_<dims>d.cu so the 16 variants compile in parallel.
template <typename S, int D> cudaError_t run_encode(const LaunchArgs& a, cudaStream_t st);
template <typename S, int D> cudaError_t run_decode(const LaunchArgs& a, cudaStream_t st);
template <typename S, int D> cudaError_t run_parse(const Job& job, cudaStream_t st);

// largest dynamic shared memory a tile may use before staging moves to global memory
constexpr size_t kMaxTileSmem = 160 * 1024;

}  // namespace zg
