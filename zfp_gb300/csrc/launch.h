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

// a tile image plus bit planes larger than this is staged in global memory
// instead (GB300 allows 227 KB of shared memory per CTA, static included)
constexpr size_t kMaxTileSmem = 216 * 1024;

// shared memory the encoder keeps for bit planes: 1-3D blocks only
inline size_t plane_bytes(size_t esize, int dims) { return dims <= 3 ? esize * 8 * kTile * 8 : 0; }

}  // namespace zg
