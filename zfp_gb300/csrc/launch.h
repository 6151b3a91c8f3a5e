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
  int multi_lossy;        // with `jobs`: no job of the array is reversible (the lossy-only kernels)
  LaunchScratch sc;
  uint32_t total_tiles;
  int use_ticket;
  uint32_t img_words;     // shared-memory words per CTA for the tile image / staged stream words
  int grid;
  uint32_t want_words;    // decode planning: stream words a typical tile stages (0: unknown)
};

// Launchers, one explicit instantiation per (scalar type, dimensionality) in
// kern_<type>_<dims>d.cu so the 16 variants compile in parallel.
template <typename S, int D> cudaError_t run_encode(const LaunchArgs& a, cudaStream_t st);
template <typename S, int D> cudaError_t run_decode(const LaunchArgs& a, cudaStream_t st);
template <typename S, int D> cudaError_t run_parse(const Job& job, cudaStream_t st);

// Shared-memory words a CTA of the kernel run_encode / run_decode would pick
// for `a` can hold besides its bit planes without lowering the number of
// CTAs its registers allow per SM.  Callers size img_words with it: up to
// this many words the tile image (encode) or staged stream (decode) costs no
// occupancy.
template <typename S, int D> uint32_t stage_room(const LaunchArgs& a, bool encode);

// 64-bit words of storage for `logical` words of tile image or staged stream:
// the kernels keep a spare word after every 16 (shared-memory bank spreading)
inline uint64_t image_words(uint64_t logical) { return logical + logical / 16 + 1; }

// shared memory a CTA may take for its tile image or staged stream words
// beside its bit planes (GB300 allows 227 KB per CTA, static included)
constexpr size_t kMaxTileSmem = 216 * 1024;

// shared memory the kernels keep for bit planes: 1-3D blocks only
inline size_t plane_bytes(size_t esize, int dims) { return dims <= 3 ? esize * 8 * kTile * 8 : 0; }

}  // namespace zg
