// job.h -- launch descriptors shared by the host runtime and the kernels.
//
// A launch codes one or more fields ("jobs").  Each job is cut into tiles of
// kTile zfp blocks, one block per thread of a CTA; the tiles of all jobs are
// numbered consecutively so a persistent launch can pull them from one
// counter.
#pragma once

#include <cstdint>

namespace zg {

constexpr int kTile = 128;  // zfp blocks per tile = threads per CTA

enum JobFlags : uint32_t {
  kFixedRate = 1u,   // every block takes exactly maxbits bits (offset = block * maxbits)
  kVecOk = 2u,       // full rows of 4 values can be moved with 16-byte vector accesses
  kWriteIndex = 4u,  // encode: record each block's start bit in `offsets`
  kVerify = 8u,      // decode: check every block ends where the next begins
  kVec32 = 16u,      // with kVecOk, 64-bit rows (32 bytes) are 32-byte aligned: one access per row
  kStreamHost = 32u, // encode: the stream is host memory written in place over the host link, where
                     // only whole coalesced lines go at speed: tiles are staged in shared memory
                     // whenever they fit (by the kLossyHost / kRevHost kernels)
};

enum JobStatus : uint32_t {
  kStatusOverflow = 1u,  // output would pass the end of the stream buffer
  kStatusTimeout = 2u,   // a bounded wait on a predecessor tile gave up
  kStatusIndex = 4u,     // decode: a block did not end at the recorded next offset
};

struct JobResult {
  unsigned long long end_bit;  // encode: bit after the last block
  unsigned int status;         // JobStatus bits
  unsigned int pad;
};

struct Job {
  void* field;              // element (0,0,0,0); source for encode, destination for decode
  int64_t s[4];             // strides in elements (resolved; unused axes 0)
  uint32_t n[4];            // extents (1 for unused axes)
  uint32_t nb[4];           // blocks per axis (1 for unused axes)
  uint64_t nblocks;
  uint32_t minbits, maxbits, maxprec;
  int32_t minexp;
  uint32_t flags;           // JobFlags
  uint32_t tile0;           // first tile of this job in the launch
  uint32_t ntiles;
  uint32_t pad;             // keeps the 64-bit fields below 8-byte aligned
  uint64_t* words;          // stream words, index 0 = beginning of the stream buffer
  uint64_t cap_words;       // words addressable at `words`
  uint64_t bit0;            // stream bit where the job's first block starts
  uint64_t head_word;       // encode: bits already present below bit0 in word bit0/64
  uint64_t end_bit;         // decode: bit after the last block (variable rate)
  uint64_t* offsets;        // per-block start bits (variable-rate index)
  JobResult* result;
};

// per-launch scratch in device memory, zeroed before every launch
struct LaunchScratch {
  unsigned long long* tile_state;  // per tile: 2-bit status | 62-bit bit count
  unsigned long long* side;        // per tile boundary: tail part, head part
  unsigned int* side_cnt;          // per tile boundary: arrivals
  unsigned int* ticket;            // next tile to hand out
  long long wait_cycles;           // bound on each look-back wait, in SM clock cycles (0: kDefaultWaitCycles)
};

// ~2 s at GB300 clocks: a predecessor tile that has not published its bit
// count by then is taken to be lost, and the launch fails instead of hanging
constexpr long long kDefaultWaitCycles = 4000000000ll;

inline size_t scratch_bytes(uint32_t total_tiles) {
  const size_t t = (size_t)total_tiles + 1;
  return t * 8 + t * 16 + t * 4 + 64;
}

}  // namespace zg
