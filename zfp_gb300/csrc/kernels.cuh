// kernels.cuh -- encode/decode/parse kernels over tiles of zfp blocks.
//
// One CTA = one tile of kTile blocks, one block per thread (see codec.cuh).
//
// Encode of a tile:
//   gather (strided, partial blocks padded as src/template/encode.c:9-27)
//   -> prepare the block in registers -> block length (variable rate only)
//   -> CTA exclusive scan of lengths -> tile position in the stream:
//        fixed rate : tile * kTile * maxbits
//        otherwise  : decoupled look-back over predecessor tiles (bounded
//                     waits; tiles are handed out in order by a counter so a
//                     predecessor is always running or finished)
//   -> every thread writes its block into a shared-memory image of the tile
//   -> the image is shifted to the stream's bit alignment and stored with
//      coalesced 64-bit words; the two words a tile shares with its
//      neighbours are merged through a two-party handshake, never by
//      zeroing the output first.
// Decode of a tile: the tile's stream words are staged into shared memory
// with coalesced loads, each thread decodes its block from there and
// scatters it.  Block starts come from `block * maxbits` (fixed rate) or the
// index written at encode time, which the decoder verifies: a block must end
// exactly where the next one starts, which proves by induction that every
// recorded start is the true one.
#pragma once

#include <cuda_runtime.h>

#include "codec.cuh"
#include "job.h"

namespace zg {

// ---------------------------------------------------------------------------
// block coordinates, gather and scatter

__device__ __forceinline__ void block_coords(const Job& job, uint64_t b, uint32_t (&c)[4]) {
  if (job.nblocks <= 0xffffffffull) {
    uint32_t r = (uint32_t)b;
    c[0] = r % job.nb[0]; r /= job.nb[0];
    c[1] = r % job.nb[1]; r /= job.nb[1];
    c[2] = r % job.nb[2]; r /= job.nb[2];
    c[3] = r;
  } else {
    uint64_t r = b;
    c[0] = (uint32_t)(r % job.nb[0]); r /= job.nb[0];
    c[1] = (uint32_t)(r % job.nb[1]); r /= job.nb[1];
    c[2] = (uint32_t)(r % job.nb[2]); r /= job.nb[2];
    c[3] = (uint32_t)r;
  }
}

// position i of a partial block row holding cnt valid values reads source
// index i (i < cnt), else the padding pattern [a], [a b b a], [a b c a]
__device__ __forceinline__ int pad_index(int i, int cnt) {
  return i < cnt ? i : (cnt == 2 && i == 2) ? 1 : 0;
}

template <typename B, int D>
__device__ __forceinline__ void gather(const Job& job, uint64_t b, B (&raw)[1 << (2 * D)]) {
  constexpr int N = 1 << (2 * D);
  constexpr int EX = 4, EY = D >= 2 ? 4 : 1, EZ = D >= 3 ? 4 : 1, EW = D >= 4 ? 4 : 1;
  uint32_t c[4];
  block_coords(job, b, c);
  const int64_t s0 = job.s[0], s1 = job.s[1], s2 = job.s[2], s3 = job.s[3];
  const B* base = (const B*)job.field + (int64_t)(4 * c[0]) * s0 + (int64_t)(4 * c[1]) * s1 +
                  (int64_t)(4 * c[2]) * s2 + (int64_t)(4 * c[3]) * s3;
  int cnt[4];
  bool full = true;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const uint32_t left = job.n[a] - 4 * c[a];
    cnt[a] = a < D ? (left < 4 ? (int)left : 4) : 1;
    full &= a >= D || cnt[a] == 4;
  }
  if (full && (job.flags & kVecOk)) {
#pragma unroll (N <= 64 ? N / 4 : 1)
    for (int r = 0; r < N / 4; r++) {
      const int y = r & 3, z = (r >> 2) & 3, w = r >> 4;
      const B* row = base + y * s1 + z * s2 + w * s3;
      if constexpr (sizeof(B) == 4) {
        const uint4 q = __ldg((const uint4*)row);
        raw[4 * r + 0] = q.x; raw[4 * r + 1] = q.y; raw[4 * r + 2] = q.z; raw[4 * r + 3] = q.w;
      } else if (job.flags & kVec32) {
        const ulonglong4_32a q = *(const ulonglong4_32a*)row;
        raw[4 * r + 0] = q.x; raw[4 * r + 1] = q.y; raw[4 * r + 2] = q.z; raw[4 * r + 3] = q.w;
      } else {
        const ulonglong2 q0 = __ldg((const ulonglong2*)row);
        const ulonglong2 q1 = __ldg((const ulonglong2*)row + 1);
        raw[4 * r + 0] = q0.x; raw[4 * r + 1] = q0.y; raw[4 * r + 2] = q1.x; raw[4 * r + 3] = q1.y;
      }
    }
  } else if (full) {
#pragma unroll (N <= 64 ? EW : 1)
    for (int w = 0; w < EW; w++)
#pragma unroll (N <= 64 ? EZ : 1)
      for (int z = 0; z < EZ; z++)
#pragma unroll (N <= 64 ? EY : 1)
        for (int y = 0; y < EY; y++)
#pragma unroll
          for (int x = 0; x < EX; x++)
            raw[x + 4 * y + 16 * z + 64 * w] = __ldg(base + x * s0 + y * s1 + z * s2 + w * s3);
  } else {
#pragma unroll (N <= 64 ? EW : 1)
    for (int w = 0; w < EW; w++)
#pragma unroll (N <= 64 ? EZ : 1)
      for (int z = 0; z < EZ; z++)
#pragma unroll (N <= 64 ? EY : 1)
        for (int y = 0; y < EY; y++)
#pragma unroll
          for (int x = 0; x < EX; x++)
            raw[x + 4 * y + 16 * z + 64 * w] =
                __ldg(base + pad_index(x, cnt[0]) * s0 + pad_index(y, cnt[1]) * s1 +
                      pad_index(z, cnt[2]) * s2 + pad_index(w, cnt[3]) * s3);
  }
}

template <typename B, int D>
__device__ __forceinline__ void scatter(const Job& job, uint64_t b, const B (&raw)[1 << (2 * D)]) {
  constexpr int N = 1 << (2 * D);
  constexpr int EX = 4, EY = D >= 2 ? 4 : 1, EZ = D >= 3 ? 4 : 1, EW = D >= 4 ? 4 : 1;
  uint32_t c[4];
  block_coords(job, b, c);
  const int64_t s0 = job.s[0], s1 = job.s[1], s2 = job.s[2], s3 = job.s[3];
  B* base = (B*)job.field + (int64_t)(4 * c[0]) * s0 + (int64_t)(4 * c[1]) * s1 +
            (int64_t)(4 * c[2]) * s2 + (int64_t)(4 * c[3]) * s3;
  int cnt[4];
  bool full = true;
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const uint32_t left = job.n[a] - 4 * c[a];
    cnt[a] = a < D ? (left < 4 ? (int)left : 4) : 1;
    full &= a >= D || cnt[a] == 4;
  }
  if (full && (job.flags & kVecOk)) {
#pragma unroll (N <= 64 ? N / 4 : 1)
    for (int r = 0; r < N / 4; r++) {
      const int y = r & 3, z = (r >> 2) & 3, w = r >> 4;
      B* row = base + y * s1 + z * s2 + w * s3;
      if constexpr (sizeof(B) == 4) {
        *(uint4*)row = make_uint4(raw[4 * r + 0], raw[4 * r + 1], raw[4 * r + 2], raw[4 * r + 3]);
      } else if (job.flags & kVec32) {
        // one 32-byte store per row: a warp's row stores then fill whole
        // sectors, which matters when the field is host memory
        ulonglong4_32a q;
        q.x = raw[4 * r + 0]; q.y = raw[4 * r + 1]; q.z = raw[4 * r + 2]; q.w = raw[4 * r + 3];
        *(ulonglong4_32a*)row = q;
      } else {
        ((ulonglong2*)row)[0] = make_ulonglong2(raw[4 * r + 0], raw[4 * r + 1]);
        ((ulonglong2*)row)[1] = make_ulonglong2(raw[4 * r + 2], raw[4 * r + 3]);
      }
    }
  } else if (full) {
#pragma unroll (N <= 64 ? EW : 1)
    for (int w = 0; w < EW; w++)
#pragma unroll (N <= 64 ? EZ : 1)
      for (int z = 0; z < EZ; z++)
#pragma unroll (N <= 64 ? EY : 1)
        for (int y = 0; y < EY; y++)
#pragma unroll
          for (int x = 0; x < EX; x++)
            base[x * s0 + y * s1 + z * s2 + w * s3] = raw[x + 4 * y + 16 * z + 64 * w];
  } else {
    // fixed trip counts with predicated stores keep raw[] in registers
#pragma unroll (N <= 64 ? EW : 1)
    for (int w = 0; w < EW; w++)
#pragma unroll (N <= 64 ? EZ : 1)
      for (int z = 0; z < EZ; z++)
#pragma unroll (N <= 64 ? EY : 1)
        for (int y = 0; y < EY; y++)
#pragma unroll
          for (int x = 0; x < EX; x++)
            if (x < cnt[0] && y < cnt[1] && z < cnt[2] && w < cnt[3])
              base[x * s0 + y * s1 + z * s2 + w * s3] = raw[x + 4 * y + 16 * z + 64 * w];
  }
}

// ---------------------------------------------------------------------------
// shared-memory bit sink: a block starts at an arbitrary bit of the tile
// image; its first and last words may be shared with neighbouring blocks and
// are combined with atomicOr, every word in between belongs to it alone.
// The image is zeroed beforehand, so padding only moves the cursor.

// Tile images and staged stream words are stored with one spare 64-bit word
// after every 16: a block of 512 bits (rate 8 in 3D) would otherwise put the
// same word of every thread's block in the same shared-memory bank.  The
// logical word w lives at img_phys(w); a buffer of `phys` words holds
// img_cap(phys) logical words.
__host__ __device__ constexpr uint32_t img_phys(uint32_t w) { return w + (w >> 4); }
__host__ __device__ constexpr uint32_t img_cap(uint32_t phys) { return (uint32_t)((uint64_t)phys * 16 / 17); }


// atomic OR of a 64-bit word as two 32-bit atomics (the 32-bit ones are
// native shared-memory operations), skipping empty halves
__device__ __forceinline__ void or_shared(uint64_t* p, uint64_t v) {
  if ((uint32_t)v) atomicOr((unsigned*)p, (unsigned)v);
  if (v >> 32) atomicOr((unsigned*)p + 1, (unsigned)(v >> 32));
}

struct SmemSink {
  uint64_t* buf;
  uint32_t word;
  unsigned fill;
  uint64_t acc;
  bool first;
  uint32_t cap;       // words in the image; stores past it are dropped and flagged
  unsigned* status;

  __device__ __forceinline__ void store(uint64_t w) {
    if (word >= cap) {
      atomicOr(status, (unsigned)kStatusOverflow);
      word++;
      return;
    }
    if (first) {
      or_shared(&buf[img_phys(word)], w);
      first = false;
    } else {
      buf[img_phys(word)] = w;
    }
    word++;
  }
  // v must have no bits at or above n
  __device__ __forceinline__ void put(uint64_t v, unsigned n) {
    acc |= v << fill;
    const unsigned t = fill + n;
    if (t >= 64) {
      store(acc);
      acc = fill ? v >> (64 - fill) : 0;
      fill = t - 64;
    } else {
      fill = t;
    }
  }
  __device__ __forceinline__ void pad(unsigned n) {
    const unsigned t = fill + n;
    if (t >= 64) {
      store(acc);
      acc = 0;
      word += t / 64 - 1;
      fill = t % 64;
    } else {
      fill = t;
    }
  }
  __device__ __forceinline__ void finish() {
    if (!fill) return;
    if (word < cap) or_shared(&buf[img_phys(word)], acc);
    else atomicOr(status, (unsigned)kStatusOverflow);
  }
};

// One block written straight into the stream from bit `fill` of word
// `dst` on; the caller has checked that the block's words lie inside the
// stream buffer.  Words the block covers whole are stored; its first word,
// when it starts inside it, and its last word, when it ends inside it, hold
// bits of the neighbouring blocks too: those are OR-ed into the tile's seam
// table (shared memory, entries at shared addresses `head` and `tail`) and
// stored once every block of the tile has added its part.
constexpr uint32_t kNoSeam = ~0u;

// (no "memory" clobber: the barrier after the tile's blocks orders these
// with the reads of the table, and the coder's loads of its bit planes stay
// free to be scheduled around them)
__device__ __forceinline__ void seam_or(uint32_t addr, uint64_t v) {
  asm volatile("red.shared.or.b64 [%0], %1;" ::"r"(addr), "l"(v));
}

struct SeamSink {
  uint64_t* dst;
  unsigned fill;
  uint64_t acc;
  uint32_t head;      // kNoSeam when the block starts on a word
  uint32_t tail;

  __device__ __forceinline__ void store(uint64_t w) {
    if (head != kNoSeam) {
      seam_or(head, w);
      head = kNoSeam;
    } else {
      *dst = w;
    }
    dst++;
  }
  // v must have no bits at or above n
  __device__ __forceinline__ void put(uint64_t v, unsigned n) {
    acc |= v << fill;
    const unsigned t = fill + n;
    if (t >= 64) {
      store(acc);
      acc = fill ? v >> (64 - fill) : 0;
      fill = t - 64;
    } else {
      fill = t;
    }
  }
  __device__ __forceinline__ void pad(unsigned n) {
    unsigned t = fill + n;
    while (t >= 64) {
      store(acc);
      acc = 0;
      t -= 64;
    }
    fill = t;
  }
  // a block ending inside the word that it starts inside has the same entry
  // for both
  __device__ __forceinline__ void finish() {
    if (fill) seam_or(tail, acc);
  }
};

// ---------------------------------------------------------------------------
// CTA-wide exclusive scan of one value per thread

__device__ __forceinline__ uint32_t cta_exclusive_scan(uint32_t v, uint32_t& total, uint32_t* s_warp) {
  const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= (unsigned)o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  uint32_t before = 0, sum = 0;
#pragma unroll
  for (int w = 0; w < kTile / 32; w++) {
    const uint32_t t = s_warp[w];
    before += (unsigned)w < warp ? t : 0;
    sum += t;
  }
  total = sum;
  return before + x - v;
}

// ---------------------------------------------------------------------------
// decoupled look-back (variable-rate streams)

constexpr unsigned long long kStateAgg = 1ull << 62;
constexpr unsigned long long kStateIncl = 2ull << 62;
constexpr unsigned long long kStateValue = (1ull << 62) - 1;

__device__ __forceinline__ void publish_state(unsigned long long* slot, unsigned long long v) {
  __threadfence();
  *(volatile unsigned long long*)slot = v;
}

// The tile's own bit total, published by one thread as soon as it is known
// (the job's first tile publishes it as its inclusive prefix).
__device__ __forceinline__ void publish_aggregate(const Job& job, const LaunchScratch& sc, uint32_t gt,
                                                  uint64_t aggregate) {
  publish_state(sc.tile_state + gt, (gt == job.tile0 ? kStateIncl : kStateAgg) | aggregate);
}

// Called by all lanes of one warp after publish_aggregate.  Returns the
// number of stream bits taken by the job's tiles before `gt`.
__device__ __forceinline__ uint64_t look_back(const Job& job, const LaunchScratch& sc, uint32_t gt,
                                              uint64_t aggregate) {
  const unsigned lane = threadIdx.x & 31;
  if (gt == job.tile0) return 0;
  uint64_t exclusive = 0;
  int64_t pred = (int64_t)gt - 1 - lane;
  const long long t0 = clock64();
  const long long wait_limit = sc.wait_cycles > 0 ? sc.wait_cycles : kDefaultWaitCycles;
  bool timed_out = false;
  for (;;) {
    unsigned long long st = kStateIncl;  // before the job's first tile: inclusive 0
    if (pred >= (int64_t)job.tile0) {
      const volatile unsigned long long* slot = sc.tile_state + pred;
      st = *slot;
      while (!(st >> 62)) {
        if (clock64() - t0 > wait_limit) {
          timed_out = true;
          st = kStateIncl;
          break;
        }
        __nanosleep(32);
        st = *slot;
      }
    }
    const unsigned incl = __ballot_sync(0xffffffffu, (st >> 62) == 2);
    const unsigned limit = incl ? (unsigned)(__ffs(incl) - 1) : 31u;
    uint64_t part = lane <= limit ? (st & kStateValue) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    exclusive += part;
    if (incl) break;
    pred -= 32;
  }
  if (__any_sync(0xffffffffu, timed_out) && lane == 0) atomicOr(&job.result->status, (unsigned)kStatusTimeout);
  if (lane == 0) publish_state(sc.tile_state + gt, kStateIncl | (exclusive + aggregate));
  return exclusive;
}

// ---------------------------------------------------------------------------
// tile image -> stream words

__device__ __forceinline__ void store_word(const Job& job, uint64_t w, uint64_t v) {
  if (w < job.cap_words) job.words[w] = v;
  else atomicOr(&job.result->status, (unsigned)kStatusOverflow);
}

// a word shared by tiles t-1 (low part) and t (high part): whoever arrives
// second stores the union
__device__ __forceinline__ void merge_word(const Job& job, const LaunchScratch& sc, uint32_t t,
                                           int part, uint64_t w, uint64_t v) {
  sc.side[2 * (size_t)t + part] = v;
  __threadfence();
  if (atomicAdd(&sc.side_cnt[t], 1u) == 1u) {
    __threadfence();
    v |= *(volatile unsigned long long*)&sc.side[2 * (size_t)t + (1 - part)];
    store_word(job, w, v);
  }
}

__device__ __forceinline__ void write_tile(const Job& job, const LaunchScratch& sc, uint32_t lt, uint32_t gt,
                                           const uint64_t* img, uint32_t nimg, uint64_t G, uint32_t total) {
  const uint64_t E = G + total;
  const uint64_t hw = G >> 6, tw = E >> 6;
  const unsigned sh = (unsigned)(G & 63), te = (unsigned)(E & 63);
  const bool first = lt == 0, last = lt + 1 == job.ntiles;
  // A tile codes no bits only when every block of the job does (maxbits 0):
  // then nothing but the caller's bits ahead of the stream goes out.
  if (!total) {
    if (first && sh && threadIdx.x == 0) store_word(job, hw, job.head_word & ((1ull << sh) - 1));
    return;
  }
  const uint32_t cnt = (uint32_t)((te ? tw + 1 : tw) - hw);   // stream words this tile touches
  const bool in_bounds = hw + cnt <= job.cap_words;
  // stream word hw + j: image word j shifted up by sh, with the top of word j - 1 below
  auto word = [&](uint32_t j) -> uint64_t {
    const uint64_t cur = j < nimg ? img[img_phys(j)] : 0ull;
    if (!sh) return cur;
    const uint64_t prev = j && j - 1 < nimg ? img[img_phys(j - 1)] : 0ull;
    return (cur << sh) | (prev >> (64 - sh));
  };
  // a tile that does not start (end) on a word shares its first (last) word
  // with the previous (next) tile of the job; every word in between is its
  // own.  Otherwise every block codes at least one bit, a tile other than a
  // job's last holds at least 128 bits, and those two shared words are
  // distinct.
  const uint32_t jlo = sh ? 1u : 0u;
  const uint32_t jhi = te && !last ? cnt - 1 : cnt;
  for (uint32_t j = jlo + threadIdx.x; j < jhi; j += kTile) {
    const uint64_t v = word(j);
    if (in_bounds) job.words[hw + j] = v;
    else store_word(job, hw + j, v);
  }
  if (threadIdx.x == 0 && sh) {
    const uint64_t v = word(0);
    if (first) store_word(job, hw, v | (job.head_word & ((1ull << sh) - 1)));
    else merge_word(job, sc, gt, 1, hw, v);
  }
  if (threadIdx.x == kTile - 1 && te && !last) merge_word(job, sc, gt + 1, 0, tw, word(cnt - 1));
}

// ---------------------------------------------------------------------------
// encode one tile

// Variable-rate tiles of more code than this are written straight into the
// stream even where the image would hold them: their blocks, each tens of
// words apart, store into the image with many bank conflicts, and the
// look-back that direct writing waits for is spread over more work.
constexpr uint32_t kStageMaxWords = 2048;

// Bit planes first (with each block's length, for variable rates), then the
// tile's place in the stream: its first bit G follows from the tile number
// at a fixed rate, else from the decoupled look-back.
//
// A variable-rate tile whose code fits the shared-memory image (`img`,
// `img_words` words) and kStageMaxWords is coded there while the look-back
// runs, and copied out at G by write_tile: the look-back's wait for the
// tiles before it overlaps the coding.  The host-stream kernels stage every
// tile the image holds, fixed-rate and large ones included, so that only
// whole lines cross the host link.
//
// Every other tile -- fixed-rate ones, whose G needs no look-back, and
// variable-rate ones too large for the image or the cap -- is coded
// straight into the stream (SeamSink).  Boundary i of the tile (block i's first bit; boundary
// nb is the tile's end) lies in stream word W_i; a word holding a boundary
// inside it is shared, and its seam entry is that of the first boundary in
// the word.  Blocks of 64 bits or more put every boundary in a word of its
// own; shorter ones (zero blocks of the lossy modes) can put several in
// one, found through the table of the boundaries' words.  The first and
// last words of the tile may be shared with the neighbouring tiles of the
// job: those go through merge_word.
template <typename S, int D, int kSel>
__device__ __forceinline__ void encode_tile(const Job& job, const LaunchScratch& sc, uint32_t gt, uint64_t* img,
                                            uint32_t img_words, uint64_t* planes, const uint32_t* gtab) {
  using B = typename Traits<S>::Bits;
  using U = typename Traits<S>::UInt;
  constexpr int N = 1 << (2 * D);
  constexpr int P = 8 * sizeof(U);
  __shared__ uint32_t s_warp[kTile / 32];
  __shared__ unsigned long long s_base;
  __shared__ unsigned long long s_seam[kTile + 1];
  __shared__ uint32_t s_word[kTile + 1];   // W_i - W_0, when a tile has blocks under 64 bits
  const uint32_t lt = gt - job.tile0;
  const uint32_t bi = threadIdx.x;
  const uint64_t b = (uint64_t)lt * kTile + bi;
  const bool active = b < job.nblocks;
  const uint64_t left = job.nblocks - (uint64_t)lt * kTile;
  const uint32_t nb = left < kTile ? (uint32_t)left : kTile;
  const bool fixed = kSel == kFixedOnly || (job.flags & kFixedRate);
  const bool first = lt == 0, last = lt + 1 == job.ntiles;
  const BlockParams p{job.minbits, job.maxbits, job.maxprec, job.minexp};
  uint64_t* my_planes = planes + bi;   // plane k of this block at my_planes[k * kTile]

  uint32_t len = 0;
  BlockHead h;
  [[maybe_unused]] WideCode<S> wc;  // 4D only (local memory)
  if (active) {
    B raw[N];
    gather<B, D>(job, b, raw);
    if constexpr (N <= 64) {
      U u[N];
      prepare_coeffs<S, D, kSel>(h, p, raw, u);
      if (h.coded) store_planes<N, kSel == kLossyFloor>(u, my_planes, kTile, h.maxprec);
      len = fixed ? job.maxbits : block_bits<P, N>(h, my_planes, kTile);
    } else {
      U u[N];
      prepare_coeffs<S, D, kSel>(wc.h, p, raw, u);
      wc.set(u);
      len = fixed ? job.maxbits : wc.length();
    }
  }
  uint32_t total;
  const uint32_t excl = cta_exclusive_scan(len, total, s_warp);
  if (bi == 0) {
    if (fixed) s_base = (unsigned long long)lt * kTile * job.maxbits;
    else publish_aggregate(job, sc, gt, total);
  }

  const uint32_t need = (total + 63) / 64 + 1;
  // The fixed-precision kernel is launched only where the image holds the
  // largest possible tile (see with_encoder), so it is built with this path
  // alone: measured 6% faster at precision 20 than with both paths.
  constexpr bool kStagedOnly = kSel == kLossyFloor;
  // fixed-rate and large tiles are staged only by the host-stream kernels,
  // whose stream is written across the host link: making the path
  // reachable for fixed-rate tiles cost the device-memory fp64 encoder 8%
  // through its register allocation
  constexpr bool kHost = kSel == kLossyHost || kSel == kRevHost;
  const bool stage = !fixed || kHost;
  if (kStagedOnly || (stage && total && need <= img_cap(img_words) && (kHost || need <= kStageMaxWords))) {
    const uint32_t nw = kStagedOnly ? min(need, img_cap(img_words)) : need;   // stores past it are flagged
    for (uint32_t i = bi; i < nw; i += kTile) img[img_phys(i)] = 0;
    __syncthreads();
    if (active) {
      SmemSink out{img, excl >> 6, excl & 63u, 0ull, true, nw, &job.result->status};
      if constexpr (N <= 64) emit_block_seq<P, N>(out, h, my_planes, kTile, gtab);
      else wc.emit(out, gtab);
      out.finish();
    }
    // the last warp resolves the tile's place after its own blocks, by when
    // the tiles before have mostly published theirs
    if (!fixed && bi >= kTile - 32) {
      const uint64_t before = look_back(job, sc, gt, total);
      if (bi == kTile - 32) s_base = before;
    }
    __syncthreads();
    const uint64_t G = job.bit0 + s_base;
    write_tile(job, sc, lt, gt, img, nw, G, total);
    if (active && (job.flags & kWriteIndex)) job.offsets[b] = G + excl;
    if (bi == 0 && last) job.result->end_bit = G + total;
    return;
  }

  s_seam[bi] = 0;
  if (bi == 0) s_seam[kTile] = 0;
  if (!fixed && bi >= kTile - 32) {
    const uint64_t before = look_back(job, sc, gt, total);
    if (bi == kTile - 32) s_base = before;
  }
  const bool small = __syncthreads_or(active && len < 64);

  const uint64_t G = job.bit0 + s_base, E = G + total;
  const uint64_t pos = G + excl, end = pos + len;
  if (active && (job.flags & kWriteIndex)) job.offsets[b] = pos;
  if (bi == 0 && last) job.result->end_bit = E;
  // A block codes no bits only when every block of the job does (maxbits
  // 0): then nothing but the caller's bits ahead of the stream goes out.
  // Otherwise every block has a bit at least.
  if (!total) {
    if (bi == 0 && first && (G & 63)) store_word(job, G >> 6, job.head_word & ((1ull << (G & 63)) - 1));
    return;
  }
  // seam entries of this block's boundaries (its first bit and its end)
  uint32_t lo = bi, hi = bi + 1;
  if (small) {
    const uint64_t w0 = G >> 6;
    if (active) s_word[bi] = (uint32_t)((pos >> 6) - w0);
    if (bi + 1 == nb) s_word[nb] = (uint32_t)((E >> 6) - w0);
    __syncthreads();
    if (active) {
      const uint32_t w = s_word[bi];
      while (lo && s_word[lo - 1] == w) lo--;
      hi = s_word[bi + 1] == w ? lo : bi + 1;
    }
  }

  if (active) {
    if ((end + 63) >> 6 <= job.cap_words) {
      const uint32_t seam0 = (uint32_t)__cvta_generic_to_shared(s_seam);
      SeamSink out{job.words + (pos >> 6), (unsigned)(pos & 63), 0ull, (pos & 63) ? seam0 + 8 * lo : kNoSeam,
                   seam0 + 8 * hi};
      if constexpr (N <= 64) emit_block_seq<P, N>(out, h, my_planes, kTile, gtab);
      else wc.emit(out, gtab);
      out.finish();
    } else {
      atomicOr(&job.result->status, (unsigned)kStatusOverflow);
    }
  }
  __syncthreads();

  // shared words out: each by the first boundary in it
  auto seam_out = [&](uint32_t i, uint64_t w, uint64_t v) {
    const unsigned sh = (unsigned)(G & 63);
    if (i == 0 && sh) {
      if (first) store_word(job, w, v | (job.head_word & ((1ull << sh) - 1)));
      else merge_word(job, sc, gt, 1, w, v);
    } else if (w == (E >> 6) && (E & 63) && !last) {
      merge_word(job, sc, gt + 1, 0, w, v);
    } else {
      store_word(job, w, v);
    }
  };
  if (active) {
    if (lo == bi && ((pos & 63) || hi == lo)) seam_out(bi, pos >> 6, s_seam[bi]);
    if (bi + 1 == nb && hi == nb && (end & 63)) seam_out(nb, end >> 6, s_seam[nb]);
  }
}

// dynamic shared memory for the bit planes of one tile (1-3D blocks)
template <typename S, int D, bool kEncode>
constexpr size_t plane_smem_bytes() {
  return (1 << (2 * D)) <= 64 ? (size_t)8 * sizeof(typename Traits<S>::UInt) * kTile * 8 : 0;
}

// 64-bit 2D/3D blocks whose coded planes all lie in the top half (maxprec <=
// 32: every lossy mode but high precision) never touch planes 0-31 -- the
// encoder transposes only the high words and the decoder keeps `top_only`
// -- so a single-job launch gives them only the upper half of the plane
// buffer.  Kernels of mode kLossyFloor (chosen for fixed-precision jobs)
// skip every plane below P - maxprec and get maxprec planes.  Host and
// kernel decide both from the same job.
template <typename S, int D>
ZG_HD constexpr bool half_planes(unsigned maxprec) {
  return sizeof(typename Traits<S>::UInt) == 8 && D >= 2 && D <= 3 && maxprec <= 32;
}

template <typename S, int D, bool kFloorKernel>
ZG_HD constexpr unsigned plane_floor(bool multi, unsigned maxprec) {
  constexpr unsigned P = 8 * sizeof(typename Traits<S>::UInt);
  return multi ? 0u : kFloorKernel ? (maxprec < P ? P - maxprec : 0u) : half_planes<S, D>(maxprec) ? 32u : 0u;
}

// the decoder of 64-bit 2D and 3D blocks works through 32 planes at a time
// (uncode_coeffs), whatever the job
template <typename S, int D>
ZG_HD constexpr bool half_decode_planes() {
  return sizeof(typename Traits<S>::UInt) == 8 && (D == 2 || D == 3);
}

template <typename S, int D, bool kEncode, bool kFloorKernel = false>
ZG_HD constexpr size_t plane_smem_bytes(bool multi, unsigned maxprec) {
  constexpr unsigned P = 8 * sizeof(typename Traits<S>::UInt);
  return !kEncode && half_decode_planes<S, D>()
             ? plane_smem_bytes<S, D, kEncode>() / 2
             : plane_smem_bytes<S, D, kEncode>() / P * (P - plane_floor<S, D, kFloorKernel>(multi, maxprec));
}

// plane k of thread 0 at planes[k * kTile]: the buffer starts at the floor
template <typename S, int D, bool kMulti, int kSel>
__device__ __forceinline__ uint64_t* plane_base(uint64_t* buf, const Job& one) {
  return buf - (size_t)plane_floor<S, D, kSel == kLossyFloor>(kMulti, one.maxprec) * kTile;
}

// ---------------------------------------------------------------------------
// decode one tile

template <typename S, int D, int kSel>
__device__ __forceinline__ void decode_tile(const Job& job, uint32_t gt, uint64_t* img, uint32_t img_words,
                                            uint64_t* planes) {
  using B = typename Traits<S>::Bits;
  constexpr int N = 1 << (2 * D);
  const uint32_t lt = gt - job.tile0;
  const uint64_t b0 = (uint64_t)lt * kTile;
  const uint64_t b = b0 + threadIdx.x;
  const bool active = b < job.nblocks;
  const bool fixed = kSel == kFixedOnly || (job.flags & kFixedRate);
  const uint64_t nblk = job.nblocks - b0 < (uint64_t)kTile ? job.nblocks - b0 : (uint64_t)kTile;

  uint64_t Gs, Ge, start = 0, expect = 0;
  if (fixed) {
    Gs = job.bit0 + b0 * job.maxbits;
    Ge = Gs + nblk * job.maxbits;
    start = Gs + (uint64_t)threadIdx.x * job.maxbits;
  } else {
    Gs = job.offsets[b0];
    Ge = b0 + nblk < job.nblocks ? job.offsets[b0 + nblk] : job.end_bit;
    if (active) {
      start = job.offsets[b];
      expect = b + 1 < job.nblocks ? job.offsets[b + 1] : job.end_bit;
    }
  }
  const uint64_t w0 = Gs >> 6;
  const uint64_t nwords = Ge >= Gs ? ((Ge + 63) >> 6) - w0 + 2 : ~0ull;
  const bool staged = nwords <= img_cap(img_words);
  if (staged) {
    for (uint64_t i = threadIdx.x; i < nwords; i += kTile)
      img[img_phys((uint32_t)i)] = w0 + i < job.cap_words ? __ldg((const unsigned long long*)job.words + w0 + i) : 0ull;
  } else {
    // each thread walks its block's words one dependent load at a time:
    // bring the tile's lines into L2 first (16 words a line)
    for (uint64_t i = 16 * threadIdx.x; i < nwords && w0 + i < job.cap_words; i += 16 * kTile)
      asm volatile("prefetch.global.L2 [%0];" ::"l"(__cvta_generic_to_global(job.words + w0 + i)));
  }
  __syncthreads();
  if (!active) return;

  const BlockParams p{job.minbits, job.maxbits, job.maxprec, job.minexp};
  const PlaneBuf pb{planes + threadIdx.x, kTile};
  B raw[N];
  uint64_t end;
  if (staged) {
    SharedSource in;
    in.base = img;
    in.cap = nwords;
    in.seek(start - (w0 << 6));
    decode_block<S, D, kSel>(in, p, raw, pb);
    end = in.tell() + (w0 << 6);
  } else {
    WordSource in;
    in.base = job.words;
    in.cap = job.cap_words;
    in.seek(start);
    decode_block<S, D, kSel>(in, p, raw, pb);
    end = in.tell();
  }
  if ((job.flags & kVerify) && end != expect) atomicOr(&job.result->status, (unsigned)kStatusIndex);
  scatter<B, D>(job, b, raw);
}

// ---------------------------------------------------------------------------
// kernels.  A launch covers `total_tiles` tiles of one job (passed by value)
// or of several jobs (device array, sorted by tile0).  With `use_ticket` the
// CTAs pull tiles from a counter in order; otherwise tile = blockIdx.x.

template <bool kMulti>
__device__ __forceinline__ const Job* resolve_job(const Job& one, const Job* jobs, int njobs, uint32_t gt, Job* s_job) {
  if (!kMulti) return &one;
  if (threadIdx.x == 0) {
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].tile0 <= gt) lo = mid;
      else hi = mid - 1;
    }
    *s_job = jobs[lo];
  }
  __syncthreads();
  return s_job;
}

template <typename S, int D, bool kMulti, int kSel>
__device__ __forceinline__ void encode_body(const Job& one, const Job* jobs, int njobs, const LaunchScratch& sc,
                                            uint32_t total_tiles, int use_ticket, uint32_t img_words) {
  extern __shared__ uint64_t smem_img[];
  uint64_t* planes = plane_base<S, D, kMulti, kSel>(smem_img + img_words, one);
  __shared__ uint32_t s_tile;
  __shared__ Job s_job;
  __shared__ uint32_t s_gtab[256];   // group-test codes of every byte (emit_block_seq)
  for (uint32_t i = threadIdx.x; i < 256; i += kTile) s_gtab[i] = group_code_entry(i);
  for (uint32_t iter = blockIdx.x;; iter += gridDim.x) {
    if (threadIdx.x == 0) s_tile = use_ticket ? atomicAdd(sc.ticket, 1u) : iter;
    __syncthreads();
    const uint32_t gt = s_tile;
    if (gt >= total_tiles) break;
    const Job* job = resolve_job<kMulti>(one, jobs, njobs, gt, &s_job);
    encode_tile<S, D, kSel>(*job, sc, gt, smem_img, img_words, planes, s_gtab);
    __syncthreads();
  }
}

template <typename S, int D, bool kMulti, int kSel>
__global__ void __launch_bounds__(kTile) encode_kernel(const __grid_constant__ Job one, const Job* jobs, int njobs,
                                                       LaunchScratch sc, uint32_t total_tiles, int use_ticket,
                                                       uint32_t img_words) {
  encode_body<S, D, kMulti, kSel>(one, jobs, njobs, sc, total_tiles, use_ticket, img_words);
}

// The same encoder held to more CTAs per SM (see decode_kernel_occ).
template <typename S, int D, bool kMulti, int kSel, int kMinCtas>
__global__ void __launch_bounds__(kTile, kMinCtas) encode_kernel_occ(const __grid_constant__ Job one, const Job* jobs,
                                                                     int njobs, LaunchScratch sc, uint32_t total_tiles,
                                                                     int use_ticket, uint32_t img_words) {
  encode_body<S, D, kMulti, kSel>(one, jobs, njobs, sc, total_tiles, use_ticket, img_words);
}

// img_words: shared memory for staging a tile's stream words; tiles that do
// not fit are read from the stream directly
template <typename S, int D, bool kMulti, int kSel>
__device__ __forceinline__ void decode_body(const Job& one, const Job* jobs, int njobs, uint32_t total_tiles,
                                            uint32_t img_words) {
  extern __shared__ uint64_t smem_img[];
  uint64_t* img = smem_img;
  uint64_t* planes = half_decode_planes<S, D>() ? smem_img + img_words
                                                : plane_base<S, D, kMulti, kSel>(smem_img + img_words, one);
  __shared__ Job s_job;
  for (uint32_t gt = blockIdx.x; gt < total_tiles; gt += gridDim.x) {
    const Job* job = resolve_job<kMulti>(one, jobs, njobs, gt, &s_job);
    decode_tile<S, D, kSel>(*job, gt, img, img_words, planes);
    __syncthreads();
  }
}

template <typename S, int D, bool kMulti, int kSel>
__global__ void __launch_bounds__(kTile) decode_kernel(const __grid_constant__ Job one, const Job* jobs, int njobs,
                                                       uint32_t total_tiles, uint32_t img_words) {
  decode_body<S, D, kMulti, kSel>(one, jobs, njobs, total_tiles, img_words);
}

// The same decoder held to more CTAs per SM.  Three (168 registers) for
// 64-bit lossy blocks and 32-bit reversible blocks, where the compiler's own
// choice (about 180 registers, two CTAs) leaves the SM short of warps:
// measured 10-17% faster on the former.  Five (96
// registers) for 32-bit fixed-rate blocks whose tile fits the smaller
// shared-memory share: measured 10% faster at rate 8.
template <typename S, int D, bool kMulti, int kSel, int kMinCtas>
__global__ void __launch_bounds__(kTile, kMinCtas) decode_kernel_occ(const __grid_constant__ Job one, const Job* jobs,
                                                                     int njobs, uint32_t total_tiles,
                                                                     uint32_t img_words) {
  decode_body<S, D, kMulti, kSel>(one, jobs, njobs, total_tiles, img_words);
}

// Recover block offsets of a variable-rate stream that carries no index by
// walking it block after block (one thread; used only for streams this
// library did not write).
// Block offsets of a variable-rate stream that carries no index: the chain
// of block lengths is sequential, so one thread walks it with the
// length-only decoder (skip_block).  A wider window staged by the warp in
// shared memory was measured no faster: the walk is bound by its own
// dependent instructions (about 5 us per 3D block), not by memory.
template <typename S, int D>
__global__ void parse_kernel(const __grid_constant__ Job job) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const BlockParams p{job.minbits, job.maxbits, job.maxprec, job.minexp};
  WordSource in;
  in.base = job.words;
  in.cap = job.cap_words;
  in.seek(job.bit0);
  for (uint64_t b = 0; b < job.nblocks; b++) {
    job.offsets[b] = in.tell();
    skip_block<S, D>(in, p);
  }
  job.result->end_bit = in.tell();
}

// ---------------------------------------------------------------------------
// Speculative parallel parse.  A wrong start, parsed on, often lands on a
// true block boundary after a few hundred blocks, and from there on its
// boundaries are the true ones.  So:
//  1. parse_probe: one thread parses the first blocks for the mean length;
//  2. parse_spec: worker w (one thread each) starts at bit0 + w * seg and
//     records the starts of `k` consecutive blocks and the end of the last;
//  3. parse_stitch: one thread follows the true chain from bit0.  At a true
//     position it looks for that exact position among the records of the
//     workers that cover it; found, it adopts the rest of that worker's
//     records (all true: the parse is deterministic), else it parses one
//     block itself and tries again a few blocks later.
// Every adopted offset therefore follows from a position reached by the
// true chain: the result is the sequential parse's, only faster.

// a worker records the chain over this many worker spacings, so up to this
// many workers cover any position
constexpr uint32_t kParseCover = 16;

template <typename S, int D>
__global__ void parse_probe(const __grid_constant__ Job job, uint32_t count, unsigned long long* mean_bits) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const BlockParams p{job.minbits, job.maxbits, job.maxprec, job.minexp};
  WordSource in;
  in.base = job.words;
  in.cap = job.cap_words;
  in.seek(job.bit0);
  for (uint32_t b = 0; b < count; b++) skip_block<S, D>(in, p);
  *mean_bits = (in.tell() - job.bit0 + count - 1) / count;
}

template <typename S, int D>
__global__ void parse_spec(const __grid_constant__ Job job, uint64_t seg, uint32_t k, uint32_t workers,
                           unsigned long long* rec) {
  const uint32_t w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= workers) return;
  const BlockParams p{job.minbits, job.maxbits, job.maxprec, job.minexp};
  WordSource in;
  in.base = job.words;
  in.cap = job.cap_words;
  in.seek(job.bit0 + (uint64_t)w * seg);
  unsigned long long* r = rec + (size_t)w * (k + 1);
  for (uint32_t j = 0; j < k; j++) {
    r[j] = in.tell();
    skip_block<S, D>(in, p);
  }
  r[k] = in.tell();
}

// index of `pos` among the k sorted starts r[0..k), or k
__device__ __forceinline__ uint32_t find_start(const unsigned long long* r, uint32_t k, uint64_t pos) {
  uint32_t lo = 0, hi = k;
  while (lo < hi) {
    const uint32_t mid = (lo + hi) / 2;
    if (r[mid] < pos) lo = mid + 1;
    else hi = mid;
  }
  return lo < k && r[lo] == pos ? lo : k;
}

template <typename S, int D>
__global__ void parse_stitch(const __grid_constant__ Job job, uint64_t seg, uint32_t k, uint32_t workers,
                             const unsigned long long* rec) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const BlockParams p{job.minbits, job.maxbits, job.maxprec, job.minexp};
  uint64_t pos = job.bit0, b = 0;
  uint32_t miss = 0, wait = 0;   // blocks parsed here since the last search; before the next
  while (b < job.nblocks) {
    if (miss >= wait) {
      // workers that started at or before pos, latest first
      const uint64_t w_hi = (pos - job.bit0) / seg;
      bool adopted = false;
      for (uint64_t d = 0; d < kParseCover && d <= w_hi && !adopted; d++) {
        const uint64_t w = w_hi - d;
        if (w >= workers) continue;
        const unsigned long long* r = rec + (size_t)w * (k + 1);
        if (r[k] <= pos) break;   // this and earlier workers end before pos
        const uint32_t j = find_start(r, k, pos);
        if (j == k) continue;
        uint32_t i = j;
        for (; i < k && b < job.nblocks; i++) job.offsets[b++] = r[i];
        pos = r[i];   // start of the next block: the end of the last one taken
        adopted = true;
      }
      miss = 0;
      if (adopted) {
        wait = 0;
        continue;
      }
      wait = wait ? (wait < 64 ? 2 * wait : 64) : 8;   // searching again soon rarely pays
    }
    WordSource in;
    in.base = job.words;
    in.cap = job.cap_words;
    in.seek(pos);
    job.offsets[b++] = pos;
    skip_block<S, D>(in, p);
    pos = in.tell();
    miss++;
  }
  job.result->end_bit = pos;
}

}  // namespace zg
