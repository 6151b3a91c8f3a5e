// index.cu -- zfp's block-index formats (include/zfp/index.hpp) as a side
// channel for variable-rate streams.  A stream written elsewhere carries no
// block offsets, and zfp_decompress then has to recover them by parsing it;
// a caller that kept zfp's own index of the stream (a compressed array's
// verbatim, hybrid4 or hybrid8 index) can hand it over instead
// (zfp_gb300_index_import), and an index of a stream this library wrote can
// be taken out in those formats (zfp_gb300_index_export).
//
// The packing below restates the formats of index.hpp in code of our own,
// because a different packing would not be the reference's index.  Offsets
// here are bit offsets relative to the first block, nblocks + 1 of them, the
// last one being the index's range (its stream's length in bits).
#include <cuda_runtime.h>

#include <cstring>
#include <vector>

#include "../../include/zfp_gb300.h"
#include "gpu_internal.h"
#include "runtime.h"

namespace zg {
namespace {

constexpr uint64_t kMaxBlockBits = 16658;  // ZFP_MAX_BITS, include/zfp.h:19

// hybrid4 (index.hpp:160-305): records of 4 blocks, {uint32 hi; uint16 lo[4]}:
// the chunk's base offset is hi << 12 plus lo[0], block k at (hi << 12) + lo[k]
struct Hybrid4Record {
  uint32_t hi;
  uint16_t lo[4];
};
static_assert(sizeof(Hybrid4Record) == 12, "hybrid4 record is 12 bytes");
constexpr unsigned kH4Shift = 12;

// hybrid8<dims> (index.hpp:307-505): two words per 8 blocks; the chunk base
// offset splits into ptr >> 8 (top of the first word) and ptr & 255 (top
// byte of the second); below them the sizes of blocks 0-6, each split into
// hbits = 2 (dims - 1) high bits (first word) and 8 low bits (second word),
// block 0 highest.  Block 7's size is implied by the next chunk.
constexpr unsigned kH8Low = 8;
unsigned h8_high(unsigned dims) { return 2 * (dims - 1); }

size_t bytes_of(int format, size_t n) {
  switch (format) {
    case ZFP_GB300_INDEX_VERBATIM: return 8 * (n + 1);
    case ZFP_GB300_INDEX_HYBRID4: return sizeof(Hybrid4Record) * ((n + 3) / 4);
    case ZFP_GB300_INDEX_HYBRID8: return 16 * ((n + 7) / 8);
    default: return 0;
  }
}

// offset of block i (relative), blocks past n padded with zero sizes
inline uint64_t off_at(const uint64_t* off, size_t n, size_t i) { return off[i < n ? i : n]; }

const char* pack(int format, unsigned dims, const uint64_t* off, size_t n, void* out) {
  if (off[0] != 0) return "index offsets must start at 0";
  for (size_t i = 0; i < n; i++)
    if (off[i + 1] < off[i]) return "index offsets must not decrease";
  switch (format) {
    case ZFP_GB300_INDEX_VERBATIM:
      std::memcpy(out, off, 8 * (n + 1));
      return nullptr;
    case ZFP_GB300_INDEX_HYBRID4: {
      auto* rec = static_cast<Hybrid4Record*>(out);
      for (size_t c = 0; c < (n + 3) / 4; c++) {
        const uint64_t ptr = off_at(off, n, 4 * c);
        if (ptr >> (32 + kH4Shift)) return "block offset too large for a hybrid4 index";
        Hybrid4Record r;
        r.hi = (uint32_t)(ptr >> kH4Shift);
        const uint64_t base = (uint64_t)r.hi << kH4Shift;
        for (unsigned k = 0; k < 4; k++) {
          const size_t b = 4 * c + k;
          if (b < n && off[b + 1] - off[b] > kMaxBlockBits) return "block too large for a hybrid4 index";
          r.lo[k] = (uint16_t)(off_at(off, n, b) - base);
        }
        std::memcpy(rec + c, &r, sizeof r);
      }
      return nullptr;
    }
    case ZFP_GB300_INDEX_HYBRID8: {
      if (dims < 1 || dims > 4) return "hybrid8 index needs dims 1-4";
      const unsigned hb = h8_high(dims);
      auto* w = static_cast<uint64_t*>(out);
      for (size_t c = 0; c < (n + 7) / 8; c++) {
        const uint64_t ptr = off_at(off, n, 8 * c);
        const uint64_t h = ptr >> kH8Low;
        uint64_t hi = h << (7 * hb), lo = (ptr & 0xffu) << (7 * kH8Low);
        if ((hi >> (7 * hb)) != h) return "block offset too large for a hybrid8 index";
        for (unsigned k = 0; k < 8; k++) {
          const size_t b = 8 * c + k;
          const uint64_t size = b < n ? off[b + 1] - off[b] : 0;
          if (size >> (hb + kH8Low)) return "block too large for a hybrid8 index";
          if (k < 7) {
            hi += (size >> kH8Low) << ((6 - k) * hb);
            lo += (size & 0xffu) << ((6 - k) * kH8Low);
          }
        }
        w[2 * c] = hi;
        w[2 * c + 1] = lo;
      }
      return nullptr;
    }
    default:
      return "unknown index format";
  }
}

const char* unpack(int format, unsigned dims, const void* in, size_t n, uint64_t range, uint64_t* off) {
  switch (format) {
    case ZFP_GB300_INDEX_VERBATIM:
      std::memcpy(off, in, 8 * (n + 1));
      break;
    case ZFP_GB300_INDEX_HYBRID4: {
      const auto* rec = static_cast<const Hybrid4Record*>(in);
      for (size_t i = 0; i < n; i++) {
        Hybrid4Record r;
        std::memcpy(&r, rec + i / 4, sizeof r);
        off[i] = ((uint64_t)r.hi << kH4Shift) + r.lo[i % 4];
      }
      off[n] = range;
      break;
    }
    case ZFP_GB300_INDEX_HYBRID8: {
      if (dims < 1 || dims > 4) return "hybrid8 index needs dims 1-4";
      const unsigned hb = h8_high(dims);
      const uint64_t hmask = (1ull << hb) - 1;
      const auto* w = static_cast<const uint64_t*>(in);
      for (size_t c = 0; c < (n + 7) / 8; c++) {
        const uint64_t hi = w[2 * c], lo = w[2 * c + 1];
        uint64_t at = ((hi >> (7 * hb)) << kH8Low) + (lo >> (7 * kH8Low));
        for (unsigned k = 0; k < 8 && 8 * c + k < n; k++) {
          off[8 * c + k] = at;
          if (k < 7)
            at += (((hi >> ((6 - k) * hb)) & hmask) << kH8Low) + ((lo >> ((6 - k) * kH8Low)) & 0xffu);
        }
      }
      off[n] = range;
      break;
    }
    default:
      return "unknown index format";
  }
  if (n && off[0] != 0) return "index does not start at offset 0";
  for (size_t i = 0; i < n; i++)
    if (off[i + 1] < off[i]) return "index offsets decrease (or the range is too small)";
  return nullptr;
}

// the stream position zfp_decompress would start at
uint64_t read_position(const zfp_stream* z) {
  const StreamState ss = get_stream_state(z->stream);
  return (uint64_t)(ss.ptr - ss.begin) * 64 - ss.bits;
}

}  // namespace
}  // namespace zg

extern "C" {

size_t zfp_gb300_index_bytes(int format, size_t nblocks) { return zg::bytes_of(format, nblocks); }

size_t zfp_gb300_index_pack(int format, unsigned dims, const uint64_t* offsets, size_t nblocks, void* index,
                            size_t bytes) {
  const size_t need = zg::bytes_of(format, nblocks);
  if (!need) return zg::fail("zfp_gb300_index_pack: unknown index format");
  if (!offsets || !index || bytes < need) return zg::fail("zfp_gb300_index_pack: buffer too small");
  if (const char* why = zg::pack(format, dims, offsets, nblocks, index)) return zg::fail(why);
  zg::set_error("");
  return need;
}

zfp_bool zfp_gb300_index_unpack(int format, unsigned dims, const void* index, size_t bytes, size_t nblocks,
                                uint64_t range, uint64_t* offsets) {
  const size_t need = zg::bytes_of(format, nblocks);
  if (!need || !index || !offsets || bytes < need) {
    zg::set_error("zfp_gb300_index_unpack: unknown format or index too short");
    return zfp_false;
  }
  if (const char* why = zg::unpack(format, dims, index, nblocks, range, offsets)) {
    zg::set_error(why);
    return zfp_false;
  }
  zg::set_error("");
  return zfp_true;
}

size_t zfp_gb300_index_export(const zfp_stream* zfp, const zfp_field* field, int format, void* index,
                              size_t bytes, uint64_t* range) {
  using namespace zg;
  if (!zfp || !zfp->stream) return fail("zfp_gb300_index_export: no bit stream");
  FieldInfo fi;
  if (const char* why = field_info(field, fi)) return fail(why);
  const size_t need = bytes_of(format, fi.nblocks);
  if (!need) return fail("zfp_gb300_index_export: unknown index format");
  if (!index || bytes < need) return fail("zfp_gb300_index_export: buffer too small");
  const StreamState ss = get_stream_state(zfp->stream);
  const uint64_t bit0 = read_position(zfp);
  std::vector<uint64_t> off(fi.nblocks + 1);
  if (is_fixed_rate(fi, zfp)) {
    for (uint64_t i = 0; i <= fi.nblocks; i++) off[i] = i * zfp->maxbits;
  } else {
    IndexEntry e;
    if (!registry_find(ss.begin, bit0, fi, zfp, e))
      return fail("zfp_gb300_index_export: no index of a stream this library wrote at this position");
    cudaError_t err;
    if (e.index->written && (err = cudaEventSynchronize(e.index->written)) != cudaSuccess)
      return fail_cuda("zfp_gb300_index_export: wait", err);
    if ((err = cudaMemcpy(off.data(), e.index->ptr, fi.nblocks * 8, cudaMemcpyDeviceToHost)) != cudaSuccess)
      return fail_cuda("zfp_gb300_index_export: download", err);
    for (uint64_t i = 0; i < fi.nblocks; i++) off[i] -= bit0;
    off[fi.nblocks] = e.end_bit - bit0;
  }
  if (const char* why = pack(format, fi.dims, off.data(), fi.nblocks, index)) return fail(why);
  if (range) *range = off[fi.nblocks];
  set_error("");
  return need;
}

zfp_bool zfp_gb300_index_import(zfp_stream* zfp, const zfp_field* field, int format, const void* index,
                                size_t bytes, uint64_t range) {
  using namespace zg;
  if (!zfp || !zfp->stream) {
    set_error("zfp_gb300_index_import: no bit stream");
    return zfp_false;
  }
  FieldInfo fi;
  if (const char* why = field_info(field, fi)) {
    set_error(why);
    return zfp_false;
  }
  if (is_fixed_rate(fi, zfp)) {  // offsets follow from the rate; nothing to keep
    set_error("");
    return zfp_true;
  }
  const size_t need = bytes_of(format, fi.nblocks);
  if (!need || !index || bytes < need) {
    set_error("zfp_gb300_index_import: unknown format or index too short");
    return zfp_false;
  }
  std::vector<uint64_t> off(fi.nblocks + 1);
  if (const char* why = unpack(format, fi.dims, index, fi.nblocks, range, off.data())) {
    set_error(why);
    return zfp_false;
  }
  init_pool_once();
  const StreamState ss = get_stream_state(zfp->stream);
  const uint64_t bit0 = read_position(zfp);
  for (uint64_t i = 0; i < fi.nblocks; i++) off[i] += bit0;
  cudaError_t err;
  IndexRef idx = make_index(fi.nblocks, nullptr, err);
  if (!idx || (err = cudaMemcpyAsync(idx->ptr, off.data(), fi.nblocks * 8, cudaMemcpyHostToDevice, nullptr)) !=
                  cudaSuccess ||
      (err = cudaStreamSynchronize(nullptr)) != cudaSuccess) {
    fail_cuda("zfp_gb300_index_import: upload", err);
    return zfp_false;
  }
  Job j = base_job(fi, zfp, nullptr);
  // zfp_decompress checks every block against it and parses the stream
  // itself if the index does not describe it
  registry_insert(make_entry(ss.begin, bit0, off[fi.nblocks] + bit0, fi, j, idx));
  set_error("");
  return zfp_true;
}

}  // extern "C"
