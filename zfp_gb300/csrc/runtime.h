// runtime.h -- glue between the host API (zfp_api.cpp) and the GPU codec
// (gpu_codec.cu, kern_*.cu).
#pragma once

#include <cstddef>
#include <cstdint>

#include "../../include/zfp.h"

namespace zg {

// the fields of a bit stream that the GPU path reads and updates
struct StreamState {
  uint64_t* begin;
  uint64_t* ptr;
  uint64_t* end;
  size_t bits;
  uint64_t buffer;
};

StreamState get_stream_state(const bitstream* s);
// leave the stream as stream_flush / stream_align would after a call that
// ended at end_bit: pointer past the last touched word, no buffered bits
void set_stream_flushed(bitstream* s, uint64_t end_bit);

void set_error(const char* msg);
bool ensure_exec_params(zfp_stream* z);
void release_exec_params(zfp_stream* z);

// exact_end: leave the stream at the exact end bit instead of flushed /
// aligned (the reference's block functions do: stream_pad / stream_align is
// the caller's); bits_out receives the bits coded
size_t gpu_compress(zfp_stream* z, const zfp_field* f, bool exact_end = false, uint64_t* bits_out = nullptr);
size_t gpu_decompress(zfp_stream* z, zfp_field* f, bool exact_end = false, uint64_t* bits_out = nullptr);

// the reference's writer state after writing up to end_bit without a flush:
// the last partial word's bits held in `buffer` (read back from the stream's
// memory, which the GPU already wrote; device memory if `device`)
bool set_stream_written(bitstream* s, uint64_t end_bit, bool device);
// the reader state of stream_rseek(end_bit): the rest of the current word in `buffer`
bool set_stream_read_at(bitstream* s, uint64_t end_bit, bool device);

}  // namespace zg
