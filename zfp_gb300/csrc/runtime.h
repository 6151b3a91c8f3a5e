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

size_t gpu_compress(zfp_stream* z, const zfp_field* f);
size_t gpu_decompress(zfp_stream* z, zfp_field* f);

}  // namespace zg
