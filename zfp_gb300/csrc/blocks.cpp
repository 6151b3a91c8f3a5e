// blocks.cpp -- zfp's low-level block codec (reference include/zfp.h:636-775,
// src/template/encode*.c / decode*.c public entry points) on the GPU.
//
// The reference's compressed-array classes (include/zfp/codec/zfpcodec.hpp)
// code one 4^d block per call of zfp_encode_block_<type>_<dims> /
// zfp_decode_block_<type>_<dims> at the stream's current bit, without
// flushing, and return the bits written or read.  Here every such call is
// the whole-array path on a field of one block: a full block is the field
// 4 x ... x 4 (contiguous, or with the caller's strides), a partial block
// the field nx x ny x ... with its strides, which the kernels pad or scatter
// exactly as the reference's partial-block functions do.  A run of `count`
// full blocks stored one after another (4^d values each, x fastest) is the
// field 4 x ... x 4 x (4 * count) -- blocks are coded in raster order, x
// fastest -- so zfp_gb300_encode_blocks / zfp_gb300_decode_blocks code
// thousands of blocks in one launch, bit for bit as `count` successive
// calls would.  These functions use the GPU whatever the stream's execution
// policy (the reference's block functions do not look at it either); the
// stream is left at the exact end bit, its last partial word buffered, as
// the reference's bit stream leaves it.
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../include/zfp.h"
#include "../../include/zfp_gb300.h"
#include "gpu_internal.h"
#include "runtime.h"

namespace zg {

// code one field of n[] values with strides s[] (0: contiguous), encoding or decoding
static size_t code_field(zfp_stream* z, zfp_type type, unsigned dims, void* p, const size_t* n,
                         const ptrdiff_t* s, bool encode) {
  if (!z || !z->stream || !p || dims < 1 || dims > 4) {
    fail("zfp block codec: bad arguments");
    return 0;
  }
  zfp_field f;
  std::memset(&f, 0, sizeof f);
  f.type = type;
  f.data = p;
  size_t* ext[4] = {&f.nx, &f.ny, &f.nz, &f.nw};
  ptrdiff_t* str[4] = {&f.sx, &f.sy, &f.sz, &f.sw};
  for (unsigned a = 0; a < dims; a++) {
    *ext[a] = n[a];
    *str[a] = s ? s[a] : 0;
  }
  // run on the GPU with default controls when the stream has none of its own
  ExecParams tmp{kExecMagic, nullptr, 0};
  const zfp_execution saved = z->exec;
  const bool borrow = !exec_params(z);
  if (borrow) {
    z->exec.policy = zfp_exec_cuda;
    z->exec.params = &tmp;
  }
  uint64_t bits = 0;
  const size_t r = encode ? gpu_compress(z, &f, true, &bits) : gpu_decompress(z, &f, true, &bits);
  if (borrow) z->exec = saved;
  return r ? (size_t)bits : 0;
}

static size_t code_block(zfp_stream* z, zfp_type type, unsigned dims, void* p, const size_t* n, const ptrdiff_t* s,
                         bool encode) {
  for (unsigned a = 0; a < dims; a++)
    if (n[a] < 1 || n[a] > 4) {
      fail("zfp block codec: a block has 1 to 4 values per dimension");
      return 0;
    }
  return code_field(z, type, dims, p, n, s, encode);
}

}  // namespace zg

extern "C" {

size_t zfp_gb300_encode_blocks(zfp_stream* zfp, zfp_type type, unsigned int dims, const void* blocks, size_t count) {
  size_t n[4] = {4, 4, 4, 4};
  if (!count || dims < 1 || dims > 4) return zg::fail("zfp_gb300_encode_blocks: bad arguments");
  n[dims - 1] = 4 * count;
  return zg::code_field(zfp, type, dims, const_cast<void*>(blocks), n, nullptr, true);
}

size_t zfp_gb300_decode_blocks(zfp_stream* zfp, zfp_type type, unsigned int dims, void* blocks, size_t count) {
  size_t n[4] = {4, 4, 4, 4};
  if (!count || dims < 1 || dims > 4) return zg::fail("zfp_gb300_decode_blocks: bad arguments");
  n[dims - 1] = 4 * count;
  return zg::code_field(zfp, type, dims, blocks, n, nullptr, false);
}

// The reference's entry points, one per scalar type and dimensionality
// (include/zfp.h:640-775): full contiguous blocks, full strided blocks,
// partial strided blocks, each for encoding and decoding.
#define ZG_BLOCK_1(T, NAME, ZT)                                                                              \
  size_t zfp_encode_block_##NAME##_1(zfp_stream* z, const T* b) {                                           \
    const size_t n[1] = {4};                                                                                \
    return zg::code_block(z, ZT, 1, (void*)b, n, nullptr, true);                                             \
  }                                                                                                          \
  size_t zfp_encode_block_strided_##NAME##_1(zfp_stream* z, const T* p, ptrdiff_t sx) {                      \
    const size_t n[1] = {4};                                                                                \
    const ptrdiff_t s[1] = {sx};                                                                             \
    return zg::code_block(z, ZT, 1, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_encode_partial_block_strided_##NAME##_1(zfp_stream* z, const T* p, size_t nx, ptrdiff_t sx) {   \
    const size_t n[1] = {nx};                                                                               \
    const ptrdiff_t s[1] = {sx};                                                                             \
    return zg::code_block(z, ZT, 1, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_##NAME##_1(zfp_stream* z, T* b) {                                                 \
    const size_t n[1] = {4};                                                                                \
    return zg::code_block(z, ZT, 1, b, n, nullptr, false);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_strided_##NAME##_1(zfp_stream* z, T* p, ptrdiff_t sx) {                            \
    const size_t n[1] = {4};                                                                                \
    const ptrdiff_t s[1] = {sx};                                                                             \
    return zg::code_block(z, ZT, 1, p, n, s, false);                                                         \
  }                                                                                                          \
  size_t zfp_decode_partial_block_strided_##NAME##_1(zfp_stream* z, T* p, size_t nx, ptrdiff_t sx) {         \
    const size_t n[1] = {nx};                                                                               \
    const ptrdiff_t s[1] = {sx};                                                                             \
    return zg::code_block(z, ZT, 1, p, n, s, false);                                                         \
  }

#define ZG_BLOCK_2(T, NAME, ZT)                                                                              \
  size_t zfp_encode_block_##NAME##_2(zfp_stream* z, const T* b) {                                           \
    const size_t n[2] = {4, 4};                                                                             \
    return zg::code_block(z, ZT, 2, (void*)b, n, nullptr, true);                                             \
  }                                                                                                          \
  size_t zfp_encode_block_strided_##NAME##_2(zfp_stream* z, const T* p, ptrdiff_t sx, ptrdiff_t sy) {        \
    const size_t n[2] = {4, 4};                                                                             \
    const ptrdiff_t s[2] = {sx, sy};                                                                         \
    return zg::code_block(z, ZT, 2, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_encode_partial_block_strided_##NAME##_2(zfp_stream* z, const T* p, size_t nx, size_t ny,        \
                                                     ptrdiff_t sx, ptrdiff_t sy) {                           \
    const size_t n[2] = {nx, ny};                                                                           \
    const ptrdiff_t s[2] = {sx, sy};                                                                         \
    return zg::code_block(z, ZT, 2, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_##NAME##_2(zfp_stream* z, T* b) {                                                 \
    const size_t n[2] = {4, 4};                                                                             \
    return zg::code_block(z, ZT, 2, b, n, nullptr, false);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_strided_##NAME##_2(zfp_stream* z, T* p, ptrdiff_t sx, ptrdiff_t sy) {              \
    const size_t n[2] = {4, 4};                                                                             \
    const ptrdiff_t s[2] = {sx, sy};                                                                         \
    return zg::code_block(z, ZT, 2, p, n, s, false);                                                         \
  }                                                                                                          \
  size_t zfp_decode_partial_block_strided_##NAME##_2(zfp_stream* z, T* p, size_t nx, size_t ny, ptrdiff_t sx, \
                                                     ptrdiff_t sy) {                                         \
    const size_t n[2] = {nx, ny};                                                                           \
    const ptrdiff_t s[2] = {sx, sy};                                                                         \
    return zg::code_block(z, ZT, 2, p, n, s, false);                                                         \
  }

#define ZG_BLOCK_3(T, NAME, ZT)                                                                              \
  size_t zfp_encode_block_##NAME##_3(zfp_stream* z, const T* b) {                                           \
    const size_t n[3] = {4, 4, 4};                                                                          \
    return zg::code_block(z, ZT, 3, (void*)b, n, nullptr, true);                                             \
  }                                                                                                          \
  size_t zfp_encode_block_strided_##NAME##_3(zfp_stream* z, const T* p, ptrdiff_t sx, ptrdiff_t sy,          \
                                             ptrdiff_t sz) {                                                 \
    const size_t n[3] = {4, 4, 4};                                                                          \
    const ptrdiff_t s[3] = {sx, sy, sz};                                                                     \
    return zg::code_block(z, ZT, 3, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_encode_partial_block_strided_##NAME##_3(zfp_stream* z, const T* p, size_t nx, size_t ny,        \
                                                     size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz) {  \
    const size_t n[3] = {nx, ny, nz};                                                                       \
    const ptrdiff_t s[3] = {sx, sy, sz};                                                                     \
    return zg::code_block(z, ZT, 3, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_##NAME##_3(zfp_stream* z, T* b) {                                                 \
    const size_t n[3] = {4, 4, 4};                                                                          \
    return zg::code_block(z, ZT, 3, b, n, nullptr, false);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_strided_##NAME##_3(zfp_stream* z, T* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz) { \
    const size_t n[3] = {4, 4, 4};                                                                          \
    const ptrdiff_t s[3] = {sx, sy, sz};                                                                     \
    return zg::code_block(z, ZT, 3, p, n, s, false);                                                         \
  }                                                                                                          \
  size_t zfp_decode_partial_block_strided_##NAME##_3(zfp_stream* z, T* p, size_t nx, size_t ny, size_t nz,   \
                                                     ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz) {             \
    const size_t n[3] = {nx, ny, nz};                                                                       \
    const ptrdiff_t s[3] = {sx, sy, sz};                                                                     \
    return zg::code_block(z, ZT, 3, p, n, s, false);                                                         \
  }

#define ZG_BLOCK_4(T, NAME, ZT)                                                                              \
  size_t zfp_encode_block_##NAME##_4(zfp_stream* z, const T* b) {                                           \
    const size_t n[4] = {4, 4, 4, 4};                                                                       \
    return zg::code_block(z, ZT, 4, (void*)b, n, nullptr, true);                                             \
  }                                                                                                          \
  size_t zfp_encode_block_strided_##NAME##_4(zfp_stream* z, const T* p, ptrdiff_t sx, ptrdiff_t sy,          \
                                             ptrdiff_t sz, ptrdiff_t sw) {                                   \
    const size_t n[4] = {4, 4, 4, 4};                                                                       \
    const ptrdiff_t s[4] = {sx, sy, sz, sw};                                                                 \
    return zg::code_block(z, ZT, 4, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_encode_partial_block_strided_##NAME##_4(zfp_stream* z, const T* p, size_t nx, size_t ny,        \
                                                     size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy,       \
                                                     ptrdiff_t sz, ptrdiff_t sw) {                           \
    const size_t n[4] = {nx, ny, nz, nw};                                                                   \
    const ptrdiff_t s[4] = {sx, sy, sz, sw};                                                                 \
    return zg::code_block(z, ZT, 4, (void*)p, n, s, true);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_##NAME##_4(zfp_stream* z, T* b) {                                                 \
    const size_t n[4] = {4, 4, 4, 4};                                                                       \
    return zg::code_block(z, ZT, 4, b, n, nullptr, false);                                                   \
  }                                                                                                          \
  size_t zfp_decode_block_strided_##NAME##_4(zfp_stream* z, T* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz,  \
                                             ptrdiff_t sw) {                                                 \
    const size_t n[4] = {4, 4, 4, 4};                                                                       \
    const ptrdiff_t s[4] = {sx, sy, sz, sw};                                                                 \
    return zg::code_block(z, ZT, 4, p, n, s, false);                                                         \
  }                                                                                                          \
  size_t zfp_decode_partial_block_strided_##NAME##_4(zfp_stream* z, T* p, size_t nx, size_t ny, size_t nz,   \
                                                     size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz,    \
                                                     ptrdiff_t sw) {                                         \
    const size_t n[4] = {nx, ny, nz, nw};                                                                   \
    const ptrdiff_t s[4] = {sx, sy, sz, sw};                                                                 \
    return zg::code_block(z, ZT, 4, p, n, s, false);                                                         \
  }

#define ZG_BLOCKS(T, NAME, ZT) ZG_BLOCK_1(T, NAME, ZT) ZG_BLOCK_2(T, NAME, ZT) ZG_BLOCK_3(T, NAME, ZT) ZG_BLOCK_4(T, NAME, ZT)

ZG_BLOCKS(int32, int32, zfp_type_int32)
ZG_BLOCKS(int64, int64, zfp_type_int64)
ZG_BLOCKS(float, float, zfp_type_float)
ZG_BLOCKS(double, double, zfp_type_double)

}  // extern "C"
