/*
 * zfp.h -- high-level C API of libzfp_gb300, a drop-in for the reference's
 * whole-array compression path on one GB300 GPU.
 *
 * The types, constants and entry points below have the reference's names,
 * layouts and meaning (reference include/zfp.h; line numbers cited per
 * entry), so a program written against the reference links against
 * libzfp_gb300 unchanged.  What differs is execution: zfp_compress and
 * zfp_decompress run the GB300 CUDA codec when the stream's policy is
 * zfp_exec_cuda, for every mode (fixed rate, precision, accuracy,
 * reversible, expert), scalar type and dimensionality 1-4, with host or
 * device field/stream buffers; streams are bit-identical to the reference's
 * serial encoder.  There is no CPU fallback: with the serial policy (the
 * default of zfp_stream_open, as in the reference) both return 0, and
 * zfp_exec_omp cannot be selected.
 */
#ifndef ZFP_GB300_ZFP_H
#define ZFP_GB300_ZFP_H

#include <stddef.h>
#include <stdint.h>

#include "bitstream.h"
#include "zfp/version.h"              /* versions (reference include/zfp/version.h): codec 5, library 1.0.1 */
#include "zfp/internal/zfp/types.h"   /* int32, uint, ... (reference include/zfp.h:13) */

/* default compression parameters (include/zfp.h:18-21) */
#define ZFP_MIN_BITS 1
#define ZFP_MAX_BITS 16658
#define ZFP_MAX_PREC 64
#define ZFP_MIN_EXP -1074

/* header masks (include/zfp.h:24-28) */
#define ZFP_HEADER_NONE 0x0u
#define ZFP_HEADER_MAGIC 0x1u
#define ZFP_HEADER_META 0x2u
#define ZFP_HEADER_MODE 0x4u
#define ZFP_HEADER_FULL 0x7u

/* header field sizes (include/zfp.h:44-52) */
#define ZFP_META_NULL ((uint64_t)-1)
#define ZFP_MAGIC_BITS 32
#define ZFP_META_BITS 52
#define ZFP_MODE_SHORT_BITS 12
#define ZFP_MODE_LONG_BITS 64
#define ZFP_HEADER_MAX_BITS 148
#define ZFP_MODE_SHORT_MAX ((1u << ZFP_MODE_SHORT_BITS) - 2)

typedef int zfp_bool;                           /* include/zfp.h:57-64 */
enum { zfp_false = 0, zfp_true = 1 };

typedef enum {                                  /* include/zfp.h:68-72 */
  zfp_exec_serial = 0,
  zfp_exec_omp = 1,
  zfp_exec_cuda = 2
} zfp_exec_policy;

typedef struct {                                /* include/zfp.h:75-78 */
  unsigned int threads;
  unsigned int chunk_size;
} zfp_exec_params_omp;

typedef struct {                                /* include/zfp.h:80-83 */
  zfp_exec_policy policy;
  void* params;
} zfp_execution;

typedef struct {                                /* include/zfp.h:86-93 */
  unsigned int minbits;
  unsigned int maxbits;
  unsigned int maxprec;
  int minexp;
  bitstream* stream;
  zfp_execution exec;
} zfp_stream;

typedef enum {                                  /* include/zfp.h:96-103 */
  zfp_mode_null = 0,
  zfp_mode_expert = 1,
  zfp_mode_fixed_rate = 2,
  zfp_mode_fixed_precision = 3,
  zfp_mode_fixed_accuracy = 4,
  zfp_mode_reversible = 5
} zfp_mode;

typedef struct {                                /* include/zfp.h:106-119 */
  zfp_mode mode;
  union {
    double rate;
    unsigned int precision;
    double tolerance;
    struct {
      unsigned int minbits;
      unsigned int maxbits;
      unsigned int maxprec;
      int minexp;
    } expert;
  } arg;
} zfp_config;

typedef enum {                                  /* include/zfp.h:122-128 */
  zfp_type_none = 0,
  zfp_type_int32 = 1,
  zfp_type_int64 = 2,
  zfp_type_float = 3,
  zfp_type_double = 4
} zfp_type;

typedef struct {                                /* include/zfp.h:131-136 */
  zfp_type type;
  size_t nx, ny, nz, nw;
  ptrdiff_t sx, sy, sz, sw;
  void* data;
} zfp_field;

#ifdef __cplusplus
extern "C" {
#endif

extern const unsigned int zfp_codec_version;    /* include/zfp.h:144 */
extern const unsigned int zfp_library_version;  /* include/zfp.h:145 */
extern const char* const zfp_version_string;    /* include/zfp.h:146 */

size_t zfp_type_size(zfp_type type);                                   /* include/zfp.h:151 */

/* compressed stream (include/zfp.h:159-332) */
zfp_stream* zfp_stream_open(bitstream* stream);                        /* :159 */
void zfp_stream_close(zfp_stream* zfp);                                /* :165 */
bitstream* zfp_stream_bit_stream(const zfp_stream* zfp);               /* :173 */
zfp_mode zfp_stream_compression_mode(const zfp_stream* zfp);           /* :179 */
double zfp_stream_rate(const zfp_stream* zfp, unsigned int dims);      /* :185 */
unsigned int zfp_stream_precision(const zfp_stream* zfp);              /* :192 */
double zfp_stream_accuracy(const zfp_stream* zfp);                     /* :198 */
uint64_t zfp_stream_mode(const zfp_stream* zfp);                       /* :204 */
void zfp_stream_params(const zfp_stream* zfp, unsigned int* minbits, unsigned int* maxbits,
                       unsigned int* maxprec, int* minexp);            /* :210 */
size_t zfp_stream_compressed_size(const zfp_stream* zfp);              /* :220 */
size_t zfp_stream_maximum_size(const zfp_stream* zfp, const zfp_field* field); /* :226 */
void zfp_stream_rewind(zfp_stream* zfp);                               /* :235 */
void zfp_stream_set_bit_stream(zfp_stream* zfp, bitstream* stream);    /* :241 */
void zfp_stream_set_reversible(zfp_stream* zfp);                       /* :248 */
double zfp_stream_set_rate(zfp_stream* zfp, double rate, zfp_type type, unsigned int dims,
                           zfp_bool align);                            /* :254 */
unsigned int zfp_stream_set_precision(zfp_stream* zfp, unsigned int precision); /* :264 */
double zfp_stream_set_accuracy(zfp_stream* zfp, double tolerance);     /* :271 */
zfp_mode zfp_stream_set_mode(zfp_stream* zfp, uint64_t mode);          /* :278 */
zfp_bool zfp_stream_set_params(zfp_stream* zfp, unsigned int minbits, unsigned int maxbits,
                               unsigned int maxprec, int minexp);      /* :285 */
zfp_exec_policy zfp_stream_execution(const zfp_stream* zfp);           /* :297 */
unsigned int zfp_stream_omp_threads(const zfp_stream* zfp);            /* :303 */
unsigned int zfp_stream_omp_chunk_size(const zfp_stream* zfp);         /* :309 */
zfp_bool zfp_stream_set_execution(zfp_stream* zfp, zfp_exec_policy policy);   /* :315 */
zfp_bool zfp_stream_set_omp_threads(zfp_stream* zfp, unsigned int threads);   /* :322 */
zfp_bool zfp_stream_set_omp_chunk_size(zfp_stream* zfp, unsigned int chunk_size); /* :329 */

/* configurations (include/zfp.h:338-371) */
zfp_config zfp_config_none(void);                                      /* :338 */
zfp_config zfp_config_rate(double rate, zfp_bool align);               /* :342 */
zfp_config zfp_config_precision(unsigned int precision);               /* :349 */
zfp_config zfp_config_accuracy(double tolerance);                      /* :355 */
zfp_config zfp_config_reversible(void);                                /* :361 */
zfp_config zfp_config_expert(unsigned int minbits, unsigned int maxbits,
                             unsigned int maxprec, int minexp);        /* :365 */

/* fields (include/zfp.h:376-582) */
zfp_field* zfp_field_alloc(void);                                      /* :376 */
zfp_field* zfp_field_1d(void* pointer, zfp_type type, size_t nx);      /* :380 */
zfp_field* zfp_field_2d(void* pointer, zfp_type type, size_t nx, size_t ny);             /* :388 */
zfp_field* zfp_field_3d(void* pointer, zfp_type type, size_t nx, size_t ny, size_t nz);  /* :397 */
zfp_field* zfp_field_4d(void* pointer, zfp_type type, size_t nx, size_t ny, size_t nz,
                        size_t nw);                                    /* :407 */
void zfp_field_free(zfp_field* field);                                 /* :418 */
void* zfp_field_pointer(const zfp_field* field);                       /* :426 */
void* zfp_field_begin(const zfp_field* field);                         /* :432 */
zfp_type zfp_field_type(const zfp_field* field);                       /* :438 */
unsigned int zfp_field_precision(const zfp_field* field);              /* :444 */
unsigned int zfp_field_dimensionality(const zfp_field* field);         /* :450 */
size_t zfp_field_size(const zfp_field* field, size_t* size);           /* :456 */
size_t zfp_field_size_bytes(const zfp_field* field);                   /* :463 */
size_t zfp_field_blocks(const zfp_field* field);                       /* :469 */
zfp_bool zfp_field_stride(const zfp_field* field, ptrdiff_t* stride);  /* :475 */
zfp_bool zfp_field_is_contiguous(const zfp_field* field);              /* :482 */
uint64_t zfp_field_metadata(const zfp_field* field);                   /* :488 */
void zfp_field_set_pointer(zfp_field* field, void* pointer);           /* :496 */
zfp_type zfp_field_set_type(zfp_field* field, zfp_type type);          /* :503 */
void zfp_field_set_size_1d(zfp_field* field, size_t nx);               /* :510 */
void zfp_field_set_size_2d(zfp_field* field, size_t nx, size_t ny);    /* :517 */
void zfp_field_set_size_3d(zfp_field* field, size_t nx, size_t ny, size_t nz);            /* :525 */
void zfp_field_set_size_4d(zfp_field* field, size_t nx, size_t ny, size_t nz, size_t nw); /* :534 */
void zfp_field_set_stride_1d(zfp_field* field, ptrdiff_t sx);          /* :544 */
void zfp_field_set_stride_2d(zfp_field* field, ptrdiff_t sx, ptrdiff_t sy);               /* :551 */
void zfp_field_set_stride_3d(zfp_field* field, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz); /* :559 */
void zfp_field_set_stride_4d(zfp_field* field, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz,
                             ptrdiff_t sw);                            /* :568 */
zfp_bool zfp_field_set_metadata(zfp_field* field, uint64_t meta);      /* :578 */

/* compression and decompression: the hot path (include/zfp.h:587-597) */
size_t zfp_compress(zfp_stream* zfp, const zfp_field* field);          /* :587, src/zfp.c:1052 */
size_t zfp_decompress(zfp_stream* zfp, zfp_field* field);              /* :594, src/zfp.c:1123 */

/* header I/O on host-resident streams (include/zfp.h:601-613) */
size_t zfp_write_header(zfp_stream* zfp, const zfp_field* field, unsigned int mask); /* :601 */
size_t zfp_read_header(zfp_stream* zfp, zfp_field* field, unsigned int mask);        /* :609 */

size_t zfp_stream_flush(zfp_stream* zfp);                              /* :619 */
size_t zfp_stream_align(zfp_stream* zfp);                              /* :625 */


/* low-level block codec (include/zfp.h:636-775): one 4^d block per call at the
 * stream's current bit, not flushed; returns the bits written / read.  Runs on
 * the GPU whatever the stream's execution policy; the stream is left as the
 * reference's bit stream would be (last partial word buffered). */
size_t zfp_encode_block_int32_1(zfp_stream* stream, const int32* block);
size_t zfp_encode_block_strided_int32_1(zfp_stream* stream, const int32* p, ptrdiff_t sx);
size_t zfp_encode_partial_block_strided_int32_1(zfp_stream* stream, const int32* p, size_t nx, ptrdiff_t sx);
size_t zfp_encode_block_int32_2(zfp_stream* stream, const int32* block);
size_t zfp_encode_block_strided_int32_2(zfp_stream* stream, const int32* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_partial_block_strided_int32_2(zfp_stream* stream, const int32* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_block_int32_3(zfp_stream* stream, const int32* block);
size_t zfp_encode_block_strided_int32_3(zfp_stream* stream, const int32* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_partial_block_strided_int32_3(zfp_stream* stream, const int32* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_block_int32_4(zfp_stream* stream, const int32* block);
size_t zfp_encode_block_strided_int32_4(zfp_stream* stream, const int32* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_partial_block_strided_int32_4(zfp_stream* stream, const int32* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_block_int64_1(zfp_stream* stream, const int64* block);
size_t zfp_encode_block_strided_int64_1(zfp_stream* stream, const int64* p, ptrdiff_t sx);
size_t zfp_encode_partial_block_strided_int64_1(zfp_stream* stream, const int64* p, size_t nx, ptrdiff_t sx);
size_t zfp_encode_block_int64_2(zfp_stream* stream, const int64* block);
size_t zfp_encode_block_strided_int64_2(zfp_stream* stream, const int64* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_partial_block_strided_int64_2(zfp_stream* stream, const int64* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_block_int64_3(zfp_stream* stream, const int64* block);
size_t zfp_encode_block_strided_int64_3(zfp_stream* stream, const int64* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_partial_block_strided_int64_3(zfp_stream* stream, const int64* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_block_int64_4(zfp_stream* stream, const int64* block);
size_t zfp_encode_block_strided_int64_4(zfp_stream* stream, const int64* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_partial_block_strided_int64_4(zfp_stream* stream, const int64* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_block_float_1(zfp_stream* stream, const float* block);
size_t zfp_encode_block_strided_float_1(zfp_stream* stream, const float* p, ptrdiff_t sx);
size_t zfp_encode_partial_block_strided_float_1(zfp_stream* stream, const float* p, size_t nx, ptrdiff_t sx);
size_t zfp_encode_block_float_2(zfp_stream* stream, const float* block);
size_t zfp_encode_block_strided_float_2(zfp_stream* stream, const float* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_partial_block_strided_float_2(zfp_stream* stream, const float* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_block_float_3(zfp_stream* stream, const float* block);
size_t zfp_encode_block_strided_float_3(zfp_stream* stream, const float* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_partial_block_strided_float_3(zfp_stream* stream, const float* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_block_float_4(zfp_stream* stream, const float* block);
size_t zfp_encode_block_strided_float_4(zfp_stream* stream, const float* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_partial_block_strided_float_4(zfp_stream* stream, const float* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_block_double_1(zfp_stream* stream, const double* block);
size_t zfp_encode_block_strided_double_1(zfp_stream* stream, const double* p, ptrdiff_t sx);
size_t zfp_encode_partial_block_strided_double_1(zfp_stream* stream, const double* p, size_t nx, ptrdiff_t sx);
size_t zfp_encode_block_double_2(zfp_stream* stream, const double* block);
size_t zfp_encode_block_strided_double_2(zfp_stream* stream, const double* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_partial_block_strided_double_2(zfp_stream* stream, const double* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_encode_block_double_3(zfp_stream* stream, const double* block);
size_t zfp_encode_block_strided_double_3(zfp_stream* stream, const double* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_partial_block_strided_double_3(zfp_stream* stream, const double* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_encode_block_double_4(zfp_stream* stream, const double* block);
size_t zfp_encode_block_strided_double_4(zfp_stream* stream, const double* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_encode_partial_block_strided_double_4(zfp_stream* stream, const double* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_block_int32_1(zfp_stream* stream, int32* block);
size_t zfp_decode_block_strided_int32_1(zfp_stream* stream, int32* p, ptrdiff_t sx);
size_t zfp_decode_partial_block_strided_int32_1(zfp_stream* stream, int32* p, size_t nx, ptrdiff_t sx);
size_t zfp_decode_block_int32_2(zfp_stream* stream, int32* block);
size_t zfp_decode_block_strided_int32_2(zfp_stream* stream, int32* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_partial_block_strided_int32_2(zfp_stream* stream, int32* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_block_int32_3(zfp_stream* stream, int32* block);
size_t zfp_decode_block_strided_int32_3(zfp_stream* stream, int32* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_partial_block_strided_int32_3(zfp_stream* stream, int32* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_block_int32_4(zfp_stream* stream, int32* block);
size_t zfp_decode_block_strided_int32_4(zfp_stream* stream, int32* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_partial_block_strided_int32_4(zfp_stream* stream, int32* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_block_int64_1(zfp_stream* stream, int64* block);
size_t zfp_decode_block_strided_int64_1(zfp_stream* stream, int64* p, ptrdiff_t sx);
size_t zfp_decode_partial_block_strided_int64_1(zfp_stream* stream, int64* p, size_t nx, ptrdiff_t sx);
size_t zfp_decode_block_int64_2(zfp_stream* stream, int64* block);
size_t zfp_decode_block_strided_int64_2(zfp_stream* stream, int64* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_partial_block_strided_int64_2(zfp_stream* stream, int64* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_block_int64_3(zfp_stream* stream, int64* block);
size_t zfp_decode_block_strided_int64_3(zfp_stream* stream, int64* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_partial_block_strided_int64_3(zfp_stream* stream, int64* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_block_int64_4(zfp_stream* stream, int64* block);
size_t zfp_decode_block_strided_int64_4(zfp_stream* stream, int64* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_partial_block_strided_int64_4(zfp_stream* stream, int64* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_block_float_1(zfp_stream* stream, float* block);
size_t zfp_decode_block_strided_float_1(zfp_stream* stream, float* p, ptrdiff_t sx);
size_t zfp_decode_partial_block_strided_float_1(zfp_stream* stream, float* p, size_t nx, ptrdiff_t sx);
size_t zfp_decode_block_float_2(zfp_stream* stream, float* block);
size_t zfp_decode_block_strided_float_2(zfp_stream* stream, float* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_partial_block_strided_float_2(zfp_stream* stream, float* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_block_float_3(zfp_stream* stream, float* block);
size_t zfp_decode_block_strided_float_3(zfp_stream* stream, float* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_partial_block_strided_float_3(zfp_stream* stream, float* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_block_float_4(zfp_stream* stream, float* block);
size_t zfp_decode_block_strided_float_4(zfp_stream* stream, float* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_partial_block_strided_float_4(zfp_stream* stream, float* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_block_double_1(zfp_stream* stream, double* block);
size_t zfp_decode_block_strided_double_1(zfp_stream* stream, double* p, ptrdiff_t sx);
size_t zfp_decode_partial_block_strided_double_1(zfp_stream* stream, double* p, size_t nx, ptrdiff_t sx);
size_t zfp_decode_block_double_2(zfp_stream* stream, double* block);
size_t zfp_decode_block_strided_double_2(zfp_stream* stream, double* p, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_partial_block_strided_double_2(zfp_stream* stream, double* p, size_t nx, size_t ny, ptrdiff_t sx, ptrdiff_t sy);
size_t zfp_decode_block_double_3(zfp_stream* stream, double* block);
size_t zfp_decode_block_strided_double_3(zfp_stream* stream, double* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_partial_block_strided_double_3(zfp_stream* stream, double* p, size_t nx, size_t ny, size_t nz, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz);
size_t zfp_decode_block_double_4(zfp_stream* stream, double* block);
size_t zfp_decode_block_strided_double_4(zfp_stream* stream, double* p, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);
size_t zfp_decode_partial_block_strided_double_4(zfp_stream* stream, double* p, size_t nx, size_t ny, size_t nz, size_t nw, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw);

#ifdef __cplusplus
}
#endif

#endif
