/*
 * bitstream.h -- bit stream API of libzfp_gb300.
 *
 * Same ABI as the reference's include/zfp/bitstream.h:27-100 (64-bit words,
 * bits filled from the least significant end, include/zfp/bitstream.inl).
 * These functions run on the host and touch the stream buffer from the
 * host, so they are for host-resident buffers (e.g. writing a header before
 * zfp_compress); the codec itself, zfp_compress/zfp_decompress, accepts
 * host or device buffers.
 */
#ifndef ZFP_GB300_BITSTREAM_H
#define ZFP_GB300_BITSTREAM_H

#include <stddef.h>
#include <stdint.h>

typedef struct bitstream bitstream;   /* opaque; layout bitstream.inl:133-143 */
typedef uint64_t bitstream_offset;    /* bit offset, bitstream.h:11 */
typedef bitstream_offset bitstream_size;
typedef size_t bitstream_count;

#ifdef __cplusplus
extern "C" {
#endif

extern const size_t stream_word_bits;                         /* src/bitstream.c:4 */

bitstream* stream_open(void* buffer, size_t bytes);           /* bitstream.h:30 */
void stream_close(bitstream* stream);                         /* bitstream.h:33 */
bitstream* stream_clone(const bitstream* stream);             /* bitstream.h:36 */
bitstream_count stream_alignment(void);                       /* bitstream.h:39, bitstream.inl:183 */
void* stream_data(const bitstream* stream);                   /* bitstream.h:42, bitstream.inl:190 */
size_t stream_size(const bitstream* stream);                  /* bitstream.h:45, bitstream.inl:197 */
size_t stream_capacity(const bitstream* stream);              /* bitstream.h:48, bitstream.inl:204 */
size_t stream_stride_block(const bitstream* stream);          /* bitstream.h:51 */
ptrdiff_t stream_stride_delta(const bitstream* stream);       /* bitstream.h:54 */
unsigned int stream_read_bit(bitstream* stream);              /* bitstream.h:57, bitstream.inl:226 */
unsigned int stream_write_bit(bitstream* stream, unsigned int bit);  /* bitstream.h:60, bitstream.inl:241 */
uint64_t stream_read_bits(bitstream* stream, bitstream_count n);     /* bitstream.h:63, bitstream.inl:254 */
uint64_t stream_write_bits(bitstream* stream, uint64_t value, bitstream_count n); /* bitstream.h:66, bitstream.inl:289 */
bitstream_offset stream_rtell(const bitstream* stream);       /* bitstream.h:69, bitstream.inl:317 */
bitstream_offset stream_wtell(const bitstream* stream);       /* bitstream.h:72, bitstream.inl:324 */
void stream_rewind(bitstream* stream);                        /* bitstream.h:75, bitstream.inl:331 */
void stream_rseek(bitstream* stream, bitstream_offset offset);      /* bitstream.h:78, bitstream.inl:340 */
void stream_wseek(bitstream* stream, bitstream_offset offset);      /* bitstream.h:81, bitstream.inl:356 */
void stream_skip(bitstream* stream, bitstream_size n);        /* bitstream.h:84, bitstream.inl:374 */
void stream_pad(bitstream* stream, bitstream_size n);         /* bitstream.h:87, bitstream.inl:381 */
bitstream_count stream_align(bitstream* stream);              /* bitstream.h:90, bitstream.inl:393 */
bitstream_count stream_flush(bitstream* stream);              /* bitstream.h:93, bitstream.inl:403 */
void stream_copy(bitstream* dst, bitstream* src, bitstream_size n); /* bitstream.h:96, bitstream.inl:413 */

#ifdef __cplusplus
}
#endif

#endif
