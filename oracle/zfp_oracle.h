/*
 * zfp_oracle.h -- CPU restatement of zfp 1.0.1's serial block codec.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the GPU
 * codec in zfp_gb300/ is compared against (tests/, __graft_entry__.smoke)
 * and the CPU baseline that bench.py times beside it.  The product never
 * links, loads or calls it.
 *
 * Parity pin: the oracle is checked bit for bit against streams and arrays
 * produced by the reference library itself (compiled from the reference's
 * own sources by oracle/Makefile into oracle/_ref/) and against the golden
 * fixtures under tests/golden/ that were generated from that library.
 *
 * Conventions follow the reference's zfp_field / zfp_stream
 * (include/zfp.h:86-136): scalar types use zfp_type numbering, sizes are
 * zero for unused dimensions, strides are in elements and zero means
 * "contiguous default" independently per axis (src/template/compress.c:60-68).
 */
#ifndef ZFP_ORACLE_H
#define ZFP_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_INT32 = 1, ORC_INT64 = 2, ORC_FLOAT = 3, ORC_DOUBLE = 4 };

typedef struct {
  int type;          /* ORC_INT32 .. ORC_DOUBLE */
  size_t n[4];       /* nx, ny, nz, nw (0 = unused dimension) */
  ptrdiff_t s[4];    /* strides in elements (0 = default for that axis) */
  void* data;        /* pointer to element (0,0,0,0) */
} orc_field;

typedef struct {
  unsigned minbits;  /* zfp_stream.minbits */
  unsigned maxbits;  /* zfp_stream.maxbits */
  unsigned maxprec;  /* zfp_stream.maxprec */
  int minexp;        /* zfp_stream.minexp (< -1074 selects reversible mode) */
} orc_params;

/* dimensionality (0..4) and number of 4^d blocks of a field */
int orc_dims(const orc_field* f);
size_t orc_blocks(const orc_field* f);

/* Compress the field into the word buffer starting at absolute bit offset
 * bit0.  Bits [0, bit0 % 64) of words[bit0 / 64] are kept; everything after
 * is written, and the last partial word is zero padded (stream_flush).
 * If block_end is non-NULL it receives the end bit offset of every block.
 * Returns the end bit offset (before flushing). */
uint64_t orc_compress(const orc_field* f, const orc_params* p,
                      uint64_t* words, uint64_t bit0, uint64_t* block_end);

/* Same output, blocks split into chunks encoded by `threads` OpenMP threads
 * into private buffers and concatenated afterwards (the reference's OpenMP
 * driver, src/template/ompcompress.c:155-210 + src/share/parallel.c). */
uint64_t orc_compress_par(const orc_field* f, const orc_params* p,
                          uint64_t* words, uint64_t bit0, int threads, uint64_t* block_end);

/* Decompress from the word buffer starting at bit offset bit0 into the
 * field.  Returns the end bit offset. */
uint64_t orc_decompress(const orc_field* f, const orc_params* p,
                        const uint64_t* words, uint64_t bit0);

/* Decompress with `threads` OpenMP threads, each block from its start bit
 * block_start[b] (NULL: fixed rate, block b at bit0 + b * maxbits).  The
 * reference has no parallel decompressor (src/zfp.c:1137-1138); this one
 * exists so that full-size fields can be checked quickly.  Returns the
 * largest block end bit. */
uint64_t orc_decompress_par(const orc_field* f, const orc_params* p, const uint64_t* words,
                            uint64_t bit0, const uint64_t* block_start, int threads);

/* Upper bound on the encoded bits of one block for these parameters,
 * the per-block term of zfp_stream_maximum_size (src/zfp.c:712-742). */
unsigned orc_block_maxbits(const orc_field* f, const orc_params* p);

#ifdef __cplusplus
}
#endif

#endif
