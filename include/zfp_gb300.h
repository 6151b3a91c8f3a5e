/*
 * zfp_gb300.h -- GPU controls of libzfp_gb300 that have no counterpart in
 * the reference API.  Everything here is optional: a program that only
 * uses zfp.h gets the same results, synchronously, on the legacy default
 * CUDA stream.
 */
#ifndef ZFP_GB300_EXT_H
#define ZFP_GB300_EXT_H

#include <stddef.h>
#include <stdint.h>

#include "zfp.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Run this stream's GPU work on `cuda_stream` (a cudaStream_t; NULL = the
 * legacy default stream).  Selects zfp_exec_cuda if not selected.  Returns
 * zfp_false if the policy cannot be set. */
zfp_bool zfp_gb300_stream_set_cuda_stream(zfp_stream* zfp, void* cuda_stream);

/* With async != 0, a fixed-rate compression or decompression whose field
 * and stream both live in device memory returns as soon as the work is
 * queued on the stream's CUDA stream (its size is known in advance);
 * everything else still returns after the GPU has finished.  Default 0. */
zfp_bool zfp_gb300_stream_set_async(zfp_stream* zfp, int async);

/* Wait for all GPU work queued for this zfp_stream; zfp_false on a CUDA error. */
zfp_bool zfp_gb300_stream_synchronize(zfp_stream* zfp);

/* Reason for the last failure (return value 0) seen by this thread, or "". */
const char* zfp_gb300_last_error(void);

/* Bytes copied between host and device memory by this thread's last
 * zfp_compress / zfp_decompress.  Device buffers, and page-locked host
 * buffers mapped into the device (cudaHostAlloc, cudaHostRegister), are
 * read and written in place by the kernels, so they cost no copy; other
 * host buffers are staged through device memory. */
size_t zfp_gb300_last_staged_bytes(void);

/* ---- failure detection ---------------------------------------------------
 * No counterpart in the reference (its encoders never wait on each other).
 * A variable-rate encoder tile waits, on the GPU, for the bit counts of the
 * tiles before it.  Every such wait is bounded: past this many SM clock
 * cycles the tile takes its predecessor to be lost, the call returns 0 with
 * "GPU wait timed out" in zfp_gb300_last_error(), and the CUDA context stays
 * usable.  0 selects the default, 4e9 cycles (about 2 s at GB300 clocks).
 * Applies to launches made after the call, in this process; returns the
 * previous setting. */
unsigned long long zfp_gb300_set_wait_limit(unsigned long long cycles);

/* Test hook for the bounded wait above, acting on the host: when enabled,
 * the next variable-rate zfp_compress hands out its tiles from the second
 * one on, so the second tile waits for a predecessor that never runs.  That
 * call fails as described above and clears the hook. */
void zfp_gb300_test_skip_first_tile(int enable);

/* ---- batches: many fields in one launch --------------------------------
 * A batch codes `count` independent fields, each with its own zfp_stream
 * (mode, parameters and bit stream, positioned where that stream's next
 * zfp_compress / zfp_decompress would start).  Field data and stream
 * buffers must be device memory.  Fields of the same scalar type and
 * dimensionality run as one persistent launch whose CTAs pull tiles of
 * blocks from a shared counter, so thousands of small, uneven fields keep
 * every SM busy; the launches are captured in a CUDA graph on the first run
 * and replayed afterwards.  The streams, fields and their buffers must stay
 * valid and unchanged in shape until the batch is freed. */
typedef struct zfp_gb300_batch zfp_gb300_batch;

/* direction: 0 = compress, 1 = decompress.  NULL on failure. */
zfp_gb300_batch* zfp_gb300_batch_create(zfp_stream* const* streams, const zfp_field* const* fields,
                                        size_t count, int direction);

/* Queue the batch on `cuda_stream` (NULL = legacy default stream); returns
 * without waiting. */
zfp_bool zfp_gb300_batch_run(zfp_gb300_batch* batch, void* cuda_stream);

/* Wait for the last run, leave every bit stream as zfp_compress /
 * zfp_decompress would and store each field's stream size in bytes in
 * sizes[i] (0 if that field failed).  Returns zfp_false if any failed. */
zfp_bool zfp_gb300_batch_finish(zfp_gb300_batch* batch, size_t* sizes);

void zfp_gb300_batch_free(zfp_gb300_batch* batch);

/* CTAs per SM of the persistent batch launch; 0 (default) lets the built-in
 * autotuner choose on the batch's first run: it times CTAs per SM (1, 2, 3,
 * 4, 6, 8) against how much of each CTA's shared memory stages tile images
 * and stream words (all of the room its occupancy leaves, or half), three
 * runs each, and keeps the best median.  A value set here uses full staging. */
zfp_bool zfp_gb300_batch_set_ctas_per_sm(zfp_gb300_batch* batch, int ctas_per_sm);

/* The launch shape in use once the batch has run (zfp_false before): CTAs per
 * SM and the staging share in percent. */
zfp_bool zfp_gb300_batch_get_tuning(const zfp_gb300_batch* batch, int* ctas_per_sm, int* staging_pct);

/* ---- serving: continuous batching of independent requests --------------
 * A server runs compress / decompress requests on device-resident fields
 * and streams as they arrive.  A dispatcher thread keeps `lanes` CUDA
 * streams busy.  Requests are sorted by the raw size of their field into
 * classes (up to 2 MiB, up to 32 MiB, larger), each with its own queue; the
 * first lanes serve one class each (small, medium, large), the others the
 * large class, and a class without a lane of its own is served by the
 * largest class that has one.  Whenever a lane is free it admits waiting
 * requests of its class in arrival order while the bytes of all admitted,
 * unfinished requests (field span plus stream capacity) stay within
 * `hbm_budget`, and launches them as one batch (one persistent launch per
 * scalar type, dimensionality and reversibility); a request completes with its batch, so
 * small requests never wait for large ones.  Requests that arrive while
 * batches run join the next batch on the next free lane of their class, so
 * work from different batches overlaps on the GPU.  Results are the same
 * streams/arrays zfp_compress / zfp_decompress produce. */
typedef struct zfp_gb300_server zfp_gb300_server;

zfp_gb300_server* zfp_gb300_server_create(size_t hbm_budget, int lanes);

/* direction 0 = compress, 1 = decompress.  Returns a ticket (> 0), or 0 if
 * the request cannot be served (host memory, larger than the budget, ...).
 * The zfp_stream, its bit stream and the field must stay valid until the
 * request has been waited for. */
uint64_t zfp_gb300_server_submit(zfp_gb300_server* server, zfp_stream* zfp, const zfp_field* field,
                                 int direction);

/* Block until the request is done; leaves its bit stream as zfp_compress /
 * zfp_decompress would and returns the stream size in bytes (0 on failure).
 * If seconds is not NULL it receives the time from submission to the end of
 * the request's GPU work. */
size_t zfp_gb300_server_wait(zfp_gb300_server* server, uint64_t ticket, double* seconds);

/* Counters since the server was created: the most bytes ever admitted at
 * once (never above the budget), batches launched, requests completed.
 * Any pointer may be NULL.  Returns 0 for a NULL server. */
int zfp_gb300_server_stats(zfp_gb300_server* server, size_t* peak_bytes, uint64_t* batches, uint64_t* served);

/* Finish everything submitted, stop the dispatcher and release the server. */
void zfp_gb300_server_free(zfp_gb300_server* server);

/* ---- many blocks per call: zfp's block codec in one launch ---------------
 * No counterpart in the reference, which codes one block per call
 * (zfp_encode_block_* / zfp_decode_block_*, declared in zfp.h and also
 * provided here).  `count` full 4^d blocks stored one after another (4^d
 * values each, x fastest) are coded in one GPU launch at the stream's
 * current bit, bit for bit as `count` successive zfp_encode_block_<type>_<dims>
 * calls would write them (and read back as `count` zfp_decode_block calls
 * would): the stream is left at the exact end bit, not flushed.  Blocks and
 * stream may be host or device memory.  Returns the bits written / read, 0
 * on failure. */
size_t zfp_gb300_encode_blocks(zfp_stream* zfp, zfp_type type, unsigned int dims, const void* blocks, size_t count);
size_t zfp_gb300_decode_blocks(zfp_stream* zfp, zfp_type type, unsigned int dims, void* blocks, size_t count);

/* ---- compression without device allocation -----------------------------
 * No counterpart in the reference: zfp_compress there has no GPU scratch.
 * Same stream as zfp_compress (zfp_exec_cuda), for callers that cannot let
 * the library allocate device memory -- for example a program whose device
 * memory belongs to another allocator, or a latency-critical loop that must
 * not trigger an allocation.  Field and stream buffers must be in device
 * memory; nothing is staged, and the encoder's scratch is a fixed 1 MiB
 * device array inside the library (held by every GPU that loads it), which
 * limits a call to 4,194,304 zfp blocks (e.g. 512^3 float).  Larger or
 * host-resident inputs return 0 with a reason in zfp_gb300_last_error().  The first call on a device (in
 * each CUDA context of it) does a set-up step: it looks up that array's
 * device address.  Make that first call before any CUDA stream capture
 * begins.  Each call waits for its own GPU work before it returns.  All
 * calls share the array, which keeps the last call's contents (each call
 * clears what it uses): calls whose GPU work overlaps (other CUDA streams or
 * host threads) race and must be ordered by the caller.  No block index is
 * kept, and one kept for an earlier stream at the same place is dropped, so
 * zfp_decompress of a variable-rate stream written here recovers block
 * offsets by parsing the stream. */
size_t zfp_gb300_compress_noalloc(zfp_stream* zfp, const zfp_field* field);

/* ---- block indexes: zfp's index formats as a side channel ---------------
 * A variable-rate stream carries no block offsets; zfp_decompress of one this
 * library did not write (or no longer remembers) recovers them by parsing the
 * stream on the GPU.  A caller holding zfp's own index of the stream -- the
 * formats of the reference's compressed arrays, include/zfp/index.hpp --
 * can pass it instead, and can take such an index out of a stream this
 * library wrote.  Offsets are bit offsets from the field's first block; an
 * index's range is the stream length in bits (hybrid indexes do not store
 * it).  The stream must be positioned where zfp_decompress would start (after
 * zfp_stream_rewind, or after reading a header). */
#define ZFP_GB300_INDEX_VERBATIM 1  /* uint64 offset per block, plus the range (index.hpp:62) */
#define ZFP_GB300_INDEX_HYBRID4  2  /* 12-byte record per 4 blocks (index.hpp:160) */
#define ZFP_GB300_INDEX_HYBRID8  3  /* two uint64 per 8 blocks, packed for the field's dimensionality (index.hpp:307) */

/* Bytes of an index of `nblocks` blocks in `format` (0: unknown format). */
size_t zfp_gb300_index_bytes(int format, size_t nblocks);

/* Pack nblocks + 1 offsets (offsets[0] = 0, offsets[nblocks] = range) into
 * `format` (dims: the field's dimensionality, used by hybrid8).  Returns the
 * bytes written, 0 if a block or offset is too large for the format. */
size_t zfp_gb300_index_pack(int format, unsigned dims, const uint64_t* offsets, size_t nblocks, void* index,
                            size_t bytes);

/* Unpack an index into nblocks + 1 offsets (range: the stream length in bits,
 * ignored for the verbatim format, which stores it). */
zfp_bool zfp_gb300_index_unpack(int format, unsigned dims, const void* index, size_t bytes, size_t nblocks,
                                uint64_t range, uint64_t* offsets);

/* The index of the stream at zfp's position, which this library wrote for
 * `field` (variable rate: as recorded at compression; fixed rate: from the
 * rate).  Returns the bytes written (0 on failure); *range gets the range. */
size_t zfp_gb300_index_export(const zfp_stream* zfp, const zfp_field* field, int format, void* index,
                              size_t bytes, uint64_t* range);

/* Let the next zfp_decompress of the stream at zfp's position use this index
 * (same field and compression parameters) instead of parsing the stream.
 * Every block is still checked against it while decoding; an index that
 * does not describe the stream costs one parse, not a wrong result. */
zfp_bool zfp_gb300_index_import(zfp_stream* zfp, const zfp_field* field, int format, const void* index,
                                size_t bytes, uint64_t range);

#ifdef __cplusplus
}
#endif

#endif
