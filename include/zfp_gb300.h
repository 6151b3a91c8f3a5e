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

#ifdef __cplusplus
}
#endif

#endif
