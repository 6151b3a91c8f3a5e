/* percall_loop.c -- libzfp_gb300_loop.so: a plain C client of the public
 * API (include/zfp.h) that makes one zfp_compress or zfp_decompress call per
 * field, in order, `reps` times over the whole list.  It is the per-array
 * arm the batched launch (zfp_gb300_batch_*) is measured against: the loop
 * a C program using the reference's API would run, with no interpreter in
 * it.  Returns the number of calls that failed (0 on success). */
#include <stddef.h>

#include "../../include/zfp.h"

size_t zfp_gb300_loop_calls(zfp_stream* const* streams, zfp_field* const* fields, size_t count, int direction,
                            int reps) {
  size_t failed = 0;
  for (int r = 0; r < reps; r++)
    for (size_t i = 0; i < count; i++) {
      zfp_stream_rewind(streams[i]);
      const size_t size = direction ? zfp_decompress(streams[i], fields[i]) : zfp_compress(streams[i], fields[i]);
      failed += size == 0;
    }
  return failed;
}
