/*
 * Test infrastructure only (never linked by the product): a thin C layer over
 * the reference's own test utilities -- its seeded smooth-random field
 * generator (tests/utils/genSmoothRandNums.c) and its stream and array
 * hashes (tests/utils/zfpHash.c) -- compiled from the sources where they lie
 * by `make -C oracle kat`.  It lets tests/test_kat.py feed the oracle the
 * exact arrays the reference's end-to-end tests compress and compare the
 * oracle's streams and decoded arrays with the checksums those tests ship
 * (tests/constants/checksums/*.h, keys from tests/utils/zfpChecksums.c).
 */
#include <stddef.h>
#include <stdint.h>
#include <stdlib.h>

#include "utils/genSmoothRandNums.h"
#include "utils/zfpHash.h"

/* element counts of the reference's end-to-end tests
   (tests/src/endtoend/zfpEndtoendBase.c:19-23) */
#define KAT_FLOAT_ELEMENTS 1000000
#define KAT_INT_ELEMENTS 4096

/* type: zfp_type (1 int32, 2 int64, 3 float, 4 double).  Returns the array
   (free with kat_free), its side length and total length. */
void* kat_generate(int type, int dims, size_t* side, size_t* total)
{
  void* arr = NULL;
  switch (type) {
    case 1: generateSmoothRandInts32(KAT_INT_ELEMENTS, dims, 32 - 2, (int32**)&arr, side, total); break;
    case 2: generateSmoothRandInts64(KAT_INT_ELEMENTS, dims, 64 - 2, (int64**)&arr, side, total); break;
    case 3: generateSmoothRandFloats(KAT_FLOAT_ELEMENTS, dims, (float**)&arr, side, total); break;
    default: generateSmoothRandDoubles(KAT_FLOAT_ELEMENTS, dims, (double**)&arr, side, total); break;
  }
  return arr;
}

void kat_free(void* p) { free(p); }

uint64_t kat_hash_stream(uint64_t* words, size_t bytes) { return hashBitstream((uint64*)words, bytes); }

uint64_t kat_hash_array(int bits, const void* arr, size_t n, ptrdiff_t stride)
{
  return bits == 32 ? (uint64_t)hashArray32((const uint32*)arr, n, stride)
                    : (uint64_t)hashArray64((const uint64*)arr, n, stride);
}
