/* zfp/bitstream.h -- the reference's include path for the bit stream API
 * (reference include/zfp/bitstream.h); the declarations are in
 * bitstream.h one level up. */
#ifndef ZFP_GB300_ZFP_BITSTREAM_H
#define ZFP_GB300_ZFP_BITSTREAM_H
#include "../bitstream.h"
#endif
