/* zfp/internal/zfp/macros.h -- MIN/MAX, which the reference's headers
 * provide to its tools (reference include/zfp/internal/zfp/macros.h). */
#ifndef ZFP_MACROS_H
#define ZFP_MACROS_H

#define MIN(x, y) ((x) < (y) ? (x) : (y))
#define MAX(x, y) ((x) > (y) ? (x) : (y))

#endif
