/*
 * zfp/internal/zfp/types.h -- the scalar type names the reference's public
 * headers give their users (reference include/zfp/internal/zfp/types.h):
 * programs written against the reference use them (int32, uint, ...), so
 * they are defined here with the same names, as the fixed-width standard
 * types of C99 / C++11 (the only compilers this library supports).
 */
#ifndef ZFP_TYPES_H
#define ZFP_TYPES_H

typedef unsigned char uchar;
typedef unsigned short ushort;
typedef unsigned int uint;
typedef unsigned long ulong;

#if defined(__cplusplus)
  #include <cinttypes>
  #include <cstdint>
  typedef std::int8_t int8;
  typedef std::uint8_t uint8;
  typedef std::int16_t int16;
  typedef std::uint16_t uint16;
  typedef std::int32_t int32;
  typedef std::uint32_t uint32;
  typedef std::int64_t int64;
  typedef std::uint64_t uint64;
#else
  #include <inttypes.h>
  #include <stdint.h>
  typedef int8_t int8;
  typedef uint8_t uint8;
  typedef int16_t int16;
  typedef uint16_t uint16;
  typedef int32_t int32;
  typedef uint32_t uint32;
  typedef int64_t int64;
  typedef uint64_t uint64;
#endif

/* 64-bit literals and printf/scanf conversions */
#define INT64C(x) INT64_C(x)
#define UINT64C(x) UINT64_C(x)
#define INT64PRId PRId64
#define INT64PRIi PRIi64
#define UINT64PRIo PRIo64
#define UINT64PRIu PRIu64
#define UINT64PRIx PRIx64
#define INT64SCNd SCNd64
#define INT64SCNi SCNi64
#define UINT64SCNo SCNo64
#define UINT64SCNu SCNu64
#define UINT64SCNx SCNx64

#endif
