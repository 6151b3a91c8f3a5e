/*
 * zfp/version.h -- version macros of the API this library implements
 * (reference include/zfp/version.h): library 1.0.1, codec 5.  Programs test
 * these to pick code paths, so names and values are the reference's.
 */
#ifndef ZFP_VERSION_H
#define ZFP_VERSION_H

#define ZFP_VERSION_MAJOR 1
#define ZFP_VERSION_MINOR 0
#define ZFP_VERSION_PATCH 1
#define ZFP_VERSION_TWEAK 0
#define ZFP_VERSION_DEVELOP 1
#define ZFP_CODEC 5

#define _zfp_str_(x) #x
#define _zfp_str(x) _zfp_str_(x)

/* one integer per version: 4 bits each for major, minor, patch, tweak */
#define ZFP_MAKE_VERSION(major, minor, patch, tweak) \
  (((major) << 12) + ((minor) << 8) + ((patch) << 4) + (tweak))
#define ZFP_MAKE_VERSION_STRING(major, minor, patch) \
  _zfp_str(major) "." _zfp_str(minor) "." _zfp_str(patch)
#define ZFP_MAKE_FULLVERSION_STRING(major, minor, patch, tweak) \
  _zfp_str(major) "." _zfp_str(minor) "." _zfp_str(patch) "." _zfp_str(tweak)

#define ZFP_VERSION ZFP_MAKE_VERSION(ZFP_VERSION_MAJOR, ZFP_VERSION_MINOR, ZFP_VERSION_PATCH, ZFP_VERSION_TWEAK)
/* the tweak number is part of the string only when it is not zero */
#define ZFP_VERSION_STRING ZFP_MAKE_VERSION_STRING(ZFP_VERSION_MAJOR, ZFP_VERSION_MINOR, ZFP_VERSION_PATCH)

#endif
