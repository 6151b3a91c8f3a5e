// codec.cuh -- zfp fixed-/variable-rate block codec, one zfp block per thread.
//
// Everything here is __host__ __device__ so the per-block logic can be run on
// the CPU against the oracle; the kernels (kernels.cuh) supply the
// bit sinks/sources, gather/scatter and the stream assembly.
//
// Design (GB300-first, not a translation of src/cuda_zfp):
//  * a thread owns one 4^d block; for d <= 3 the whole block lives in
//    registers (all loops unrolled, coefficient permutation resolved at
//    compile time);
//  * bit planes are formed by a register bit-matrix transpose (byte-permute
//    for the 16/8-bit levels, masked swaps below) instead of per-bit loops;
//  * group tests are coded a byte of coefficient bits at a time from a
//    table (emit_block_seq) and decoded a window of whole events at a
//    time (event_window), never bit by bit;
//  * the rate-limited and whole-plane coders of the reference are one coder
//    here: the rate-limited stream is the whole-plane stream cut at maxbits
//    (src/template/encode.c:92-256), which is exactly what a per-bit budget
//    produces.
// Bit-level format: src/template/encodef.c:63-90 (lossy floating point),
// encode.c:260-280 (integers), revencode*.c (reversible),
// include/zfp/bitstream.inl:226-313 (64-bit words, LSB first).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

#if defined(__CUDACC__)
#define ZG_HD __host__ __device__ __forceinline__
#else
#define ZG_HD inline
#endif

namespace zg {

// ---------------------------------------------------------------------------
// scalar traits (src/traits{f,d,i,l}.h)

template <typename S> struct Traits;
template <> struct Traits<float> {
  using Bits = uint32_t; using Int = int32_t; using UInt = uint32_t;
  static constexpr bool kFloat = true;
  static constexpr int kPrec = 32, kEBits = 8, kEBias = 127, kPBits = 5, kMant = 23;
};
template <> struct Traits<double> {
  using Bits = uint64_t; using Int = int64_t; using UInt = uint64_t;
  static constexpr bool kFloat = true;
  static constexpr int kPrec = 64, kEBits = 11, kEBias = 1023, kPBits = 6, kMant = 52;
};
template <> struct Traits<int32_t> {
  using Bits = uint32_t; using Int = int32_t; using UInt = uint32_t;
  static constexpr bool kFloat = false;
  static constexpr int kPrec = 32, kEBits = 0, kEBias = 0, kPBits = 5, kMant = 0;
};
template <> struct Traits<int64_t> {
  using Bits = uint64_t; using Int = int64_t; using UInt = uint64_t;
  static constexpr bool kFloat = false;
  static constexpr int kPrec = 64, kEBits = 0, kEBias = 0, kPBits = 6, kMant = 0;
};

constexpr int kMinExp = -1074;  // ZFP_MIN_EXP; minexp below it selects reversible mode

struct BlockParams {
  uint32_t minbits, maxbits, maxprec;
  int32_t minexp;
};

// Which code paths a kernel carries: both (jobs of mixed modes), or only
// the lossy / only the reversible one -- each specialisation keeps the
// other path's registers out of the kernel.
// kLossyFloor: lossy blocks whose planes below P - maxprec have no room in
// the plane buffer (store_planes, decode_planes and uncode_coeffs skip them)
// kLossyHost / kRevHost: lossy / reversible blocks of an encode into host
// memory (kernels.cuh stages every tile the image holds, which the
// device-memory kernels do not do for fixed-rate or large tiles)
// kFixedOnly: fixed-rate blocks only (the 64-bit 3D decoder: no block index
// or variable-rate paths in the kernel)
enum ModeSel { kAnyMode = 0, kLossyOnly = 1, kRevOnly = 2, kLossyFloor = 3, kLossyHost = 4, kFixedOnly = 5, kRevHost = 6 };

template <int kSel>
ZG_HD bool is_rev(const BlockParams& p) {
  return kSel == kRevOnly || kSel == kRevHost || (kSel == kAnyMode && p.minexp < kMinExp);
}

// ---------------------------------------------------------------------------
// bit helpers with host equivalents

ZG_HD unsigned ctz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return (unsigned)(__ffsll((long long)x) - 1);
#else
  return (unsigned)__builtin_ctzll(x);
#endif
}

ZG_HD uint32_t byte_perm(uint32_t x, uint32_t y, uint32_t s) {
#if defined(__CUDA_ARCH__)
  return __byte_perm(x, y, s);
#else
  uint64_t xy = ((uint64_t)y << 32) | x;
  uint32_t r = 0;
  for (int i = 0; i < 4; i++)
    r |= (uint32_t)((xy >> (8 * ((s >> (4 * i)) & 7))) & 0xff) << (8 * i);
  return r;
#endif
}

ZG_HD uint64_t low_bits(uint64_t v, unsigned n) { return n >= 64 ? v : v & ((uint64_t(1) << n) - 1); }

ZG_HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}

// count of leading zeros of a nonzero word
ZG_HD int clz64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __clzll((long long)x);
#else
  return __builtin_clzll(x);
#endif
}

ZG_HD unsigned ctz32(uint32_t x) {      // x nonzero
#if defined(__CUDA_ARCH__)
  return (unsigned)__clz(__brev(x));
#else
  return (unsigned)__builtin_ctz(x);
#endif
}

ZG_HD unsigned clz32(uint32_t x) {      // x nonzero
#if defined(__CUDA_ARCH__)
  return (unsigned)__clz(x);
#else
  return (unsigned)__builtin_clz(x);
#endif
}

ZG_HD unsigned popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return (unsigned)__popc(x);
#else
  return (unsigned)__builtin_popcount(x);
#endif
}

// bit j of the result: parity of bits 0..j of x
ZG_HD uint32_t prefix_xor32(uint32_t x) {
  x ^= x << 1;
  x ^= x << 2;
  x ^= x << 4;
  x ^= x << 8;
  x ^= x << 16;
  return x;
}

// ---------------------------------------------------------------------------
// coefficient order (src/template/codec{2,3,4}.c): by total sequency
// i+j+k(+l), then by i^2+j^2+k^2(+l^2); ties in the order the format fixes.
// Index = i + 4j + 16k + 64l.  The tables are packed at compile time into
// 64-bit constants so that, in unrolled code, perm<D>(i) folds to a
// register index.

namespace detail {
constexpr unsigned char kOrder2[16] = {0, 1, 4, 5, 2, 8, 6, 9, 3, 12, 10, 7, 13, 11, 14, 15};
constexpr unsigned char kOrder3[64] = {
    0, 1, 4, 16, 20, 17, 5, 2, 8, 32, 21, 6, 18, 24, 9, 33,
    36, 3, 12, 48, 22, 25, 37, 40, 34, 10, 7, 19, 28, 13, 49, 52,
    41, 38, 26, 23, 29, 53, 11, 35, 44, 14, 50, 56, 42, 27, 39, 45,
    30, 54, 57, 60, 51, 15, 43, 46, 58, 61, 55, 31, 62, 59, 47, 63};
constexpr uint64_t pack2() {
  uint64_t v = 0;
  for (int i = 0; i < 16; i++) v |= (uint64_t)kOrder2[i] << (4 * i);
  return v;
}
constexpr uint64_t pack3(int w) {
  uint64_t v = 0;
  for (int j = 0; j < 10 && 10 * w + j < 64; j++) v |= (uint64_t)kOrder3[10 * w + j] << (6 * j);
  return v;
}
constexpr uint64_t kP2 = pack2();
constexpr uint64_t kP3_0 = pack3(0), kP3_1 = pack3(1), kP3_2 = pack3(2), kP3_3 = pack3(3),
                   kP3_4 = pack3(4), kP3_5 = pack3(5), kP3_6 = pack3(6);
}  // namespace detail

// 4D order is only read by the rolled 4D path (runtime index); one copy per
// translation unit since the library is built without relocatable device code
#define ZG_ORDER4_DATA \
    0, 1, 4, 16, 64, 5, 80, 17, 68, 65, 20, 2, 8, 32, 128, 84, \
    81, 69, 21, 6, 18, 66, 24, 72, 9, 96, 33, 36, 129, 132, 144, 3, \
    12, 48, 192, 85, 82, 70, 22, 73, 25, 88, 37, 100, 97, 148, 145, 133, \
    10, 160, 34, 136, 130, 40, 7, 19, 67, 28, 76, 13, 112, 49, 52, 193, \
    196, 208, 86, 89, 101, 149, 161, 137, 41, 134, 38, 164, 26, 152, 146, 104, \
    98, 74, 83, 71, 23, 77, 29, 92, 53, 116, 113, 212, 209, 197, 11, 35, \
    131, 44, 140, 14, 176, 50, 56, 194, 200, 224, 90, 165, 102, 153, 150, 105, \
    168, 162, 138, 42, 87, 93, 117, 213, 27, 75, 99, 39, 135, 147, 108, 45, \
    141, 156, 30, 78, 177, 180, 54, 114, 120, 57, 198, 210, 216, 201, 225, 228, \
    15, 240, 51, 204, 195, 60, 169, 166, 154, 106, 91, 103, 151, 109, 157, 94, \
    181, 118, 121, 214, 217, 229, 163, 139, 43, 142, 46, 172, 58, 184, 178, 232, \
    226, 202, 241, 205, 61, 199, 55, 244, 31, 220, 211, 124, 115, 79, 170, 167, \
    155, 107, 158, 110, 173, 122, 185, 182, 233, 230, 218, 95, 245, 119, 221, 215, \
    125, 242, 206, 62, 203, 59, 248, 47, 236, 227, 188, 179, 143, 171, 174, 186, \
    234, 246, 222, 126, 219, 123, 249, 111, 237, 231, 189, 183, 159, 252, 243, 207, \
    63, 175, 250, 187, 238, 235, 190, 253, 247, 223, 127, 254, 251, 239, 191, 255,
#if defined(__CUDACC__)
static __device__ __constant__ unsigned char kOrder4Dev[256] = {ZG_ORDER4_DATA};
#endif
static const unsigned char kOrder4Host[256] = {ZG_ORDER4_DATA};
#undef ZG_ORDER4_DATA

template <int D>
ZG_HD int perm(int i) {
  if (D == 1) return i;
  if (D == 2) return (int)((detail::kP2 >> (4 * i)) & 15);
  if (D == 3) {
    const uint64_t w = i < 10 ? detail::kP3_0 : i < 20 ? detail::kP3_1 : i < 30 ? detail::kP3_2
                     : i < 40 ? detail::kP3_3 : i < 50 ? detail::kP3_4 : i < 60 ? detail::kP3_5
                     : detail::kP3_6;
    return (int)((w >> (6 * (i % 10))) & 63);
  }
#if defined(__CUDA_ARCH__)
  return kOrder4Dev[i];
#else
  return kOrder4Host[i];
#endif
}

// ---------------------------------------------------------------------------
// IEEE-754 helpers (replace libm frexp/ldexp with exact bit arithmetic)

template <typename S> ZG_HD S from_bits(typename Traits<S>::Bits b) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(S) == 4) return __int_as_float((int)b);
  else return __longlong_as_double((long long)b);
#else
  S s; std::memcpy(&s, &b, sizeof s); return s;
#endif
}
template <typename S> ZG_HD typename Traits<S>::Bits to_bits(S s) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(S) == 4) return (uint32_t)__float_as_int(s);
  else return (uint64_t)__double_as_longlong(s);
#else
  typename Traits<S>::Bits b; std::memcpy(&b, &s, sizeof b); return b;
#endif
}

// 2^e rounded like ldexp(1, e): inf above range, exact subnormals, 0 below
// half of the smallest subnormal
template <typename S> ZG_HD S pow2(int e) {
  using T = Traits<S>;
  using B = typename T::Bits;
  constexpr int kEminSub = 1 - T::kEBias - T::kMant;
  B b;
  if (e > T::kEBias) b = B((B(1) << T::kEBits) - 1) << T::kMant;
  else if (e >= 1 - T::kEBias) b = B(e + T::kEBias) << T::kMant;
  else if (e >= kEminSub) b = B(1) << (e - kEminSub);
  else b = 0;
  return from_bits<S>(b);
}

template <typename S> ZG_HD S fmul(S a, S b) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(S) == 4) return __fmul_rn(a, b);
  else return __dmul_rn(a, b);
#else
  return a * b;
#endif
}

// truncating float -> integer of the same width; valid for |x| < 2^(p-1)
template <typename S> ZG_HD typename Traits<S>::Int trunc_int(S x) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(S) == 4) return __float2int_rz(x);
  else return __double2ll_rz(x);
#else
  return (typename Traits<S>::Int)x;
#endif
}

// truncation toward zero, in the same format
template <typename S> ZG_HD S ftrunc(S x) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(S) == 4) return truncf(x);
  else return trunc(x);
#else
  return std::trunc(x);
#endif
}

// round-to-nearest integer -> float of the same width
template <typename S> ZG_HD S int_to_float(typename Traits<S>::Int i) {
#if defined(__CUDA_ARCH__)
  if constexpr (sizeof(S) == 4) return __int2float_rn(i);
  else return __ll2double_rn(i);
#else
  return (S)i;
#endif
}

// number of bit planes to code (src/template/codecf.c:6-13)
ZG_HD unsigned coded_precision(int emax, unsigned maxprec, int minexp, int dims) {
  long long p = (long long)emax - minexp + 2 * dims + 2;
  if (p < 0) p = 0;
  return (unsigned long long)p < maxprec ? (unsigned)p : maxprec;
}

// Largest normalised exponent of the block's finite/infinite |values|
// (src/template/encodef.c:11-40).  NaNs never win the reference's
// `max < f` test; an infinite maximum gets exponent 0 (glibc frexp).
// `special` reports a NaN or infinity anywhere in the block.
template <typename S, int N>
ZG_HD int block_emax(const typename Traits<S>::Bits (&raw)[N], bool& special) {
  using T = Traits<S>;
  using B = typename T::Bits;
  constexpr B kAbs = ~(B(1) << (8 * sizeof(B) - 1));
  constexpr B kInf = B((B(1) << T::kEBits) - 1) << T::kMant;
  B top = 0;
  if constexpr (sizeof(B) == 8) {
    // the exponent sits in the high word: 32-bit maxima, plus an OR of the
    // low words to tell subnormals from zeros
    uint32_t hi = 0, lo = 0;
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) {
      const uint32_t a = (uint32_t)(raw[i] >> 32) & 0x7fffffffu;
      hi = a > hi ? a : hi;
      lo |= (uint32_t)raw[i];
    }
    top = ((B)hi << 32) | (hi ? 0u : lo);   // same exponent field and zero test as the true maximum
  } else {
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) {
      B a = raw[i] & kAbs;
      top = a > top ? a : top;
    }
  }
  special = top >= kInf;
  if (special) {
    top = 0;
    for (int i = 0; i < N; i++) {
      B a = raw[i] & kAbs;
      if (a <= kInf && a > top) top = a;
    }
  }
  if (top == 0) return -T::kEBias;
  if (top == kInf) return 0;
  int biased = (int)(top >> T::kMant);
  return biased ? biased - (T::kEBias - 1) : 1 - T::kEBias;
}

// |x| = m * 2^q for a finite bit pattern (m = 0 for both zeros)
template <typename S>
ZG_HD typename Traits<S>::Bits significand(typename Traits<S>::Bits b, int& q) {
  using T = Traits<S>;
  using B = typename T::Bits;
  const int e = (int)((b >> T::kMant) & ((B(1) << T::kEBits) - 1));
  q = (e ? e : 1) - (T::kEBias + T::kMant);
  const B m = b & ((B(1) << T::kMant) - 1);
  return e ? m | (B(1) << T::kMant) : m;
}

// trunc(x * 2^se) from the bits alone, for finite x with |x| * 2^se below
// 2^(P-1).  Equal to the rounded product followed by truncation: scaling by
// a power of two is exact unless the product falls below the normal range,
// and such a product truncates to 0 either way.  Double precision uses it
// because the FP64 pipe of this GPU is narrow.
template <typename S>
ZG_HD typename Traits<S>::Int scale_trunc(typename Traits<S>::Bits b, int se) {
  using T = Traits<S>;
  using B = typename T::Bits;
  constexpr int W = 8 * sizeof(B);
  int q;
  const B m = significand<S>(b, q);
  const int t = q + se;
  const B a = t >= 0 ? B(m << t) : (-t < W ? B(m >> -t) : B(0));
  const B neg = B(0) - (b >> (W - 1));   // all ones for negative x
  return (typename T::Int)((a ^ neg) - neg);
}

// bits of (S)v * 2^e with round-to-nearest-even at the conversion, for
// results in the normal range (the product itself is then exact)
template <typename S>
ZG_HD typename Traits<S>::Bits int_scale(typename Traits<S>::Int v, int e) {
  using T = Traits<S>;
  using B = typename T::Bits;
  constexpr int W = 8 * sizeof(B);
  constexpr int kDrop = W - 1 - T::kMant;
  const B neg = B(0) - B(v < 0);
  const B a = (B(v) ^ neg) - neg;
  if (!a) return 0;
  const int lz = clz64((uint64_t)a) - (64 - W);
  const B n = a << lz;
  B mant = n >> kDrop;                                   // with the leading one at bit kMant
  const B rem = n & ((B(1) << kDrop) - 1), half = B(1) << (kDrop - 1);
  mant += B((rem > half) | ((rem == half) & (unsigned)(mant & 1)));   // a carry lands in the exponent
  const int ex = W - 1 - lz + e;                         // exponent of the leading one
  return (B(ex + T::kEBias - 1) << T::kMant) + mant + (neg & (B(1) << (W - 1)));
}

// block-floating-point cast (src/template/encodef.c:44-59).  Out-of-range
// or NaN products give the x86 integer-indefinite value, as the reference
// does on x86-64; that only happens in blocks with NaN/inf or with a scale
// factor that overflows (tiny blocks), so the common path has no checks.
template <typename S>
ZG_HD typename Traits<S>::Int cast_slow(typename Traits<S>::Bits b, S s) {
  using T = Traits<S>;
  using I = typename T::Int;
  const S lim = pow2<S>(T::kPrec - 1);
  const S x = fmul<S>(s, from_bits<S>(b));
  return (x < lim && x > -lim) ? trunc_int<S>(x) : (I)((typename T::UInt)1 << (T::kPrec - 1));
}

template <typename S, int N>
ZG_HD void fwd_cast(const typename Traits<S>::Bits (&raw)[N], typename Traits<S>::Int (&v)[N],
                    int emax, bool special) {
  using T = Traits<S>;
  const int se = T::kPrec - 2 - emax;
  const S s = pow2<S>(se);
  if (!special && se <= T::kEBias) {
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) {
      if constexpr (sizeof(S) == 8) v[i] = scale_trunc<S>(raw[i], se);
      else v[i] = trunc_int<S>(fmul<S>(s, from_bits<S>(raw[i])));
    }
  } else {
    for (int i = 0; i < N; i++) v[i] = cast_slow<S>(raw[i], s);
  }
}

// inverse cast (src/template/codecf.c:17-32)
template <typename S, int N>
ZG_HD void inv_cast(const typename Traits<S>::Int (&v)[N], typename Traits<S>::Bits (&raw)[N], int emax) {
  using T = Traits<S>;
  const int e = emax - (T::kPrec - 2);
  if constexpr (sizeof(S) == 8) {
    // every product normal: smallest |v| = 1 and largest 2^(P-1) stay in range
    if (e >= 1 - T::kEBias && e + T::kPrec - 1 <= T::kEBias) {
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) raw[i] = int_scale<S>(v[i], e);
      return;
    }
  }
  const S s = pow2<S>(e);
#pragma unroll (N <= 64 ? N : 1)
  for (int i = 0; i < N; i++) raw[i] = to_bits<S>(fmul<S>(s, int_to_float<S>(v[i])));
}

// Reversible floating-point blocks: does the block-floating-point cast
// round-trip bit for bit (src/template/revencodef.c:9-16)?  When no value is
// special and 2^(emax-(P-2)) is a normal number, both casts only scale by
// powers of two, so the answer is yes exactly when no value is -0 and every
// nonzero value's lowest set bit is worth at least 2^(emax-(P-2)).  Otherwise
// each value is cast and cast back.  Nothing is kept, so the caller's raw
// array is the only live copy of the block.
template <typename S, int N>
ZG_HD bool bfp_exact(const typename Traits<S>::Bits (&raw)[N], int emax, bool special) {
  using T = Traits<S>;
  using B = typename T::Bits;
  const int lo = emax - (T::kPrec - 2);
  bool exact = true;
  if (!special && lo >= 1 - T::kEBias) {
    if constexpr (sizeof(S) == 4) {
      // float: on the FP32 pipe.  x * 2^(P-2-emax) is exact unless it falls
      // below the normal range, and is then nonzero only if it is not an
      // integer; a value that vanishes there (y == 0, x != 0) is not exact.
      const S s = pow2<S>(T::kPrec - 2 - emax);
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) {
        const S y = fmul<S>(s, from_bits<S>(raw[i]));
        const bool zero = (B)(raw[i] << 1) == 0;
        exact &= zero ? raw[i] == 0 : (y == ftrunc<S>(y)) & (y != S(0));
      }
    } else {
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) {
        int q;
        const B m = significand<S>(raw[i], q);
        exact &= m ? q + (int)ctz64((uint64_t)m) >= lo : raw[i] == 0;
      }
    }
  } else {
    const S s = pow2<S>(T::kPrec - 2 - emax), r = pow2<S>(lo);
    for (int i = 0; i < N; i++)
      exact &= to_bits<S>(fmul<S>(r, int_to_float<S>(cast_slow<S>(raw[i], s)))) == raw[i];
  }
  return exact;
}

// ---------------------------------------------------------------------------
// lifting steps (src/template/encode.c:31-56, decode.c:9-45,
// revencode.c:7-33, revdecode.c:7-33); integers wrap like the reference

template <typename I>
ZG_HD void fwd_lift(I& a, I& b, I& c, I& d) {
  using U = typename std::make_unsigned<I>::type;
  a = (I)((U)a + (U)d); a >>= 1; d = (I)((U)d - (U)a);
  c = (I)((U)c + (U)b); c >>= 1; b = (I)((U)b - (U)c);
  a = (I)((U)a + (U)c); a >>= 1; c = (I)((U)c - (U)a);
  d = (I)((U)d + (U)b); d >>= 1; b = (I)((U)b - (U)d);
  d = (I)((U)d + (U)(b >> 1)); b = (I)((U)b - (U)(d >> 1));
}

template <typename I>
ZG_HD void inv_lift(I& a, I& b, I& c, I& d) {
  using U = typename std::make_unsigned<I>::type;
  b = (I)((U)b + (U)(d >> 1)); d = (I)((U)d - (U)(b >> 1));
  b = (I)((U)b + (U)d); d = (I)((U)d - ((U)b - (U)d));
  c = (I)((U)c + (U)a); a = (I)((U)a - ((U)c - (U)a));
  b = (I)((U)b + (U)c); c = (I)((U)c - ((U)b - (U)c));
  d = (I)((U)d + (U)a); a = (I)((U)a - ((U)d - (U)a));
}

template <typename I>
ZG_HD void rev_fwd_lift(I& a, I& b, I& c, I& d) {
  using U = typename std::make_unsigned<I>::type;
  U x = (U)a, y = (U)b, z = (U)c, w = (U)d;
  w -= z; z -= y; y -= x;
  w -= z; z -= y;
  w -= z;
  a = (I)x; b = (I)y; c = (I)z; d = (I)w;
}

template <typename I>
ZG_HD void rev_inv_lift(I& a, I& b, I& c, I& d) {
  using U = typename std::make_unsigned<I>::type;
  U x = (U)a, y = (U)b, z = (U)c, w = (U)d;
  w += z;
  z += y; w += z;
  y += x; z += y; w += z;
  a = (I)x; b = (I)y; c = (I)z; d = (I)w;
}

// Separable transform over a 4^D block: axes x, y, z, w in that order for
// the forward direction, the reverse order for the inverse
// (src/template/encode3.c:35-50, decode3.c:27-42, encode4.c:42-65).
enum LiftKind { kFwd, kInv, kRevFwd, kRevInv };

template <LiftKind K, typename I>
ZG_HD void lift(I& a, I& b, I& c, I& d) {
  if constexpr (K == kFwd) fwd_lift(a, b, c, d);
  else if constexpr (K == kInv) inv_lift(a, b, c, d);
  else if constexpr (K == kRevFwd) rev_fwd_lift(a, b, c, d);
  else rev_inv_lift(a, b, c, d);
}

template <LiftKind K, int D, typename I>
ZG_HD void xform(I (&v)[1 << (2 * D)]);

// 4D: lifts along x, y and z never mix the four w-slices of 64 values, so
// each slice goes through the 3D transform in registers (all of its
// indexes compile-time), and the w lifts -- one per (x, y, z) position
// across the slices -- come after (forward) or before (inverse) them.  The
// block array itself stays in local memory; only whole slices and one
// position's four values cross it.
template <LiftKind K, typename I>
ZG_HD void xform4(I (&v)[256]) {
  constexpr bool kInverse = (K == kInv || K == kRevInv);
  auto w_lifts = [&]() {
#pragma unroll 4
    for (int j = 0; j < 64; j++) lift<K>(v[j], v[j + 64], v[j + 128], v[j + 192]);
  };
  if (kInverse) w_lifts();
#pragma unroll 1
  for (int w = 0; w < 4; w++) {
    I r[64];
#pragma unroll
    for (int j = 0; j < 64; j++) r[j] = v[64 * w + j];
    xform<K, 3>(r);
#pragma unroll
    for (int j = 0; j < 64; j++) v[64 * w + j] = r[j];
  }
  if (!kInverse) w_lifts();
}

template <LiftKind K, int D, typename I>
ZG_HD void xform(I (&v)[1 << (2 * D)]) {
  constexpr int N = 1 << (2 * D);
  constexpr bool kInverse = (K == kInv || K == kRevInv);
  if constexpr (D == 4) {
    xform4<K>(v);
  } else {
#pragma unroll
    for (int step = 0; step < D; step++) {
      const int axis = kInverse ? D - 1 - step : step;
      const int s = 1 << (2 * axis);
#pragma unroll
      for (int i = 0; i < N; i++)
        if (((i >> (2 * axis)) & 3) == 0) lift<K>(v[i], v[i + s], v[i + 2 * s], v[i + 3 * s]);
    }
  }
}

// negabinary (src/template/encode.c:76-79, decode.c:64-67)
template <typename U> ZG_HD U nb_mask() { return (U)0xaaaaaaaaaaaaaaaaull; }
template <typename I> ZG_HD typename std::make_unsigned<I>::type to_nb(I x) {
  using U = typename std::make_unsigned<I>::type;
  return ((U)x + nb_mask<U>()) ^ nb_mask<U>();
}
template <typename I> ZG_HD I from_nb(typename std::make_unsigned<I>::type u) {
  using U = typename std::make_unsigned<I>::type;
  return (I)((u ^ nb_mask<U>()) - nb_mask<U>());
}

// ---------------------------------------------------------------------------
// bit planes: P[k] bit i = bit k of coefficient i (coefficients in coding
// order).  32x32 bit-matrix transpose: byte permutes for the 16- and 8-bit
// levels, masked swaps for 4, 2, 1.  It is its own inverse.

ZG_HD void transpose32(uint32_t (&a)[32]) {
#pragma unroll
  for (int i = 0; i < 16; i++) {
    uint32_t x = a[i], y = a[i + 16];
    a[i] = byte_perm(x, y, 0x5410);
    a[i + 16] = byte_perm(x, y, 0x7632);
  }
#pragma unroll
  for (int i = 0; i < 32; i++)
    if ((i & 8) == 0) {
      uint32_t x = a[i], y = a[i + 8];
      a[i] = byte_perm(x, y, 0x6240);
      a[i + 8] = byte_perm(x, y, 0x7351);
    }
#pragma unroll
  for (int i = 0; i < 32; i++)
    if ((i & 4) == 0) {
      uint32_t t = ((a[i] >> 4) ^ a[i + 4]) & 0x0f0f0f0fu;
      a[i] ^= t << 4; a[i + 4] ^= t;
    }
#pragma unroll
  for (int i = 0; i < 32; i++)
    if ((i & 2) == 0) {
      uint32_t t = ((a[i] >> 2) ^ a[i + 2]) & 0x33333333u;
      a[i] ^= t << 2; a[i + 2] ^= t;
    }
#pragma unroll
  for (int i = 0; i < 32; i++)
    if ((i & 1) == 0) {
      uint32_t t = ((a[i] >> 1) ^ a[i + 1]) & 0x55555555u;
      a[i] ^= t << 1; a[i + 1] ^= t;
    }
}

// coefficients (N <= 64) -> planes
template <int N, typename U, int P>
ZG_HD void make_planes(const U (&u)[N], uint64_t (&pl)[P]) {
  static_assert(N <= 64, "wide blocks use the rolled coder");
  if constexpr (N == 4) {
#pragma unroll
    for (int k = 0; k < P; k++) {
      uint64_t x = 0;
#pragma unroll
      for (int i = 0; i < 4; i++) x |= (uint64_t)((u[i] >> k) & 1u) << i;
      pl[k] = x;
    }
  } else {
    uint32_t a[32];
#pragma unroll
    for (int half = 0; half < (int)sizeof(U) / 4; half++) {      // which 32-bit half of U
#pragma unroll
      for (int grp = 0; grp < (N + 31) / 32; grp++) {            // coefficients 0..31 / 32..63
#pragma unroll
        for (int i = 0; i < 32; i++) {
          const int c = 32 * grp + i;
          a[i] = c < N ? (uint32_t)((uint64_t)u[c < N ? c : 0] >> (32 * half)) : 0u;
        }
        transpose32(a);
#pragma unroll
        for (int k = 0; k < 32; k++) {
          if (grp == 0) pl[32 * half + k] = a[k];
          else pl[32 * half + k] |= (uint64_t)a[k] << 32;
        }
      }
    }
  }
}

// planes -> coefficients
template <int N, typename U, int P>
ZG_HD void take_planes(const uint64_t (&pl)[P], U (&u)[N]) {
  static_assert(N <= 64, "wide blocks use the rolled coder");
  if constexpr (N == 4) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
      U x = 0;
#pragma unroll
      for (int k = 0; k < P; k++) x |= (U)((pl[k] >> i) & 1u) << k;
      u[i] = x;
    }
  } else {
    uint32_t a[32];
#pragma unroll
    for (int i = 0; i < N; i++) u[i] = 0;
#pragma unroll
    for (int half = 0; half < (int)sizeof(U) / 4; half++) {
#pragma unroll
      for (int grp = 0; grp < (N + 31) / 32; grp++) {
#pragma unroll
        for (int k = 0; k < 32; k++) a[k] = (uint32_t)(pl[32 * half + k] >> (32 * grp));
        transpose32(a);
#pragma unroll
        for (int i = 0; i < 32; i++) {
          const int c = 32 * grp + i;
          if (c < N) u[c < N ? c : 0] |= (U)((uint64_t)a[i] << (32 * half));
        }
      }
    }
  }
}

// 32-bit half h (0 = low) of the plane word at p.  The kernels keep planes
// in shared memory and store halves with 32-bit accesses; the host writes
// half 0 first, as a whole word.
ZG_HD void set_half(uint64_t* p, int h, uint32_t v) {
#if defined(__CUDA_ARCH__)
  reinterpret_cast<uint32_t*>(p)[h] = v;
#else
  if (h) *p |= (uint64_t)v << 32;
  else *p = v;
#endif
}

// coefficients -> planes stored at plane[k * stride].  Each 32x32 transpose
// (one 32-bit half of 32 coefficients) is stored as soon as it is done, so
// no array of all planes is held in registers next to the coefficients.
// 64-bit coefficients whose coded planes all lie in the top half
// (maxprec <= 32: every lossy mode but high precision) transpose only their
// high words.  With kFloor, planes below P - maxprec (never coded) are not
// stored: the kernel gives the buffer no room for them.
template <int N, bool kFloor = false, typename U>
ZG_HD void store_planes(const U (&u)[N], uint64_t* plane, int stride, unsigned maxprec = 8 * sizeof(U)) {
  constexpr int P = 8 * sizeof(U);
  const int kmin = kFloor && (unsigned)P > maxprec ? P - (int)maxprec : 0;   // planes below are never coded
  if constexpr (N == 4) {
    uint64_t pl[P];
    make_planes<N>(u, pl);
#pragma unroll
    for (int k = 0; k < P; k++)
      if (k >= kmin) plane[k * stride] = pl[k];
  } else {
    constexpr int G = (N + 31) / 32, H = P / 32;
    const bool top = P == 64 && maxprec <= 32;
#pragma unroll
    for (int half = 0; half < H; half++) {
      if (top && half == 0) continue;
#pragma unroll
      for (int grp = 0; grp < G; grp++) {
        uint32_t a[32];
#pragma unroll
        for (int i = 0; i < 32; i++) {
          const int c = 32 * grp + i;
          a[i] = c < N ? (uint32_t)((uint64_t)u[c < N ? c : 0] >> (32 * half)) : 0u;
        }
        transpose32(a);
#pragma unroll
        for (int k = 0; k < 32; k++) {
          if (32 * half + k < kmin) continue;
          uint64_t* q = plane + (32 * half + k) * stride;
          if (G == 1) *q = a[k];
          else set_half(q, grp, a[k]);
        }
      }
    }
  }
}


// ---------------------------------------------------------------------------
// embedded plane decoder for N <= 64 coefficients (one 64-bit word per plane)

// Whole events of a 32-bit window of group-test code that starts at a
// positive test.  Past a plane's verbatim bits its code is a run of events
// "1 0^z 1" (positive test, z zero scan bits, the one found) ended by a 0
// (src/template/decode.c:100-113).  The prefix parity of the window is 1
// exactly inside an event (from its test up to its found one), so a 0 of
// parity 0 ends the plane and the ones of parity 0 are the found ones.
// e: bits of the whole events (up to the stop, else up to the last found
// one; 0 if the window holds none); scan: scan bits among them (each stands
// for the next coefficient, n, n+1, ...; so after them n grows by scan);
// found: their found ones; used: bits to consume (the stop included).
struct EventWindow {
  uint32_t found;
  unsigned e, scan, used;
  bool stop;
};

ZG_HD EventWindow event_window(uint32_t w) {
  const uint32_t px = prefix_xor32(w);
  const uint32_t stop = ~(w | px);
  const uint32_t found = w & ~px;
  EventWindow ev;
  ev.e = stop ? ctz32(stop) : found ? 32 - clz32(found) : 0;
  const uint32_t seg = ev.e >= 32 ? ~0u : (1u << ev.e) - 1;
  ev.scan = ev.e - popc32(w & px & seg);
  ev.found = found & seg;
  ev.stop = stop != 0;
  ev.used = ev.e + (stop != 0);
  return ev;
}

struct PlaneBuf {
  uint64_t* p;
  int stride;
};

// The decoder of src/template/decode.c:80-278, rolled over planes: planes k
// down to klo, while budget is left, stored at pb.p[(k - kbase) *
// pb.stride]; on return k is the first plane not decoded.  A positive group
// test and the scan that follows it are read with one peek, or, with kWin,
// a 32-bit window of whole events at a time (event_window): measured faster
// for lossy blocks, which have several events per plane, and slower for
// reversible ones, which have about one per plane before every coefficient
// is significant.  When the budget ends inside a positive group test the
// reference still deposits a one at the scan position; so does this.
template <int N, class Source, bool kWin>
ZG_HD void decode_plane_range(Source& in, unsigned& bits, unsigned& n, int& k, int klo, int kbase, PlaneBuf pb) {
  for (; k >= klo && bits; k--) {
    const unsigned m = n < bits ? n : bits;
    uint64_t x = in.read(m);
    bits -= m;
    while (bits && n < (unsigned)N) {
      if (kWin && bits >= 32 && n + 1 < (unsigned)N) {
        const uint32_t w = in.peek32();
        if (!(w & 1)) {        // negative test: rest of the plane is zero
          in.skip(1);
          bits--;
          break;
        }
        if (w != 1) {          // else no found one in the window
          const EventWindow ev = event_window(w);
          // found one of rank i (from 1) at window bit j: coefficient
          // n + j - i.  Events are taken while their found one lies below
          // the last coefficient (which is implied, never scanned).
          const int room = N - 2 - (int)n;
          uint32_t f = ev.found, y = 0;
          int i = 1, last = -1;
          for (; f; i++) {
            const int j = (int)ctz32(f);
            if (j - i > room) break;
            y |= 1u << (j - i);
            last = j;
            f &= f - 1;
          }
          x |= (uint64_t)y << n;
          if (!f) {            // every event of the window
            n += ev.scan;
            in.skip(ev.used);
            bits -= ev.used;
            if (ev.stop) break;
            continue;
          }
          if (last >= 0) {     // the events before one that reaches the limit
            n += (unsigned)(last + 2 - i);
            in.skip((unsigned)last + 1);
            bits -= (unsigned)last + 1;
            continue;
          }
        }
      }
      // one event at a time: near the budget or the last coefficient, or a
      // scan longer than the window
      const uint64_t w = in.peek64();
      if (!(w & 1)) {          // negative test: rest of the plane is zero
        in.skip(1);
        bits--;
        break;
      }
      // group-test bit plus at most cap = min(bits - 1, N - 1 - n) scan
      // bits; a sentinel at the limit stops the count of trailing zeros
      const unsigned cap = N - 1 - n < bits - 1 ? N - 1 - n : bits - 1;
      const unsigned z = ctz64((w >> 1) | (uint64_t(1) << cap));
      const unsigned adv = z + (z < cap ? 2u : 1u);   // a found one is consumed; at the limit it is implied
      in.skip(adv);
      bits -= adv;
      n += z;
      x |= uint64_t(1) << n;
      n++;
    }
    pb.p[(k - kbase) * pb.stride] = x;
  }
}

// All planes of a block; planes below the last one decoded are zero (with
// kFloor only down to P - maxprec: the ones below are never touched, the
// reader takes them as zero and the kernel gives them no room).  For 64-bit
// coefficients, when every decoded plane lies in the top half, only the top
// half is stored (zeros included) and `top_only` is set: the low words are
// zero.
template <int P, int N, class Source, bool kWin = true, bool kFloor = false>
ZG_HD unsigned decode_planes(Source& in, unsigned budget, unsigned maxprec, PlaneBuf pb, bool& top_only) {
  const int kmin = (unsigned)P > maxprec ? P - (int)maxprec : 0;
  unsigned bits = budget, n = 0;
  int k = P - 1;
  decode_plane_range<N, Source, kWin>(in, bits, n, k, kmin, 0, pb);
  top_only = P == 64 && N > 4 && k >= 31;
  const int kz = top_only ? (kFloor && kmin > 32 ? kmin : 32) : (kFloor ? kmin : 0);
  for (; k >= kz; k--) pb.p[k * pb.stride] = 0;
  return budget - bits;
}

// group-test code of bytes and 16-bit chunks (see the table-driven coder below)
// E(b) in bits 0-15 (every one of the byte b followed by a '1'), popc(b) in bits 16-19
ZG_HD constexpr uint32_t group_code_entry(uint32_t b) {
  uint32_t e = 0, j = 0;
  for (uint32_t p = 0; p < 8; p++)
    if ((b >> p) & 1u) {
      e |= 3u << (p + j);
      j++;
    }
  return e | (j << 16);
}

struct GroupCodeTable {
  uint32_t e[256];
};

constexpr GroupCodeTable make_group_code_table() {
  GroupCodeTable t{};
  for (uint32_t b = 0; b < 256; b++) t.e[b] = group_code_entry(b);
  return t;
}

constexpr GroupCodeTable kGroupCodeHost = make_group_code_table();

// code of 16 group-test bits c of a plane (at most 32 bits), length in len;
// `last`: the plane's last one is in this chunk, at position t of it, and
// `implied` says whether it is the block's last coefficient (then it and its
// test are not written; otherwise the test after it is negative)
ZG_HD uint32_t group_chunk(uint32_t c, const uint32_t* gtab, bool last, unsigned t, bool implied, unsigned& len) {
  const uint32_t e0 = gtab[c & 0xffu], e1 = gtab[c >> 8];
  const unsigned p0 = e0 >> 16, pc = p0 + (e1 >> 16);
  uint32_t code = (e0 & 0xffffu) | ((e1 & 0xffffu) << (8 + p0));
  len = 16 + pc;
  if (last) {
    if (implied) {
      len = t + pc - 1;
      code &= len < 32 ? (1u << len) - 1 : ~0u;
    } else {
      len = t + pc + 1;
      code &= ~(1u << (len - 1));
    }
  }
  return code;
}

// 4D blocks (256 coefficients): bit planes of four 64-bit words, plane k at
// pl[4k .. 4k+3] with coefficient i at bit i % 64 of word i / 64, formed and
// taken apart with the same 32x32 register transposes as 1-3D blocks (eight
// groups of 32 coefficients per 32-bit half of the values).

template <typename U, int P>
ZG_HD void make_planes_wide(const U (&u)[256], uint64_t (&pl)[4 * P]) {
  for (int grp = 0; grp < 8; grp++) {
#pragma unroll
    for (int half = 0; half < P / 32; half++) {
      uint32_t a[32];
#pragma unroll
      for (int i = 0; i < 32; i++) a[i] = (uint32_t)((uint64_t)u[32 * grp + i] >> (32 * half));
      transpose32(a);
#pragma unroll
      for (int k = 0; k < 32; k++) {
        uint64_t& w = pl[4 * (32 * half + k) + grp / 2];
        if (grp & 1) w |= (uint64_t)a[k] << 32;
        else w = a[k];
      }
    }
  }
}

template <typename U, int P>
ZG_HD void take_planes_wide(const uint64_t (&pl)[4 * P], U (&u)[256]) {
  for (int grp = 0; grp < 8; grp++) {
    U acc[32];
#pragma unroll
    for (int i = 0; i < 32; i++) acc[i] = 0;
#pragma unroll
    for (int half = 0; half < P / 32; half++) {
      uint32_t a[32];
#pragma unroll
      for (int k = 0; k < 32; k++) a[k] = (uint32_t)(pl[4 * (32 * half + k) + grp / 2] >> (32 * (grp & 1)));
      transpose32(a);
#pragma unroll
      for (int i = 0; i < 32; i++) acc[i] |= (U)((uint64_t)a[i] << (32 * half));
    }
#pragma unroll
    for (int i = 0; i < 32; i++) u[32 * grp + i] = acc[i];
  }
}

// bits [pos, pos + 16) of a 256-bit plane (zeros past its end)
ZG_HD uint32_t plane_bits16(const uint64_t* x, unsigned pos) {
  const unsigned w = pos >> 6, o = pos & 63;
  uint64_t v = x[w] >> o;
  if (o > 48 && w < 3) v |= x[w + 1] << (64 - o);
  return (uint32_t)v & 0xffffu;
}

// highest set bit of a 256-bit plane, or -1
ZG_HD int plane_top(const uint64_t* x) {
  for (int w = 3; w >= 0; w--)
    if (x[w]) return 64 * w + 63 - clz64(x[w]);
  return -1;
}

// ones of a 256-bit plane in [lo, hi]
ZG_HD unsigned plane_popc(const uint64_t* x, unsigned lo, unsigned hi) {
  unsigned c = 0;
  for (unsigned w = lo >> 6; w <= hi >> 6; w++) {
    uint64_t v = x[w];
    if (w == lo >> 6) v &= ~0ull << (lo & 63);
    if (w == hi >> 6 && (hi & 63) != 63) v &= (2ull << (hi & 63)) - 1;
    c += (unsigned)popc64(v);
  }
  return c;
}

// The coder of emit_block_seq (the same group-test expansion, a 16-bit
// chunk at a time from the byte table) over 256-bit planes: per plane the
// verbatim bits in 64-bit pieces, the opening test, then the chunks up to
// the top one.  With `count` nothing is written and only the length is
// returned: a plane's length is O(1) from its top one and popcount.
template <int P, bool kCount, class Sink>
ZG_HD unsigned code_planes_wide(Sink& out, unsigned budget, unsigned maxprec, const uint64_t* pl,
                                const uint32_t* gtab) {
  constexpr unsigned N = 256;
  const int kmin = (unsigned)P > maxprec ? P - (int)maxprec : 0;
  unsigned left = budget, n = 0;
  auto put = [&](uint64_t v, unsigned len) {   // cut at the budget; false once it is spent
    if (len >= left) {
      if (!kCount) out.put(low_bits(v, left), left);
      left = 0;
      return false;
    }
    if (!kCount) out.put(v, len);
    left -= len;
    return true;
  };
  for (int k = P - 1; k >= kmin && left; k--) {
    const uint64_t* x = pl + 4 * k;
    int top = plane_top(x);
    if (top < (int)n) top = -1;                  // no coefficient becomes significant
    if (kCount) {
      unsigned len = n;
      if (n < N) {
        len += 1;
        if (top >= 0) {
          const unsigned m = plane_popc(x, n, (unsigned)top);
          len += (unsigned)top == N - 1 ? (unsigned)top - n + m - 1 : (unsigned)top - n + 1 + m;
        }
      }
      if (len >= left) return budget;
      left -= len;
      if (top >= 0) n = (unsigned)top + 1;
      continue;
    }
    bool more = true;
    for (unsigned w = 0; w * 64 < n && more; w++) {
      const unsigned c = n - 64 * w < 64 ? n - 64 * w : 64;
      more = put(low_bits(x[w], c), c);
    }
    if (!more) break;
    if (n >= N) continue;
    if (!put(top >= 0, 1)) break;
    if (top < 0) continue;
    const bool implied = (unsigned)top == N - 1;
    const unsigned rem = (unsigned)top - n;
    for (unsigned c = 0; more; c += 16) {
      unsigned clen;
      const uint32_t code = group_chunk(plane_bits16(x, n + c), gtab, rem < c + 16, rem - c, implied, clen);
      more = put(code, clen) && rem >= c + 16;
    }
    if (!left) break;
    n = (unsigned)top + 1;
  }
  return budget - left;
}

// The decoder of src/template/decode.c:80-278 over 256-bit planes: verbatim
// bits in 64-bit pieces, then one significance event at a time, each scan
// 64 bits per peek (4D blocks have up to 255 coefficients to scan).
template <int P, class Source>
ZG_HD unsigned decode_planes_wide(Source& in, unsigned budget, unsigned maxprec, uint64_t (&pl)[4 * P]) {
  constexpr unsigned N = 256;
  const int kmin = (unsigned)P > maxprec ? P - (int)maxprec : 0;
  unsigned bits = budget, n = 0;
  for (int k = 0; k < 4 * P; k++) pl[k] = 0;
  for (int k = P - 1; k >= kmin && bits; k--) {
    uint64_t* x = pl + 4 * k;
    const unsigned m = n < bits ? n : bits;
    for (unsigned w = 0; w * 64 < m; w++) {
      const unsigned c = m - 64 * w < 64 ? m - 64 * w : 64;
      x[w] = in.read(c);
    }
    bits -= m;
    while (bits && n < N) {
      bits--;
      const bool positive = in.peek64() & 1u;
      in.skip(1);
      if (!positive) break;                      // rest of the plane is zero
      // scan at most cap coefficient bits for the next one; none: it is
      // implied (the last coefficient) or the budget ended inside the test
      const unsigned cap = N - 1 - n < bits ? N - 1 - n : bits;
      unsigned z = 0;
      bool found = false;
      while (z < cap) {
        const unsigned c = cap - z < 64 ? cap - z : 64;
        uint64_t w = in.peek64();
        if (c < 64) w |= uint64_t(1) << c;
        const unsigned t = w ? ctz64(w) : 64u;
        if (t < c) {
          in.skip(t + 1);
          z += t;
          found = true;
          break;
        }
        in.skip(c);
        z += c;
      }
      bits -= z + (found ? 1u : 0u);
      n += z;
      x[n >> 6] |= uint64_t(1) << (n & 63);
      n++;
    }
  }
  return budget - bits;
}

// ---------------------------------------------------------------------------
// integer block codec (src/template/encode.c:260-280, decode.c:282-298,
// revencode.c:57-79, revdecode.c:37-55)

// 32 planes in slots 0-31 of pb -> 32-bit values (slot j = bit j), one
// 32x32 transpose per 32 coefficients, loaded a transpose at a time
template <int N>
ZG_HD void take_half_planes(PlaneBuf pb, uint32_t (&v)[N]) {
#pragma unroll
  for (int grp = 0; grp < (N + 31) / 32; grp++) {
    uint32_t a[32];
#pragma unroll
    for (int j = 0; j < 32; j++) a[j] = (uint32_t)(pb.p[j * pb.stride] >> (32 * grp));
    transpose32(a);
#pragma unroll
    for (int i = 0; i < 32; i++)
      if (32 * grp + i < N) v[32 * grp + i < N ? 32 * grp + i : 0] = a[i];
  }
}

template <int D, typename I, class Source, bool kWin = true, bool kFloor = false>
ZG_HD unsigned uncode_coeffs(Source& in, unsigned budget, unsigned maxprec,
                             typename std::make_unsigned<I>::type (&u)[1 << (2 * D)], PlaneBuf pb) {
  using U = typename std::make_unsigned<I>::type;
  constexpr int N = 1 << (2 * D);
  constexpr int P = 8 * sizeof(U);
  if constexpr (P == 64 && (N == 64 || N == 16)) {
    // 64-bit 2D and 3D blocks: the buffer holds 32 planes.  Planes 63-32
    // are decoded into it and their 32-bit halves transposed at once, then
    // the same slots take planes 31-0.
    const int kmin = (unsigned)P > maxprec ? P - (int)maxprec : 0;
    unsigned bits = budget, n = 0;
    int k = P - 1;
    decode_plane_range<N, Source, kWin>(in, bits, n, k, kmin > 32 ? kmin : 32, 32, pb);
    for (int kk = k; kk >= 32; kk--) pb.p[(kk - 32) * pb.stride] = 0;
    uint32_t hi[N];
    take_half_planes<N>(pb, hi);
    if (k >= kmin && bits) {
      decode_plane_range<N, Source, kWin>(in, bits, n, k, kmin, 0, pb);
      for (int kk = k; kk >= 0; kk--) pb.p[kk * pb.stride] = 0;
      uint32_t lo[N];
      take_half_planes<N>(pb, lo);
#pragma unroll
      for (int i = 0; i < N; i++) u[i] = ((U)hi[i] << 32) | lo[i];
    } else {
#pragma unroll
      for (int i = 0; i < N; i++) u[i] = (U)hi[i] << 32;
    }
    return budget - bits;
  } else if constexpr (N <= 64) {
    bool top_only;
    const unsigned bits = decode_planes<P, N, Source, kWin, kFloor>(in, budget, maxprec, pb, top_only);
    const int kmin = kFloor && (unsigned)P > maxprec ? P - (int)maxprec : 0;
    if constexpr (P == 64 && N > 4) {
      if (top_only) {
        uint64_t pl[32];
#pragma unroll
        for (int k = 0; k < 32; k++) pl[k] = 32 + k >= kmin ? pb.p[(32 + k) * pb.stride] : 0;
        uint32_t hi[N];
        take_planes<N>(pl, hi);
#pragma unroll
        for (int i = 0; i < N; i++) u[i] = (U)hi[i] << 32;
        return bits;
      }
    }
    uint64_t pl[P];
#pragma unroll
    for (int k = 0; k < P; k++) pl[k] = k >= kmin ? pb.p[k * pb.stride] : 0;
    take_planes<N>(pl, u);
    return bits;
  } else {
    uint64_t pl[4 * P];
    const unsigned bits = decode_planes_wide<P>(in, budget, maxprec, pl);
    take_planes_wide<U, P>(pl, u);
    return bits;
  }
}

template <int D, typename I, bool kFloor = false, class Source>
ZG_HD unsigned decode_ints(Source& in, unsigned minbits, unsigned maxbits, unsigned maxprec,
                           I (&v)[1 << (2 * D)], PlaneBuf pb) {
  using U = typename std::make_unsigned<I>::type;
  constexpr int N = 1 << (2 * D);
  U u[N];
  unsigned bits = uncode_coeffs<D, I, Source, true, kFloor>(in, maxbits, maxprec, u, pb);
  if (bits < minbits) { in.skip_long(minbits - bits); bits = minbits; }
#pragma unroll (N <= 64 ? N : 1)
  for (int i = 0; i < N; i++) v[perm<D>(i)] = from_nb<I>(u[i]);
  xform<kInv, D>(v);
  return bits;
}

template <int D, typename I, class Source>
ZG_HD unsigned rev_decode_ints(Source& in, unsigned minbits, unsigned maxbits, I (&v)[1 << (2 * D)], PlaneBuf pb) {
  using U = typename std::make_unsigned<I>::type;
  constexpr int N = 1 << (2 * D);
  constexpr unsigned kPBits = sizeof(I) == 4 ? 5 : 6;
  const unsigned prec = (unsigned)in.read(kPBits) + 1;
  U u[N];
  unsigned bits = kPBits + uncode_coeffs<D, I, Source, false>(in, maxbits - kPBits, prec, u, pb);
  if (bits < minbits) { in.skip_long(minbits - bits); bits = minbits; }
#pragma unroll (N <= 64 ? N : 1)
  for (int i = 0; i < N; i++) v[perm<D>(i)] = from_nb<I>(u[i]);
  xform<kRevInv, D>(v);
  return bits;
}

// ---------------------------------------------------------------------------
// whole-block front ends.  `raw` holds the gathered block as bit patterns.

ZG_HD unsigned umin(unsigned a, unsigned b) { return a < b ? a : b; }

template <typename S, int D, bool kFloor = false, class Source>
ZG_HD unsigned decode_float_lossy(Source& in, const BlockParams& p,
                                  typename Traits<S>::Bits (&raw)[1 << (2 * D)], PlaneBuf pb) {
  using T = Traits<S>;
  constexpr int N = 1 << (2 * D);
  unsigned bits = 1;
  if (in.read(1)) {
    bits += T::kEBits;
    const int emax = (int)in.read(T::kEBits) - T::kEBias;
    const unsigned maxprec = coded_precision(emax, p.maxprec, p.minexp, D);
    typename T::Int v[N];
    bits += decode_ints<D, typename T::Int, kFloor>(in, p.minbits - umin(bits, p.minbits), p.maxbits - bits,
                                                   maxprec, v, pb);
    inv_cast<S, N>(v, raw, emax);
  } else {
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) raw[i] = 0;
    if (p.minbits > bits) { in.skip_long(p.minbits - bits); bits = p.minbits; }
  }
  return bits;
}

template <typename S, int D, class Source>
ZG_HD unsigned decode_float_rev(Source& in, const BlockParams& p,
                                typename Traits<S>::Bits (&raw)[1 << (2 * D)], PlaneBuf pb) {
  using T = Traits<S>;
  using B = typename T::Bits;
  using I = typename T::Int;
  constexpr int N = 1 << (2 * D);
  constexpr B kTc = ~(B(1) << (8 * sizeof(B) - 1));
  unsigned bits = 1;
  if (in.read(1)) {
    I v[N];
    bits++;
    const bool reinterpreted = in.read(1);   // one copy of the plane decoder for both kinds
    int emax = 0;
    if (!reinterpreted) {
      bits += T::kEBits;
      emax = (int)in.read(T::kEBits) - T::kEBias;
    }
    bits += rev_decode_ints<D>(in, p.minbits - umin(bits, p.minbits), p.maxbits - bits, v, pb);
    if (reinterpreted) {
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) raw[i] = v[i] < 0 ? ((B)v[i] ^ kTc) : (B)v[i];
    } else if (emax != -T::kEBias) {
      inv_cast<S, N>(v, raw, emax);
    } else {
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) raw[i] = 0;
    }
  } else {
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) raw[i] = 0;
    if (p.minbits > bits) { in.skip_long(p.minbits - bits); bits = p.minbits; }
  }
  return bits;
}

// ---------------------------------------------------------------------------
// encoder: a block is first prepared (header, coding budget and bit planes
// held in registers) and then emitted.  Kernels that need the block's length
// before writing it (variable-rate streams) run length() between the two.

struct CountSink {
  unsigned n = 0;
  ZG_HD void put(uint64_t, unsigned k) { n += k; }
  ZG_HD void pad(unsigned k) { n += k; }
};

// Everything about a block except its bit planes: header bits, the budget
// left for the plane coder, the planes to code and the minimum size.
struct BlockHead {
  uint64_t hdr;        // header bits, first bit in the LSB
  unsigned hdr_bits;
  unsigned budget;     // bits granted to the plane coder (unsigned wrap as in the reference)
  unsigned maxprec;    // bit planes to code
  unsigned pad_to;     // the block is padded with zeros to at least this many bits
  bool coded;          // false: header only
};

// reorder by sequency and map to negabinary (src/template/encode.c:83-88)
template <int D, typename I>
ZG_HD void reorder(const I (&v)[1 << (2 * D)], typename std::make_unsigned<I>::type (&u)[1 << (2 * D)]) {
  constexpr int N = 1 << (2 * D);
#pragma unroll (N <= 64 ? N : 1)
  for (int i = 0; i < N; i++) u[i] = to_nb<I>(v[perm<D>(i)]);
}

// precision of a reversible block: top plane down to the lowest set bit of
// any coefficient (src/template/revencode.c:37-53), clamped to [1, maxprec]
template <typename U, int N>
ZG_HD unsigned rev_precision(const U (&u)[N], unsigned maxprec) {
  U all = 0;
#pragma unroll (N <= 64 ? N : 1)
  for (int i = 0; i < N; i++) all |= u[i];
  unsigned prec = all ? 8 * sizeof(U) - ctz64((uint64_t)all) : 0;
  if (prec > maxprec) prec = maxprec;
  if (prec < 1) prec = 1;
  return prec;
}

// Front end of one gathered block of scalar type S (bit patterns in `raw`):
// fills the head and, for coded blocks, the reordered negabinary
// coefficients.  Lossy floating point: src/template/encodef.c:63-90;
// reversible floating point: revencodef.c:45-80; integers: encode.c:260-280,
// revencode.c:57-79.
template <typename S, int D, int kSel = kAnyMode>
ZG_HD void prepare_coeffs(BlockHead& h, const BlockParams& p, const typename Traits<S>::Bits (&raw)[1 << (2 * D)],
                          typename Traits<S>::UInt (&u)[1 << (2 * D)]) {
  using T = Traits<S>;
  using B = typename T::Bits;
  using I = typename T::Int;
  using U = typename T::UInt;
  constexpr int N = 1 << (2 * D);
  const bool rev = is_rev<kSel>(p);
  I v[N];
  h.pad_to = p.minbits;
  h.coded = true;
  if constexpr (T::kFloat) {
    bool special;
    const int emax = block_emax<S, N>(raw, special);
    if (!rev) {
      const unsigned maxprec = coded_precision(emax, p.maxprec, p.minexp, D);
      const unsigned e = maxprec ? (unsigned)(emax + T::kEBias) : 0u;
      if (!e) {                                    // single zero bit, padded to minbits
        h.hdr = 0; h.hdr_bits = 1; h.coded = false;
        return;
      }
      h.hdr = 2 * (uint64_t)e + 1;
      h.hdr_bits = 1 + T::kEBits;
      h.budget = p.maxbits - h.hdr_bits;
      h.maxprec = maxprec;
      fwd_cast<S, N>(raw, v, emax, special);
      xform<kFwd, D>(v);
      reorder<D>(v, u);
      return;
    }
    constexpr B kTc = ~(B(1) << (8 * sizeof(B) - 1));
    bool exact;
    if (emax != -T::kEBias) {
      exact = bfp_exact<S, N>(raw, emax, special);
    } else {
      exact = true;
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) exact &= raw[i] == 0;
    }
    unsigned outer;
    if (exact) {
      const unsigned e = (unsigned)(emax + T::kEBias);
      if (!e) {                                    // all-zero block: one bit, never padded
        h.hdr = 0; h.hdr_bits = 1; h.coded = false; h.pad_to = 0;
        return;
      }
      fwd_cast<S, N>(raw, v, emax, special);
      h.hdr = 1 | ((uint64_t)e << 2);
      outer = 2 + T::kEBits;
    } else {                                       // reinterpret sign-magnitude as two's complement
#pragma unroll (N <= 64 ? N : 1)
      for (int i = 0; i < N; i++) v[i] = (I)raw[i] < 0 ? (I)(raw[i] ^ kTc) : (I)raw[i];
      h.hdr = 3;
      outer = 2;
    }
    xform<kRevFwd, D>(v);
    reorder<D>(v, u);
    const unsigned prec = rev_precision<U, N>(u, p.maxprec);
    h.hdr |= (uint64_t)(prec - 1) << outer;
    h.hdr_bits = outer + T::kPBits;
    h.budget = p.maxbits - outer - T::kPBits;
    h.maxprec = prec;
  } else {
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) v[i] = (I)raw[i];
    if (!rev) {
      h.hdr = 0; h.hdr_bits = 0;
      h.budget = p.maxbits;
      h.maxprec = p.maxprec;
      xform<kFwd, D>(v);
      reorder<D>(v, u);
    } else {
      xform<kRevFwd, D>(v);
      reorder<D>(v, u);
      const unsigned prec = rev_precision<U, N>(u, p.maxprec);
      h.hdr = prec - 1;
      h.hdr_bits = T::kPBits;
      h.budget = p.maxbits - T::kPBits;
      h.maxprec = prec;
    }
  }
}

// ---------------------------------------------------------------------------
// plane-array coder (N <= 64): planes live in an array plane[k * stride]
// (shared memory in the kernels, a local array on the host), the coder is a
// rolled loop over planes.  Because the stream of a plane depends only on
// the plane word and the count n of coefficients already significant, its
// length is known in O(1) (popc/clz) and every plane that fits the budget is
// written with no per-bit budget test; only the plane where the budget ends
// takes the bit-exact truncating path.

// bits of plane x given n significant coefficients; updates n
template <int N>
ZG_HD unsigned plane_bits(uint64_t x, unsigned& n) {
  unsigned len = n;
  if (n < (unsigned)N) {
    const uint64_t r = x >> n;
    if (!r) {
      len += 1;
    } else {
      // the top one of x is the top one of r: n verbatim bits, then a test
      // and a bit per coefficient up to it, a test after each one, and a
      // closing negative test (none when the last coefficient is reached,
      // whose one is then implied)
      const unsigned top = 64 - (unsigned)clz64(x);
      len = top + (unsigned)popc64(r) + (top < (unsigned)N ? 1u : 0u) - (top < (unsigned)N ? 0u : 1u);
      n = top;
    }
  }
  return len;
}

// write plane x completely (it fits the budget)
template <int N, class Sink>
ZG_HD void put_plane(Sink& out, uint64_t x, unsigned& n) {
  out.put(n ? x & (~0ull >> (64 - n)) : 0ull, n);
  if (n >= (unsigned)N) return;
  uint64_t r = x >> n;
  while (r) {
    const unsigned z = ctz64(r);
    if (n + z == (unsigned)N - 1) {   // positive test, z zeros, implied one
      out.put(1, z + 1);
      n = N;
      return;
    }
    out.put(1 | (2ull << z), z + 2);  // positive test, z zeros, the one
    n += z + 1;
    r >>= z + 1;
  }
  out.put(0, 1);                      // negative test: rest of the plane is zero
}

// write the first `bits` bits of plane x's code (the budget ends inside it)
template <int N, class Sink>
ZG_HD void put_plane_cut(Sink& out, uint64_t x, unsigned n, unsigned bits) {
  const unsigned m = n < bits ? n : bits;
  out.put(m ? x & (~0ull >> (64 - m)) : 0ull, m);
  bits -= m;
  if (n >= (unsigned)N) return;
  uint64_t r = x >> n;
  while (bits) {
    bits--;
    if (!r) { out.put(0, 1); return; }
    out.put(1, 1);
    const unsigned z = ctz64(r);
    if (n + z == (unsigned)N - 1) {
      out.put(0, z < bits ? z : bits);
      return;
    }
    const unsigned len = z + 1, e = len < bits ? len : bits;
    out.put(e > z ? (1ull << z) : 0ull, e);
    bits -= e;
    if (e < len) return;
    n += len;
    r >>= len;
  }
}

// total bits of a prepared block
template <int P, int N>
ZG_HD unsigned block_bits(const BlockHead& h, const uint64_t* plane, int stride) {
  unsigned bits = h.hdr_bits;
  if (h.coded) {
    const int kmin = (unsigned)P > h.maxprec ? P - (int)h.maxprec : 0;
    unsigned n = 0, code = 0;
    for (int k = P - 1; k >= kmin && code < h.budget; k--) {
      if (n >= (unsigned)N) {                 // all coefficients significant: N verbatim bits per plane
        code += (unsigned)(k - kmin + 1) * N;
        break;
      }
      code += plane_bits<N>(plane[k * stride], n);
    }
    bits += code < h.budget ? code : h.budget;
  }
  return bits > h.pad_to ? bits : h.pad_to;
}

// write a prepared block; returns its bits
template <int P, int N, class Sink>
ZG_HD unsigned emit_block(Sink& out, const BlockHead& h, const uint64_t* plane, int stride) {
  out.put(h.hdr, h.hdr_bits);
  unsigned bits = h.hdr_bits;
  if (h.coded) {
    const int kmin = (unsigned)P > h.maxprec ? P - (int)h.maxprec : 0;
    unsigned left = h.budget, n = 0;
    for (int k = P - 1; k >= kmin && left; k--) {
      const uint64_t x = plane[k * stride];
      unsigned n2 = n;
      const unsigned len = plane_bits<N>(x, n2);
      if (len <= left) {
        put_plane<N>(out, x, n);
        left -= len;
      } else {
        put_plane_cut<N>(out, x, n, left);
        left = 0;
      }
    }
    bits += h.budget - left;
  }
  if (bits < h.pad_to) {
    out.pad(h.pad_to - bits);
    bits = h.pad_to;
  }
  return bits;
}

// ---------------------------------------------------------------------------
// Table-driven sequential coder (N <= 64).
//
// Past its n verbatim bits, plane x's code is a pure function of r = x >> n
// (src/template/encode.c:92-132): a positive test '1' if r != 0 (else a
// single '0'), then r's bits from the bottom up to its top one, each one
// followed by a test bit -- '1' (more ones follow) or, after the last one,
// '0'.  A last one at coefficient N-1 is implied: neither it nor a test
// after it is written.  So the code of r is the expansion E(r) of r in
// which every one becomes '11', with the bit after the last one cleared or
// the last one's two bits dropped.  E is computed a byte at a time from a
// 256-entry table (group_code_entry): E(b) with popc(b) above it; a 16-bit
// chunk of r is two lookups, whatever its number of ones.  The coder walks
// the planes in one flat loop whose iterations each start a plane (its
// verbatim bits and opening test: one put) and code one 16-bit chunk of its
// r (one put); most planes need one iteration.  Every put is cut at the bit
// budget, which truncates the code exactly where the reference's per-bit
// budget stops its coder (src/template/encode.c:92-256).

template <int P, int N, class Sink>
ZG_HD unsigned emit_block_seq(Sink& out, const BlockHead& h, const uint64_t* plane, int stride, const uint32_t* gtab) {
  out.put(h.hdr, h.hdr_bits);
  unsigned bits = h.hdr_bits;
  if (h.coded) {
    const int kmin = (unsigned)P > h.maxprec ? P - (int)h.maxprec : 0;
    unsigned left = h.budget;        // bits the plane coder may still write
    unsigned n = 0;                  // coefficients already significant
    int k = P - 1;
    uint64_t r = 0;                  // group-test bits of the current plane not yet coded (next chunk at bit 0)
    int rem = -1;                    // position in r of the plane's last one; -1: none pending
    bool implied = false;            // that one is coefficient N-1
    while (left) {
      if (rem < 0) {                 // next plane: verbatim bits and the opening test
        if (k < kmin) break;
        const uint64_t x = plane[k * stride];
        k--;
        uint64_t v = x;
        unsigned len = N;
        if (n < (unsigned)N) {
          const uint64_t g = x >> n;
          v = low_bits(x, n) | ((uint64_t)(g != 0) << n);
          len = n + 1;
          if (g) {
            const unsigned top = 63u - (unsigned)clz64(g);
            implied = n + top == (unsigned)N - 1;
            rem = (int)top;
            r = g;
            n += top + 1;
          }
        }
        if (len >= left) {
          out.put(low_bits(v, left), left);
          left = 0;
          break;
        }
        out.put(v, len);
        left -= len;
        if (rem < 0) continue;
      }
      // the next 16 bits of r
      const uint32_t c = (uint32_t)r & 0xffffu;
      const uint32_t e0 = gtab[c & 0xffu], e1 = gtab[c >> 8];
      const unsigned p0 = e0 >> 16, pc = p0 + (e1 >> 16);
      uint32_t code = (e0 & 0xffffu) | ((e1 & 0xffffu) << (8 + p0));
      unsigned len = 16 + pc;
      if (rem < 16) {                // the plane's last chunk: up to its last one
        if (implied) {
          len = (unsigned)rem + pc - 1;                 // the one and its test are not written
          code &= len < 32 ? (1u << len) - 1 : ~0u;
        } else {
          len = (unsigned)rem + pc + 1;                 // the test after the last one is negative
          code &= ~(1u << (len - 1));
        }
        rem = -1;
      } else {
        r >>= 16;
        rem -= 16;
      }
      if (len >= left) {
        out.put(low_bits(code, left), left);
        left = 0;
        break;
      }
      out.put(code, len);
      left -= len;
    }
    bits += h.budget - left;
  }
  if (bits < h.pad_to) {
    out.pad(h.pad_to - bits);
    bits = h.pad_to;
  }
  return bits;
}

// 4D blocks: the header, and the coefficients as 256-bit bit planes
template <typename S>
struct WideCode {
  using U = typename Traits<S>::UInt;
  static constexpr int P = 8 * sizeof(U);
  BlockHead h;
  uint64_t pl[4 * P];
  ZG_HD void set(const U (&u)[256]) {
    if (h.coded) make_planes_wide<U, P>(u, pl);
  }
  template <class Sink>
  ZG_HD unsigned emit(Sink& out, const uint32_t* gtab) const {
    out.put(h.hdr, h.hdr_bits);
    unsigned bits = h.hdr_bits;
    if (h.coded) bits += code_planes_wide<P, false>(out, h.budget, h.maxprec, pl, gtab);
    if (bits < h.pad_to) { out.pad(h.pad_to - bits); bits = h.pad_to; }
    return bits;
  }
  ZG_HD unsigned length() const {
    CountSink c;
    unsigned bits = h.hdr_bits;
    if (h.coded) bits += code_planes_wide<P, true>(c, h.budget, h.maxprec, pl, nullptr);
    return bits > h.pad_to ? bits : h.pad_to;
  }
};

// whole-block encoder (one significance event per put for 1-3D blocks; gtab:
// the group-code table, used by 4D blocks)
template <typename S, int D, class Sink>
ZG_HD unsigned encode_block(Sink& out, const BlockParams& p, const typename Traits<S>::Bits (&raw)[1 << (2 * D)],
                            const uint32_t* gtab) {
  using U = typename Traits<S>::UInt;
  constexpr int N = 1 << (2 * D);
  if constexpr (N <= 64) {
    BlockHead h;
    U u[N];
    uint64_t plane[8 * sizeof(U)];
    prepare_coeffs<S, D>(h, p, raw, u);
    if (h.coded) store_planes<N>(u, plane, 1, h.maxprec);
    return emit_block<8 * sizeof(U), N>(out, h, plane, 1);
  } else {
    WideCode<S> wc;
    U u[256];
    prepare_coeffs<S, D>(wc.h, p, raw, u);
    wc.set(u);
    return wc.emit(out, gtab);
  }
}

// ---------------------------------------------------------------------------
// Length-only decoding, for recovering block offsets of a variable-rate
// stream that carries no index: the same bits are consumed as by
// decode_block, but planes are not formed and nothing is transformed.

// bits of the plane code (the group-test rules of decode_planes and
// decode_planes_wide, any N), scanning with 64-bit peeks
template <int N, int P, class Source>
ZG_HD unsigned skip_planes(Source& in, unsigned budget, unsigned maxprec) {
  const int kmin = (unsigned)P > maxprec ? P - (int)maxprec : 0;
  unsigned bits = budget, n = 0;
  for (int k = P - 1; k >= kmin && bits; k--) {
    unsigned m = n < bits ? n : bits;        // verbatim bits
    bits -= m;
    while (m) {
      const unsigned c = m < 64 ? m : 64;
      in.skip(c);
      m -= c;
    }
    while (bits && n < (unsigned)N) {
      if (bits >= 32 && n + 1 < (unsigned)N) {
        const uint32_t w = in.peek32();
        if ((w & 1) && w != 1) {
          const EventWindow ev = event_window(w);
          if (ev.e && n + ev.scan < (unsigned)N) {
            n += ev.scan;
            in.skip(ev.used);
            bits -= ev.used;
            if (ev.stop) break;
            continue;
          }
        }
      }
      const bool positive = in.peek64() & 1;
      in.skip(1);
      bits--;
      if (!positive) break;                   // rest of the plane is zero
      // scan at most cap bits for the next one; none: it is implied at the limit
      const unsigned cap = N - 1 - n < bits ? N - 1 - n : bits;
      unsigned z = 0;
      bool found = false;
      while (z < cap) {
        const unsigned c = cap - z < 64 ? cap - z : 64;
        const uint64_t w = in.peek64();
        const uint64_t sw = c < 64 ? (w | (uint64_t(1) << c)) : w;
        const unsigned t = sw ? ctz64(sw) : 64u;
        if (t < c) {
          in.skip(t + 1);
          z += t;
          found = true;
          break;
        }
        in.skip(c);
        z += c;
      }
      bits -= z + (found ? 1u : 0u);
      n += z + 1;
    }
  }
  return budget - bits;
}

// bits of a whole block (decode_block's header and padding rules)
template <typename S, int D, class Source>
ZG_HD unsigned skip_block(Source& in, const BlockParams& p) {
  using T = Traits<S>;
  using U = typename T::UInt;
  constexpr int N = 1 << (2 * D), P = 8 * sizeof(U);
  constexpr unsigned kPBits = sizeof(U) == 4 ? 5 : 6;
  const bool rev = p.minexp < kMinExp;
  unsigned bits = 0, minbits = p.minbits, maxbits = p.maxbits, maxprec = p.maxprec;
  if constexpr (T::kFloat) {
    bits = 1;
    if (!in.read(1)) {                        // all-zero block
      if (minbits > bits) { in.skip_long(minbits - bits); bits = minbits; }
      return bits;
    }
    if (rev) {
      bits++;
      if (!in.read(1)) {                      // block-floating-point: exponent follows
        bits += T::kEBits;
        in.skip(T::kEBits);
      }
    } else {
      bits += T::kEBits;
      const int emax = (int)in.read(T::kEBits) - T::kEBias;
      maxprec = coded_precision(emax, p.maxprec, p.minexp, D);
    }
    minbits = p.minbits - umin(bits, p.minbits);
    maxbits = p.maxbits - bits;
  }
  unsigned code;
  if (rev) {
    const unsigned prec = (unsigned)in.read(kPBits) + 1;
    code = kPBits + skip_planes<N, P>(in, maxbits - kPBits, prec);
  } else {
    code = skip_planes<N, P>(in, maxbits, maxprec);
  }
  if (code < minbits) { in.skip_long(minbits - code); code = minbits; }
  return bits + code;
}

template <typename S, int D, int kSel = kAnyMode, class Source>
ZG_HD unsigned decode_block(Source& in, const BlockParams& p, typename Traits<S>::Bits (&raw)[1 << (2 * D)],
                            PlaneBuf pb) {
  using T = Traits<S>;
  constexpr int N = 1 << (2 * D);
  const bool rev = is_rev<kSel>(p);
  constexpr bool kFloor = kSel == kLossyFloor;
  if constexpr (T::kFloat) {
    return rev ? decode_float_rev<S, D>(in, p, raw, pb) : decode_float_lossy<S, D, kFloor>(in, p, raw, pb);
  } else {
    typename T::Int v[N];
    const unsigned bits = rev ? rev_decode_ints<D>(in, p.minbits, p.maxbits, v, pb)
                              : decode_ints<D, typename T::Int, kFloor>(in, p.minbits, p.maxbits, p.maxprec, v, pb);
#pragma unroll (N <= 64 ? N : 1)
    for (int i = 0; i < N; i++) raw[i] = (typename T::Bits)v[i];
    return bits;
  }
}

// same, with the planes in a local array
template <typename S, int D, class Source>
ZG_HD unsigned decode_block(Source& in, const BlockParams& p, typename Traits<S>::Bits (&raw)[1 << (2 * D)]) {
  uint64_t plane[8 * sizeof(typename Traits<S>::UInt)];
  return decode_block<S, D>(in, p, raw, PlaneBuf{plane, 1});
}

// ---------------------------------------------------------------------------
// bit source over a word array: a 128-bit window, loads past `cap` words
// read as zero so a corrupt or truncated stream cannot fault.  kGlobal
// selects read-only global loads; otherwise plain (e.g. shared-memory) loads.

template <bool kGlobal>
struct WordSourceT {
  const uint64_t* base;
  uint64_t cap;     // readable words
  uint64_t next;    // index of the next word to load; the current position is (next - 2) * 64 + pos
  uint64_t lo, hi;
  unsigned pos;     // bit offset of the current position inside lo

  ZG_HD uint64_t load(uint64_t i) const {
#if defined(__CUDA_ARCH__)
    // shared staging keeps a spare word after every 16 (bank spreading)
    if constexpr (kGlobal) return i < cap ? __ldg((const unsigned long long*)base + i) : 0ull;
    else return i < cap ? base[i + (i >> 4)] : 0ull;
#else
    return i < cap ? base[i] : 0ull;
#endif
  }
  ZG_HD uint64_t tell() const { return (next - 2) * 64 + pos; }
  ZG_HD void seek(uint64_t bit) {
    const uint64_t w = bit >> 6;
    lo = load(w);
    hi = load(w + 1);
    next = w + 2;
    pos = (unsigned)(bit & 63);
  }
  ZG_HD uint64_t peek64() const { return pos ? (lo >> pos) | (hi << (64 - pos)) : lo; }
  ZG_HD uint32_t peek32() const {
#if defined(__CUDA_ARCH__)
    const bool up = pos >= 32;
    const uint32_t a = up ? (uint32_t)(lo >> 32) : (uint32_t)lo;
    const uint32_t b = up ? (uint32_t)hi : (uint32_t)(lo >> 32);
    return __funnelshift_r(a, b, pos);
#else
    return (uint32_t)peek64();
#endif
  }
  ZG_HD uint64_t peek(unsigned n) const { return low_bits(peek64(), n); }   // n <= 64
  ZG_HD void skip(unsigned n) {               // n <= 64
    pos += n;
    if (pos >= 64) {
      lo = hi;
      hi = load(next++);
      pos -= 64;
    }
  }
  ZG_HD uint64_t read(unsigned n) {
    const uint64_t v = peek(n);
    skip(n);
    return v;
  }
  ZG_HD void skip_long(uint64_t n) { seek(tell() + n); }
};

using WordSource = WordSourceT<true>;
using SharedSource = WordSourceT<false>;

}  // namespace zg
