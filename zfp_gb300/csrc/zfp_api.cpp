// zfp_api.cpp -- host side of the drop-in C API: bit streams, stream and
// field bookkeeping, mode setters, headers.  Semantics follow the reference
// (src/zfp.c, include/zfp/bitstream.inl) function by function, with each
// function citing what it mirrors; zfp_compress / zfp_decompress hand over
// to the GPU codec in gpu_codec.cu.
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "../../include/zfp.h"
#include "../../include/zfp_gb300.h"
#include "runtime.h"

// ---------------------------------------------------------------------------
// bit stream: 64-bit words, LSB first (include/zfp/bitstream.inl:133-143)

struct bitstream {
  size_t bits;        // buffered bits, 0 <= bits < 64
  uint64_t buffer;    // buffered bits (buffer < 2^bits)
  uint64_t* ptr;      // next word to read or write
  uint64_t* begin;
  uint64_t* end;
};

static const size_t kWord = 64;

extern "C" {

const size_t stream_word_bits = kWord;

bitstream* stream_open(void* buffer, size_t bytes) {
  bitstream* s = (bitstream*)std::malloc(sizeof(bitstream));
  if (s) {
    s->begin = (uint64_t*)buffer;
    s->end = s->begin + bytes / sizeof(uint64_t);
    s->ptr = s->begin;
    s->buffer = 0;
    s->bits = 0;
  }
  return s;
}

void stream_close(bitstream* s) { std::free(s); }

bitstream* stream_clone(const bitstream* s) {
  bitstream* c = (bitstream*)std::malloc(sizeof(bitstream));
  if (c) *c = *s;
  return c;
}

bitstream_count stream_alignment(void) { return kWord; }
void* stream_data(const bitstream* s) { return s->begin; }
size_t stream_size(const bitstream* s) { return (size_t)(s->ptr - s->begin) * sizeof(uint64_t); }
size_t stream_capacity(const bitstream* s) { return (size_t)(s->end - s->begin) * sizeof(uint64_t); }
size_t stream_stride_block(const bitstream*) { return 1; }
ptrdiff_t stream_stride_delta(const bitstream*) { return 0; }

unsigned int stream_read_bit(bitstream* s) {
  if (!s->bits) {
    s->buffer = *s->ptr++;
    s->bits = kWord;
  }
  s->bits--;
  const unsigned int bit = (unsigned int)(s->buffer & 1u);
  s->buffer >>= 1;
  return bit;
}

unsigned int stream_write_bit(bitstream* s, unsigned int bit) {
  s->buffer += (uint64_t)bit << s->bits;
  if (++s->bits == kWord) {
    *s->ptr++ = s->buffer;
    s->buffer = 0;
    s->bits = 0;
  }
  return bit;
}

uint64_t stream_read_bits(bitstream* s, bitstream_count n) {
  uint64_t value = s->buffer;
  if (s->bits < n) {
    const uint64_t w = *s->ptr++;
    value += w << s->bits;          // s->bits < n <= 64
    s->bits += kWord - n;
    if (!s->bits) {
      s->buffer = 0;
    } else {
      s->buffer = w >> (kWord - s->bits);
      value &= (((uint64_t)2) << (n - 1)) - 1;
    }
  } else {
    s->bits -= n;
    s->buffer >>= n;
    value &= n >= kWord ? ~0ull : (((uint64_t)1) << n) - 1;
  }
  return value;
}

uint64_t stream_write_bits(bitstream* s, uint64_t value, bitstream_count n) {
  s->buffer += value << s->bits;
  s->bits += n;
  if (s->bits >= kWord) {
    value >>= 1;
    n--;
    s->bits -= kWord;
    *s->ptr++ = s->buffer;
    s->buffer = value >> (n - s->bits);
  }
  s->buffer &= (((uint64_t)1) << s->bits) - 1;
  return value >> n;
}

bitstream_offset stream_rtell(const bitstream* s) { return (bitstream_offset)(s->ptr - s->begin) * kWord - s->bits; }
bitstream_offset stream_wtell(const bitstream* s) { return (bitstream_offset)(s->ptr - s->begin) * kWord + s->bits; }

void stream_rewind(bitstream* s) {
  s->ptr = s->begin;
  s->buffer = 0;
  s->bits = 0;
}

void stream_rseek(bitstream* s, bitstream_offset offset) {
  const size_t n = (size_t)(offset % kWord);
  s->ptr = s->begin + (size_t)(offset / kWord);
  if (n) {
    s->buffer = *s->ptr++ >> n;
    s->bits = kWord - n;
  } else {
    s->buffer = 0;
    s->bits = 0;
  }
}

void stream_wseek(bitstream* s, bitstream_offset offset) {
  const size_t n = (size_t)(offset % kWord);
  s->ptr = s->begin + (size_t)(offset / kWord);
  if (n) {
    s->buffer = *s->ptr & ((((uint64_t)1) << n) - 1);
    s->bits = n;
  } else {
    s->buffer = 0;
    s->bits = 0;
  }
}

void stream_skip(bitstream* s, bitstream_size n) { stream_rseek(s, stream_rtell(s) + n); }

void stream_pad(bitstream* s, bitstream_size n) {
  bitstream_offset bits = s->bits;
  for (bits += n; bits >= kWord; bits -= kWord) {
    *s->ptr++ = s->buffer;
    s->buffer = 0;
  }
  s->bits = (size_t)bits;
}

bitstream_count stream_align(bitstream* s) {
  const size_t bits = s->bits;
  if (bits) stream_skip(s, bits);
  return bits;
}

bitstream_count stream_flush(bitstream* s) {
  const size_t bits = (kWord - s->bits) % kWord;
  if (bits) stream_pad(s, bits);
  return bits;
}

void stream_copy(bitstream* dst, bitstream* src, bitstream_size n) {
  while (n > kWord) {
    stream_write_bits(dst, stream_read_bits(src, kWord), kWord);
    n -= kWord;
  }
  if (n) stream_write_bits(dst, stream_read_bits(src, (size_t)n), (size_t)n);
}

// ---------------------------------------------------------------------------
// library identity (src/zfp.c:12-14)

const unsigned int zfp_codec_version = ZFP_CODEC;
const unsigned int zfp_library_version = 0x1010u;
const char* const zfp_version_string = "zfp version 1.0.1 (libzfp_gb300: GB300 CUDA codec)";

size_t zfp_type_size(zfp_type type) {  // src/zfp.c:90-105
  switch (type) {
    case zfp_type_int32: return 4;
    case zfp_type_int64: return 8;
    case zfp_type_float: return 4;
    case zfp_type_double: return 8;
    default: return 0;
  }
}

// ---------------------------------------------------------------------------
// fields (src/zfp.c:16-39, 107-463)

static void field_strides(const zfp_field* f, ptrdiff_t s[4]) {
  s[0] = f->sx ? f->sx : 1;
  s[1] = f->sy ? f->sy : (ptrdiff_t)f->nx;
  s[2] = f->sz ? f->sz : (ptrdiff_t)(f->nx * f->ny);
  s[3] = f->sw ? f->sw : (ptrdiff_t)(f->nx * f->ny * f->nz);
}

// lowest/highest element offset from the base pointer (src/zfp.c:17-39)
static size_t field_span(const zfp_field* f, ptrdiff_t* lo, ptrdiff_t* hi) {
  ptrdiff_t s[4];
  field_strides(f, s);
  const size_t n[4] = {f->nx, f->ny, f->nz, f->nw};
  ptrdiff_t mn = 0, mx = 0;
  for (int a = 0; a < 4; a++) {
    const ptrdiff_t d = n[a] ? s[a] * (ptrdiff_t)(n[a] - 1) : 0;
    mn += d < 0 ? d : 0;
    mx += d > 0 ? d : 0;
  }
  if (lo) *lo = mn;
  if (hi) *hi = mx;
  return (size_t)(mx - mn + 1);
}

zfp_field* zfp_field_alloc(void) {
  zfp_field* f = (zfp_field*)std::malloc(sizeof(zfp_field));
  if (f) {
    f->type = zfp_type_none;
    f->nx = f->ny = f->nz = f->nw = 0;
    f->sx = f->sy = f->sz = f->sw = 0;
    f->data = nullptr;
  }
  return f;
}

static zfp_field* field_make(void* p, zfp_type t, size_t nx, size_t ny, size_t nz, size_t nw) {
  zfp_field* f = zfp_field_alloc();
  if (f) {
    f->type = t;
    f->nx = nx; f->ny = ny; f->nz = nz; f->nw = nw;
    f->data = p;
  }
  return f;
}

zfp_field* zfp_field_1d(void* p, zfp_type t, size_t nx) { return field_make(p, t, nx, 0, 0, 0); }
zfp_field* zfp_field_2d(void* p, zfp_type t, size_t nx, size_t ny) { return field_make(p, t, nx, ny, 0, 0); }
zfp_field* zfp_field_3d(void* p, zfp_type t, size_t nx, size_t ny, size_t nz) { return field_make(p, t, nx, ny, nz, 0); }
zfp_field* zfp_field_4d(void* p, zfp_type t, size_t nx, size_t ny, size_t nz, size_t nw) {
  return field_make(p, t, nx, ny, nz, nw);
}
void zfp_field_free(zfp_field* f) { std::free(f); }
void* zfp_field_pointer(const zfp_field* f) { return f->data; }

void* zfp_field_begin(const zfp_field* f) {
  if (!f->data) return nullptr;
  ptrdiff_t lo;
  field_span(f, &lo, nullptr);
  return (char*)f->data + lo * (ptrdiff_t)zfp_type_size(f->type);
}

zfp_type zfp_field_type(const zfp_field* f) { return f->type; }
unsigned int zfp_field_precision(const zfp_field* f) { return (unsigned int)(8 * zfp_type_size(f->type)); }
unsigned int zfp_field_dimensionality(const zfp_field* f) {
  return f->nx ? f->ny ? f->nz ? f->nw ? 4 : 3 : 2 : 1 : 0;
}

size_t zfp_field_size(const zfp_field* f, size_t* size) {
  const unsigned int d = zfp_field_dimensionality(f);
  if (size) {
    if (d >= 4) size[3] = f->nw;
    if (d >= 3) size[2] = f->nz;
    if (d >= 2) size[1] = f->ny;
    if (d >= 1) size[0] = f->nx;
  }
  auto m1 = [](size_t v) { return v ? v : (size_t)1; };
  return m1(f->nx) * m1(f->ny) * m1(f->nz) * m1(f->nw);
}

size_t zfp_field_size_bytes(const zfp_field* f) { return field_span(f, nullptr, nullptr) * zfp_type_size(f->type); }

size_t zfp_field_blocks(const zfp_field* f) {
  const size_t bx = (f->nx + 3) / 4, by = (f->ny + 3) / 4, bz = (f->nz + 3) / 4, bw = (f->nw + 3) / 4;
  switch (zfp_field_dimensionality(f)) {
    case 1: return bx;
    case 2: return bx * by;
    case 3: return bx * by * bz;
    case 4: return bx * by * bz * bw;
    default: return 0;
  }
}

zfp_bool zfp_field_stride(const zfp_field* f, ptrdiff_t* stride) {
  if (stride) {
    ptrdiff_t s[4];
    field_strides(f, s);
    const unsigned int d = zfp_field_dimensionality(f);
    for (unsigned int a = 0; a < d; a++) stride[a] = s[a];
  }
  return f->sx || f->sy || f->sz || f->sw;
}

zfp_bool zfp_field_is_contiguous(const zfp_field* f) {
  return field_span(f, nullptr, nullptr) == zfp_field_size(f, nullptr);
}

// 52-bit metadata: extents, dimensionality, type (src/zfp.c:287-330)
uint64_t zfp_field_metadata(const zfp_field* f) {
  uint64_t meta = 0;
  const unsigned int d = zfp_field_dimensionality(f);
  const size_t n[4] = {f->nx, f->ny, f->nz, f->nw};
  const unsigned int width = d == 1 ? 48 : d == 2 ? 24 : d == 3 ? 16 : 12;
  if (d < 1 || d > 4) return ZFP_META_NULL;
  for (int a = (int)d - 1; a >= 0; a--) {
    const uint64_t v = (uint64_t)(n[a] - 1);
    if (v >> width) return ZFP_META_NULL;
    meta = (meta << width) + v;
  }
  meta = (meta << 2) + (d - 1);
  meta = (meta << 2) + (uint64_t)(f->type - 1);
  return meta;
}

void zfp_field_set_pointer(zfp_field* f, void* p) { f->data = p; }

zfp_type zfp_field_set_type(zfp_field* f, zfp_type t) {
  switch (t) {
    case zfp_type_int32: case zfp_type_int64: case zfp_type_float: case zfp_type_double:
      f->type = t;
      return t;
    default:
      return zfp_type_none;
  }
}

void zfp_field_set_size_1d(zfp_field* f, size_t nx) { f->nx = nx; f->ny = f->nz = f->nw = 0; }
void zfp_field_set_size_2d(zfp_field* f, size_t nx, size_t ny) { f->nx = nx; f->ny = ny; f->nz = f->nw = 0; }
void zfp_field_set_size_3d(zfp_field* f, size_t nx, size_t ny, size_t nz) {
  f->nx = nx; f->ny = ny; f->nz = nz; f->nw = 0;
}
void zfp_field_set_size_4d(zfp_field* f, size_t nx, size_t ny, size_t nz, size_t nw) {
  f->nx = nx; f->ny = ny; f->nz = nz; f->nw = nw;
}
void zfp_field_set_stride_1d(zfp_field* f, ptrdiff_t sx) { f->sx = sx; f->sy = f->sz = f->sw = 0; }
void zfp_field_set_stride_2d(zfp_field* f, ptrdiff_t sx, ptrdiff_t sy) { f->sx = sx; f->sy = sy; f->sz = f->sw = 0; }
void zfp_field_set_stride_3d(zfp_field* f, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz) {
  f->sx = sx; f->sy = sy; f->sz = sz; f->sw = 0;
}
void zfp_field_set_stride_4d(zfp_field* f, ptrdiff_t sx, ptrdiff_t sy, ptrdiff_t sz, ptrdiff_t sw) {
  f->sx = sx; f->sy = sy; f->sz = sz; f->sw = sw;
}

zfp_bool zfp_field_set_metadata(zfp_field* f, uint64_t meta) {
  if (meta >> ZFP_META_BITS) return zfp_false;
  f->type = (zfp_type)((meta & 3u) + 1);
  meta >>= 2;
  const unsigned int d = (unsigned int)(meta & 3u) + 1;
  meta >>= 2;
  const unsigned int width = d == 1 ? 48 : d == 2 ? 24 : d == 3 ? 16 : 12;
  size_t n[4] = {0, 0, 0, 0};
  for (unsigned int a = 0; a < d; a++) {
    // one-dimensional extents are limited to 32 bits (src/zfp.c:297-299)
    const uint64_t mask = d == 1 ? 0xffffffffull : (1ull << width) - 1;
    n[a] = (size_t)(meta & mask) + 1;
    meta >>= width;
  }
  f->nx = n[0]; f->ny = n[1]; f->nz = n[2]; f->nw = n[3];
  f->sx = f->sy = f->sz = f->sw = 0;
  return zfp_true;
}

// ---------------------------------------------------------------------------
// configurations (src/zfp.c:328-393)

zfp_config zfp_config_none(void) { zfp_config c; c.mode = zfp_mode_null; return c; }
zfp_config zfp_config_rate(double rate, zfp_bool align) {
  zfp_config c; c.mode = zfp_mode_fixed_rate; c.arg.rate = align ? -rate : rate; return c;
}
zfp_config zfp_config_precision(unsigned int precision) {
  zfp_config c; c.mode = zfp_mode_fixed_precision; c.arg.precision = precision; return c;
}
zfp_config zfp_config_accuracy(double tolerance) {
  zfp_config c; c.mode = zfp_mode_fixed_accuracy; c.arg.tolerance = tolerance; return c;
}
zfp_config zfp_config_reversible(void) { zfp_config c; c.mode = zfp_mode_reversible; return c; }
zfp_config zfp_config_expert(unsigned int minbits, unsigned int maxbits, unsigned int maxprec, int minexp) {
  zfp_config c;
  c.mode = zfp_mode_expert;
  c.arg.expert.minbits = minbits;
  c.arg.expert.maxbits = maxbits;
  c.arg.expert.maxprec = maxprec;
  c.arg.expert.minexp = minexp;
  return c;
}

// ---------------------------------------------------------------------------
// compressed stream (src/zfp.c:397-958)

zfp_stream* zfp_stream_open(bitstream* stream) {
  zfp_stream* z = (zfp_stream*)std::malloc(sizeof(zfp_stream));
  if (z) {
    z->stream = stream;
    z->minbits = ZFP_MIN_BITS;
    z->maxbits = ZFP_MAX_BITS;
    z->maxprec = ZFP_MAX_PREC;
    z->minexp = ZFP_MIN_EXP;
    z->exec.policy = zfp_exec_serial;
    z->exec.params = nullptr;
  }
  return z;
}

void zfp_stream_close(zfp_stream* z) {
  zg::release_exec_params(z);
  std::free(z);
}

bitstream* zfp_stream_bit_stream(const zfp_stream* z) { return z->stream; }

zfp_mode zfp_stream_compression_mode(const zfp_stream* z) {  // src/zfp.c:567-608
  if (z->minbits > z->maxbits || !(0 < z->maxprec && z->maxprec <= 64)) return zfp_mode_null;
  if (z->minbits == ZFP_MIN_BITS && z->maxbits == ZFP_MAX_BITS && z->maxprec == ZFP_MAX_PREC &&
      z->minexp == ZFP_MIN_EXP)
    return zfp_mode_expert;
  if (z->minbits == z->maxbits && 1 <= z->maxbits && z->maxbits <= ZFP_MAX_BITS &&
      z->maxprec >= ZFP_MAX_PREC && z->minexp == ZFP_MIN_EXP)
    return zfp_mode_fixed_rate;
  if (z->minbits <= ZFP_MIN_BITS && z->maxbits >= ZFP_MAX_BITS && z->maxprec >= 1 && z->minexp == ZFP_MIN_EXP)
    return zfp_mode_fixed_precision;
  if (z->minbits <= ZFP_MIN_BITS && z->maxbits >= ZFP_MAX_BITS && z->maxprec >= ZFP_MAX_PREC &&
      z->minexp >= ZFP_MIN_EXP)
    return zfp_mode_fixed_accuracy;
  if (z->minbits <= ZFP_MIN_BITS && z->maxbits >= ZFP_MAX_BITS && z->maxprec >= ZFP_MAX_PREC &&
      z->minexp < ZFP_MIN_EXP)
    return zfp_mode_reversible;
  return zfp_mode_expert;
}

double zfp_stream_rate(const zfp_stream* z, unsigned int dims) {
  return zfp_stream_compression_mode(z) == zfp_mode_fixed_rate ? (double)z->maxbits / (1u << (2 * dims)) : 0.0;
}

unsigned int zfp_stream_precision(const zfp_stream* z) {
  return zfp_stream_compression_mode(z) == zfp_mode_fixed_precision ? z->maxprec : 0;
}

double zfp_stream_accuracy(const zfp_stream* z) {
  return zfp_stream_compression_mode(z) == zfp_mode_fixed_accuracy ? std::ldexp(1.0, z->minexp) : 0.0;
}

// 12-bit short or 64-bit long mode encoding (src/zfp.c:630-690)
uint64_t zfp_stream_mode(const zfp_stream* z) {
  switch (zfp_stream_compression_mode(z)) {
    case zfp_mode_fixed_rate:
      if (z->maxbits <= 2048) return z->maxbits - 1;
      break;
    case zfp_mode_fixed_precision:
      if (z->maxprec <= 128) return (z->maxprec - 1) + 2048;
      break;
    case zfp_mode_fixed_accuracy:
      if (z->minexp <= 843) return (uint64_t)(z->minexp - ZFP_MIN_EXP) + (2048 + 128 + 1);
      break;
    case zfp_mode_reversible:
      return 2048 + 128;
    default:
      break;
  }
  auto clamp = [](long long v, long long lo, long long hi) { return v < lo ? lo : v > hi ? hi : v; };
  const uint64_t minbits = (uint64_t)clamp(z->minbits < 0x8000u ? z->minbits : 0x8000u, 1, 0x8000) - 1;
  const uint64_t maxbits = (uint64_t)clamp(z->maxbits < 0x8000u ? z->maxbits : 0x8000u, 1, 0x8000) - 1;
  const uint64_t maxprec = (uint64_t)clamp(z->maxprec < 0x80u ? z->maxprec : 0x80u, 1, 0x80) - 1;
  const uint64_t minexp = (uint64_t)clamp((long long)z->minexp + 16495, 0, 0x7fff);
  uint64_t mode = 0;
  mode = (mode << 15) + minexp;
  mode = (mode << 7) + maxprec;
  mode = (mode << 15) + maxbits;
  mode = (mode << 15) + minbits;
  mode = (mode << 12) + 0xfffu;
  return mode;
}

void zfp_stream_params(const zfp_stream* z, unsigned int* minbits, unsigned int* maxbits, unsigned int* maxprec,
                       int* minexp) {
  if (minbits) *minbits = z->minbits;
  if (maxbits) *maxbits = z->maxbits;
  if (maxprec) *maxprec = z->maxprec;
  if (minexp) *minexp = z->minexp;
}

size_t zfp_stream_compressed_size(const zfp_stream* z) { return stream_size(z->stream); }

// worst-case stream size including a full header (src/zfp.c:712-742)
size_t zfp_stream_maximum_size(const zfp_stream* z, const zfp_field* f) {
  const bool rev = z->minexp < ZFP_MIN_EXP;
  const unsigned int d = zfp_field_dimensionality(f);
  const size_t blocks = zfp_field_blocks(f);
  const unsigned int values = 1u << (2 * d);
  unsigned int maxbits = 0;
  if (!d) return 0;
  switch (f->type) {
    case zfp_type_int32: maxbits += rev ? 5 : 0; break;
    case zfp_type_int64: maxbits += rev ? 6 : 0; break;
    case zfp_type_float: maxbits += rev ? 1 + 1 + 8 + 5 : 1 + 8; break;
    case zfp_type_double: maxbits += rev ? 1 + 1 + 11 + 6 : 1 + 11; break;
    default: return 0;
  }
  const unsigned int prec = zfp_field_precision(f);
  maxbits += values - 1 + values * (z->maxprec < prec ? z->maxprec : prec);
  if (maxbits > z->maxbits) maxbits = z->maxbits;
  if (maxbits < z->minbits) maxbits = z->minbits;
  return ((ZFP_HEADER_MAX_BITS + blocks * maxbits + kWord - 1) & ~(kWord - 1)) / 8;
}

void zfp_stream_set_bit_stream(zfp_stream* z, bitstream* s) { z->stream = s; }

void zfp_stream_set_reversible(zfp_stream* z) {
  z->minbits = ZFP_MIN_BITS;
  z->maxbits = ZFP_MAX_BITS;
  z->maxprec = ZFP_MAX_PREC;
  z->minexp = ZFP_MIN_EXP - 1;
}

double zfp_stream_set_rate(zfp_stream* z, double rate, zfp_type type, unsigned int dims, zfp_bool align) {
  const unsigned int n = 1u << (2 * dims);
  unsigned int bits = (unsigned int)std::floor(n * rate + 0.5);
  if (type == zfp_type_float && bits < 1 + 8u) bits = 1 + 8u;
  if (type == zfp_type_double && bits < 1 + 11u) bits = 1 + 11u;
  if (align) bits = (bits + (unsigned int)kWord - 1) & ~((unsigned int)kWord - 1);
  z->minbits = bits;
  z->maxbits = bits;
  z->maxprec = ZFP_MAX_PREC;
  z->minexp = ZFP_MIN_EXP;
  return (double)bits / n;
}

unsigned int zfp_stream_set_precision(zfp_stream* z, unsigned int precision) {
  z->minbits = ZFP_MIN_BITS;
  z->maxbits = ZFP_MAX_BITS;
  z->maxprec = precision ? (precision < ZFP_MAX_PREC ? precision : ZFP_MAX_PREC) : ZFP_MAX_PREC;
  z->minexp = ZFP_MIN_EXP;
  return z->maxprec;
}

double zfp_stream_set_accuracy(zfp_stream* z, double tolerance) {
  int emin = ZFP_MIN_EXP;
  if (tolerance > 0) {
    std::frexp(tolerance, &emin);   // tolerance = x * 2^emin, 0.5 <= x < 1
    emin--;
  }
  z->minbits = ZFP_MIN_BITS;
  z->maxbits = ZFP_MAX_BITS;
  z->maxprec = ZFP_MAX_PREC;
  z->minexp = emin;
  return tolerance > 0 ? std::ldexp(1.0, emin) : 0;
}

zfp_bool zfp_stream_set_params(zfp_stream* z, unsigned int minbits, unsigned int maxbits, unsigned int maxprec,
                               int minexp) {
  if (minbits > maxbits || !(0 < maxprec && maxprec <= 64)) return zfp_false;
  z->minbits = minbits;
  z->maxbits = maxbits;
  z->maxprec = maxprec;
  z->minexp = minexp;
  return zfp_true;
}

zfp_mode zfp_stream_set_mode(zfp_stream* z, uint64_t mode) {  // src/zfp.c:830-880
  unsigned int minbits, maxbits, maxprec;
  int minexp;
  if (mode <= ZFP_MODE_SHORT_MAX) {
    if (mode < 2048) {
      minbits = maxbits = (unsigned int)mode + 1;
      maxprec = ZFP_MAX_PREC;
      minexp = ZFP_MIN_EXP;
    } else if (mode < 2048 + 128) {
      minbits = ZFP_MIN_BITS;
      maxbits = ZFP_MAX_BITS;
      maxprec = (unsigned int)mode + 1 - 2048;
      minexp = ZFP_MIN_EXP;
    } else if (mode == 2048 + 128) {
      minbits = ZFP_MIN_BITS;
      maxbits = ZFP_MAX_BITS;
      maxprec = ZFP_MAX_PREC;
      minexp = ZFP_MIN_EXP - 1;
    } else {
      minbits = ZFP_MIN_BITS;
      maxbits = ZFP_MAX_BITS;
      maxprec = ZFP_MAX_PREC;
      minexp = (int)mode + ZFP_MIN_EXP - (2048 + 128 + 1);
    }
  } else {
    mode >>= 12; minbits = (unsigned int)(mode & 0x7fffu) + 1;
    mode >>= 15; maxbits = (unsigned int)(mode & 0x7fffu) + 1;
    mode >>= 15; maxprec = (unsigned int)(mode & 0x007fu) + 1;
    mode >>= 7;  minexp = (int)(mode & 0x7fffu) - 16495;
  }
  if (!zfp_stream_set_params(z, minbits, maxbits, maxprec, minexp)) return zfp_mode_null;
  return zfp_stream_compression_mode(z);
}

size_t zfp_stream_flush(zfp_stream* z) { return stream_flush(z->stream); }
size_t zfp_stream_align(zfp_stream* z) { return stream_align(z->stream); }
void zfp_stream_rewind(zfp_stream* z) { stream_rewind(z->stream); }

zfp_exec_policy zfp_stream_execution(const zfp_stream* z) { return z->exec.policy; }
unsigned int zfp_stream_omp_threads(const zfp_stream*) { return 0u; }
unsigned int zfp_stream_omp_chunk_size(const zfp_stream*) { return 0u; }

// serial (the default) and cuda can be selected; OpenMP is not part of this
// library, so selecting it fails exactly as in a reference build without
// OpenMP (src/zfp.c:918-955)
zfp_bool zfp_stream_set_execution(zfp_stream* z, zfp_exec_policy policy) {
  switch (policy) {
    case zfp_exec_serial:
      zg::release_exec_params(z);
      z->exec.policy = policy;
      return zfp_true;
    case zfp_exec_cuda:
      if (!zg::ensure_exec_params(z)) return zfp_false;
      z->exec.policy = policy;
      return zfp_true;
    default:
      return zfp_false;
  }
}

zfp_bool zfp_stream_set_omp_threads(zfp_stream* z, unsigned int) { return zfp_stream_set_execution(z, zfp_exec_omp); }
zfp_bool zfp_stream_set_omp_chunk_size(zfp_stream* z, unsigned int) { return zfp_stream_set_execution(z, zfp_exec_omp); }

// ---------------------------------------------------------------------------
// compression (src/zfp.c:1052-1180): GPU only

size_t zfp_compress(zfp_stream* z, const zfp_field* f) {
  if (z->exec.policy != zfp_exec_cuda) {
    zg::set_error("zfp_compress: execution policy is not zfp_exec_cuda (this library has no CPU codec)");
    return 0;
  }
  return zg::gpu_compress(z, f);
}

size_t zfp_decompress(zfp_stream* z, zfp_field* f) {
  if (z->exec.policy != zfp_exec_cuda) {
    zg::set_error("zfp_decompress: execution policy is not zfp_exec_cuda (this library has no CPU codec)");
    return 0;
  }
  return zg::gpu_decompress(z, f);
}

// ---------------------------------------------------------------------------
// header (src/zfp.c:1183-1249)

size_t zfp_write_header(zfp_stream* z, const zfp_field* f, unsigned int mask) {
  size_t bits = 0;
  uint64_t meta = 0;
  if (mask & ZFP_HEADER_META) {
    meta = zfp_field_metadata(f);
    if (meta == ZFP_META_NULL) return 0;
  }
  if (mask & ZFP_HEADER_MAGIC) {
    stream_write_bits(z->stream, 'z', 8);
    stream_write_bits(z->stream, 'f', 8);
    stream_write_bits(z->stream, 'p', 8);
    stream_write_bits(z->stream, zfp_codec_version, 8);
    bits += ZFP_MAGIC_BITS;
  }
  if (mask & ZFP_HEADER_META) {
    stream_write_bits(z->stream, meta, ZFP_META_BITS);
    bits += ZFP_META_BITS;
  }
  if (mask & ZFP_HEADER_MODE) {
    const uint64_t mode = zfp_stream_mode(z);
    const size_t size = mode > ZFP_MODE_SHORT_MAX ? ZFP_MODE_LONG_BITS : ZFP_MODE_SHORT_BITS;
    stream_write_bits(z->stream, mode, size);
    bits += size;
  }
  return bits;
}

size_t zfp_read_header(zfp_stream* z, zfp_field* f, unsigned int mask) {
  size_t bits = 0;
  if (mask & ZFP_HEADER_MAGIC) {
    if (stream_read_bits(z->stream, 8) != 'z' || stream_read_bits(z->stream, 8) != 'f' ||
        stream_read_bits(z->stream, 8) != 'p' || stream_read_bits(z->stream, 8) != zfp_codec_version)
      return 0;
    bits += ZFP_MAGIC_BITS;
  }
  if (mask & ZFP_HEADER_META) {
    const uint64_t meta = stream_read_bits(z->stream, ZFP_META_BITS);
    if (!zfp_field_set_metadata(f, meta)) return 0;
    bits += ZFP_META_BITS;
  }
  if (mask & ZFP_HEADER_MODE) {
    uint64_t mode = stream_read_bits(z->stream, ZFP_MODE_SHORT_BITS);
    bits += ZFP_MODE_SHORT_BITS;
    if (mode > ZFP_MODE_SHORT_MAX) {
      const size_t size = ZFP_MODE_LONG_BITS - ZFP_MODE_SHORT_BITS;
      mode += stream_read_bits(z->stream, size) << ZFP_MODE_SHORT_BITS;
      bits += size;
    }
    if (zfp_stream_set_mode(z, mode) == zfp_mode_null) return 0;
  }
  return bits;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// internal access to the bit stream state for the GPU path

namespace zg {

StreamState get_stream_state(const bitstream* s) {
  StreamState st;
  st.begin = s->begin;
  st.ptr = s->ptr;
  st.end = s->end;
  st.bits = s->bits;
  st.buffer = s->buffer;
  return st;
}

void set_stream_flushed(bitstream* s, uint64_t end_bit) {
  s->ptr = s->begin + (end_bit + 63) / 64;
  s->bits = 0;
  s->buffer = 0;
}

static bool read_word(const uint64_t* p, bool device, uint64_t& w) {
  if (!device) {
    w = *p;
    return true;
  }
  if (cudaMemcpy(&w, p, sizeof w, cudaMemcpyDeviceToHost) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return true;
}

// writer state (include/zfp/bitstream.inl:133-143): `bits` buffered bits in
// `buffer`, ptr at the word they will go to
bool set_stream_written(bitstream* s, uint64_t end_bit, bool device) {
  s->ptr = s->begin + end_bit / 64;
  s->bits = end_bit % 64;
  s->buffer = 0;
  if (!s->bits) return true;
  uint64_t w;
  if (!read_word(s->ptr, device, w)) return false;
  s->buffer = w & ((uint64_t(1) << s->bits) - 1);
  return true;
}

// reader state of stream_rseek (include/zfp/bitstream.inl:340-352)
bool set_stream_read_at(bitstream* s, uint64_t end_bit, bool device) {
  const unsigned n = (unsigned)(end_bit % 64);
  s->ptr = s->begin + end_bit / 64;
  s->buffer = 0;
  s->bits = 0;
  if (!n) return true;
  uint64_t w;
  if (!read_word(s->ptr, device, w)) return false;
  s->ptr++;
  s->buffer = w >> n;
  s->bits = 64 - n;
  return true;
}

}  // namespace zg
