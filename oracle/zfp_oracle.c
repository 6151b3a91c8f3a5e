/*
 * zfp_oracle.c -- CPU restatement of zfp 1.0.1's serial block codec.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the GPU codec and the CPU
 * baseline that bench.py times.  Nothing in zfp_gb300/ links or loads it.
 * Parity of this file is pinned against the reference library compiled
 * from its own sources (oracle/Makefile, target `ref`) and against the
 * fixtures in tests/golden/.
 *
 * Layout of the restatement:
 *   bit I/O          include/zfp/bitstream.inl:226-409 (64-bit words, LSB first)
 *   coefficient order src/template/codec{1,2,3,4}.c (PERM tables)
 *   gather/scatter   src/template/encode{1..4}.c, decode{1..4}.c,
 *                    pad_block src/template/encode.c:9-27
 *   array drivers    src/template/compress.c, decompress.c (raster order)
 *   parallel driver  src/template/ompcompress.c:155-210, src/share/parallel.c
 *   integer codec    oracle_int.inc;  floating front end  oracle_float.inc
 */
#include "zfp_oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CAT_(a, b) a##b
#define CAT(a, b) CAT_(a, b)
#define ORC_MIN_EXP (-1074)
#define NBMASK_32 0xaaaaaaaau
#define NBMASK_64 0xaaaaaaaaaaaaaaaaull
#define PBITS_32 5
#define PBITS_64 6

/* ------------------------------------------------------------------ */
/* coefficient order: by total sequency i+j+k+l, then by i^2+j^2+k^2+l^2.
 * The tie order inside equal keys is part of the stream format and is
 * given as data (index = i + 4j + 16k + 64l). */

static const uint8_t order1[4] = {0, 1, 2, 3};
static const uint8_t order2[16] = {
  0, 1, 4, 5, 2, 8, 6, 9, 3, 12, 10, 7, 13, 11, 14, 15};
static const uint8_t order3[64] = {
  0, 1, 4, 16, 20, 17, 5, 2, 8, 32, 21, 6, 18, 24, 9, 33,
  36, 3, 12, 48, 22, 25, 37, 40, 34, 10, 7, 19, 28, 13, 49, 52,
  41, 38, 26, 23, 29, 53, 11, 35, 44, 14, 50, 56, 42, 27, 39, 45,
  30, 54, 57, 60, 51, 15, 43, 46, 58, 61, 55, 31, 62, 59, 47, 63};
static const uint8_t order4[256] = {
  0, 1, 4, 16, 64, 5, 80, 17, 68, 65, 20, 2, 8, 32, 128, 84,
  81, 69, 21, 6, 18, 66, 24, 72, 9, 96, 33, 36, 129, 132, 144, 3,
  12, 48, 192, 85, 82, 70, 22, 73, 25, 88, 37, 100, 97, 148, 145, 133,
  10, 160, 34, 136, 130, 40, 7, 19, 67, 28, 76, 13, 112, 49, 52, 193,
  196, 208, 86, 89, 101, 149, 161, 137, 41, 134, 38, 164, 26, 152, 146, 104,
  98, 74, 83, 71, 23, 77, 29, 92, 53, 116, 113, 212, 209, 197, 11, 35,
  131, 44, 140, 14, 176, 50, 56, 194, 200, 224, 90, 165, 102, 153, 150, 105,
  168, 162, 138, 42, 87, 93, 117, 213, 27, 75, 99, 39, 135, 147, 108, 45,
  141, 156, 30, 78, 177, 180, 54, 114, 120, 57, 198, 210, 216, 201, 225, 228,
  15, 240, 51, 204, 195, 60, 169, 166, 154, 106, 91, 103, 151, 109, 157, 94,
  181, 118, 121, 214, 217, 229, 163, 139, 43, 142, 46, 172, 58, 184, 178, 232,
  226, 202, 241, 205, 61, 199, 55, 244, 31, 220, 211, 124, 115, 79, 170, 167,
  155, 107, 158, 110, 173, 122, 185, 182, 233, 230, 218, 95, 245, 119, 221, 215,
  125, 242, 206, 62, 203, 59, 248, 47, 236, 227, 188, 179, 143, 171, 174, 186,
  234, 246, 222, 126, 219, 123, 249, 111, 237, 231, 189, 183, 159, 252, 243, 207,
  63, 175, 250, 187, 238, 235, 190, 253, 247, 223, 127, 254, 251, 239, 191, 255};

static const uint8_t* coeff_order(int dims)
{
  switch (dims) {
    case 1: return order1;
    case 2: return order2;
    case 3: return order3;
    default: return order4;
  }
}

/* number of bit planes to code (src/template/codecf.c:6-13, default build) */
static unsigned coded_precision(int emax, unsigned maxprec, int minexp, int dims)
{
  long long p = (long long)emax - minexp + 2 * dims + 2;
  if (p < 0)
    p = 0;
  return (unsigned)p < maxprec ? (unsigned)p : maxprec;
}

/* ------------------------------------------------------------------ */
/* bit I/O: 64-bit words, bits filled from the least significant end */

typedef struct {
  uint64_t* base;
  uint64_t* p;      /* next word to store */
  uint64_t acc;     /* pending bits */
  unsigned fill;    /* number of pending bits, < 64 */
} bw_t;

static void bw_init(bw_t* w, uint64_t* words, uint64_t bit0)
{
  w->base = words;
  w->p = words + (bit0 >> 6);
  w->fill = (unsigned)(bit0 & 63);
  w->acc = w->fill ? (*w->p & ((1ull << w->fill) - 1)) : 0;
}

static inline void bw_put(bw_t* w, uint64_t v, unsigned n)
{
  unsigned t;
  if (!n)
    return;
  if (n < 64)
    v &= (1ull << n) - 1;
  w->acc |= v << w->fill;
  t = w->fill + n;
  if (t >= 64) {
    *w->p++ = w->acc;
    w->acc = w->fill ? v >> (64 - w->fill) : 0;
    t -= 64;
  }
  w->fill = t;
}

static void bw_pad(bw_t* w, uint64_t n)
{
  while (n) {
    unsigned c = n < 64 ? (unsigned)n : 64;
    bw_put(w, 0, c);
    n -= c;
  }
}

static uint64_t bw_tell(const bw_t* w)
{
  return (uint64_t)(w->p - w->base) * 64 + w->fill;
}

static void bw_flush(bw_t* w)
{
  if (w->fill) {
    *w->p++ = w->acc;
    w->acc = 0;
    w->fill = 0;
  }
}

typedef struct {
  const uint64_t* words;
  uint64_t pos;     /* absolute bit offset of the next bit */
} br_t;

static inline uint64_t br_get(br_t* r, unsigned n)
{
  uint64_t i, v;
  unsigned o;
  if (!n)
    return 0;
  i = r->pos >> 6;
  o = (unsigned)(r->pos & 63);
  v = r->words[i] >> o;
  if (o && o + n > 64)
    v |= r->words[i + 1] << (64 - o);
  r->pos += n;
  return n == 64 ? v : v & ((1ull << n) - 1);
}

static inline void br_skip(br_t* r, uint64_t n)
{
  r->pos += n;
}

/* plane helpers for the group tests: bit i of a plane of <= 256 bits */
static inline unsigned plane_bit(const uint64_t* plane, unsigned i)
{
  return (unsigned)((plane[i >> 6] >> (i & 63)) & 1u);
}

static inline unsigned plane_any_from(const uint64_t* plane, unsigned from, unsigned size)
{
  unsigned i;
  for (i = from; i < size; i++)
    if (plane_bit(plane, i))
      return 1;
  return 0;
}

/* ------------------------------------------------------------------ */
/* integer codec, one instance per width */

#define FN(name) CAT(name, W)

#define W 32
#define IT int32_t
#define UT uint32_t
#include "oracle_int.inc"
#undef W
#undef IT
#undef UT

#define W 64
#define IT int64_t
#define UT uint64_t
#include "oracle_int.inc"
#undef W
#undef IT
#undef UT

/* floating-point front end, one instance per scalar type */

#define FFN(name) CAT(name, FSUF)

#define FT float
#define FSUF _f
#define W 32
#define IT int32_t
#define UT uint32_t
#define EBITS_F 8
#include "oracle_float.inc"
#undef FT
#undef FSUF
#undef W
#undef IT
#undef UT
#undef EBITS_F

#define FT double
#define FSUF _d
#define W 64
#define IT int64_t
#define UT uint64_t
#define EBITS_F 11
#include "oracle_float.inc"
#undef FT
#undef FSUF
#undef W
#undef IT
#undef UT
#undef EBITS_F

/* ------------------------------------------------------------------ */
/* field geometry */

typedef struct {
  int dims;
  int type;
  size_t esize;
  size_t n[4];      /* extents, 1 for unused axes */
  size_t nb[4];     /* blocks per axis */
  ptrdiff_t s[4];   /* resolved strides */
  size_t blocks;
} geom_t;

int orc_dims(const orc_field* f)
{
  return f->n[0] ? f->n[1] ? f->n[2] ? f->n[3] ? 4 : 3 : 2 : 1 : 0;
}

static int make_geom(const orc_field* f, geom_t* g)
{
  int a;
  g->dims = orc_dims(f);
  g->type = f->type;
  switch (f->type) {
    case ORC_INT32: case ORC_FLOAT: g->esize = 4; break;
    case ORC_INT64: case ORC_DOUBLE: g->esize = 8; break;
    default: return 0;
  }
  if (!g->dims)
    return 0;
  g->blocks = 1;
  for (a = 0; a < 4; a++) {
    g->n[a] = a < g->dims ? f->n[a] : 1;
    g->nb[a] = a < g->dims ? (f->n[a] + 3) / 4 : 1;
    g->blocks *= g->nb[a];
  }
  /* each stride defaults independently (src/template/compress.c:60-68) */
  g->s[0] = f->s[0] ? f->s[0] : 1;
  g->s[1] = f->s[1] ? f->s[1] : (ptrdiff_t)f->n[0];
  g->s[2] = f->s[2] ? f->s[2] : (ptrdiff_t)(f->n[0] * f->n[1]);
  g->s[3] = f->s[3] ? f->s[3] : (ptrdiff_t)(f->n[0] * f->n[1] * f->n[2]);
  return 1;
}

size_t orc_blocks(const orc_field* f)
{
  geom_t g;
  return make_geom(f, &g) ? g.blocks : 0;
}

/* index of the source value that fills position i of a block row holding
 * n valid values: [a], [a b b a], [a b c a] padding (encode.c:9-27) */
static const uint8_t pad_map[5][4] = {
  {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 1, 1, 0}, {0, 1, 2, 0}, {0, 1, 2, 3}};

static void block_origin(const geom_t* g, size_t b, size_t org[4], size_t cnt[4])
{
  int a;
  for (a = 0; a < 4; a++) {
    size_t i = b % g->nb[a];
    b /= g->nb[a];
    org[a] = 4 * i;
    cnt[a] = g->n[a] - org[a] < 4 ? g->n[a] - org[a] : 4;
  }
}

/* gather one (possibly partial) block as raw bit patterns */
static void gather_block(const geom_t* g, const void* data, size_t b, void* out)
{
  size_t org[4], cnt[4];
  const char* base;
  int x, y, z, w, i = 0;
  int ex = g->dims >= 1 ? 4 : 1, ey = g->dims >= 2 ? 4 : 1;
  int ez = g->dims >= 3 ? 4 : 1, ew = g->dims >= 4 ? 4 : 1;
  block_origin(g, b, org, cnt);
  base = (const char*)data + (ptrdiff_t)g->esize *
         ((ptrdiff_t)org[0] * g->s[0] + (ptrdiff_t)org[1] * g->s[1] +
          (ptrdiff_t)org[2] * g->s[2] + (ptrdiff_t)org[3] * g->s[3]);
  for (w = 0; w < ew; w++)
    for (z = 0; z < ez; z++)
      for (y = 0; y < ey; y++)
        for (x = 0; x < ex; x++, i++) {
          ptrdiff_t off = pad_map[cnt[0]][x] * g->s[0] + pad_map[cnt[1]][y] * g->s[1] +
                          pad_map[cnt[2]][z] * g->s[2] + pad_map[cnt[3]][w] * g->s[3];
          if (g->esize == 4)
            ((uint32_t*)out)[i] = *(const uint32_t*)(base + 4 * off);
          else
            ((uint64_t*)out)[i] = *(const uint64_t*)(base + 8 * off);
        }
}

/* store the valid part of one decoded block (decode3.c:5-23) */
static void scatter_block(const geom_t* g, void* data, size_t b, const void* in)
{
  size_t org[4], cnt[4];
  char* base;
  size_t x, y, z, w;
  block_origin(g, b, org, cnt);
  base = (char*)data + (ptrdiff_t)g->esize *
         ((ptrdiff_t)org[0] * g->s[0] + (ptrdiff_t)org[1] * g->s[1] +
          (ptrdiff_t)org[2] * g->s[2] + (ptrdiff_t)org[3] * g->s[3]);
  for (w = 0; w < cnt[3]; w++)
    for (z = 0; z < cnt[2]; z++)
      for (y = 0; y < cnt[1]; y++)
        for (x = 0; x < cnt[0]; x++) {
          ptrdiff_t off = (ptrdiff_t)x * g->s[0] + (ptrdiff_t)y * g->s[1] +
                          (ptrdiff_t)z * g->s[2] + (ptrdiff_t)w * g->s[3];
          size_t i = x + 4 * y + 16 * z + 64 * w;
          if (g->esize == 4)
            *(uint32_t*)(base + 4 * off) = ((const uint32_t*)in)[i];
          else
            *(uint64_t*)(base + 8 * off) = ((const uint64_t*)in)[i];
        }
}

static unsigned encode_one(bw_t* w, const geom_t* g, const orc_params* p, void* raw)
{
  switch (g->type) {
    case ORC_INT32: return encode_int_field_block32(w, p, (int32_t*)raw, g->dims);
    case ORC_INT64: return encode_int_field_block64(w, p, (int64_t*)raw, g->dims);
    case ORC_FLOAT: return encode_field_block_f(w, p, (const float*)raw, g->dims);
    default: return encode_field_block_d(w, p, (const double*)raw, g->dims);
  }
}

static unsigned decode_one(br_t* r, const geom_t* g, const orc_params* p, void* raw)
{
  switch (g->type) {
    case ORC_INT32: return decode_int_field_block32(r, p, (int32_t*)raw, g->dims);
    case ORC_INT64: return decode_int_field_block64(r, p, (int64_t*)raw, g->dims);
    case ORC_FLOAT: return decode_field_block_f(r, p, (float*)raw, g->dims);
    default: return decode_field_block_d(r, p, (double*)raw, g->dims);
  }
}

uint64_t orc_compress(const orc_field* f, const orc_params* p,
                      uint64_t* words, uint64_t bit0, uint64_t* block_end)
{
  geom_t g;
  bw_t w;
  size_t b;
  uint64_t end;
  uint64_t raw[256];
  if (!make_geom(f, &g))
    return bit0;
  bw_init(&w, words, bit0);
  for (b = 0; b < g.blocks; b++) {
    gather_block(&g, f->data, b, raw);
    encode_one(&w, &g, p, raw);
    if (block_end)
      block_end[b] = bw_tell(&w);
  }
  end = bw_tell(&w);
  bw_flush(&w);
  return end;
}

uint64_t orc_decompress(const orc_field* f, const orc_params* p,
                        const uint64_t* words, uint64_t bit0)
{
  geom_t g;
  br_t r;
  size_t b;
  uint64_t raw[256];
  if (!make_geom(f, &g))
    return bit0;
  r.words = words;
  r.pos = bit0;
  for (b = 0; b < g.blocks; b++) {
    decode_one(&r, &g, p, raw);
    scatter_block(&g, f->data, b, raw);
  }
  return r.pos;
}

unsigned orc_block_maxbits(const orc_field* f, const orc_params* p)
{
  int dims = orc_dims(f);
  int rev = p->minexp < ORC_MIN_EXP;
  unsigned values = 1u << (2 * dims);
  unsigned bits = 0, prec = 0;
  switch (f->type) {
    case ORC_INT32: bits = rev ? 5 : 0; prec = 32; break;
    case ORC_INT64: bits = rev ? 6 : 0; prec = 64; break;
    case ORC_FLOAT: bits = rev ? 1 + 1 + 8 + 5 : 1 + 8; prec = 32; break;
    case ORC_DOUBLE: bits = rev ? 1 + 1 + 11 + 6 : 1 + 11; prec = 64; break;
    default: return 0;
  }
  bits += values - 1 + values * (p->maxprec < prec ? p->maxprec : prec);
  if (bits > p->maxbits)
    bits = p->maxbits;
  if (bits < p->minbits)
    bits = p->minbits;
  return bits;
}

/* Parallel driver: contiguous block ranges per chunk, each coded into a
 * private buffer, then copied one after the other into the output.  The
 * output is identical to orc_compress. */
uint64_t orc_compress_par(const orc_field* f, const orc_params* p,
                          uint64_t* words, uint64_t bit0, int threads, uint64_t* block_end)
{
  geom_t g;
  size_t chunks, c;
  uint64_t** buf;
  uint64_t* len;
  unsigned maxb;
  bw_t out;
  uint64_t end;
  if (!make_geom(f, &g))
    return bit0;
  if (threads < 1)
    threads = 1;
  chunks = (size_t)threads * 4;
  if (chunks > g.blocks)
    chunks = g.blocks;
  maxb = orc_block_maxbits(f, p);
  buf = (uint64_t**)calloc(chunks, sizeof(uint64_t*));
  len = (uint64_t*)calloc(chunks, sizeof(uint64_t));
#ifdef _OPENMP
  #pragma omp parallel for schedule(static, 1) num_threads(threads)
#endif
  for (c = 0; c < chunks; c++) {
    size_t b0 = g.blocks * c / chunks, b1 = g.blocks * (c + 1) / chunks, b;
    size_t nw = ((b1 - b0) * (uint64_t)maxb + 127) / 64;
    uint64_t raw[256];
    bw_t w;
    buf[c] = (uint64_t*)malloc(nw * sizeof(uint64_t));
    bw_init(&w, buf[c], 0);
    for (b = b0; b < b1; b++) {
      gather_block(&g, f->data, b, raw);
      encode_one(&w, &g, p, raw);
      if (block_end)
        block_end[b] = bw_tell(&w);   /* chunk-relative for now */
    }
    len[c] = bw_tell(&w);
    bw_flush(&w);
  }
  bw_init(&out, words, bit0);
  for (c = 0; c < chunks; c++) {
    uint64_t i;
    if (block_end) {
      size_t b0 = g.blocks * c / chunks, b1 = g.blocks * (c + 1) / chunks, b;
      uint64_t base = bw_tell(&out);
      for (b = b0; b < b1; b++)
        block_end[b] += base;
    }
    for (i = 0; i < len[c]; i += 64)
      bw_put(&out, buf[c][i >> 6], len[c] - i < 64 ? (unsigned)(len[c] - i) : 64);
    free(buf[c]);
  }
  free(buf);
  free(len);
  end = bw_tell(&out);
  bw_flush(&out);
  return end;
}

/* Parallel decompression given every block's start bit (block_start[b]);
 * with block_start == NULL the stream must be fixed rate (minbits ==
 * maxbits) and block b starts at bit0 + b * maxbits. */
uint64_t orc_decompress_par(const orc_field* f, const orc_params* p, const uint64_t* words,
                            uint64_t bit0, const uint64_t* block_start, int threads)
{
  geom_t g;
  long long b;
  uint64_t end = bit0;
  if (!make_geom(f, &g))
    return bit0;
  if (threads < 1)
    threads = 1;
#ifdef _OPENMP
  #pragma omp parallel for schedule(static, 256) num_threads(threads) reduction(max : end)
#endif
  for (b = 0; b < (long long)g.blocks; b++) {
    uint64_t raw[256];
    br_t r;
    r.words = words;
    r.pos = block_start ? block_start[b] : bit0 + (uint64_t)b * p->maxbits;
    decode_one(&r, &g, p, raw);
    scatter_block(&g, f->data, (size_t)b, raw);
    if (r.pos > end)
      end = r.pos;
  }
  return end;
}
