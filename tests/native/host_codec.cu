// host_codec.cu -- runs the GPU block codec (zfp_gb300/csrc/codec.cuh) on the
// CPU over whole fields, block after block in raster order, so the tests can
// compare its per-block logic with the oracle without a GPU.  Test-only; the
// product library never contains this file.
#include <cstddef>
#include <cstdint>
#include <cstring>

#include "../../zfp_gb300/csrc/codec.cuh"
#include "../../zfp_gb300/csrc/kernels.cuh"
#include "../../zfp_gb300/csrc/launch.h"

namespace {

// Like the kernels' sinks, put() requires v to have no bits at or above n;
// a violation is recorded (and makes the field compare fail) instead of
// being masked away.
static bool g_unclean_put = false;

struct VecSink {
  uint64_t* words;
  uint64_t pos;
  ZG_HD void put(uint64_t v, unsigned n) {
#if !defined(__CUDA_ARCH__)
    if (n < 64 && (v >> n)) g_unclean_put = true;
#endif
    if (!n) return;
    const unsigned o = (unsigned)(pos & 63);
    words[pos >> 6] |= v << o;
    if (o && o + n > 64) words[(pos >> 6) + 1] |= v >> (64 - o);
    pos += n;
  }
  ZG_HD void pad(unsigned n) { pos += n; }
  ZG_HD void finish() {}
};

static bool g_or_overrun = false;   // the kernel's coder wrote past the length it returned
static int g_coder = 0;   // 0: emit_block (one put per significance event), 1: emit_block_seq (table coder)

// Kernels may give a launch's plane buffer no room below plane P - maxprec
// (the planes a job's blocks never code).  The harness fills its plane
// arrays with this pattern: a coder that read such a plane would produce a
// different stream or array, and one that wrote it is recorded here.
static const uint64_t kPlaneJunk = 0xa5a5a5a5a5a5a5a5ull;
static bool g_floor_touched = false;

static void check_floor(const uint64_t* plane, int P, unsigned maxprec, int limit) {
  const int floor = (unsigned)P > maxprec ? P - (int)maxprec : 0;
  for (int k = 0; k < floor && k < limit; k++)
    if (plane[k] != kPlaneJunk) g_floor_touched = true;
}

struct Geom {
  int dims;
  size_t n[4], nb[4];
  ptrdiff_t s[4];
  size_t blocks;
};

Geom geom(int dims, const size_t* n, const ptrdiff_t* s) {
  Geom g;
  g.dims = dims;
  g.blocks = 1;
  for (int a = 0; a < 4; a++) {
    g.n[a] = a < dims ? n[a] : 1;
    g.nb[a] = (g.n[a] + 3) / 4;
    g.blocks *= g.nb[a];
  }
  g.s[0] = s[0] ? s[0] : 1;
  g.s[1] = s[1] ? s[1] : (ptrdiff_t)n[0];
  g.s[2] = s[2] ? s[2] : (ptrdiff_t)(n[0] * g.n[1]);
  g.s[3] = s[3] ? s[3] : (ptrdiff_t)(n[0] * g.n[1] * g.n[2]);
  return g;
}

int pad_index(int i, size_t cnt) { return i < (int)cnt ? i : (cnt == 2 && i == 2) ? 1 : 0; }

template <typename B, int D>
void gather(const Geom& g, const B* data, size_t b, B (&raw)[1 << (2 * D)], size_t org[4], size_t cnt[4]) {
  for (int a = 0; a < 4; a++) {
    size_t i = b % g.nb[a];
    b /= g.nb[a];
    org[a] = 4 * i;
    cnt[a] = g.n[a] - org[a] < 4 ? g.n[a] - org[a] : 4;
  }
  const int e[4] = {D >= 1 ? 4 : 1, D >= 2 ? 4 : 1, D >= 3 ? 4 : 1, D >= 4 ? 4 : 1};
  int i = 0;
  for (int w = 0; w < e[3]; w++)
    for (int z = 0; z < e[2]; z++)
      for (int y = 0; y < e[1]; y++)
        for (int x = 0; x < e[0]; x++, i++) {
          ptrdiff_t off = (ptrdiff_t)(org[0] + pad_index(x, cnt[0])) * g.s[0] +
                          (ptrdiff_t)(org[1] + pad_index(y, cnt[1])) * g.s[1] +
                          (ptrdiff_t)(org[2] + pad_index(z, cnt[2])) * g.s[2] +
                          (ptrdiff_t)(org[3] + pad_index(w, cnt[3])) * g.s[3];
          raw[i] = data[off];
        }
}

template <typename S, int D>
uint64_t compress_t(const Geom& g, const zg::BlockParams& p, const void* data, uint64_t* words, uint64_t bit0) {
  using B = typename zg::Traits<S>::Bits;
  VecSink out{words, bit0};
  for (size_t b = 0; b < g.blocks; b++) {
    B raw[1 << (2 * D)];
    size_t org[4], cnt[4];
    gather<B, D>(g, (const B*)data, b, raw, org, cnt);
    if constexpr ((1 << (2 * D)) <= 64) {
      if (g_coder == 1) {
        using U = typename zg::Traits<S>::UInt;
        constexpr int N = 1 << (2 * D), P = 8 * sizeof(U);
        zg::BlockHead h;
        U u[N];
        uint64_t plane[P];
        for (int k = 0; k < P; k++) plane[k] = kPlaneJunk;
        zg::prepare_coeffs<S, D>(h, p, raw, u);
        if (h.coded) zg::store_planes<N, true>(u, plane, 1, h.maxprec);   // as the kLossyFloor kernels
        const uint64_t at = out.pos;
        const unsigned bits = zg::emit_block_seq<P, N>(out, h, plane, 1, zg::kGroupCodeHost.e);
        if (out.pos != at + bits) g_or_overrun = true;
        check_floor(plane, P, p.maxprec, P);
        continue;
      }
    }
    zg::encode_block<S, D>(out, p, raw, zg::kGroupCodeHost.e);
  }
  return out.pos;
}

template <typename S, int D>
uint64_t decompress_t(const Geom& g, const zg::BlockParams& p, void* data, const uint64_t* words,
                      uint64_t cap, uint64_t bit0) {
  using B = typename zg::Traits<S>::Bits;
  zg::WordSource in;
  in.base = words;
  in.cap = cap;
  in.seek(bit0);
  for (size_t b = 0; b < g.blocks; b++) {
    B raw[1 << (2 * D)];
    constexpr int P = 8 * sizeof(typename zg::Traits<S>::UInt);
    uint64_t plane[P];
    for (int k = 0; k < P; k++) plane[k] = kPlaneJunk;
    // lossy blocks decode as the kLossyFloor kernels do (planes below P -
    // maxprec untouched); 64-bit 2D and 3D blocks go through 32 slots regardless
    if (p.minexp < zg::kMinExp) {
      zg::decode_block<S, D, zg::kRevOnly>(in, p, raw, zg::PlaneBuf{plane, 1});
    } else {
      zg::decode_block<S, D, zg::kLossyFloor>(in, p, raw, zg::PlaneBuf{plane, 1});
      if (!(P == 64 && (D == 2 || D == 3))) check_floor(plane, P, p.maxprec, P);
    }
    size_t org[4], cnt[4];
    size_t bb = b;
    for (int a = 0; a < 4; a++) {
      size_t i = bb % g.nb[a];
      bb /= g.nb[a];
      org[a] = 4 * i;
      cnt[a] = g.n[a] - org[a] < 4 ? g.n[a] - org[a] : 4;
    }
    for (size_t w = 0; w < cnt[3]; w++)
      for (size_t z = 0; z < cnt[2]; z++)
        for (size_t y = 0; y < cnt[1]; y++)
          for (size_t x = 0; x < cnt[0]; x++) {
            ptrdiff_t off = (ptrdiff_t)(org[0] + x) * g.s[0] + (ptrdiff_t)(org[1] + y) * g.s[1] +
                            (ptrdiff_t)(org[2] + z) * g.s[2] + (ptrdiff_t)(org[3] + w) * g.s[3];
            ((B*)data)[off] = raw[x + 4 * y + 16 * z + 64 * w];
          }
  }
  return in.tell();
}

template <typename S>
uint64_t compress_s(const Geom& g, const zg::BlockParams& p, const void* d, uint64_t* w, uint64_t b0) {
  switch (g.dims) {
    case 1: return compress_t<S, 1>(g, p, d, w, b0);
    case 2: return compress_t<S, 2>(g, p, d, w, b0);
    case 3: return compress_t<S, 3>(g, p, d, w, b0);
    default: return compress_t<S, 4>(g, p, d, w, b0);
  }
}

template <typename S>
uint64_t decompress_s(const Geom& g, const zg::BlockParams& p, void* d, const uint64_t* w, uint64_t cap, uint64_t b0) {
  switch (g.dims) {
    case 1: return decompress_t<S, 1>(g, p, d, w, cap, b0);
    case 2: return decompress_t<S, 2>(g, p, d, w, cap, b0);
    case 3: return decompress_t<S, 3>(g, p, d, w, cap, b0);
    default: return decompress_t<S, 4>(g, p, d, w, cap, b0);
  }
}

}  // namespace

extern "C" void zgh_set_coder(int c) { g_coder = c; }

extern "C" int zgh_floor_touched(void) {
  const int r = g_floor_touched;
  g_floor_touched = false;
  return r;
}

extern "C" int zgh_or_overrun(void) {
  const int r = g_or_overrun;
  g_or_overrun = false;
  return r;
}

extern "C" int zgh_unclean_put(void) {
  const int r = g_unclean_put;
  g_unclean_put = false;
  return r;
}

extern "C" uint64_t zgh_compress(int type, int dims, const size_t* n, const ptrdiff_t* s,
                                 const void* data, const unsigned* prm, uint64_t* words, uint64_t bit0) {
  Geom g = geom(dims, n, s);
  zg::BlockParams p{prm[0], prm[1], prm[2], (int32_t)prm[3]};
  switch (type) {
    case 1: return compress_s<int32_t>(g, p, data, words, bit0);
    case 2: return compress_s<int64_t>(g, p, data, words, bit0);
    case 3: return compress_s<float>(g, p, data, words, bit0);
    default: return compress_s<double>(g, p, data, words, bit0);
  }
}

extern "C" uint64_t zgh_decompress(int type, int dims, const size_t* n, const ptrdiff_t* s, void* data,
                                   const unsigned* prm, const uint64_t* words, uint64_t cap, uint64_t bit0) {
  Geom g = geom(dims, n, s);
  zg::BlockParams p{prm[0], prm[1], prm[2], (int32_t)prm[3]};
  switch (type) {
    case 1: return decompress_s<int32_t>(g, p, data, words, cap, bit0);
    case 2: return decompress_s<int64_t>(g, p, data, words, cap, bit0);
    case 3: return decompress_s<float>(g, p, data, words, cap, bit0);
    default: return decompress_s<double>(g, p, data, words, cap, bit0);
  }
}

// the integer casts against the hardware multiply they replace:
// out[i] = bits of (double)v[i] * 2^e, trunc[i] = trunc(x[i] * 2^se)
extern "C" void zgh_int_scale(const int64_t* v, size_t n, int e, uint64_t* out) {
  for (size_t i = 0; i < n; i++) out[i] = zg::int_scale<double>(v[i], e);
}
extern "C" void zgh_scale_trunc(const uint64_t* x, size_t n, int se, int64_t* out) {
  for (size_t i = 0; i < n; i++) out[i] = zg::scale_trunc<double>(x[i], se);
}
extern "C" int zgh_bfp_exact64(const uint64_t* raw, int emax, int special) {
  uint64_t b[64];
  for (int i = 0; i < 64; i++) b[i] = raw[i];
  return zg::bfp_exact<double, 64>(b, emax, special != 0);
}
extern "C" int zgh_bfp_exact32(const uint32_t* raw, int emax, int special) {
  uint32_t b[64];
  for (int i = 0; i < 64; i++) b[i] = raw[i];
  return zg::bfp_exact<float, 64>(b, emax, special != 0);
}

// shared-memory image layout (kernels.cuh / launch.h): every logical word
// of a buffer sized by image_words() lands inside it, for all sizes up to n
extern "C" int zgh_image_layout_ok(uint32_t n) {
  for (uint32_t logical = 1; logical <= n; logical++) {
    const uint32_t phys = (uint32_t)zg::image_words(logical);
    if (zg::img_cap(phys) < logical) return 0;
    if (zg::img_phys(zg::img_cap(phys) - 1) >= phys) return 0;
    if (zg::img_phys(logical - 1) >= phys) return 0;
  }
  return 1;
}

// block offsets by the length-only decoder (skip_block), as the GPU parse
// kernel recovers them for streams without an index: ends[b] = first bit
// after block b
template <typename S, int D>
uint64_t parse_t(const Geom& g, const zg::BlockParams& p, const uint64_t* words, uint64_t cap, uint64_t bit0,
                 uint64_t* ends) {
  zg::WordSource in;
  in.base = words;
  in.cap = cap;
  in.seek(bit0);
  for (size_t b = 0; b < g.blocks; b++) {
    zg::skip_block<S, D>(in, p);
    ends[b] = in.tell();
  }
  return in.tell();
}

template <typename S>
uint64_t parse_s(const Geom& g, const zg::BlockParams& p, const uint64_t* w, uint64_t cap, uint64_t b0, uint64_t* e) {
  switch (g.dims) {
    case 1: return parse_t<S, 1>(g, p, w, cap, b0, e);
    case 2: return parse_t<S, 2>(g, p, w, cap, b0, e);
    case 3: return parse_t<S, 3>(g, p, w, cap, b0, e);
    default: return parse_t<S, 4>(g, p, w, cap, b0, e);
  }
}

extern "C" uint64_t zgh_parse(int type, int dims, const size_t* n, const unsigned* prm, const uint64_t* words,
                              uint64_t cap, uint64_t bit0, uint64_t* ends) {
  const ptrdiff_t s[4] = {0, 0, 0, 0};
  Geom g = geom(dims, n, s);
  zg::BlockParams p{prm[0], prm[1], prm[2], (int32_t)prm[3]};
  switch (type) {
    case 1: return parse_s<int32_t>(g, p, words, cap, bit0, ends);
    case 2: return parse_s<int64_t>(g, p, words, cap, bit0, ends);
    case 3: return parse_s<float>(g, p, words, cap, bit0, ends);
    default: return parse_s<double>(g, p, words, cap, bit0, ends);
  }
}
