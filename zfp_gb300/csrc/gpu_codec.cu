// gpu_codec.cu -- zfp_compress / zfp_decompress on the GPU.
//
// The reference's CUDA hook (src/cuda_zfp/cuZFP.cu:357-491) accepted only
// fixed-rate 1-3D contiguous fields; this path takes every mode, type,
// dimensionality, stride layout and stream offset the serial codec takes
// (src/zfp.c:1052-1180) and produces the same bits.  Per call:
//   1. classify field and stream buffers: device memory and page-locked
//      host memory mapped into the device (read and written in place by the
//      kernels, over the host link) are used as they are; other host data
//      is staged through device memory from the stream-ordered pool;
//   2. describe the field as one Job and launch the encode/decode kernel on
//      the zfp_stream's CUDA stream;
//   3. leave the bit stream as the serial path leaves it (flushed on
//      compress, aligned on decompress) and return the byte size.
// Variable-rate streams carry no block index (docs/source/execution.rst:289-
// 300); the encoder records one in device memory, kept in a small registry
// keyed by stream buffer and start bit, and the decoder verifies it.  For a
// stream with no entry (written elsewhere) the offsets are recovered on the
// GPU by a sequential parse.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <atomic>
#include <climits>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/zfp_gb300.h"
#include "job.h"
#include "launch.h"
#include "runtime.h"
#include "gpu_internal.h"

namespace zg {

// ---------------------------------------------------------------------------
// errors and per-stream GPU settings

static thread_local std::string g_last_error;

void set_error(const char* msg) { g_last_error = msg ? msg : ""; }

size_t fail(const char* msg) {
  set_error(msg);
  return 0;
}

size_t fail_cuda(const char* where, cudaError_t e) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  set_error(m.c_str());
  return 0;
}


bool ensure_exec_params(zfp_stream* z) {
  if (z->exec.policy == zfp_exec_cuda && z->exec.params) return true;
  if (z->exec.params) std::free(z->exec.params);
  ExecParams* p = (ExecParams*)std::malloc(sizeof(ExecParams));
  if (!p) return false;
  p->magic = kExecMagic;
  p->stream = nullptr;
  p->async = 0;
  z->exec.params = p;
  return true;
}

void release_exec_params(zfp_stream* z) {
  if (z->exec.params) std::free(z->exec.params);
  z->exec.params = nullptr;
}

ExecParams* exec_params(zfp_stream* z) {
  ExecParams* p = (ExecParams*)z->exec.params;
  return (p && p->magic == kExecMagic) ? p : nullptr;
}

// ---------------------------------------------------------------------------
// memory

bool is_device_ptr(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Page-locked host memory (cudaHostAlloc / cudaHostRegister) that the
// device addresses at the same virtual address: kernels may read and write
// it directly.  The whole range [p, p + bytes) must lie inside one such
// allocation (the driver's allocation range), so no kernel touches a page
// outside it; anything else is staged.
bool is_mapped_host(const void* p, size_t bytes) {
  if (!p || !bytes) return false;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (a.type != cudaMemoryTypeHost || a.devicePointer != p || a.hostPointer != p) return false;
  // the driver call is looked up at run time so the library loads without libcuda
  using GetAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
  static GetAttr get_attr = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      fn = nullptr;
    }
    return (GetAttr)fn;
  }();
  if (!get_attr) return false;
  CUdeviceptr start = 0;
  size_t size = 0;
  if (get_attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)p) != CUDA_SUCCESS ||
      get_attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)p) != CUDA_SUCCESS)
    return false;
  const uintptr_t b = (uintptr_t)p;
  return start && b >= (uintptr_t)start && bytes <= size && b - (uintptr_t)start <= size - bytes;
}

static thread_local size_t g_staged = 0;   // bytes copied host<->device by this thread's last call

void init_pool_once() {
  static std::once_flag flag;
  std::call_once(flag, [] {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = ~0ull;  // keep freed blocks for reuse instead of returning them
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  });
}


// ---------------------------------------------------------------------------
// field description


const char* field_info(const zfp_field* f, FieldInfo& fi) {
  switch (f->type) {
    case zfp_type_int32: case zfp_type_float: fi.esize = 4; break;
    case zfp_type_int64: case zfp_type_double: fi.esize = 8; break;
    default: return "unsupported scalar type";
  }
  fi.type = f->type;
  fi.dims = f->nx ? f->ny ? f->nz ? f->nw ? 4 : 3 : 2 : 1 : 0;
  if (!fi.dims) return "field has no dimensions";
  const size_t n[4] = {f->nx, f->ny, f->nz, f->nw};
  const ptrdiff_t sd[4] = {f->sx ? f->sx : 1, f->sy ? f->sy : (ptrdiff_t)f->nx,
                           f->sz ? f->sz : (ptrdiff_t)(f->nx * f->ny),
                           f->sw ? f->sw : (ptrdiff_t)(f->nx * f->ny * f->nz)};
  fi.nblocks = 1;
  for (int a = 0; a < 4; a++) {
    if (a < fi.dims) {
      if (n[a] >= (1ull << 32) - 4) return "field extent too large";
      fi.n[a] = (uint32_t)n[a];
      fi.nb[a] = (fi.n[a] + 3) / 4;
      fi.s[a] = sd[a];
      const ptrdiff_t d = sd[a] * (ptrdiff_t)(n[a] - 1);
      fi.lo += d < 0 ? d : 0;
      fi.hi += d > 0 ? d : 0;
    }
    fi.nblocks *= fi.nb[a];
  }
  if (!f->data) return "field has no data pointer";
  return nullptr;
}

// header bits a block can carry before its bit planes
uint32_t header_max(int type, bool rev) {
  switch (type) {
    case zfp_type_int32: return rev ? 5 : 0;
    case zfp_type_int64: return rev ? 6 : 0;
    case zfp_type_float: return rev ? 1 + 1 + 8 + 5 : 1 + 8;
    default: return rev ? 1 + 1 + 11 + 6 : 1 + 11;
  }
}

// upper bound on the bits of one block (the block term of
// zfp_stream_maximum_size, src/zfp.c:712-742, widened where a maxbits
// below the header size makes the reference's budget wrap around)
uint64_t block_bound(const FieldInfo& fi, const zfp_stream* z) {
  const bool rev = z->minexp < ZFP_MIN_EXP;
  const uint64_t values = 1ull << (2 * fi.dims);
  const uint64_t prec = 8 * fi.esize;
  const uint64_t hm = header_max(fi.type, rev);
  const uint64_t coder = values - 1 + values * std::min<uint64_t>(z->maxprec, prec);
  uint64_t b = hm + coder;
  if (z->maxbits >= hm) b = std::min<uint64_t>(b, z->maxbits);
  return std::max<uint64_t>(b, z->minbits);
}

bool is_fixed_rate(const FieldInfo& fi, const zfp_stream* z) {
  const bool rev = z->minexp < ZFP_MIN_EXP;
  return !rev && z->minbits == z->maxbits && z->maxbits >= header_max(fi.type, false) && z->maxbits > 0;
}

bool vector_ok(const FieldInfo& fi, const void* data) {
  if (fi.s[0] != 1 || ((uintptr_t)data & 15)) return false;
  for (int a = 1; a < fi.dims; a++)
    if ((fi.s[a] * (int64_t)fi.esize) % 16) return false;
  return true;
}

uint32_t vector_flags(const FieldInfo& fi, const void* data) {
  if (!vector_ok(fi, data)) return 0;
  bool wide = fi.esize == 8 && !((uintptr_t)data & 31);
  for (int a = 1; a < fi.dims; a++)
    if ((fi.s[a] * (int64_t)fi.esize) % 32) wide = false;
  return kVecOk | (wide ? kVec32 : 0u);
}

// ---------------------------------------------------------------------------
// index registry for variable-rate streams


// the registry lives for the whole process (never destroyed, so no CUDA
// call runs from a static destructor at exit)
static std::mutex g_reg_mu;
static std::vector<IndexEntry>& g_reg = *new std::vector<IndexEntry>();
static uint64_t g_tick = 0;
static const size_t kRegistryBytes = 4ull << 30;

static cudaStream_t free_stream() {
  static cudaStream_t st = [] {
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      cudaGetLastError();
      s = nullptr;
    }
    return s;
  }();
  return st;
}

DevIndex::~DevIndex() {
  if (!ptr) return;
  cudaStream_t fs = free_stream();
  if (written) {
    cudaStreamWaitEvent(fs, written, 0);
    cudaEventDestroy(written);
  }
  if (cudaFreeAsync(ptr, fs) != cudaSuccess) cudaGetLastError();
}

IndexRef make_index(size_t nblocks, cudaStream_t st, cudaError_t& err) {
  auto idx = std::make_shared<DevIndex>();
  err = cudaMallocAsync((void**)&idx->ptr, nblocks ? nblocks * 8 : 8, st);
  if (err != cudaSuccess) {
    idx->ptr = nullptr;
    return nullptr;
  }
  return idx;
}

IndexEntry make_entry(const void* begin, uint64_t bit0, uint64_t end_bit, const FieldInfo& fi, const Job& j,
                      IndexRef index) {
  IndexEntry e;
  e.begin = begin;
  e.bit0 = bit0;
  e.end_bit = end_bit;
  e.nblocks = fi.nblocks;
  e.type = fi.type;
  e.dims = fi.dims;
  e.minbits = j.minbits;
  e.maxbits = j.maxbits;
  e.maxprec = j.maxprec;
  e.minexp = j.minexp;
  e.index = std::move(index);
  return e;
}

// Indexes dropped by calls that must not free device memory (the no-alloc
// entry point): held here until the next call that may free them.
static std::vector<IndexRef>& g_parked = *new std::vector<IndexRef>();

// drop entries of the same buffer whose stream range overlaps [bit0, end);
// their memory is released when the last holder lets go -- or, with `park`,
// not before the next registry call without it
static void drop_overlapping(const void* begin, uint64_t bit0, uint64_t end, bool park) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  if (!park) g_parked.clear();
  for (size_t i = 0; i < g_reg.size();) {
    IndexEntry& e = g_reg[i];
    if (e.begin == begin && e.bit0 < end && bit0 < e.end_bit) {
      if (park) g_parked.push_back(std::move(e.index));
      g_reg.erase(g_reg.begin() + i);
    } else {
      i++;
    }
  }
}

void registry_invalidate(const void* begin, uint64_t bit0, uint64_t end) { drop_overlapping(begin, bit0, end, false); }

void registry_invalidate_parked(const void* begin, uint64_t bit0, uint64_t end) {
  drop_overlapping(begin, bit0, end, true);
}

void registry_insert(const IndexEntry& ne) {
  registry_invalidate(ne.begin, ne.bit0, ne.end_bit);
  std::lock_guard<std::mutex> lk(g_reg_mu);
  size_t bytes = ne.nblocks * 8;
  for (auto& e : g_reg) bytes += e.nblocks * 8;
  while (bytes > kRegistryBytes && !g_reg.empty()) {
    auto it = std::min_element(g_reg.begin(), g_reg.end(),
                               [](const IndexEntry& a, const IndexEntry& b) { return a.tick < b.tick; });
    bytes -= it->nblocks * 8;
    g_reg.erase(it);
  }
  g_reg.push_back(ne);
  g_reg.back().tick = ++g_tick;
}

bool registry_find(const void* begin, uint64_t bit0, const FieldInfo& fi, const zfp_stream* z, IndexEntry& out) {
  std::lock_guard<std::mutex> lk(g_reg_mu);
  for (auto& e : g_reg)
    if (e.begin == begin && e.bit0 == bit0 && e.nblocks == fi.nblocks && e.type == fi.type &&
        e.dims == fi.dims && e.minbits == z->minbits && e.maxbits == z->maxbits && e.maxprec == z->maxprec &&
        e.minexp == z->minexp) {
      e.tick = ++g_tick;
      out = e;
      return true;
    }
  return false;
}

// ---------------------------------------------------------------------------
// launch helpers

Job base_job(const FieldInfo& fi, const zfp_stream* z, void* field) {
  Job j;
  std::memset(&j, 0, sizeof j);
  j.field = field;
  for (int a = 0; a < 4; a++) {
    j.s[a] = fi.s[a];
    j.n[a] = fi.n[a];
    j.nb[a] = fi.nb[a];
  }
  j.nblocks = fi.nblocks;
  j.minbits = z->minbits;
  j.maxbits = z->maxbits;
  j.maxprec = z->maxprec;
  j.minexp = z->minexp;
  j.tile0 = 0;
  j.ntiles = (uint32_t)((fi.nblocks + kTile - 1) / kTile);
  return j;
}

int persistent_grid() {
  static int sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 148;
  }();
  return sms * 4;
}

// Launch geometry; a.one / a.jobs must be set (they select the kernel).
// `bound_bits` bounds one block's code, so a tile's image never exceeds
// `words`.  Up to the kernel's occupancy room the tile's image (encode) or
// stream words (decode) are staged in shared memory; larger tiles are coded
// straight into the stream, or read from it directly.  A fixed-rate encode
// stages nothing: its tiles' places are known without the look-back.  An
// encode into host memory (written in place over the host link, which only
// whole lines cross at speed) stages whole tiles wherever shared memory
// holds them, at the cost of CTAs per SM: such a call is bound by the link.
static void plan_launch(LaunchArgs& a, int type, int dims, bool encode, uint64_t bound_bits, uint32_t total_tiles) {
  const uint64_t words = image_words((uint64_t)kTile * bound_bits / 64 + 4);
  const bool fixed_encode = encode && !a.jobs && (a.one.flags & kFixedRate);
  const bool host_encode = encode && !a.jobs && (a.one.flags & kStreamHost);
  const size_t esize = type == zfp_type_float || type == zfp_type_int32 ? 4 : 8;
  const size_t planes = plane_bytes(esize, dims);   // at most what the kernel keeps
  const uint32_t room = host_encode ? (uint32_t)((kMaxTileSmem > planes ? kMaxTileSmem - planes : 0) / 8)
                        : fixed_encode ? 0
                                       : stage_room_any(type, dims, a, encode);
  a.total_tiles = total_tiles;
  a.grid = (int)total_tiles;
  a.img_words = (uint32_t)std::min<uint64_t>(words, room);
}

template <class F>
static cudaError_t by_type(int type, int dims, F&& f) {
  auto d = [&](auto tag) -> cudaError_t {
    using S = decltype(tag);
    switch (dims) {
      case 1: return f(S{}, std::integral_constant<int, 1>{});
      case 2: return f(S{}, std::integral_constant<int, 2>{});
      case 3: return f(S{}, std::integral_constant<int, 3>{});
      case 4: return f(S{}, std::integral_constant<int, 4>{});
      default: return cudaErrorInvalidValue;
    }
  };
  switch (type) {
    case zfp_type_int32: return d(int32_t{});
    case zfp_type_int64: return d(int64_t{});
    case zfp_type_float: return d(float{});
    default: return d(double{});
  }
}

cudaError_t launch_encode_any(int type, int dims, const LaunchArgs& a, cudaStream_t st) {
  return by_type(type, dims, [&](auto s, auto d) { return run_encode<decltype(s), decltype(d)::value>(a, st); });
}

cudaError_t launch_decode_any(int type, int dims, const LaunchArgs& a, cudaStream_t st) {
  return by_type(type, dims, [&](auto s, auto d) { return run_decode<decltype(s), decltype(d)::value>(a, st); });
}

uint32_t stage_room_any(int type, int dims, const LaunchArgs& a, bool encode) {
  uint32_t r = 0;
  by_type(type, dims, [&](auto s, auto d) {
    r = stage_room<decltype(s), decltype(d)::value>(a, encode);
    return cudaSuccess;
  });
  return r;
}

cudaError_t launch_parse_any(int type, int dims, const Job& j, cudaStream_t st) {
  return by_type(type, dims, [&](auto s, auto d) { return run_parse<decltype(s), decltype(d)::value>(j, st); });
}

// bound on the encoder's look-back waits (0: the kernels' default), and the
// failure-detection test hook: the next variable-rate zfp_compress skips its
// first tile
static std::atomic<long long> g_wait_cycles{0};
static std::atomic<int> g_skip_first_tile{0};

long long wait_cycles() { return g_wait_cycles.load(std::memory_order_relaxed); }

// scratch for one launch: result slot + look-back / boundary state, zeroed
struct LaunchMem {
  DevBuf buf;
  JobResult* result = nullptr;
  LaunchScratch sc{};
  cudaError_t make(uint32_t total_tiles, cudaStream_t st) {
    const size_t t = (size_t)total_tiles + 1;
    const size_t bytes = 64 + t * 8 + t * 16 + t * 4 + 16;
    cudaError_t e = buf.alloc(bytes, st);
    if (e != cudaSuccess) return e;
    char* p = (char*)buf.p;
    result = (JobResult*)p;
    sc.ticket = (unsigned int*)(p + 32);
    sc.tile_state = (unsigned long long*)(p + 64);
    sc.side = (unsigned long long*)(p + 64 + t * 8);
    sc.side_cnt = (unsigned int*)(p + 64 + t * 24);
    sc.wait_cycles = wait_cycles();
    return cudaMemsetAsync(p, 0, bytes, st);
  }
};

// ---------------------------------------------------------------------------
// compress

size_t gpu_compress(zfp_stream* z, const zfp_field* f, bool exact_end, uint64_t* bits_out) {
  ExecParams* ep = exec_params(z);
  if (!ep) return fail("zfp_compress: stream has no GPU execution parameters");
  if (!z->stream) return fail("zfp_compress: no bit stream");
  FieldInfo fi;
  if (const char* why = field_info(f, fi)) return fail(why);
  init_pool_once();
  const cudaStream_t st = ep->stream;
  const StreamState ss = get_stream_state(z->stream);
  if (!ss.begin) return fail("zfp_compress: bit stream has no buffer");
  const uint64_t bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 + ss.bits;
  const uint64_t cap_words = (uint64_t)(ss.end - ss.begin);
  const bool fixed = is_fixed_rate(fi, z);
  const uint64_t bound = block_bound(fi, z);
  const uint64_t max_end = bit0 + fi.nblocks * (fixed ? (uint64_t)z->maxbits : bound);
  if (fixed && (max_end + 63) / 64 > cap_words) return fail("zfp_compress: stream buffer too small");

  const size_t span = (size_t)(fi.hi - fi.lo + 1) * fi.esize;
  const char* fbegin = (const char*)f->data + fi.lo * (ptrdiff_t)fi.esize;
  const bool field_dev = is_device_ptr(f->data);
  const bool field_map = !field_dev && is_mapped_host(fbegin, span);
  const bool stream_dev = is_device_ptr(ss.begin);
  const bool stream_map = !stream_dev && is_mapped_host(ss.begin, cap_words * 8);
  cudaError_t e;
  g_staged = 0;

  // field
  DevBuf fstage;
  void* dfield = f->data;
  if (!field_dev && !field_map) {
    if ((e = fstage.alloc(span, st)) != cudaSuccess) return fail_cuda("zfp_compress: staging alloc", e);
    if ((e = cudaMemcpyAsync(fstage.p, fbegin, span, cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return fail_cuda("zfp_compress: field upload", e);
    g_staged += span;
    dfield = (char*)fstage.p - fi.lo * (ptrdiff_t)fi.esize;
  }

  // stream words
  DevBuf sstage;
  uint64_t* dwords = ss.begin;
  uint64_t dcap = cap_words;
  const uint64_t w_first = bit0 / 64;
  if (!stream_dev && !stream_map) {
    const uint64_t w_end = std::min<uint64_t>(cap_words, (max_end + 63) / 64);
    const uint64_t nw = w_end > w_first ? w_end - w_first : 0;
    if ((e = sstage.alloc(nw * 8, st)) != cudaSuccess) return fail_cuda("zfp_compress: staging alloc", e);
    dwords = (uint64_t*)sstage.p - w_first;
    dcap = w_first + nw;
  }

  Job job = base_job(fi, z, dfield);
  job.flags = (fixed ? kFixedRate : 0u) | (stream_map ? kStreamHost : 0u) | vector_flags(fi, dfield);
  job.words = dwords;
  job.cap_words = dcap;
  job.bit0 = bit0;
  job.head_word = ss.bits ? (ss.buffer & ((1ull << ss.bits) - 1)) : 0;

  IndexRef index;
  if (!fixed) {
    index = make_index(fi.nblocks, st, e);
    if (!index) return fail_cuda("zfp_compress: index alloc", e);
    job.offsets = index->ptr;
    job.flags |= kWriteIndex;
  }

  LaunchMem lm;
  if ((e = lm.make(job.ntiles, st)) != cudaSuccess) return fail_cuda("zfp_compress: scratch", e);
  job.result = lm.result;
  // test hook: hand tiles out from the second one, so that the second
  // tile's look-back waits for a tile that never runs
  if (!fixed && g_skip_first_tile.exchange(0) && (e = cudaMemsetAsync(lm.sc.ticket, 1, 1, st)) != cudaSuccess)
    return fail_cuda("zfp_compress: scratch", e);

  LaunchArgs a;
  std::memset(&a, 0, sizeof a);
  a.one = job;
  a.njobs = 1;
  a.sc = lm.sc;
  a.use_ticket = fixed ? 0 : 1;
  plan_launch(a, fi.type, fi.dims, true, fixed ? z->maxbits : bound, job.ntiles);
  if ((e = launch_encode_any(fi.type, fi.dims, a, st)) != cudaSuccess) return fail_cuda("zfp_compress: launch", e);

  if (fixed && field_dev && stream_dev && ep->async && !exact_end) {
    const uint64_t end = bit0 + fi.nblocks * (uint64_t)z->maxbits;
    registry_invalidate(ss.begin, bit0, end);
    set_stream_flushed(z->stream, end);
    return (size_t)((end + 63) / 64) * 8;
  }

  JobResult res;
  if ((e = cudaMemcpyAsync(&res, lm.result, sizeof res, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail_cuda("zfp_compress: kernel", e);
  if (res.status) {
    return fail(res.status & kStatusOverflow ? "zfp_compress: stream buffer too small"
                                             : "zfp_compress: GPU wait timed out");
  }
  const uint64_t end = res.end_bit;
  if (!stream_dev && !stream_map) {
    const uint64_t w_end = (end + 63) / 64;
    if ((e = cudaMemcpyAsync(ss.begin + w_first, dwords + w_first, (w_end - w_first) * 8, cudaMemcpyDeviceToHost,
                             st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return fail_cuda("zfp_compress: stream download", e);
    g_staged += (w_end - w_first) * 8;
  }
  if (index) {
    registry_insert(make_entry(ss.begin, bit0, end, fi, job, index));   // written: the stream was synchronised
  } else {
    registry_invalidate(ss.begin, bit0, end);
  }
  if (exact_end) {
    if (!set_stream_written(z->stream, end, stream_dev)) return fail("zfp_compress: reading the stream's last word");
  } else {
    set_stream_flushed(z->stream, end);
  }
  if (bits_out) *bits_out = end - bit0;
  set_error("");
  return (size_t)((end + 63) / 64) * 8;
}

// ---------------------------------------------------------------------------
// decompress

size_t gpu_decompress(zfp_stream* z, zfp_field* f, bool exact_end, uint64_t* bits_out) {
  ExecParams* ep = exec_params(z);
  if (!ep) return fail("zfp_decompress: stream has no GPU execution parameters");
  if (!z->stream) return fail("zfp_decompress: no bit stream");
  FieldInfo fi;
  if (const char* why = field_info(f, fi)) return fail(why);
  init_pool_once();
  const cudaStream_t st = ep->stream;
  const StreamState ss = get_stream_state(z->stream);
  if (!ss.begin) return fail("zfp_decompress: bit stream has no buffer");
  const uint64_t bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 - ss.bits;
  const uint64_t cap_words = (uint64_t)(ss.end - ss.begin);
  const bool fixed = is_fixed_rate(fi, z);
  const uint64_t bound = block_bound(fi, z);
  const size_t span = (size_t)(fi.hi - fi.lo + 1) * fi.esize;
  char* fbegin = (char*)f->data + fi.lo * (ptrdiff_t)fi.esize;
  const bool field_dev = is_device_ptr(f->data);
  const bool field_map = !field_dev && is_mapped_host(fbegin, span);
  const bool stream_dev = is_device_ptr(ss.begin);
  const bool stream_map = !stream_dev && is_mapped_host(ss.begin, cap_words * 8);
  cudaError_t e;
  g_staged = 0;

  uint64_t end = 0;
  IndexEntry ent;
  bool have_index = false;
  if (fixed) {
    end = bit0 + fi.nblocks * (uint64_t)z->maxbits;
    if ((end + 63) / 64 > cap_words) return fail("zfp_decompress: stream shorter than the field");
  } else {
    have_index = registry_find(ss.begin, bit0, fi, z, ent);
    if (have_index) end = ent.end_bit;
  }

  // stream words.  Page-locked host words are read in place, unless the
  // tiles (on average; their sizes are known from the rate or the index)
  // do not fit the decoder's shared memory: threads would then read their
  // blocks word by word across the host link, far slower than one upload.
  bool stage_stream = !stream_dev && !stream_map;
  uint32_t want_words = 0;   // a typical tile's staged words
  if ((fixed || have_index) && fi.nblocks) {
    const uint64_t ntiles = (fi.nblocks + kTile - 1) / kTile;
    const uint64_t tile_bits = fixed ? (uint64_t)kTile * z->maxbits : (end - bit0) / ntiles;
    want_words = (uint32_t)std::min<uint64_t>(image_words(tile_bits / 64 + 4), 1u << 30);
  }
  if (stream_map && want_words) {
    LaunchArgs probe;
    std::memset(&probe, 0, sizeof probe);
    probe.one = base_job(fi, z, f->data);
    probe.want_words = want_words;
    stage_stream = want_words > stage_room_any(fi.type, fi.dims, probe, false);
  }
  DevBuf sstage;
  uint64_t* dwords = ss.begin;
  uint64_t dcap = cap_words;
  const uint64_t w_first = bit0 / 64;
  if (stage_stream) {
    const uint64_t w_end = (fixed || have_index) ? std::min<uint64_t>(cap_words, (end + 63) / 64) : cap_words;
    const uint64_t nw = w_end > w_first ? w_end - w_first : 0;
    if ((e = sstage.alloc(nw * 8, st)) != cudaSuccess) return fail_cuda("zfp_decompress: staging alloc", e);
    if (nw && (e = cudaMemcpyAsync(sstage.p, ss.begin + w_first, nw * 8, cudaMemcpyHostToDevice, st)) != cudaSuccess)
      return fail_cuda("zfp_decompress: stream upload", e);
    g_staged += nw * 8;
    dwords = (uint64_t*)sstage.p - w_first;
    dcap = w_first + nw;
  }

  // field
  DevBuf fstage;
  void* dfield = f->data;
  if (!field_dev && !field_map) {
    if ((e = fstage.alloc(span, st)) != cudaSuccess) return fail_cuda("zfp_decompress: staging alloc", e);
    const uint64_t count = (uint64_t)fi.n[0] * fi.n[1] * fi.n[2] * fi.n[3];
    if (count * fi.esize != span) {  // strided with gaps: keep what lies between the values
      if ((e = cudaMemcpyAsync(fstage.p, fbegin, span, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return fail_cuda("zfp_decompress: field upload", e);
      g_staged += span;
    }
    dfield = (char*)fstage.p - fi.lo * (ptrdiff_t)fi.esize;
  }

  Job job = base_job(fi, z, dfield);
  job.flags = (fixed ? kFixedRate : 0u) | vector_flags(fi, dfield);
  job.words = dwords;
  job.cap_words = dcap;
  job.bit0 = bit0;

  LaunchMem lm;
  if ((e = lm.make(job.ntiles, st)) != cudaSuccess) return fail_cuda("zfp_decompress: scratch", e);
  job.result = lm.result;

  IndexRef parsed;
  auto parse = [&]() -> cudaError_t {
    cudaError_t pe;
    if (!parsed && !(parsed = make_index(fi.nblocks, st, pe))) return pe;
    Job pj = job;
    pj.offsets = parsed->ptr;
    if ((pe = launch_parse_any(fi.type, fi.dims, pj, st)) != cudaSuccess) return pe;
    JobResult r;
    if ((pe = cudaMemcpyAsync(&r, lm.result, sizeof r, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return pe;
    if ((pe = cudaStreamSynchronize(st)) != cudaSuccess) return pe;
    end = r.end_bit;
    job.offsets = parsed->ptr;
    job.end_bit = end;
    job.flags &= ~kVerify;
    return cudaSuccess;
  };

  if (!fixed) {
    if (have_index) {
      job.offsets = ent.index->ptr;
      job.end_bit = ent.end_bit;
      job.flags |= kVerify;
    } else if ((e = parse()) != cudaSuccess) {
      return fail_cuda("zfp_decompress: parse", e);
    }
  }

  LaunchArgs a;
  std::memset(&a, 0, sizeof a);
  a.njobs = 1;
  a.sc = lm.sc;
  a.one = job;
  a.want_words = want_words;
  plan_launch(a, fi.type, fi.dims, false, fixed ? z->maxbits : bound, job.ntiles);
  a.one = job;
  if ((e = launch_decode_any(fi.type, fi.dims, a, st)) != cudaSuccess) return fail_cuda("zfp_decompress: launch", e);

  const bool async_ok = fixed && field_dev && stream_dev && ep->async && !exact_end;
  if (!async_ok) {
    JobResult res;
    if ((e = cudaMemcpyAsync(&res, lm.result, sizeof res, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return fail_cuda("zfp_decompress: kernel", e);
    if (res.status & kStatusIndex) {
      // the recorded index does not describe this stream: recover and decode again
      if ((e = cudaMemsetAsync(lm.result, 0, sizeof(JobResult), st)) != cudaSuccess || (e = parse()) != cudaSuccess)
        return fail_cuda("zfp_decompress: parse", e);
      a.one = job;
      if ((e = launch_decode_any(fi.type, fi.dims, a, st)) != cudaSuccess ||
          (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail_cuda("zfp_decompress: kernel", e);
    }
  }
  if (!field_dev && !field_map) {
    if ((e = cudaMemcpyAsync(fbegin, fstage.p, span, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return fail_cuda("zfp_decompress: field download", e);
    g_staged += span;
  }
  if (parsed) registry_insert(make_entry(ss.begin, bit0, end, fi, job, parsed));
  if (exact_end) {
    if (!set_stream_read_at(z->stream, end, stream_dev)) return fail("zfp_decompress: reading the stream's last word");
  } else {
    set_stream_flushed(z->stream, end);
  }
  if (bits_out) *bits_out = end - bit0;
  set_error("");
  return (size_t)((end + 63) / 64) * 8;
}

}  // namespace zg

// ---------------------------------------------------------------------------
// extension API (include/zfp_gb300.h)

extern "C" {

zfp_bool zfp_gb300_stream_set_cuda_stream(zfp_stream* z, void* cuda_stream) {
  if (z->exec.policy != zfp_exec_cuda && !zfp_stream_set_execution(z, zfp_exec_cuda)) return zfp_false;
  zg::ExecParams* p = zg::exec_params(z);
  if (!p) return zfp_false;
  p->stream = (cudaStream_t)cuda_stream;
  return zfp_true;
}

zfp_bool zfp_gb300_stream_set_async(zfp_stream* z, int async) {
  if (z->exec.policy != zfp_exec_cuda && !zfp_stream_set_execution(z, zfp_exec_cuda)) return zfp_false;
  zg::ExecParams* p = zg::exec_params(z);
  if (!p) return zfp_false;
  p->async = async;
  return zfp_true;
}

zfp_bool zfp_gb300_stream_synchronize(zfp_stream* z) {
  zg::ExecParams* p = zg::exec_params(z);
  cudaError_t e = cudaStreamSynchronize(p ? p->stream : nullptr);
  if (e != cudaSuccess) {
    zg::fail_cuda("zfp_gb300_stream_synchronize", e);
    return zfp_false;
  }
  return zfp_true;
}

const char* zfp_gb300_last_error(void) { return zg::g_last_error.c_str(); }

size_t zfp_gb300_last_staged_bytes(void) { return zg::g_staged; }

}  // extern "C"

extern "C" unsigned long long zfp_gb300_set_wait_limit(unsigned long long cycles) {
  const long long v = cycles > (unsigned long long)LLONG_MAX ? LLONG_MAX : (long long)cycles;
  return (unsigned long long)zg::g_wait_cycles.exchange(v);
}

extern "C" void zfp_gb300_test_skip_first_tile(int enable) { zg::g_skip_first_tile.store(enable ? 1 : 0); }
