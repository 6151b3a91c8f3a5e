// noalloc.cu -- zfp_compress for callers that cannot allocate device memory.
//
// zfp_compress allocates: staging buffers for host data, the per-launch
// scratch of the encoder (tile states for the variable-rate look-back,
// boundary words shared by neighbouring tiles, the tile counter) and the
// block index it keeps for later decompression.  Some callers cannot let a
// library call cudaMalloc or cudaMallocAsync: programs whose device memory
// is entirely owned by another allocator (a framework's caching allocator
// that has reserved the pool), and latency-critical loops that must not
// trigger the implicit synchronisation or pool growth an allocation can
// cause.  zfp_gb300_compress_noalloc serves them: the caller passes device
// field and stream buffers, and the encoder's scratch lives in one
// file-scope device array of fixed size instead of being allocated.
//
// The array is shared by every call in the process on a given device and
// keeps what the last call left in it; each call clears the part it uses
// before launching.  Two calls whose GPU work overlaps in time (different
// CUDA streams, or different host threads) race on it and must be ordered
// by the caller.  Every GPU that loads the library holds the array until
// the process exits.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "../../include/zfp_gb300.h"
#include "gpu_internal.h"
#include "runtime.h"

namespace zg {

// up to this many tiles of kTile blocks per call (4,194,304 blocks)
constexpr uint32_t kNoAllocMaxTiles = 32768;
constexpr size_t kNoAllocBytes = 1u << 20;  // 1 MiB per device
static_assert(64 + ((size_t)kNoAllocMaxTiles + 1) * 28 <= kNoAllocBytes, "scratch layout does not fit");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

static std::mutex g_noalloc_mu;

// Set-up, per device: the device address of g_noalloc_scratch.  In host code
// the array's name is only a host-side handle, so the address is looked up
// with cudaGetSymbolAddress while that device is current.  It is kept with
// the driver context it was looked up in: after cudaDeviceReset the device's
// next context loads the module again, possibly elsewhere, and the lookup
// is repeated.
struct ScratchAddr {
  void* ctx = nullptr;
  void* addr = nullptr;
};
static ScratchAddr g_noalloc_addr[256];   // per device ordinal

static void* current_context() {
  using GetCtx = CUresult (*)(CUcontext*);
  static GetCtx get_ctx = [] {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      fn = nullptr;
    }
    return (GetCtx)fn;
  }();
  CUcontext c = nullptr;
  return get_ctx && get_ctx(&c) == CUDA_SUCCESS ? (void*)c : nullptr;
}

static void* noalloc_scratch(cudaError_t& err) {
  int dev = 0;
  err = cudaGetDevice(&dev);
  if (err != cudaSuccess || dev < 0 || dev >= 256) return nullptr;
  // the caller has already made runtime calls on this device (pointer
  // queries), so its primary context is current on this thread
  void* ctx = current_context();
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  ScratchAddr& s = g_noalloc_addr[dev];
  if (!s.addr || !ctx || s.ctx != ctx) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return nullptr;
    s.addr = p;
    s.ctx = ctx ? ctx : current_context();
  }
  return s.addr;
}

}  // namespace zg

extern "C" size_t zfp_gb300_compress_noalloc(zfp_stream* z, const zfp_field* f) {
  using namespace zg;
  ExecParams* ep = exec_params(z);
  if (!ep) return fail("zfp_gb300_compress_noalloc: the stream's execution policy is not zfp_exec_cuda");
  if (!z->stream) return fail("zfp_gb300_compress_noalloc: no bit stream");
  FieldInfo fi;
  if (const char* why = field_info(f, fi)) return fail(why);
  const StreamState ss = get_stream_state(z->stream);
  if (!ss.begin || !is_device_ptr(ss.begin) || !is_device_ptr(f->data))
    return fail("zfp_gb300_compress_noalloc: field and stream must be in device memory");
  const uint64_t ntiles = (fi.nblocks + kTile - 1) / kTile;
  if (ntiles > kNoAllocMaxTiles)
    return fail("zfp_gb300_compress_noalloc: field has more than 4194304 blocks (the scratch limit)");
  const bool fixed = is_fixed_rate(fi, z);
  const uint64_t bound = fixed ? (uint64_t)z->maxbits : block_bound(fi, z);
  const uint64_t bit0 = (uint64_t)(ss.ptr - ss.begin) * 64 + ss.bits;
  const uint64_t cap_words = (uint64_t)(ss.end - ss.begin);
  if (fixed && (bit0 + fi.nblocks * (uint64_t)z->maxbits + 63) / 64 > cap_words)
    return fail("zfp_gb300_compress_noalloc: stream buffer too small");

  cudaError_t e;
  char* scratch = (char*)noalloc_scratch(e);
  if (!scratch) return fail_cuda("zfp_gb300_compress_noalloc: cudaGetSymbolAddress", e);
  const cudaStream_t st = ep->stream;
  const size_t t = (size_t)ntiles + 1;
  const size_t used = 64 + t * 28;
  // the previous call's state must not leak into this one
  if ((e = cudaMemsetAsync(scratch, 0, used, st)) != cudaSuccess)
    return fail_cuda("zfp_gb300_compress_noalloc: clear scratch", e);

  Job job = base_job(fi, z, f->data);
  job.flags = (fixed ? kFixedRate : 0u) | vector_flags(fi, f->data);
  job.words = ss.begin;
  job.cap_words = cap_words;
  job.bit0 = bit0;
  job.head_word = ss.bits ? (ss.buffer & ((1ull << ss.bits) - 1)) : 0;
  job.result = (JobResult*)scratch;

  LaunchArgs a;
  std::memset(&a, 0, sizeof a);
  a.one = job;
  a.njobs = 1;
  a.sc.ticket = (unsigned int*)(scratch + 32);
  a.sc.tile_state = (unsigned long long*)(scratch + 64);
  a.sc.side = (unsigned long long*)(scratch + 64 + t * 8);
  a.sc.side_cnt = (unsigned int*)(scratch + 64 + t * 24);
  a.sc.wait_cycles = wait_cycles();
  a.total_tiles = (uint32_t)ntiles;
  a.use_ticket = fixed ? 0 : 1;
  // variable-rate tiles are staged in shared memory up to the kernel's
  // occupancy room, larger ones coded straight into the stream
  a.img_words = fixed ? 0u
                      : (uint32_t)std::min<uint64_t>(image_words((uint64_t)kTile * bound / 64 + 4),
                                                     stage_room_any(fi.type, fi.dims, a, true));
  a.grid = (int)ntiles;
  if ((e = launch_encode_any(fi.type, fi.dims, a, st)) != cudaSuccess)
    return fail_cuda("zfp_gb300_compress_noalloc: launch", e);

  JobResult res;
  if ((e = cudaMemcpyAsync(&res, scratch, sizeof res, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return fail_cuda("zfp_gb300_compress_noalloc: kernel", e);
  if (res.status)
    return fail(res.status & kStatusOverflow ? "zfp_gb300_compress_noalloc: stream buffer too small"
                                             : "zfp_gb300_compress_noalloc: GPU wait timed out");
  // a block index kept for an earlier stream at the same place no longer
  // describes it; the dropped index is freed by a later call, not this one
  registry_invalidate_parked(ss.begin, bit0, res.end_bit);
  set_stream_flushed(z->stream, res.end_bit);
  set_error("");
  return (size_t)((res.end_bit + 63) / 64) * 8;
}
