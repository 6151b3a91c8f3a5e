// gpu_internal.h -- helpers shared by the single-field path (gpu_codec.cu)
// and the batch path (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>

#include "../../include/zfp.h"
#include "job.h"
#include "launch.h"

namespace zg {

struct ExecParams {
  uint32_t magic;
  cudaStream_t stream;
  int async;
};
static const uint32_t kExecMagic = 0x7a673330u;  // identifies params owned by this library
ExecParams* exec_params(zfp_stream* z);

struct FieldInfo {
  int type = 0, dims = 0;
  size_t esize = 0;
  uint32_t n[4] = {1, 1, 1, 1}, nb[4] = {1, 1, 1, 1};
  int64_t s[4] = {0, 0, 0, 0};
  uint64_t nblocks = 0;
  ptrdiff_t lo = 0, hi = 0;  // lowest / highest element offset
};

const char* field_info(const zfp_field* f, FieldInfo& fi);
uint32_t header_max(int type, bool rev);
uint64_t block_bound(const FieldInfo& fi, const zfp_stream* z);
bool is_fixed_rate(const FieldInfo& fi, const zfp_stream* z);
bool vector_ok(const FieldInfo& fi, const void* data);
// kVecOk, plus kVec32 where 64-bit rows are 32-byte aligned
uint32_t vector_flags(const FieldInfo& fi, const void* data);
Job base_job(const FieldInfo& fi, const zfp_stream* z, void* field);
int persistent_grid();

bool is_device_ptr(const void* p);
// the look-back wait bound every launch uses (zfp_gb300_set_wait_limit; 0: default)
long long wait_cycles();
void init_pool_once();
size_t fail(const char* msg);
size_t fail_cuda(const char* where, cudaError_t e);

// stream-ordered device buffer
struct DevBuf {
  void* p = nullptr;
  cudaStream_t st = nullptr;
  cudaError_t alloc(size_t bytes, cudaStream_t s) {
    st = s;
    return cudaMallocAsync(&p, bytes ? bytes : 8, s);
  }
  void release() {
    if (p) cudaFreeAsync(p, st);
    p = nullptr;
  }
  ~DevBuf() { release(); }
};

// A per-block index (start bit of every block) in device memory, shared by
// the registry and by every launch that reads it.  The last holder to drop
// it frees it on a library-owned stream, after `written` (an event recorded
// behind writes that may still be in flight).  Holders keep their reference
// until the GPU work that reads the index has finished.
struct DevIndex {
  uint64_t* ptr = nullptr;
  cudaEvent_t written = nullptr;
  ~DevIndex();
};
using IndexRef = std::shared_ptr<DevIndex>;

// allocate an index for nblocks blocks (stream-ordered on st)
IndexRef make_index(size_t nblocks, cudaStream_t st, cudaError_t& err);

struct IndexEntry {
  const void* begin = nullptr;
  uint64_t bit0 = 0, end_bit = 0, nblocks = 0;
  int type = 0, dims = 0;
  uint32_t minbits = 0, maxbits = 0, maxprec = 0;
  int32_t minexp = 0;
  IndexRef index;
  uint64_t tick = 0;
};

IndexEntry make_entry(const void* begin, uint64_t bit0, uint64_t end_bit, const FieldInfo& fi, const Job& j,
                      IndexRef index);
void registry_invalidate(const void* begin, uint64_t bit0, uint64_t end);
// the same without freeing anything now: dropped indexes are kept until the
// next registry call that may free device memory
void registry_invalidate_parked(const void* begin, uint64_t bit0, uint64_t end);
void registry_insert(const IndexEntry& ne);
bool registry_find(const void* begin, uint64_t bit0, const FieldInfo& fi, const zfp_stream* z, IndexEntry& out);

cudaError_t launch_encode_any(int type, int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode_any(int type, int dims, const LaunchArgs& a, cudaStream_t st);
uint32_t stage_room_any(int type, int dims, const LaunchArgs& a, bool encode);
cudaError_t launch_parse_any(int type, int dims, const Job& j, cudaStream_t st);

}  // namespace zg
