// gpu_internal.h -- helpers shared by the single-field path (gpu_codec.cu)
// and the batch path (batch.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

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
Job base_job(const FieldInfo& fi, const zfp_stream* z, void* field);
int persistent_grid();

bool is_device_ptr(const void* p);
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

struct IndexEntry {
  const void* begin;
  uint64_t bit0, end_bit, nblocks;
  int type, dims;
  uint32_t minbits, maxbits, maxprec;
  int32_t minexp;
  uint64_t* offsets;       // device, nblocks words
  cudaStream_t stream;     // last stream that used it (frees are ordered after it)
  uint64_t tick;
};

void registry_invalidate(const void* begin, uint64_t bit0, uint64_t end);
void registry_insert(const IndexEntry& ne);
bool registry_find(const void* begin, uint64_t bit0, const FieldInfo& fi, const zfp_stream* z, cudaStream_t st,
                   IndexEntry& out);

cudaError_t launch_encode_any(int type, int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_decode_any(int type, int dims, const LaunchArgs& a, cudaStream_t st);
cudaError_t launch_parse_any(int type, int dims, const Job& j, cudaStream_t st);

}  // namespace zg
