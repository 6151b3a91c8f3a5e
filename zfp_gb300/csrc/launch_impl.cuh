// launch_impl.cuh -- kernel launch bodies, instantiated per scalar type by
// kern_{i32,i64,f32,f64}.cu.
#pragma once

#include <mutex>

#include "kernels.cuh"
#include "launch.h"

namespace zg {

template <class K>
static void allow_smem(K kernel) {
  // once per kernel: allow dynamic shared memory up to the device's opt-in
  // limit minus what the kernel declares statically
  int dev = 0, optin = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return;
  }
  cudaFuncAttributes fa;
  if (cudaFuncGetAttributes(&fa, kernel) == cudaSuccess) optin -= (int)fa.sharedSizeBytes;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin) != cudaSuccess)
    cudaGetLastError();  // keep the launch's own status clean
}

// set the shared-memory attribute once per kernel (the flag is per kernel
// because the kernel itself is the template argument)
template <auto Kernel>
static void prepare_kernel() {
  static std::once_flag flag;
  std::call_once(flag, [] { allow_smem(Kernel); });
}

// kernel variant: device job array -> multi-job kernel carrying both mode
// paths; a single job -> the variant of its mode only
template <typename S, int D>
cudaError_t run_encode(const LaunchArgs& a, cudaStream_t st) {
  const size_t smem = (a.gimg ? 0 : (size_t)a.img_words * 8) + plane_smem_bytes<S, D>();
  if (a.jobs) {
    prepare_kernel<encode_kernel<S, D, true, kAnyMode>>();
    encode_kernel<S, D, true, kAnyMode><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.sc, a.total_tiles, a.use_ticket, a.gimg, a.img_words);
  } else if (a.one.minexp < kMinExp) {
    prepare_kernel<encode_kernel<S, D, false, kRevOnly>>();
    encode_kernel<S, D, false, kRevOnly><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.sc, a.total_tiles, a.use_ticket, a.gimg, a.img_words);
  } else {
    prepare_kernel<encode_kernel<S, D, false, kLossyOnly>>();
    encode_kernel<S, D, false, kLossyOnly><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.sc, a.total_tiles, a.use_ticket, a.gimg, a.img_words);
  }
  return cudaGetLastError();
}

template <typename S, int D>
cudaError_t run_decode(const LaunchArgs& a, cudaStream_t st) {
  const size_t smem = (a.gimg ? 0 : (size_t)a.img_words * 8) + plane_smem_bytes<S, D>();
  if (a.jobs) {
    prepare_kernel<decode_kernel<S, D, true, kAnyMode>>();
    decode_kernel<S, D, true, kAnyMode><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.total_tiles, a.gimg, a.img_words);
  } else if (a.one.minexp < kMinExp) {
    prepare_kernel<decode_kernel<S, D, false, kRevOnly>>();
    decode_kernel<S, D, false, kRevOnly><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.total_tiles, a.gimg, a.img_words);
  } else {
    prepare_kernel<decode_kernel<S, D, false, kLossyOnly>>();
    decode_kernel<S, D, false, kLossyOnly><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.total_tiles, a.gimg, a.img_words);
  }
  return cudaGetLastError();
}

template <typename S, int D>
cudaError_t run_parse(const Job& job, cudaStream_t st) {
  parse_kernel<S, D><<<1, 32, 0, st>>>(job);
  return cudaGetLastError();
}

}  // namespace zg

#define ZG_INSTANTIATE(S, D)                                                   \
  namespace zg {                                                               \
  template cudaError_t run_encode<S, D>(const LaunchArgs&, cudaStream_t);      \
  template cudaError_t run_decode<S, D>(const LaunchArgs&, cudaStream_t);      \
  template cudaError_t run_parse<S, D>(const Job&, cudaStream_t);              \
  }
