// launch_impl.cuh -- kernel launch bodies, instantiated per scalar type by
// kern_{i32,i64,f32,f64}.cu.
#pragma once

#include "kernels.cuh"
#include "launch.h"

namespace zg {

template <class K>
static void allow_smem(K kernel) {
  // once per kernel: let it use the whole shared memory of an SM
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmemLimit);
}

template <typename S, int D>
cudaError_t run_encode(const LaunchArgs& a, cudaStream_t st) {
  const size_t smem = (a.gimg ? 0 : (size_t)a.img_words * 8) + plane_smem_bytes<S, D>();
  if (a.jobs) {  // device job array: the multi-job kernel
    static const bool once = (allow_smem(encode_kernel<S, D, true>), true);
    (void)once;
    encode_kernel<S, D, true><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.sc, a.total_tiles,
                                                            a.use_ticket, a.gimg, a.img_words);
  } else {
    static const bool once = (allow_smem(encode_kernel<S, D, false>), true);
    (void)once;
    encode_kernel<S, D, false><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.sc, a.total_tiles,
                                                             a.use_ticket, a.gimg, a.img_words);
  }
  return cudaGetLastError();
}

template <typename S, int D>
cudaError_t run_decode(const LaunchArgs& a, cudaStream_t st) {
  const size_t smem = a.gimg ? 0 : (size_t)a.img_words * 8;
  if (a.jobs) {  // device job array: the multi-job kernel
    static const bool once = (allow_smem(decode_kernel<S, D, true>), true);
    (void)once;
    decode_kernel<S, D, true><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.total_tiles, a.gimg,
                                                            a.img_words);
  } else {
    static const bool once = (allow_smem(decode_kernel<S, D, false>), true);
    (void)once;
    decode_kernel<S, D, false><<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.total_tiles, a.gimg,
                                                             a.img_words);
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
