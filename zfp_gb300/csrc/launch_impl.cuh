// launch_impl.cuh -- kernel launch bodies, instantiated per scalar type by
// kern_{i32,i64,f32,f64}.cu.
#pragma once

#include "kernels.cuh"
#include "launch.h"

namespace zg {

template <class K>
static void allow_smem(K kernel) {
  // once per kernel: let it use up to kMaxTileSmem of dynamic shared memory
  cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMaxTileSmem);
}

template <typename S, int D>
cudaError_t run_encode(const LaunchArgs& a, cudaStream_t st) {
  const size_t smem = a.gimg ? 0 : (size_t)a.img_words * 8;
  if (a.njobs > 1) {
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
  if (a.njobs > 1) {
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

template <typename S>
cudaError_t encode_dims(int dims, const LaunchArgs& a, cudaStream_t st) {
  switch (dims) {
    case 1: return run_encode<S, 1>(a, st);
    case 2: return run_encode<S, 2>(a, st);
    case 3: return run_encode<S, 3>(a, st);
    case 4: return run_encode<S, 4>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

template <typename S>
cudaError_t decode_dims(int dims, const LaunchArgs& a, cudaStream_t st) {
  switch (dims) {
    case 1: return run_decode<S, 1>(a, st);
    case 2: return run_decode<S, 2>(a, st);
    case 3: return run_decode<S, 3>(a, st);
    case 4: return run_decode<S, 4>(a, st);
    default: return cudaErrorInvalidValue;
  }
}

template <typename S>
cudaError_t parse_dims(int dims, const Job& job, cudaStream_t st) {
  switch (dims) {
    case 1: parse_kernel<S, 1><<<1, 32, 0, st>>>(job); break;
    case 2: parse_kernel<S, 2><<<1, 32, 0, st>>>(job); break;
    case 3: parse_kernel<S, 3><<<1, 32, 0, st>>>(job); break;
    case 4: parse_kernel<S, 4><<<1, 32, 0, st>>>(job); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace zg

#define ZG_DEFINE_LAUNCHERS(SUFFIX, S)                                                        \
  namespace zg {                                                                              \
  cudaError_t launch_encode_##SUFFIX(int d, const LaunchArgs& a, cudaStream_t st) {           \
    return encode_dims<S>(d, a, st);                                                          \
  }                                                                                           \
  cudaError_t launch_decode_##SUFFIX(int d, const LaunchArgs& a, cudaStream_t st) {           \
    return decode_dims<S>(d, a, st);                                                          \
  }                                                                                           \
  cudaError_t launch_parse_##SUFFIX(int d, const Job& j, cudaStream_t st) { return parse_dims<S>(d, j, st); } \
  }
