// launch_impl.cuh -- kernel launch bodies, instantiated per scalar type by
// kern_{i32,i64,f32,f64}.cu.
#pragma once

#include <algorithm>
#include <mutex>
#include <type_traits>

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

// Dynamic shared memory one CTA of Kernel may use for its tile image beside
// `planes` bytes of bit planes: the SM's shared memory split among as many
// CTAs as its registers allow, but no more CTAs than leave each at least
// kMinImage bytes of image (low-register 1D/2D kernels would otherwise be
// planned with no room to stage a tile at all), nor, when a typical tile's
// `want` bytes would not fit, more than leave room for it -- as long as
// four CTAs still share the SM (low-register 4D decoders with large tiles).
constexpr size_t kMinImage = 8 * 1024;

template <auto Kernel>
static size_t smem_room(size_t planes, size_t want = 0) {
  struct Limits {
    int sm_smem, ctas;
    size_t fixed;
    bool ok;
  };
  static const Limits lim = [] {
    int dev = 0, sm_smem = 0, reserved = 0;
    cudaFuncAttributes fa;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&reserved, cudaDevAttrReservedSharedMemoryPerBlock, dev) != cudaSuccess ||
        cudaFuncGetAttributes(&fa, Kernel) != cudaSuccess) {
      cudaGetLastError();
      return Limits{0, 1, 0, false};
    }
    const int regs = (fa.numRegs + 7) / 8 * 8;   // per-thread allocation granularity
    const int ctas = regs > 0 ? std::max(1, 65536 / (regs * kTile)) : 1;
    return Limits{sm_smem, ctas, (size_t)reserved + fa.sharedSizeBytes, true};
  }();
  if (!lim.ok) return kMaxTileSmem > planes ? kMaxTileSmem - planes : 0;
  const int fit = (int)((size_t)lim.sm_smem / (planes + kMinImage + lim.fixed));
  int ctas = std::max(1, std::min(lim.ctas, fit));
  if (want > kMinImage && (size_t)lim.sm_smem / ctas < planes + want + lim.fixed) {
    const int c = (int)((size_t)lim.sm_smem / (planes + want + lim.fixed));
    if (c >= 4) ctas = std::min(ctas, c);
  }
  const size_t per = (size_t)lim.sm_smem / ctas;
  const size_t room = std::min(per > lim.fixed ? per - lim.fixed : (size_t)0, kMaxTileSmem);
  return room > planes ? room - planes : 0;
}

// kFloor: the kernel keeps only the coded planes (mode kLossyFloor)
template <auto K, bool kFloorPlanes = false>
struct KernelTag {
  static constexpr auto kernel = K;
  static constexpr bool floor = kFloorPlanes;
};

// kernel variant: device job array -> multi-job kernel carrying both mode
// paths, or the lossy path alone when no job of the array is reversible (the
// reversible coder costs the lossy jobs registers: 186 for the 32-bit 3D
// decoder, which the lossy one, held to four CTAs per SM like the
// single-job kernels, does in 128); a single job -> the variant of its mode
// only.
// A 32-bit fixed-rate tile small enough for a fifth of an SM's shared memory
// (with the bit planes) goes to the five-CTA kernels; so does a 32-bit
// fixed-precision job whose largest tile fits there beside only its coded
// planes (the kLossyFloor kernels: precision up to about 20).  Decided from
// the job alone, so planning and launching pick the same kernel.
constexpr size_t kFifthShare = 228 * 1024 / 5 - 2048;   // per CTA, less reserved and static memory

template <typename S, int D>
static bool five_ctas(const Job& j) {
  if constexpr (sizeof(S) != 4 || D > 3) {
    return false;
  } else {
    const size_t tile = image_words((uint64_t)kTile * j.maxbits / 64 + 4) * 8 + plane_smem_bytes<S, D, false>();
    return (j.flags & kFixedRate) && tile <= kFifthShare;
  }
}

// bits of one block of a 32-bit fixed-precision job at most (block_bound):
// the header and every coded plane
template <typename S, int D>
static uint64_t floor_block_bound(const Job& j) {
  constexpr uint64_t N = 1u << (2 * D), hm = std::is_floating_point<S>::value ? 1 + 8 : 0;
  uint64_t b = hm + N - 1 + N * (uint64_t)j.maxprec;
  if (j.maxbits >= hm) b = std::min<uint64_t>(b, j.maxbits);
  return std::max<uint64_t>(b, j.minbits);
}

template <typename S, int D>
static bool five_ctas_floor(const Job& j) {
  if constexpr (sizeof(S) != 4 || D > 3) {
    return false;
  } else {
    if ((j.flags & kFixedRate) || j.maxprec >= 32) return false;
    const size_t tile = image_words((uint64_t)kTile * floor_block_bound<S, D>(j) / 64 + 4) * 8 +
                        plane_smem_bytes<S, D, false, true>(false, j.maxprec);
    return tile <= kFifthShare;
  }
}

// The fixed-precision encoder stages every tile whole in shared memory (it
// is built without the path that codes straight into the stream), so it is
// chosen only where the largest possible tile fits the room its occupancy
// leaves -- computed from the kernel's own attributes, the same way for
// planning and for launching.
template <typename S, int D>
static bool floor_encoder_fits(const Job& j) {
  if constexpr (sizeof(S) != 4 || D > 3) {
    return false;
  } else {
    const uint64_t words = image_words((uint64_t)kTile * floor_block_bound<S, D>(j) / 64 + 4);
    const size_t planes = plane_smem_bytes<S, D, true, true>(false, j.maxprec);
    return words * 8 <= smem_room<encode_kernel_occ<S, D, false, kLossyFloor, 5>>(planes);
  }
}

template <typename S, int D, class F>
static auto with_encoder(const LaunchArgs& a, F&& f) {
  // an encode into host memory stages its tiles (kStreamHost)
  if (!a.jobs && (a.one.flags & kStreamHost)) {
    if (a.one.minexp < kMinExp) return f(KernelTag<encode_kernel<S, D, false, kRevHost>>{});
    return f(KernelTag<encode_kernel<S, D, false, kLossyHost>>{});
  }
  if (a.jobs) {
    if (a.multi_lossy) {
      if constexpr (sizeof(S) == 4 && D == 3) return f(KernelTag<encode_kernel_occ<S, D, true, kLossyOnly, 4>>{});
      else if constexpr (sizeof(S) == 8 && D == 3) return f(KernelTag<encode_kernel_occ<S, D, true, kLossyOnly, 3>>{});
      else return f(KernelTag<encode_kernel<S, D, true, kLossyOnly>>{});
    }
    return f(KernelTag<encode_kernel<S, D, true, kAnyMode>>{});
  }
  if (a.one.minexp < kMinExp) {
    if constexpr (sizeof(S) == 8 && D <= 3) return f(KernelTag<encode_kernel_occ<S, D, false, kRevOnly, 3>>{});
    else return f(KernelTag<encode_kernel<S, D, false, kRevOnly>>{});
  }
  if constexpr (sizeof(S) == 4 && D <= 3) {
    if (five_ctas_floor<S, D>(a.one) && floor_encoder_fits<S, D>(a.one))
      return f(KernelTag<encode_kernel_occ<S, D, false, kLossyFloor, 5>, true>{});
    if (five_ctas<S, D>(a.one)) return f(KernelTag<encode_kernel_occ<S, D, false, kLossyOnly, 5>>{});
    if constexpr (D == 3) return f(KernelTag<encode_kernel_occ<S, D, false, kLossyOnly, 4>>{});
  }
  if constexpr (sizeof(S) == 8 && D == 3) return f(KernelTag<encode_kernel_occ<S, D, false, kLossyOnly, 3>>{});
  return f(KernelTag<encode_kernel<S, D, false, kLossyOnly>>{});
}

template <typename S, int D, class F>
static auto with_decoder(const LaunchArgs& a, F&& f) {
  if (a.jobs) {
    if (a.multi_lossy) {
      if constexpr (sizeof(S) == 4 && D == 3) return f(KernelTag<decode_kernel_occ<S, D, true, kLossyOnly, 4>>{});
      else if constexpr (sizeof(S) == 8 && D == 3) return f(KernelTag<decode_kernel_occ<S, D, true, kLossyOnly, 3>>{});
      else return f(KernelTag<decode_kernel<S, D, true, kLossyOnly>>{});
    }
    return f(KernelTag<decode_kernel<S, D, true, kAnyMode>>{});
  }
  if (a.one.minexp < kMinExp) {
    if constexpr (sizeof(S) == 4 && D <= 3) return f(KernelTag<decode_kernel_occ<S, D, false, kRevOnly, 3>>{});
    else return f(KernelTag<decode_kernel<S, D, false, kRevOnly>>{});
  }
  if constexpr (sizeof(S) == 8 && D <= 3) {
    // fixed rate alone: without the block-index and stream-reading paths of
    // variable rates the 3D decoder needs no spills (712 bytes otherwise), 2% faster
    if (D == 3 && (a.one.flags & kFixedRate)) return f(KernelTag<decode_kernel_occ<S, D, false, kFixedOnly, 3>>{});
    return f(KernelTag<decode_kernel_occ<S, D, false, kLossyOnly, 3>>{});
  } else {
    if (five_ctas_floor<S, D>(a.one)) return f(KernelTag<decode_kernel_occ<S, D, false, kLossyFloor, 5>, true>{});
    if (five_ctas<S, D>(a.one)) return f(KernelTag<decode_kernel_occ<S, D, false, kLossyOnly, 5>>{});
    if constexpr (sizeof(S) == 4 && D == 3) return f(KernelTag<decode_kernel_occ<S, D, false, kLossyOnly, 4>>{});
    else return f(KernelTag<decode_kernel<S, D, false, kLossyOnly>>{});
  }
}

// plane-buffer bytes the chosen kernel keeps
template <typename S, int D, bool kEncode, class Tag>
static size_t planes_of(const LaunchArgs& a) {
  return plane_smem_bytes<S, D, kEncode, Tag::floor>(a.jobs != nullptr, a.one.maxprec);
}

template <typename S, int D>
uint32_t stage_room(const LaunchArgs& a, bool encode) {
  auto words = [&](auto tag) -> uint32_t {
    using Tag = decltype(tag);
    const size_t planes = encode ? planes_of<S, D, true, Tag>(a) : planes_of<S, D, false, Tag>(a);
    return (uint32_t)(smem_room<Tag::kernel>(planes, encode ? 0 : (size_t)a.want_words * 8) / 8);
  };
  return encode ? with_encoder<S, D>(a, words) : with_decoder<S, D>(a, words);
}

template <typename S, int D>
cudaError_t run_encode(const LaunchArgs& a, cudaStream_t st) {
  return with_encoder<S, D>(a, [&](auto tag) {
    constexpr auto kernel = decltype(tag)::kernel;
    const size_t smem = (size_t)a.img_words * 8 + planes_of<S, D, true, decltype(tag)>(a);
    prepare_kernel<kernel>();
    kernel<<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.sc, a.total_tiles, a.use_ticket, a.img_words);
    return cudaGetLastError();
  });
}

template <typename S, int D>
cudaError_t run_decode(const LaunchArgs& a, cudaStream_t st) {
  return with_decoder<S, D>(a, [&](auto tag) {
    constexpr auto kernel = decltype(tag)::kernel;
    const size_t smem = (size_t)a.img_words * 8 + planes_of<S, D, false, decltype(tag)>(a);
    prepare_kernel<kernel>();
    kernel<<<a.grid, kTile, smem, st>>>(a.one, a.jobs, a.njobs, a.total_tiles, a.img_words);
    return cudaGetLastError();
  });
}

// Block offsets of a stream with no index (kernels.cuh: parse_kernel, and
// the speculative parse_probe / parse_spec / parse_stitch for long streams).
// Synchronous: returns after the offsets and end bit are written.
template <typename S, int D>
cudaError_t run_parse(const Job& job, cudaStream_t st) {
  constexpr uint32_t kProbe = 256;
  const uint64_t seg_blocks = std::max<uint64_t>(512, job.nblocks / 4096);
  const uint32_t k = (uint32_t)(kParseCover * seg_blocks);   // blocks each worker records
  if (job.nblocks <= 4ull * k) {
    parse_kernel<S, D><<<1, 32, 0, st>>>(job);
    cudaError_t e = cudaGetLastError();
    return e != cudaSuccess ? e : cudaStreamSynchronize(st);
  }
  unsigned long long* mean = nullptr;
  unsigned long long* rec = nullptr;
  cudaError_t e = cudaMallocAsync((void**)&mean, sizeof *mean, st);
  if (e != cudaSuccess) return e;
  unsigned long long mean_bits = 0;
  parse_probe<S, D><<<1, 32, 0, st>>>(job, kProbe, mean);
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(&mean_bits, mean, sizeof mean_bits, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess) {
    cudaFreeAsync(mean, st);
    return e;
  }
  const uint64_t seg = std::max<uint64_t>(mean_bits, 1) * seg_blocks;   // bits between worker starts
  // cover the stream's estimated length and a quarter more, within 512 MB of
  // records; beyond, the stitch parses alone
  const uint64_t want = std::max<uint64_t>(mean_bits, 1) * job.nblocks * 5 / 4 / seg + 4;
  const uint64_t room = (512ull << 20) / (8ull * (k + 1));
  const uint32_t workers = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(want, room), 8192);
  e = cudaMallocAsync((void**)&rec, (size_t)workers * (k + 1) * sizeof *rec, st);
  if (e == cudaSuccess) {
    parse_spec<S, D><<<(workers + 127) / 128, 128, 0, st>>>(job, seg, k, workers, rec);
    if ((e = cudaGetLastError()) == cudaSuccess) {
      parse_stitch<S, D><<<1, 32, 0, st>>>(job, seg, k, workers, rec);
      e = cudaGetLastError();
    }
    cudaFreeAsync(rec, st);
  }
  cudaFreeAsync(mean, st);
  return e != cudaSuccess ? e : cudaStreamSynchronize(st);
}

}  // namespace zg

#define ZG_INSTANTIATE(S, D)                                                   \
  namespace zg {                                                               \
  template cudaError_t run_encode<S, D>(const LaunchArgs&, cudaStream_t);      \
  template cudaError_t run_decode<S, D>(const LaunchArgs&, cudaStream_t);      \
  template cudaError_t run_parse<S, D>(const Job&, cudaStream_t);              \
  template uint32_t stage_room<S, D>(const LaunchArgs&, bool);                 \
  }
