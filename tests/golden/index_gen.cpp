// Golden-vector driver for zfp's block index formats: builds the reference's
// own index classes (include/zfp/index.hpp, compiled from the reference's
// headers by make_index_golden.py) from block sizes read on stdin and prints
// the packed index words, the range and every block offset.
//
// stdin:  format dims nblocks size_0 ... size_{nblocks-1}
//         format 1 = verbatim, 2 = hybrid4, 3 = hybrid8<dims>
// stdout: nbytes, the packed bytes as hex, range, nblocks offsets
#include <cstdio>
#include <cstring>   // the reference's memory.hpp uses std::memcpy
#include <vector>

#include "zfp.h"
#include "zfp/internal/array/exception.hpp"
#include "zfp/index.hpp"

template <class Index>
struct Open : Index {
  using Index::Index;
  const unsigned char* raw() const { return reinterpret_cast<const unsigned char*>(this->data); }
};

template <class Index>
static int run(size_t n, const std::vector<size_t>& sizes) {
  Open<Index> idx(n);
  idx.clear();
  for (size_t i = 0; i < n; i++) idx.set_block_size(i, sizes[i]);
  idx.flush();
  const size_t bytes = idx.size_bytes(ZFP_DATA_INDEX);
  std::printf("%zu\n", bytes);
  for (size_t i = 0; i < bytes; i++) std::printf("%02x", idx.raw()[i]);
  std::printf("\n%llu\n", (unsigned long long)idx.range());
  for (size_t i = 0; i < n; i++) std::printf("%llu ", (unsigned long long)idx.block_offset(i));
  std::printf("\n");
  return 0;
}

int main() {
  int format = 0, dims = 0;
  size_t n = 0;
  if (std::scanf("%d %d %zu", &format, &dims, &n) != 3) return 2;
  std::vector<size_t> sizes(n);
  for (size_t i = 0; i < n; i++)
    if (std::scanf("%zu", &sizes[i]) != 1) return 2;
  try {
    switch (format) {
      case 1: return run<zfp::index::verbatim>(n, sizes);
      case 2: return run<zfp::index::hybrid4>(n, sizes);
      case 3:
        switch (dims) {
          case 1: return run<zfp::index::hybrid8<1>>(n, sizes);
          case 2: return run<zfp::index::hybrid8<2>>(n, sizes);
          case 3: return run<zfp::index::hybrid8<3>>(n, sizes);
          default: return run<zfp::index::hybrid8<4>>(n, sizes);
        }
    }
  } catch (const zfp::exception& e) {
    std::printf("error %s\n", e.what());
    return 3;
  }
  return 2;
}
