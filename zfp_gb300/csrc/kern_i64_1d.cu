// kern_i64_1d.cu -- kernels for 1D int64_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int64_t, 1)
