// kern_i32_1d.cu -- kernels for 1D int32_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int32_t, 1)
