// kern_i32_4d.cu -- kernels for 4D int32_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int32_t, 4)
