// kern_i32_2d.cu -- kernels for 2D int32_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int32_t, 2)
