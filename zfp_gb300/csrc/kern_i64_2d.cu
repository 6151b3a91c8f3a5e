// kern_i64_2d.cu -- kernels for 2D int64_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int64_t, 2)
