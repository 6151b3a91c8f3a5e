// kern_i64_4d.cu -- kernels for 4D int64_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int64_t, 4)
