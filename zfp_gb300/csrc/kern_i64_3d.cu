// kern_i64_3d.cu -- kernels for 3D int64_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int64_t, 3)
