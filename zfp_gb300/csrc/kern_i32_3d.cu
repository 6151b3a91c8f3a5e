// kern_i32_3d.cu -- kernels for 3D int32_t fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(int32_t, 3)
