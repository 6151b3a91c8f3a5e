// kern_i32.cu -- kernels for int32_t fields.
#include "launch_impl.cuh"

ZG_DEFINE_LAUNCHERS(i32, int32_t)
