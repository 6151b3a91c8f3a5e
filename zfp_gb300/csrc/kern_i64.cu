// kern_i64.cu -- kernels for int64_t fields.
#include "launch_impl.cuh"

ZG_DEFINE_LAUNCHERS(i64, int64_t)
