// kern_f32.cu -- kernels for float fields.
#include "launch_impl.cuh"

ZG_DEFINE_LAUNCHERS(f32, float)
