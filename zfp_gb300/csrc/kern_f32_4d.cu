// kern_f32_4d.cu -- kernels for 4D float fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(float, 4)
