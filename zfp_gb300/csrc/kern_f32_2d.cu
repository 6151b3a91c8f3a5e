// kern_f32_2d.cu -- kernels for 2D float fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(float, 2)
