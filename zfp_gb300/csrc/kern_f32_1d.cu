// kern_f32_1d.cu -- kernels for 1D float fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(float, 1)
