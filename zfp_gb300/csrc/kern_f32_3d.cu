// kern_f32_3d.cu -- kernels for 3D float fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(float, 3)
