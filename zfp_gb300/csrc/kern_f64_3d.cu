// kern_f64_3d.cu -- kernels for 3D double fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(double, 3)
