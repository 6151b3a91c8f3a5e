// kern_f64_2d.cu -- kernels for 2D double fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(double, 2)
