// kern_f64_1d.cu -- kernels for 1D double fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(double, 1)
