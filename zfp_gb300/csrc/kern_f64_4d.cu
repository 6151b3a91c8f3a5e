// kern_f64_4d.cu -- kernels for 4D double fields.
#include "launch_impl.cuh"

ZG_INSTANTIATE(double, 4)
