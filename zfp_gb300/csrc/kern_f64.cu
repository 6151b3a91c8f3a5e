// kern_f64.cu -- kernels for double fields.
#include "launch_impl.cuh"

ZG_DEFINE_LAUNCHERS(f64, double)
