// FP32 instantiation of the stepper kernels (the precision form): xy, split
// and small kernels (the z pass is in kernels_f32_z.cu).
#include "launch_impl.cuh"
CB_INSTANTIATE_XY(float)
