// FP32 instantiation of the z pass.
#include "launch_impl.cuh"
CB_INSTANTIATE_Z(float)
