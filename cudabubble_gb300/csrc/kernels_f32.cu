// FP32 instantiation of the stepper kernels (the precision form).
#include "launch_impl.cuh"
template struct cb::Launch<float>;
