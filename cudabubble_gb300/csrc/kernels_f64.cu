// FP64 instantiation of the stepper kernels (the plain form) and the
// precision-independent slow-path kernels (the z pass is in kernels_f64_z.cu).
#include "launch_impl.cuh"
CB_INSTANTIATE_XY(double)

namespace cb {
cudaError_t launch_pointwise(int kind, size_t n, double* out, const double* a, const double* b, const double* c,
                             const double* d, double eps, double x0, double x1, double x2, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    pointwise_kernel<<<blocks, 256, 0, s>>>(kind, n, out, a, b, c, d, eps, x0, x1, x2);
    return cudaGetLastError();
}
}  // namespace cb
