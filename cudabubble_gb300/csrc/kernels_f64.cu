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
static __global__ void real_to_ff_kernel(const double* __restrict__ in, float2* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double v = in[i];
        const float hi = __double2float_rn(v);
        out[i] = make_float2(hi, __double2float_rn(v - (double)hi));
    }
}
cudaError_t launch_real_to_ff(const double* in, void* out, size_t n, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    real_to_ff_kernel<<<blocks, 256, 0, s>>>(in, reinterpret_cast<float2*>(out), n);
    return cudaGetLastError();
}
}  // namespace cb
