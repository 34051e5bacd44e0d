// FP64 instantiation of the stepper kernels (the plain form) and the
// precision-independent slow-path kernels (the z pass is in kernels_f64_z.cu).
#include "launch_impl.cuh"
CB_INSTANTIATE_XY(double)

#include "cb_fft.cuh"

namespace cb {
cudaError_t launch_pointwise(int kind, size_t n, double* out, const double* a, const double* b, const double* c,
                             const double* d, double eps, double x0, double x1, double x2, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    pointwise_kernel<<<blocks, 256, 0, s>>>(kind, n, out, a, b, c, d, eps, x0, x1, x2);
    return cudaGetLastError();
}
// element held by slot p of a transposed line of length L, for the x lengths the
// fused passes use (tidx<L> at run time); -1 for an unsupported length
__device__ __forceinline__ int tidx_rt(int p, int L) {
    switch (L) {
        case 8: return tidx<8>(p);
        case 12: return tidx<12>(p);
        case 16: return tidx<16>(p);
        case 24: return tidx<24>(p);
        case 32: return tidx<32>(p);
        case 48: return tidx<48>(p);
        case 64: return tidx<64>(p);
        case 96: return tidx<96>(p);
        case 128: return tidx<128>(p);
        default: return -1;
    }
}
// FP32 form's real-space field: rows of nx points as nx/2 double-float pairs
// (hi0, lo0, hi1, lo1) in the x-slot order of the fused passes' half-length x
// transform (slot q holds points 2 tidx(q) and 2 tidx(q) + 1), so each warp's
// loads and stores there are contiguous
static __global__ void real_to_ff_kernel(const double* __restrict__ in, float4* __restrict__ out, size_t nrows,
                                         int nx) {
    const int M = nx / 2;
    const size_t n = nrows * (size_t)M;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const size_t row = i / M;
        const int q = (int)(i - row * M);
        const int m = tidx_rt(q, M);
        const double v0 = in[row * nx + 2 * m], v1 = in[row * nx + 2 * m + 1];
        const float h0 = __double2float_rn(v0), h1 = __double2float_rn(v1);
        out[i] = make_float4(h0, __double2float_rn(v0 - (double)h0), h1, __double2float_rn(v1 - (double)h1));
    }
}
cudaError_t launch_real_to_ff(const double* in, void* out, size_t nrows, int nx, cudaStream_t s) {
    // only the x lengths tidx_rt knows (a -1 slot would index before the row)
    switch (nx / 2) {
        case 8: case 12: case 16: case 24: case 32: case 48: case 64: case 96: case 128: break;
        default: return cudaErrorInvalidValue;
    }
    if (nx % 2) return cudaErrorInvalidValue;
    const size_t n = nrows * (size_t)(nx / 2);
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    real_to_ff_kernel<<<blocks, 256, 0, s>>>(in, reinterpret_cast<float4*>(out), nrows, nx);
    return cudaGetLastError();
}
}  // namespace cb
