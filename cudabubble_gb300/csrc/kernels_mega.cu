// The persistent batched attempt kernel (mega.cuh) and its host-side launch helpers.
#include "mega.cuh"

namespace cb {

bool mega_size_ok(int n) {
    switch (n) {
#define CASE(N) case N: return true;
        CB_MEGA_SIZES(CASE)
#undef CASE
        default: return false;
    }
}

template <int N> constexpr size_t mega_body_bytes() {
    constexpr size_t z = (kMegaThreads / kMegaZThreads) * mega_align(z_smem_bytes<float, N, kMegaZTX>());
    constexpr size_t xy = mega_cluster_xy(N) ? xyc_smem_bytes<float, N>()
                                             : (kMegaThreads / mega_xy_threads(N)) * mega_align(xy_smem_bytes<float, N>(2));
    return z > xy ? z : xy;
}

size_t mega_smem_bytes() {
    size_t m = 0;
#define CASE(N) m = mega_body_bytes<N>() > m ? mega_body_bytes<N>() : m;
    CB_MEGA_SIZES(CASE)
#undef CASE
    return kMegaHead + m;
}

static cudaError_t mega_attr() {
    static bool done = false;
    if (done) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(mega_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)mega_smem_bytes());
    if (e == cudaSuccess) done = true;
    return e;
}

int mega_max_clusters() {
    if (mega_attr() != cudaSuccess) return 0;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(2 * 1024);
    cfg.blockDim = dim3(kMegaThreads);
    cfg.dynamicSmemBytes = mega_smem_bytes();
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, mega_kernel, &cfg) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

cudaError_t mega_launch(const MegaArgs& a, int nclusters, cudaStream_t s) {
    cudaError_t e = mega_attr();
    if (e != cudaSuccess) return e;
    mega_kernel<<<dim3(2 * nclusters), dim3(kMegaThreads), mega_smem_bytes(), s>>>(a);
    return cudaGetLastError();
}

}  // namespace cb
