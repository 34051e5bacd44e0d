// Size dispatch for the kernel templates (included by kernels_f32.cu and
// kernels_f64.cu with CB_REAL set to float or double).
#pragma once
#include <string.h>

#include "launch.h"
#include "misc_kernels.cuh"
#include "split_kernels.cuh"
#include "xy_cluster.cuh"
#include "xy_kernel.cuh"
#include "z_kernel.cuh"

namespace cb {

constexpr size_t kMaxSmem = 227 * 1024;

// [launch_k definition]
// Launch with programmatic stream serialisation: the kernel's CTAs may be scheduled
// while the previous kernel in the stream still runs, and wait in CB_PDL_WAIT for its
// results (cb_fft.cuh).  Captured into a graph, the launch becomes a programmatic edge.
// A build with -DCB_NO_PDL launches with plain stream order.
template <class... KArgs, class... Args>
static cudaError_t launch_k(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                            Args... args) {
    cudaLaunchConfig_t cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
#ifndef CB_NO_PDL
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
#else
    (void)at;
#endif
    return cudaLaunchKernelEx(&cfg, kern, args...);
}
// [end launch_k definition]

// threads of the single-CTA xy pass for planes of 96^2 and 128^2: the
// nonlinear pass (two fields both ways) gains from 32 warps per plane, the
// reductions (inverse only) do not (build-time knobs, measured on GB300)
#ifndef CB_XY_NT_LARGE
#define CB_XY_NT_LARGE 512
#endif
#ifndef CB_XY_NT_NONLIN
#define CB_XY_NT_NONLIN 1024
#endif

template <class T, int NX> struct XYCfg {
    static constexpr int NT = NX <= 32 ? 128 : (NX <= 64 ? 256 : CB_XY_NT_LARGE);
    static constexpr int NT_NONLIN = NX <= 64 ? NT : CB_XY_NT_NONLIN;
    static constexpr bool ok = xy_smem_bytes<T, NX>(2) <= kMaxSmem;   // stepping (two fields)
    static constexpr bool ok1 = xy_smem_bytes<T, NX>(1) <= kMaxSmem;  // plain transforms (one field)
    // the FP32 fused pass with curvature (a third output field)
    static constexpr bool ok_q = sizeof(T) == 4 && xy_smem_bytes<T, NX>(2, 1) <= kMaxSmem;
};

// FP32 fused pass on two-CTA clusters from 64^2 planes (a build-time knob)
#ifndef CB_XY_CLUSTER
#define CB_XY_CLUSTER 1
#endif
template <class T, int NX, int NQ = 0> constexpr bool xyc_ok() {
    return CB_XY_CLUSTER && sizeof(T) == 4 && NX >= 64 && NX % 4 == 0 && xyc_smem_bytes<T, NX, NQ>() <= 227 * 1024;
}
template <class T, int NX, int NQ = 0>
static cudaError_t xyc_go(const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s) {
    constexpr int NT = NX >= 96 ? 512 : 256;
    constexpr size_t sm = xyc_smem_bytes<T, NX, NQ>();
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(xyc_fused_kernel<T, NX, NT, NQ>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return launch_k(xyc_fused_kernel<T, NX, NT, NQ>, dim3(2 * nzmax, ninst), dim3(NT), sm, s, d, a);
}

template <class T, int NX, int NF, int NT, int NQ = 0>
static cudaError_t xy_go_nf(const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s) {
    constexpr size_t sm = xy_smem_bytes<T, NX>(NF, NQ);
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(xy_kernel<T, NX, NT, NF, NQ>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return launch_k(xy_kernel<T, NX, NT, NF, NQ>, dim3(nzmax, ninst), dim3(NT), sm, s, d, a);
}

template <class T, int NX>
static cudaError_t xy_go(const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s,
                         bool allow_cluster) {
    const bool two = a.mode == XY_REDUCE_FULL || a.mode == XY_NONLIN || a.mode == XY_FUSED;
    if constexpr (sizeof(T) == 4) {
        if (a.curv && a.mode == XY_FUSED) {  // the fused pass with its third field q
            if constexpr (xyc_ok<T, NX, 1>()) {
                if (allow_cluster) return xyc_go<T, NX, 1>(d, ninst, nzmax, a, s);
            }
            if constexpr (XYCfg<T, NX>::ok_q) return xy_go_nf<T, NX, 2, XYCfg<T, NX>::NT_NONLIN, 1>(d, ninst, nzmax, a, s);
            return cudaErrorInvalidValue;
        }
    }
    if constexpr (xyc_ok<T, NX>()) {
        if (a.mode == XY_FUSED && allow_cluster) return xyc_go<T, NX>(d, ninst, nzmax, a, s);
    }
    if constexpr (XYCfg<T, NX>::ok) {
        if (a.mode == XY_NONLIN || a.mode == XY_FUSED) return xy_go_nf<T, NX, 2, XYCfg<T, NX>::NT_NONLIN>(d, ninst, nzmax, a, s);
        if (two) return xy_go_nf<T, NX, 2, XYCfg<T, NX>::NT>(d, ninst, nzmax, a, s);
    }
    if constexpr (XYCfg<T, NX>::ok1) {
        if (!two) return xy_go_nf<T, NX, 1, XYCfg<T, NX>::NT>(d, ninst, nzmax, a, s);
    }
    return cudaErrorInvalidValue;
}

// z-pass tile of the FP32 form: columns per CTA and threads per CTA (build-time knobs;
// the FP64 form keeps 8 columns of 16-byte values and 256 threads)
#ifndef CB_Z_TX
#define CB_Z_TX 16
#endif
#ifndef CB_Z_NT
#define CB_Z_NT 256
#endif
template <class T> constexpr int ztile() { return sizeof(T) == 4 ? CB_Z_TX : 8; }
template <class T> constexpr int zthreads() { return sizeof(T) == 4 ? CB_Z_NT : 256; }

// ---- split plane path
template <int NX> constexpr int split_rpc() { return NX >= 96 ? 16 : 8; }
constexpr int kSplitThreads = 256;

template <class T, int NY>
static cudaError_t ycol_go(const InstT<T>* d, int ninst, int nzmax, const YArgs& a, cudaStream_t s) {
    constexpr int TX = sizeof(T) == 4 ? 16 : 8, NT = kSplitThreads;  // the split path's own column tile
    constexpr size_t sm = ycol_smem_bytes<T, NY, TX>();
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(ycol_kernel<T, NY, TX, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    const int ntx = (NY / 2 + 1 + TX - 1) / TX;  // square planes: nc = NY/2 + 1
    return launch_k(ycol_kernel<T, NY, TX, NT>, dim3(nzmax * ntx, ninst), dim3(NT), sm, s, d, a);
}

template <class T, int NX>
static cudaError_t xrow_go(const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s) {
    constexpr int RPC = split_rpc<NX>(), NT = kSplitThreads;
    constexpr size_t sm = xrow_smem_bytes<T, NX, RPC>();
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(xrow_kernel<T, NX, RPC, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return launch_k(xrow_kernel<T, NX, RPC, NT>, dim3(nzmax * NX / RPC, ninst), dim3(NT), sm, s, d, a);
}

// one xy mode as y pass(es) around the x-row pass
template <class T, int NX>
static cudaError_t xy_split_go(const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s) {
    YArgs y;
    memset(&y, 0, sizeof y);
    y.role = a.role;
    y.stepping = a.mode <= XY_FUSED;
    y.skip_if_stale = a.skip_if_stale;
    y.fused = a.mode == XY_FUSED;
    cudaError_t r = cudaSuccess;
    switch (a.mode) {
        case XY_NONLIN:
        case XY_FUSED:
        case XY_REDUCE_FULL:
            y.mode = Y_INV2;
            break;
        case XY_REDUCE_S:
            y.mode = Y_INV1;
            break;
        case XY_INV_PLAIN:
            y.mode = Y_INV1;
            y.cin = a.cin;
            break;
        default:  // XY_FWD_PLAIN: rows first
            y.mode = -1;
            break;
    }
    if (y.mode >= 0) {
        r = ycol_go<T, NX>(d, ninst, nzmax, y, s);
        if (r != cudaSuccess) return r;
    }
    r = xrow_go<T, NX>(d, ninst, nzmax, a, s);
    if (r != cudaSuccess) return r;
    if (a.mode == XY_NONLIN || a.mode == XY_FUSED || a.mode == XY_FWD_PLAIN) {
        y.mode = a.mode == XY_FWD_PLAIN ? Y_FWD1 : Y_FWD2;
        y.cout = a.cout;
        r = ycol_go<T, NX>(d, ninst, nzmax, y, s);
    }
    return r;
}

template <class T, int NZ, int MG, int NQ = 0>
static cudaError_t z_go_g(const InstT<T>* d, int ninst, int ntiles, const ZArgs& a, cudaStream_t s) {
    constexpr int TX = ztile<T>();
    constexpr int NT = zthreads<T>();
    constexpr size_t sm = z_smem_bytes<T, NZ, TX, NQ>();
    static bool attr = false;
    if (!attr) {
        cudaError_t e = cudaFuncSetAttribute(z_kernel<T, NZ, TX, NT, MG, NQ>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    return launch_k(z_kernel<T, NZ, TX, NT, MG, NQ>, dim3(ntiles, ninst), dim3(NT), sm, s, d, a);
}

template <class T, int NZ>
static cudaError_t z_go(const InstT<T>* d, int ninst, int ntiles, const ZArgs& a, cudaStream_t s) {
    if constexpr (sizeof(T) == 4) {
        if (a.curv) {  // FP32 stages with spontaneous curvature: the third partial q
            switch (zgroup_of(a.mode)) {
                case ZG_ETD2: return z_go_g<T, NZ, ZG_ETD2, 1>(d, ninst, ntiles, a, s);
                case ZG_ETD4: return z_go_g<T, NZ, ZG_ETD4, 1>(d, ninst, ntiles, a, s);
                case ZG_EULER: return z_go_g<T, NZ, ZG_EULER, 1>(d, ninst, ntiles, a, s);
                default: break;
            }
        }
    }
    switch (zgroup_of(a.mode)) {
        case ZG_ETD2: return z_go_g<T, NZ, ZG_ETD2>(d, ninst, ntiles, a, s);
        case ZG_ETD4: return z_go_g<T, NZ, ZG_ETD4>(d, ninst, ntiles, a, s);
        case ZG_EULER: return z_go_g<T, NZ, ZG_EULER>(d, ninst, ntiles, a, s);
        default: return z_go_g<T, NZ, ZG_PLAIN>(d, ninst, ntiles, a, s);
    }
}

#define CB_XY_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128)
#define CB_Z_SIZES(X) X(16) X(24) X(32) X(48) X(64) X(96) X(128) X(192) X(256)
// sizes the two-CTA cluster pass is built for (where its plane fits: 72.7 KB per CTA at
// 128^2, ~157 KB at 192^2)
#define CB_XYC_SIZES(X) X(64) X(96) X(128) X(192)

template <class T> bool Launch<T>::xy_cluster_ok(int nx, int curv) {
    switch (nx) {
#define CASE(n) case n: return curv ? xyc_ok<T, n, 1>() : xyc_ok<T, n>();
        CB_XYC_SIZES(CASE)
#undef CASE
        default: return false;
    }
}

template <class T> bool Launch<T>::xy_single(int nx, int nf, int curv) {
    switch (nx) {
#define CASE(n) case n: return nf == 2 ? (curv ? XYCfg<T, n>::ok_q : XYCfg<T, n>::ok) : XYCfg<T, n>::ok1;
        CB_XY_SIZES(CASE)
#undef CASE
        default: return false;
    }
}
// the FP32 fused pass with curvature runs on the cluster or one-CTA plane kernels only
// (the split passes carry no third field): true where `path` resolves to one of them
template <class T> bool Launch<T>::fused_curv_ok(int nx, int path) {
    if (sizeof(T) != 4 || path == XYP_SPLIT) return false;
    if (path == XYP_CLUSTER && xy_cluster_ok(nx, 1)) return true;
    return xy_single(nx, 2, 1);
}
template <class T> bool Launch<T>::xy_split_supported(int nx) {
    switch (nx) {
#define CASE(n) case n: return true;
        CB_Z_SIZES(CASE)
#undef CASE
        default: return false;
    }
}
template <class T> int Launch<T>::xy_rows_per_cta(int nx) { return nx >= 96 ? 16 : 8; }
template <class T> bool Launch<T>::xy_supported(int nx) { return xy_single(nx, 2) || xy_split_supported(nx); }
template <class T> bool Launch<T>::xy_plain_supported(int nx) { return xy_single(nx, 1) || xy_split_supported(nx); }
template <class T> bool Launch<T>::z_supported(int nz) {
    switch (nz) {
#define CASE(n) case n: return true;
        CB_Z_SIZES(CASE)
#undef CASE
        default: return false;
    }
}
template <class T> int Launch<T>::z_tile() { return ztile<T>(); }

template <class T>
cudaError_t Launch<T>::xy(int nx, const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s,
                          int path) {
    const int nf = (a.mode == XY_REDUCE_FULL || a.mode == XY_NONLIN || a.mode == XY_FUSED) ? 2 : 1;
    const int curv = sizeof(T) == 4 && a.curv && a.mode == XY_FUSED;
    if (path == XYP_CLUSTER && a.mode == XY_FUSED && xy_cluster_ok(nx, curv)) {
        switch (nx) {
#define CASE(n)                                                                                       \
    case n:                                                                                           \
        if (curv) {                                                                                   \
            if constexpr (xyc_ok<T, n, 1>()) return xyc_go<T, n, 1>(d, ninst, nzmax, a, s);           \
        } else {                                                                                      \
            if constexpr (xyc_ok<T, n>()) return xyc_go<T, n>(d, ninst, nzmax, a, s);                 \
        }                                                                                             \
        break;
            CB_XYC_SIZES(CASE)
#undef CASE
            default: break;
        }
    }
    if (path != XYP_SPLIT && xy_single(nx, nf, curv)) {
        switch (nx) {
#define CASE(n) case n: return xy_go<T, n>(d, ninst, nzmax, a, s, path != XYP_SINGLE);
            CB_XY_SIZES(CASE)
#undef CASE
            default: return cudaErrorInvalidValue;
        }
    }
    if (curv) return cudaErrorInvalidValue;  // the split passes carry no third field (fused_curv_ok)
    switch (nx) {
#define CASE(n) case n: return xy_split_go<T, n>(d, ninst, nzmax, a, s);
        CB_Z_SIZES(CASE)
#undef CASE
        default: return cudaErrorInvalidValue;
    }
}
template <class T>
cudaError_t Launch<T>::z(int nz, const InstT<T>* d, int ninst, int ntiles, const ZArgs& a, cudaStream_t s) {
    switch (nz) {
#define CASE(n) case n: return z_go<T, n>(d, ninst, ntiles, a, s);
        CB_Z_SIZES(CASE)
#undef CASE
        default: return cudaErrorInvalidValue;
    }
}
template <class T> cudaError_t Launch<T>::decide(const InstT<T>* d, int ninst, int raw, cudaStream_t s) {
    return launch_k(decide_kernel<T>, dim3((ninst + 127) / 128), dim3(128), 0, s, d, ninst, raw);
}
template <class T> cudaError_t Launch<T>::coef(const InstT<T>* d, int ninst, int accurate, cudaStream_t s, int raw) {
    return launch_k(prologue_fill_kernel<T>, dim3(64, ninst), dim3(256), 0, s, d, accurate, raw);
}
template <class T> cudaError_t Launch<T>::to_double(const void* in, double* out, size_t n, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    cplx_to_double_kernel<T><<<blocks, 256, 0, s>>>(reinterpret_cast<const cplx<T>*>(in), reinterpret_cast<double2*>(out), n);
    return cudaGetLastError();
}

template <class T>
cudaError_t Launch<T>::nhat_full(const InstT<T>* d, const void* spec, double* out, size_t n, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    nhat_full_kernel<T><<<blocks, 256, 0, s>>>(d, spec, reinterpret_cast<double2*>(out));
    return cudaGetLastError();
}

template <class T> cudaError_t Launch<T>::state_to_double(const void* in, double* out, size_t n, cudaStream_t s) {
    const int blocks = (int)((n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096);
    state_to_double_kernel<T><<<blocks, 256, 0, s>>>(in, reinterpret_cast<double2*>(out), n);
    return cudaGetLastError();
}

}  // namespace cb

// explicit instantiation, split in two translation units per precision so the
// z-pass instances (four mode groups x nine sizes) compile in parallel
#define CB_INSTANTIATE_XY(T)                                                                                        \
    template bool cb::Launch<T>::xy_supported(int);                                                                 \
    template bool cb::Launch<T>::xy_plain_supported(int);                                                           \
    template bool cb::Launch<T>::xy_single(int, int, int);                                                          \
    template bool cb::Launch<T>::xy_split_supported(int);                                                           \
    template bool cb::Launch<T>::xy_cluster_ok(int, int);                                                           \
    template bool cb::Launch<T>::fused_curv_ok(int, int);                                                           \
    template int cb::Launch<T>::xy_rows_per_cta(int);                                                               \
    template cudaError_t cb::Launch<T>::xy(int, const cb::InstT<T>*, int, int, const cb::XYArgs&, cudaStream_t, int); \
    template cudaError_t cb::Launch<T>::decide(const cb::InstT<T>*, int, int, cudaStream_t);                        \
    template cudaError_t cb::Launch<T>::coef(const cb::InstT<T>*, int, int, cudaStream_t, int);                    \
    template cudaError_t cb::Launch<T>::to_double(const void*, double*, size_t, cudaStream_t);                     \
    template cudaError_t cb::Launch<T>::nhat_full(const cb::InstT<T>*, const void*, double*, size_t, cudaStream_t); \
    template cudaError_t cb::Launch<T>::state_to_double(const void*, double*, size_t, cudaStream_t);
#define CB_INSTANTIATE_Z(T)                                    \
    template bool cb::Launch<T>::z_supported(int);             \
    template int cb::Launch<T>::z_tile();                      \
    template cudaError_t cb::Launch<T>::z(int, const cb::InstT<T>*, int, int, const cb::ZArgs&, cudaStream_t);
