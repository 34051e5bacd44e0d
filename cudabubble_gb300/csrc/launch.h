// Typed kernel launchers; one explicit instantiation per precision lives in
// kernels_f32.cu / kernels_f64.cu so the two compile in parallel.
#pragma once
#include <cuda_runtime.h>
#include <stddef.h>
#include "cb_inst.h"
#include "cb_kargs.h"

namespace cb {

template <class T> struct Launch {
    static bool xy_supported(int nx);        // stepping (single-CTA planes or the split path)
    static bool z_supported(int nz);
    static bool xy_plain_supported(int nx);  // plain transforms
    static bool xy_single(int nx, int nf, int curv = 0);  // one CTA per plane holds nf fields (+ q)
    static bool xy_split_supported(int nx);
    static bool xy_cluster_ok(int nx, int curv = 0);      // FP32 fused pass on two-CTA clusters (+ q)
    static bool fused_curv_ok(int nx, int path);          // FP32 fused pass with curvature on `path`
    static int xy_rows_per_cta(int nx);      // split path: rows of the x pass per CTA
    static int z_tile();
    // path: an XYPath.  XYP_SINGLE falls back to the split passes where one plane does not
    // fit a CTA; XYP_CLUSTER applies to the FP32 fused pass and is the size rule otherwise
    static cudaError_t xy(int nx, const InstT<T>* d, int ninst, int nzmax, const XYArgs& a, cudaStream_t s,
                          int path = XYP_AUTO);
    static cudaError_t z(int nz, const InstT<T>* d, int ninst, int ntiles, const ZArgs& a, cudaStream_t s);
    static cudaError_t decide(const InstT<T>* d, int ninst, int raw, cudaStream_t s);
    static cudaError_t coef(const InstT<T>* d, int ninst, int accurate, cudaStream_t s, int raw = 1);
    static cudaError_t to_double(const void* in, double* out, size_t n, cudaStream_t s);
    // the full ETD N-hat of instance 0 (its Nu buffer, plus the FP32 form's linear part on `spec`)
    static cudaError_t nhat_full(const InstT<T>* d, const void* spec, double* out, size_t n, cudaStream_t s);
    static cudaError_t state_to_double(const void* in, double* out, size_t n, cudaStream_t s);
};

cudaError_t launch_pointwise(int kind, size_t n, double* out, const double* a, const double* b, const double* c,
                             const double* d, double eps, double x0, double x1, double x2, cudaStream_t s);
// real FP64 field of nrows rows of nx points -> double-float pairs (hi = fl32(v),
// lo = fl32(v - hi)), two points per float4 in the fused passes' x-slot order
cudaError_t launch_real_to_ff(const double* in, void* out, size_t nrows, int nx, cudaStream_t s);

}  // namespace cb
