// Pointwise stages shared by the single-CTA xy pass (xy_kernel.cuh) and the
// row pass of the split plane path (split_kernels.cuh): the nonlinear
// partials G, H and the energy / area sums, on real values held as the two
// halves of complex slots.
#pragma once
#include "cb_fft.cuh"
#include "cb_inst.h"

namespace cb {

template <class T> struct Acc;
template <> struct Acc<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double part() const { return s; }
};
// FP32 values summed as a double-float pair (error-free TwoSum per add)
template <> struct Acc<float> {
    FF v{0.f, 0.f};
    __device__ __forceinline__ void add(float x) { v = ff_add(v, FF{x, 0.f}); }
    __device__ __forceinline__ void add(float x, float xlo) { v = ff_add(v, FF{x, xlo}); }  // x + xlo
    __device__ __forceinline__ FF part() const { return v; }
};

// A plain per-thread sum, handed to the same double-float / FP64 warp and block
// reductions as Acc: for totals that tolerate one FP32 rounding per add (the
// fused pass's totals of G'' and w, whose FP64 N'(0) needs ~1e-6 absolute)
template <class T> struct PSum;
template <> struct PSum<double> {
    double s = 0.0;
    __device__ __forceinline__ void add(double x) { s += x; }
    __device__ __forceinline__ double part() const { return s; }
};
template <> struct PSum<float> {
    float s = 0.f;
    __device__ __forceinline__ void add(float x) { s += x; }
    __device__ __forceinline__ FF part() const { return FF{s, 0.f}; }
};

// lambda_1 = M1 (V - alpha), lambda_2 = M2 (S - beta) (belastic.cpp:478-479) as
// the constant and f coefficients of G, formed in FP64 by one thread.
template <class T> __device__ __forceinline__ void nonlin_lambdas(const Params& p, const Ctrl* ctrl, int role, T* lam) {
    const bool euler = p.method == M_EULER;
    const Scal& sc = ctrl->sc[role];
    const double lam1 = p.M1 * (sc.V - ctrl->alpha), lam2 = p.M2 * (sc.S - ctrl->beta);
    lam[0] = euler ? (T)(0.5 * lam1) : (T)(-0.5 * lam1);
    lam[1] = euler ? (T)lam2 : (T)(-lam2 * 1.0606601717798212866);  // 3 / (2 sqrt 2)
}

// G, H of one real point from u and lap u:
// ETD  (Calc.cu:428-437 with nld from :265-284):
//   G = -lam1/2 - c3 lam2 f - eta (D t / eps^3 + (3u^2 - D - 1) f / eps^2),  H = t
// Euler (Calc.cu:410-419 with g0 from :171-180):
//   G = lam1/2 + lam2 f + eta (3u^2 - 1) f / eps^2,                         H = f
// with f = -eps lap + (u^2 - 1) u / eps and t = u (u^2 - 1 - kappa), kappa = 2,
// D = 1.5 (phasefield.cpp:259-260).  The FP32 form folds every constant hi + lo.
template <class T>
__device__ __forceinline__ void nonlin_point(const PC<T>& k, bool euler, T g_c, T g_f, T u, T lap, T& g, T& h) {
    const T kappa = (T)2.0, D = (T)1.5;
    const T u2 = u * u;
    if constexpr (sizeof(T) == 8) {
        const T f = -lap * k.eps + (u2 - (T)1) * u * k.ieps;
        if (euler) {
            if (k.C != 0.0) {  // g = -lap fc + (3u^2 - 1 + 2 eps u C) fc / eps^2 (phasefield.cpp:236-246)
                const T fc = f + (u2 - (T)1) * k.C;
                g = g_c + g_f * f + k.eta * ((T)3 * u2 - (T)1 + (T)2 * k.eps * u * k.C) * fc * k.ieps2;
                h = fc;
            } else {
                g = g_c + g_f * f + k.eta * ((T)3 * u2 - (T)1) * f * k.ieps2;
                h = f;
            }
        } else {
            const T t = u * (u2 - (T)1 - kappa);
            g = g_c + g_f * f - k.eta * (D * t * k.ieps3 + ((T)3 * u2 - D - (T)1) * k.ieps2 * f);
            h = t;
            if (k.C != 0.0) {
                // no counterpart in the reference (its nld ignores C): the curvature part
                // g_C - g0 = -lap (C (u^2 - 1)) + ((3u^2 - 1)(fc - f) + 2 eps u C fc) / eps^2
                // whole in the nonlinear term; its Laplacian rides on H (eta lap t / eps)
                const T cu = (u2 - (T)1) * k.C, fc = f + cu;
                g -= k.eta * (((T)3 * u2 - (T)1) * cu + (T)2 * k.eps * u * k.C * fc) * k.ieps2;
                h = t + k.eps * cu;
            }
        }
    } else {
        const T w = (u2 - (T)1) * u;
        const T f = k.k_ieps.mul(w) - k.k_eps.mul(lap);
        if (euler) {
            g = g_c + g_f * f + k.k_K2.mul(((T)3 * u2 - (T)1) * f);
            h = f;
        } else {
            // ETD in the linear-split form: G' = G - eta D kappa u / eps^3 and
            // H' = t + kappa u = w; the kappa u parts are applied to the exact
            // spectrum in the z pass (misc_kernels.cuh, lin_coef)
            g = g_c + g_f * f - (k.k_K3.mul(w) + k.k_K2.mul(((T)3 * u2 - D - (T)1) * f));
            h = w;
        }
        (void)kappa;
    }
}

// sums of one real point: (u^2 - 1)^2 and (full) f^2 (phasefield.cpp:293-325;
// the volume comes from the k = 0 mode in the z pass)
template <class T>
__device__ __forceinline__ void reduce_point(const PC<T>& k, bool full, T u, T lap, Acc<T>& as, Acc<T>& af) {
    const T u2m = u * u - (T)1;
    as.add(u2m * u2m);
    if (full) {
        T f;
        if constexpr (sizeof(T) == 8) f = -lap * k.eps + u2m * u * k.ieps + u2m * k.C;  // fc (phasefield.cpp:318-325)
        else f = k.k_ieps.mul(u2m * u) - k.k_eps.mul(lap);
        af.add(f * f);
    }
}

// XY_FUSED point (FP32 form): the sums of reduce_point and the lambda-free
// partials of nonlin_point (g_c = g_f = 0) from one evaluation of f
template <class T>
__device__ __forceinline__ void fused_point(const PC<T>& k, bool euler, T u, T lap, Acc<T>& as, Acc<T>& af, T& g,
                                            T& h) {
    const T D = (T)1.5;
    const T u2 = u * u;
    const T u2m = u2 - (T)1;
    const T w = u2m * u;
    T f;
    if constexpr (sizeof(T) == 8) f = -lap * k.eps + w * k.ieps;
    else f = k.k_ieps.mul(w) - k.k_eps.mul(lap);
    as.add(u2m * u2m);
    af.add(f * f);
    if constexpr (sizeof(T) == 8) {  // not used by the FP64 form; kept total
        const T t = u * (u2 - (T)3);
        if (euler) {
            g = k.eta * ((T)3 * u2 - (T)1) * f * k.ieps2;
            h = f;
        } else {
            g = -k.eta * (D * t * k.ieps3 + ((T)3 * u2 - D - (T)1) * k.ieps2 * f);
            h = t;
        }
    } else if (euler) {
        g = k.k_K2.mul(((T)3 * u2 - (T)1) * f);
        h = f;
    } else {
        g = -(k.k_K3.mul(w) + k.k_K2.mul(((T)3 * u2 - D - (T)1) * f));
        h = w;
    }
}

// ---- two real points per complex slot, two FP32 lanes per instruction
// The fused passes hold real values two to a complex slot (x = 2m, 2m + 1), and
// every pointwise step treats the two alike, so they run as lane-wise float2
// arithmetic: packed FADD2 / FMUL2 / FFMA2 on sm_100 and later, the same IEEE
// round-to-nearest operations per lane (explicit, so never contracted).
namespace lane2 {
__device__ __forceinline__ float2 bc(float v) { return make_float2(v, v); }
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
__device__ __forceinline__ float2 add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
#else
__device__ __forceinline__ float2 add(float2 a, float2 b) { return make_float2(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y)); }
__device__ __forceinline__ float2 mul(float2 a, float2 b) { return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)); }
__device__ __forceinline__ float2 fma(float2 a, float2 b, float2 c) {
    return make_float2(fmaf(a.x, b.x, c.x), fmaf(a.y, b.y, c.y));
}
#endif
__device__ __forceinline__ float2 neg(float2 a) { return make_float2(-a.x, -a.y); }
__device__ __forceinline__ float2 sub(float2 a, float2 b) { return add(a, neg(b)); }
// x * k with k = hi + lo folded before the rounding (KC<float>::mul per lane)
__device__ __forceinline__ float2 kmul(const KC<float>& k, float2 x) { return fma(x, bc(k.hi), mul(x, bc(k.lo))); }
}  // namespace lane2

// two lanes of Acc<float> (per-lane TwoSum + FastTwoSum, as ff_add), joined at the end
struct Acc2 {
    float2 hi{0.f, 0.f}, lo{0.f, 0.f};
    __device__ __forceinline__ void add(float2 x, float2 xl) {
        using namespace lane2;
        const float2 s = lane2::add(hi, x);
        const float2 bp = sub(s, hi);
        const float2 e = lane2::add(lane2::add(sub(hi, sub(s, bp)), sub(x, bp)), lane2::add(lo, xl));
        hi = lane2::add(s, e);
        lo = sub(e, sub(hi, s));
    }
    __device__ __forceinline__ FF part() const { return ff_add(FF{hi.x, lo.x}, FF{hi.y, lo.y}); }
};
// two lanes of PSum<float>
struct PSum2 {
    float2 s{0.f, 0.f};
    __device__ __forceinline__ void add(float2 x) { s = lane2::add(s, x); }
    __device__ __forceinline__ FF part() const { return ff_add(FF{s.x, 0.f}, FF{s.y, 0.f}); }
};

// u = U + v for the two points of a slot as double-float pairs (TwoSum, then
// FastTwoSum, per lane): U = (hi0, lo0, hi1, lo1) the state's real-space field,
// v the FP32 transform of u - u_state
__device__ __forceinline__ void ff_add_f2(float4 U, float2 v, float2& uh, float2& ul) {
    using namespace lane2;
    const float2 Uh = make_float2(U.x, U.z), Ul = make_float2(U.y, U.w);
    const float2 s = lane2::add(Uh, v);
    const float2 bp = sub(s, Uh);
    const float2 e = lane2::add(lane2::add(sub(Uh, sub(s, bp)), sub(v, bp)), Ul);
    uh = lane2::add(s, e);
    ul = sub(e, sub(uh, s));
}

// XY_FUSED points of the FP32 form (two per slot, lane-wise) from u = uh + ul.
// u^2 - 1 is formed as an unevaluated pair: uh^2 = p + pe exactly (TwoProd),
// p - 1 = s + se exactly (TwoSum), plus pe, se and 2 uh ul, so u^2 - 1 and
// w = (u^2 - 1) u keep their relative accuracy where u = +-1 + d with d far
// below FP32's spacing at 1.  Its square is summed to the same accuracy: that
// sum carries S, whose error moves the area penalty's lambda2 and, through it,
// the volume (a plain FP32 u^2 - 1 put ~1e-8 into S).  Otherwise as
// fused_point<float>.
//
// With CURV (spontaneous curvature C, the reference's commented-out formulas,
// phasefield.cpp:183-250) f gives way to fc = f + C (u^2 - 1) in the energy sum and in the
// Euler partial, the curvature part of the variational derivative joins G'', and the third
// output q = C (u^2 - 1) (Euler) or eps C (u^2 - 1) (ETD) carries the term whose Laplacian
// enters N: it is transformed like H and takes H's spectral multiplier (beta cx |k|^2),
// while H itself stays f (Euler) or w (ETD), the field the lambda2 term is rebuilt from.
template <bool CURV = false>
__device__ __forceinline__ void fused_point_u2(const PC<float>& k, bool euler, float2 uh, float2 ul, float2 lap,
                                               Acc2& as, Acc2& af, float2& g, float2& h, float2* q = nullptr) {
    using namespace lane2;
    const float2 one = bc(1.f), mone = bc(-1.f);
    const float2 p = mul(uh, uh);
    const float2 pe = fma(uh, uh, neg(p));
    const float2 s = lane2::add(p, mone);
    const float2 sb = sub(s, p);
    const float2 se = lane2::add(sub(p, sub(s, sb)), sub(mone, sb));
    const float2 t = lane2::add(lane2::add(se, pe), mul(mul(bc(2.f), uh), ul));
    const float2 u2m = lane2::add(s, t);
    const float2 tb = sub(u2m, s);
    const float2 u2m_lo = lane2::add(sub(s, sub(u2m, tb)), sub(t, tb));
    const float2 sq = mul(u2m, u2m);
    const float2 u2 = lane2::add(u2m, one);
    const float2 w = mul(u2m, uh);
    const float2 f = sub(kmul(k.k_ieps, w), kmul(k.k_eps, lap));
    as.add(sq, lane2::add(fma(u2m, u2m, neg(sq)), mul(mul(bc(2.f), u2m), u2m_lo)));
    if constexpr (CURV) {
        const float2 cu = mul(u2m, bc(k.C));
        const float2 fc = lane2::add(f, cu);
        af.add(mul(fc, fc), bc(0.f));
        *q = mul(u2m, bc(k.qC));
        const float2 t3 = sub(mul(bc(3.f), u2), one);  // 3 u^2 - 1
        if (euler) {  // eta (3u^2 - 1 + 2 eps u C) fc / eps^2
            g = kmul(k.k_K2, mul(lane2::add(t3, mul(bc(k.e2C), uh)), fc));
            h = f;
        } else {  // ... - eta ((3u^2 - 1) cu + 2 eps u C fc) / eps^2
            g = neg(lane2::add(kmul(k.k_K3, w), kmul(k.k_K2, mul(sub(mul(bc(3.f), u2), bc(2.5f)), f))));
            g = sub(g, kmul(k.k_K2, lane2::add(mul(t3, cu), mul(mul(bc(k.e2C), uh), fc))));
            h = w;
        }
    } else {
        (void)q;
        af.add(mul(f, f), bc(0.f));
        if (euler) {
            g = kmul(k.k_K2, mul(sub(mul(bc(3.f), u2), one), f));
            h = f;
        } else {
            g = neg(lane2::add(kmul(k.k_K3, w), kmul(k.k_K2, mul(sub(mul(bc(3.f), u2), bc(2.5f)), f))));
            h = w;
        }
    }
}

}  // namespace cb
