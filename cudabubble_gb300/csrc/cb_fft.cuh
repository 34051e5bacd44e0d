// Device primitives for the GB300 spectral stepper: complex helpers,
// register-resident DFT codelets, and in-place shared-memory line FFTs.
//
// Line FFTs of length L = R1*R2 are split into two register phases (a
// "four-step" factorisation).  Two in-place variants exist:
//   * fft_lines_NT: natural-order input  -> "transposed"-order output;
//   * fft_lines_TN: "transposed"-order input -> natural-order output.
// Element k of a transposed line lives at position tpos<L>(k) =
// (k / R1) + R2 * (k % R1).  Every phase reads and writes the same slots, so
// threads never race on a permutation and only a __syncthreads() separates
// the two phases.  A transform and its inverse are always paired NT then TN,
// so no explicit reordering pass is ever needed.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <type_traits>
#include <utility>

namespace cb {

// ------------------------------------------- programmatic dependent launch
// The stepper's kernels are launched with programmatic stream serialisation, so a
// kernel's CTAs are scheduled while the previous kernel in the stream still runs.
// Each kernel lets its successor launch at once (CB_PDL_TRIGGER) and, before it reads
// anything an earlier kernel wrote, waits for the previous grid to complete with its
// memory visible (CB_PDL_WAIT).  Work before the wait may touch only what no kernel
// of the stream writes (twiddle tables, instance descriptors).  Without a programmatic
// predecessor the wait returns at once.
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 900
#define CB_PDL_TRIGGER() asm volatile("griddepcontrol.launch_dependents;" ::: "memory")
#define CB_PDL_WAIT() asm volatile("griddepcontrol.wait;" ::: "memory")
#else
#define CB_PDL_TRIGGER() ((void)0)
#define CB_PDL_WAIT() ((void)0)
#endif

// Release / acquire fence at GPU scope for the counters the kernels sync through (the
// last CTA of a pass, the persistent batch's phase counters): fence.acq_rel orders this
// thread's (and, through the CTA barrier before it, its block's) writes before the
// counter update that follows, and the counter read before the reads that follow.  A
// build with -DCB_FENCE_SC uses __threadfence (fence.sc.gpu) instead.
#if defined(__CUDA_ARCH__) && !defined(CB_FENCE_SC)
#define CB_FENCE() asm volatile("fence.acq_rel.gpu;" ::: "memory")
#else
#define CB_FENCE() __threadfence()
#endif

// The threads a pass body runs on.  Cta: the whole CTA (threadIdx.x, __syncthreads).
// Grp: one of the equal thread groups a CTA of the persistent batched kernel splits into
// (mega.cuh), synchronised by its own named barrier `id` (1..15) over its n threads;
// the groups are whole warps.  Every body and line transform takes one and uses only its
// thread index, size and barrier.  Index and size are unsigned like threadIdx.x and
// blockDim.x: with int the block sums compiled differently and the 128^2 fused plane pass
// measured 1.2 % slower.
#if defined(__CUDA_ARCH__)
#define CB_NAMED_SYNC(id, n) asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory")
#elif defined(CB_EMULATION)
#define CB_NAMED_SYNC(id, n) ::emu::named_sync(id, n)
#else
#define CB_NAMED_SYNC(id, n) ((void)(id), (void)(n))
#endif
struct Cta {
    __device__ __forceinline__ unsigned tid() const { return threadIdx.x; }
    __device__ __forceinline__ unsigned size() const { return blockDim.x; }
    __device__ __forceinline__ void sync() const { __syncthreads(); }
};
struct Grp {
    int id, n, t;  // named barrier, threads, this thread's index in the group
    __device__ __forceinline__ unsigned tid() const { return (unsigned)t; }
    __device__ __forceinline__ unsigned size() const { return (unsigned)n; }
    __device__ __forceinline__ void sync() const { CB_NAMED_SYNC(id, n); }
};

// ---------------------------------------------------------------- complex
template <class T> struct CT;
template <> struct CT<float> { using type = float2; };
template <> struct CT<double> { using type = double2; };
template <class T> using cplx = typename CT<T>::type;

template <class C> __device__ __forceinline__ C cmk(decltype(C::x) a, decltype(C::x) b) { C r; r.x = a; r.y = b; return r; }
template <class C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <class C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <class C> __device__ __forceinline__ C cmul(C a, C b) { return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x); }
template <class C> __device__ __forceinline__ C cmulc(C a, C b) { return cmk<C>(a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y); }  // a*conj(b)
template <class C> __device__ __forceinline__ C cconj(C a) { return cmk<C>(a.x, -a.y); }
template <class C, class T> __device__ __forceinline__ C cscale(C a, T s) { return cmk<C>(a.x * s, a.y * s); }
// multiply by -i (forward) or +i (inverse)
template <bool INV, class C> __device__ __forceinline__ C cmul_mi(C a) { return INV ? cmk<C>(-a.y, a.x) : cmk<C>(a.y, -a.x); }
// FP32 complex add / subtract as one packed instruction (FADD2, sm_100 and later):
// the same two IEEE round-to-nearest additions in one issue slot
#if defined(__CUDA_ARCH__) && __CUDA_ARCH__ >= 1000
template <> __device__ __forceinline__ float2 cadd<float2>(float2 a, float2 b) { return __fadd2_rn(a, b); }
template <> __device__ __forceinline__ float2 csub<float2>(float2 a, float2 b) {
    return __fadd2_rn(a, make_float2(-b.x, -b.y));
}
#endif

// ------------------------------------------------- compile-time twiddles
// cos(pi * a / b) for b in {6, 8}: the only angles the radix <= 16 codelets
// need.  Values are the exact algebraic constants cos(pi/8), sqrt(2)/2,
// sin(pi/8), sqrt(3)/2 written to double precision.
__host__ __device__ constexpr double cospi_frac(int a, int b) {
    // reduce to [0, 2b)
    return (b == 8)
        ? ((a % 16 + 16) % 16 == 0 ? 1.0 : (a % 16 + 16) % 16 == 1 ? 0.92387953251128675613
         : (a % 16 + 16) % 16 == 2 ? 0.70710678118654752440 : (a % 16 + 16) % 16 == 3 ? 0.38268343236508977173
         : (a % 16 + 16) % 16 == 4 ? 0.0 : (a % 16 + 16) % 16 == 5 ? -0.38268343236508977173
         : (a % 16 + 16) % 16 == 6 ? -0.70710678118654752440 : (a % 16 + 16) % 16 == 7 ? -0.92387953251128675613
         : (a % 16 + 16) % 16 == 8 ? -1.0 : (a % 16 + 16) % 16 == 9 ? -0.92387953251128675613
         : (a % 16 + 16) % 16 == 10 ? -0.70710678118654752440 : (a % 16 + 16) % 16 == 11 ? -0.38268343236508977173
         : (a % 16 + 16) % 16 == 12 ? 0.0 : (a % 16 + 16) % 16 == 13 ? 0.38268343236508977173
         : (a % 16 + 16) % 16 == 14 ? 0.70710678118654752440 : 0.92387953251128675613)
        : ((a % 12 + 12) % 12 == 0 ? 1.0 : (a % 12 + 12) % 12 == 1 ? 0.86602540378443864676
         : (a % 12 + 12) % 12 == 2 ? 0.5 : (a % 12 + 12) % 12 == 3 ? 0.0
         : (a % 12 + 12) % 12 == 4 ? -0.5 : (a % 12 + 12) % 12 == 5 ? -0.86602540378443864676
         : (a % 12 + 12) % 12 == 6 ? -1.0 : (a % 12 + 12) % 12 == 7 ? -0.86602540378443864676
         : (a % 12 + 12) % 12 == 8 ? -0.5 : (a % 12 + 12) % 12 == 9 ? 0.0
         : (a % 12 + 12) % 12 == 10 ? 0.5 : 0.86602540378443864676);
}
// cos / sin of 2*pi*m/R for R in {2, 3, 4, 6, 8, 12, 16}
__host__ __device__ constexpr double cos2pi(int m, int R) {
    return (R == 16) ? cospi_frac(m, 8) : (R == 8) ? cospi_frac(2 * m, 8) : (R == 4) ? cospi_frac(4 * m, 8)
         : (R == 2) ? cospi_frac(8 * m, 8) : (R == 12) ? cospi_frac(m, 6) : (R == 6) ? cospi_frac(2 * m, 6)
         : cospi_frac(4 * m, 6);
}
__host__ __device__ constexpr double sin2pi(int m, int R) {  // sin(x) = cos(x - pi/2)
    return (R == 16) ? cospi_frac(m - 4, 8) : (R == 8) ? cospi_frac(2 * m - 4, 8) : (R == 4) ? cospi_frac(4 * m - 4, 8)
         : (R == 2) ? cospi_frac(8 * m - 4, 8) : (R == 12) ? cospi_frac(m - 3, 6) : (R == 6) ? cospi_frac(2 * m - 3, 6)
         : cospi_frac(4 * m - 3, 6);
}
// W_R^m = exp(-+ 2 pi i m / R): forward uses the minus sign
template <class C, bool INV> __device__ __forceinline__ C wconst(int m, int R) {
    using T = decltype(C::x);
    return cmk<C>((T)cos2pi(m, R), INV ? (T)sin2pi(m, R) : -(T)sin2pi(m, R));
}

template <bool INV, class C> __device__ __forceinline__ C tw_get_pre(C w) { return INV ? cconj(w) : w; }

// ------------------------------------------- gain-unbiased FP32 twiddles
// A twiddle rounded to FP32 has |w| != 1 by up to ~6e-8, and the rounding of
// a given constant has the same sign every time it is applied: the FP32
// transforms then carried a systematic gain of ~-6e-9 on the field, which the
// energy (a near-cancellation of eps lap u and (u^3 - u) / eps) amplified to
// ~5e-7.  In the FP32 form every twiddle is therefore split w = hi + lo and the
// product a * w is formed with the lo part folded in before the one rounding,
// so the only errors left are unbiased roundings.  The FP64 form keeps plain
// products.
__device__ __forceinline__ float2 cmul_comp(float2 a, float c, float s, float cl, float sl) {
    // (packed FFMA2 / FMUL2 forms need the operand broadcasts (a.x, a.x), (a.y, a.y) and
    // lane swaps of the twiddle; measured on GB300 they cost what they save)
    const float rx = fmaf(a.x, c, fmaf(-a.y, s, fmaf(-a.y, sl, a.x * cl)));
    const float ry = fmaf(a.x, s, fmaf(a.y, c, fmaf(a.y, cl, a.x * sl)));
    return make_float2(rx, ry);
}
// a * W_R^M (conjugated for INV) with compile-time M, R
template <bool INV, int M, int R, class C> __device__ __forceinline__ C wmul(C a) {
    if constexpr (sizeof(decltype(C::x)) == 8) {
        return cmul(a, wconst<C, INV>(M, R));
    } else {
        constexpr double c = cos2pi(M, R), s = INV ? sin2pi(M, R) : -sin2pi(M, R);
        constexpr float ch = (float)c, sh = (float)s;
        constexpr float cl = (float)(c - (double)ch), sl = (float)(s - (double)sh);
        if constexpr (cl == 0.f && sl == 0.f) return cmul(a, make_float2(ch, sh));
        else return cmul_comp(a, ch, sh, cl, sl);
    }
}
// a * table twiddle m (forward sign stored; conjugated for INV).  FP32 tables
// carry their lo parts in a second array `lo` of the same length.
template <bool INV> __device__ __forceinline__ double2 twmul(double2 a, const double2* hi, const double2*, int m) {
    return cmul(a, tw_get_pre<INV>(hi[m]));
}
template <bool INV> __device__ __forceinline__ float2 twmul(float2 a, const float2* hi, const float2* lo, int m) {
    const float2 h = hi[m], l = lo[m];
    return INV ? cmul_comp(a, h.x, -h.y, l.x, -l.y) : cmul_comp(a, h.x, h.y, l.x, l.y);
}
// x * k for a real constant k: FP64 plain; FP32 with k = hi + lo folded
template <class T> struct KC;
template <> struct KC<double> {
    double v;
    __device__ __forceinline__ double mul(double x) const { return x * v; }
};
template <> struct KC<float> {
    float hi, lo;
    __device__ __forceinline__ float mul(float x) const { return fmaf(x, hi, x * lo); }
};

// compile-time loop: f(std::integral_constant<int, i>) for i in [0, N)
template <class F, int... Is>
__device__ __forceinline__ void sfor_impl(F&& f, std::integer_sequence<int, Is...>) {
    (f(std::integral_constant<int, Is>{}), ...);
}
template <int N, class F> __device__ __forceinline__ void sfor(F&& f) {
    sfor_impl(f, std::make_integer_sequence<int, N>{});
}

// ------------------------------------------------------------ codelets
// In-register DFT of size R, natural order in and out:
// A[k] = sum_j a[j] * W_R^{jk}, W_R = exp(-2 pi i / R) (forward) or its conjugate.
template <int R, bool INV, class C> struct DFT;

template <bool INV, class C> struct DFT<1, INV, C> {
    static __device__ __forceinline__ void run(C*) {}
};
template <bool INV, class C> struct DFT<2, INV, C> {
    static __device__ __forceinline__ void run(C* a) {
        C t = a[0];
        a[0] = cadd(t, a[1]);
        a[1] = csub(t, a[1]);
    }
};
template <bool INV, class C> struct DFT<3, INV, C> {
    static __device__ __forceinline__ void run(C* a) {
        using T = decltype(C::x);
        C s = cadd(a[1], a[2]);
        C d = csub(a[1], a[2]);
        C m = cmk<C>(a[0].x - (T)0.5 * s.x, a[0].y - (T)0.5 * s.y);
        C r = cmul_mi<INV>(d);  // -i d (fwd) / +i d (inv)
        a[0] = cadd(a[0], s);
        C hr;
        if constexpr (sizeof(T) == 8) {
            const T h = (T)0.86602540378443864676;
            hr = cmk<C>(h * r.x, h * r.y);
        } else {  // sqrt(3)/2 = hi + lo, folded before the rounding
            constexpr double hd = 0.86602540378443864676;
            constexpr float hh = (float)hd, hl = (float)(hd - (double)hh);
            hr = cmk<C>(fmaf(r.x, hh, r.x * hl), fmaf(r.y, hh, r.y * hl));
        }
        a[1] = cmk<C>(m.x + hr.x, m.y + hr.y);
        a[2] = cmk<C>(m.x - hr.x, m.y - hr.y);
    }
};
template <bool INV, class C> struct DFT<4, INV, C> {
    static __device__ __forceinline__ void run(C* a) {
        C s0 = cadd(a[0], a[2]), d0 = csub(a[0], a[2]);
        C s1 = cadd(a[1], a[3]), d1 = cmul_mi<INV>(csub(a[1], a[3]));
        a[0] = cadd(s0, s1);
        a[2] = csub(s0, s1);
        a[1] = cadd(d0, d1);
        a[3] = csub(d0, d1);
    }
};
template <int R> struct Split {  // R = P * Q with P in {4, 3, 2}
    static constexpr int P = (R % 4 == 0 && R != 4) ? 4 : (R % 3 == 0 && R != 3) ? 3 : 2;
    static constexpr int Q = R / P;
};
// composite codelet: four-step in registers with compile-time twiddles
template <int R, bool INV, class C> struct DFT {
    static __device__ __forceinline__ void run(C* a) {
        constexpr int P = Split<R>::P, Q = Split<R>::Q;  // input j = j2 + Q*j1, output k = k1 + P*k2
        C y[R];
        sfor<Q>([&](auto J2) {
            constexpr int j2 = decltype(J2)::value;
            C t[P];
#pragma unroll
            for (int j1 = 0; j1 < P; ++j1) t[j1] = a[j2 + Q * j1];
            DFT<P, INV, C>::run(t);
            sfor<P>([&](auto K1) {
                constexpr int k1 = decltype(K1)::value;
                if constexpr (j2 * k1 == 0) y[j2 + Q * k1] = t[k1];
                else y[j2 + Q * k1] = wmul<INV, (j2 * k1) % R, R>(t[k1]);
            });
        });
#pragma unroll
        for (int k1 = 0; k1 < P; ++k1) {
            C t[Q];
#pragma unroll
            for (int j2 = 0; j2 < Q; ++j2) t[j2] = y[j2 + Q * k1];
            DFT<Q, INV, C>::run(t);
#pragma unroll
            for (int k2 = 0; k2 < Q; ++k2) a[k1 + P * k2] = t[k2];
        }
    }
};

// ------------------------------------------------- line FFT factorisation
template <int L> struct Plan;  // L = R1 * R2, both <= 16
template <> struct Plan<8> { static constexpr int R1 = 8, R2 = 1; };
template <> struct Plan<12> { static constexpr int R1 = 12, R2 = 1; };
template <> struct Plan<16> { static constexpr int R1 = 16, R2 = 1; };
template <> struct Plan<24> { static constexpr int R1 = 8, R2 = 3; };
template <> struct Plan<32> { static constexpr int R1 = 8, R2 = 4; };
template <> struct Plan<48> { static constexpr int R1 = 8, R2 = 6; };
template <> struct Plan<64> { static constexpr int R1 = 8, R2 = 8; };
// the split of the 96- and 128-point lines is a build-time schedule (CB_PLAN96_12X8,
// CB_PLAN128_8X16), chosen with the launch shapes by the schedule tuner (tune.py)
#ifdef CB_PLAN96_12X8
template <> struct Plan<96> { static constexpr int R1 = 12, R2 = 8; };
#else
template <> struct Plan<96> { static constexpr int R1 = 16, R2 = 6; };
#endif
#ifdef CB_PLAN128_8X16
template <> struct Plan<128> { static constexpr int R1 = 8, R2 = 16; };
#else
template <> struct Plan<128> { static constexpr int R1 = 16, R2 = 8; };
#endif
template <> struct Plan<192> { static constexpr int R1 = 16, R2 = 12; };
template <> struct Plan<256> { static constexpr int R1 = 16, R2 = 16; };

// slot of output element k of an NT transform (identity when R2 == 1)
template <int L> __host__ __device__ __forceinline__ int tpos(int k) {
    constexpr int R1 = Plan<L>::R1, R2 = Plan<L>::R2;
    return (R2 == 1) ? k : (k / R1) + R2 * (k % R1);
}
// element index held by slot p of a transposed line (inverse of tpos)
template <int L> __host__ __device__ __forceinline__ int tidx(int p) {
    constexpr int R1 = Plan<L>::R1, R2 = Plan<L>::R2;
    return (R2 == 1) ? p : (p / R2) + R1 * (p % R2);
}


// Line offsets: line l starts at buf + off(l).
struct LinearLines {
    int ls;
    __device__ __forceinline__ int operator()(int l) const { return l * ls; }
};
// two fields side by side in one padded plane: lines [0, n1) are rows of
// field 0, lines [n1, 2 n1) rows of field 1 (which starts `second` slots in)
template <int N1, int PITCH, int SECOND>
struct PairRows {
    __device__ __forceinline__ int operator()(int l) const {
        return (l < N1) ? l * PITCH : (l - N1) * PITCH + SECOND;
    }
};

// three fields: rows of field 0 and field 1 side by side in one padded plane (as
// PairRows), then rows of a third field in a region of its own, QOFF slots in, pitch QX
template <int N1, int PITCH, int SECOND, int QOFF, int QX>
struct TripleRows {
    __device__ __forceinline__ int operator()(int l) const {
        return (l < N1) ? l * PITCH : (l < 2 * N1) ? (l - N1) * PITCH + SECOND : QOFF + (l - 2 * N1) * QX;
    }
};

// NT: natural in -> transposed out.  Lines l in [0, nlines) at buf + off(l),
// element stride es.  All NTHR threads of the block call it; caller syncs after.
template <int L, bool INV, int NTHR, int NLINES, class C, class OFF, class G = Cta>
__device__ __forceinline__ void fft_lines_NT(C* buf, OFF off, int es, const C* tw, const C* twlo, const G& g = G()) {
    constexpr int nlines = NLINES;
    constexpr int R1 = Plan<L>::R1, R2 = Plan<L>::R2;
    const int tid = g.tid();
    if constexpr (R2 == 1) {
        for (int l = tid; l < nlines; l += NTHR) {
            C a[R1];
            C* p = buf + off(l);
#pragma unroll
            for (int j = 0; j < R1; ++j) a[j] = p[j * es];
            DFT<R1, INV, C>::run(a);
#pragma unroll
            for (int j = 0; j < R1; ++j) p[j * es] = a[j];
        }
    } else {
    // phase A: for each (line, j2) DFT_R1 over j1 of x[j2 + R2 j1], twiddle W_L^{j2 k1}
    for (int it = tid; it < nlines * R2; it += NTHR) {
        const int l = it % nlines, j2 = it / nlines;
        C* p = buf + off(l) + j2 * es;
        C a[R1];
#pragma unroll
        for (int j1 = 0; j1 < R1; ++j1) a[j1] = p[j1 * R2 * es];
        DFT<R1, INV, C>::run(a);
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) {
            C v = (k1 == 0) ? a[k1] : twmul<INV>(a[k1], tw, twlo, (j2 * k1) % L);
            p[k1 * R2 * es] = v;
        }
    }
    g.sync();
    // phase B: for each (line, k1) DFT_R2 over j2 of the contiguous block at R2*k1
    for (int it = tid; it < nlines * R1; it += NTHR) {
        const int l = it % nlines, k1 = it / nlines;
        C* p = buf + off(l) + (R2 * k1) * es;
        C a[R2];
#pragma unroll
        for (int j2 = 0; j2 < R2; ++j2) a[j2] = p[j2 * es];
        DFT<R2, INV, C>::run(a);
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) p[k2 * es] = a[k2];
    }
    }
}

// TN: transposed in -> natural out (input element j = j1 + R1 j2 sits at
// slot j2 + R2 j1, exactly where an NT transform leaves element j).
template <int L, bool INV, int NTHR, int NLINES, class C, class OFF, class G = Cta>
__device__ __forceinline__ void fft_lines_TN(C* buf, OFF off, int es, const C* tw, const C* twlo, const G& g = G()) {
    constexpr int nlines = NLINES;
    constexpr int R1 = Plan<L>::R1, R2 = Plan<L>::R2;
    const int tid = g.tid();
    if constexpr (R2 == 1) {
        fft_lines_NT<L, INV, NTHR, NLINES, C, OFF, G>(buf, off, es, tw, twlo, g);
    } else {
    // phase A: for each (line, j1) DFT_R2 over j2 (contiguous block at R2*j1), twiddle W_L^{j1 k2}
    for (int it = tid; it < nlines * R1; it += NTHR) {
        const int l = it % nlines, j1 = it / nlines;
        C* p = buf + off(l) + (R2 * j1) * es;
        C a[R2];
#pragma unroll
        for (int j2 = 0; j2 < R2; ++j2) a[j2] = p[j2 * es];
        DFT<R2, INV, C>::run(a);
#pragma unroll
        for (int k2 = 0; k2 < R2; ++k2) {
            C v = (k2 == 0) ? a[k2] : twmul<INV>(a[k2], tw, twlo, (j1 * k2) % L);
            p[k2 * es] = v;
        }
    }
    g.sync();
    // phase B: for each (line, k2) DFT_R1 over j1 at stride R2 -> X[k2 + R2 k1] at the same slots
    for (int it = tid; it < nlines * R2; it += NTHR) {
        const int l = it % nlines, k2 = it / nlines;
        C* p = buf + off(l) + k2 * es;
        C a[R1];
#pragma unroll
        for (int j1 = 0; j1 < R1; ++j1) a[j1] = p[j1 * R2 * es];
        DFT<R1, INV, C>::run(a);
#pragma unroll
        for (int k1 = 0; k1 < R1; ++k1) p[k1 * R2 * es] = a[k1];
    }
    }
}

// ------------------------------------------------------------ reductions
// Sums are carried as FP32 double-float pairs (hi + lo) up to the warp level,
// so no FP64 instruction runs per thread; only the per-warp partials of a
// block are added in FP64 (GB300's FP64 rate is a small fraction of FP32).
struct FF {
    float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b) {
    const float s = a.hi + b.hi;
    const float bp = s - a.hi;
    float e = (a.hi - (s - bp)) + (b.hi - bp);  // TwoSum
    e += a.lo + b.lo;
    FF r;
    r.hi = s + e;                                 // FastTwoSum
    r.lo = e - (r.hi - s);
    return r;
}
__device__ __forceinline__ FF warp_sum(FF v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = ff_add(v, w);
    }
    return v;
}
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// Sum of `nparts` FP64 partials (NV interleaved values each, stride NV) by a
// whole block: strided loads, a warp-shuffle tree, then the per-warp sums.
// The result is valid in thread 0.  Keeps the dependent FP64 chain short; a
// single thread walking hundreds of partials dominated the kernels' tails.
template <int NV, class G = Cta>
__device__ __forceinline__ void block_sum_parts(const double* part, int nparts, double* out, double* red,
                                                const G& g = G()) {
    double v[NV];
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = 0.0;
    for (int i = g.tid(); i < nparts; i += g.size()) {
#pragma unroll
        for (int j = 0; j < NV; ++j) v[j] += __ldcg(part + (size_t)NV * i + j);
    }
    const int lane = g.tid() & 31, w = g.tid() >> 5, nw = (g.size() + 31) >> 5;
#pragma unroll
    for (int j = 0; j < NV; ++j) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[j] += __shfl_xor_sync(0xffffffffu, v[j], o);
    }
    g.sync();
    if (lane == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) red[j * 32 + w] = v[j];
    }
    g.sync();
    if (g.tid() == 0) {
#pragma unroll
        for (int j = 0; j < NV; ++j) {
            double s = 0.0;
            for (int k = 0; k < nw; ++k) s += red[j * 32 + k];
            out[j] = s;
        }
    }
}

// Block-wide sum of NV values (FF pairs or doubles); the FP64 result is valid
// in thread 0.  `red` must hold 32*NV doubles of shared memory.
template <int NV, class V, class G = Cta>
__device__ __forceinline__ void block_sum(V* v, double* out, double* red, const G& g = G()) {
    const int lane = g.tid() & 31, w = g.tid() >> 5, nw = (g.size() + 31) >> 5;
#pragma unroll
    for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
    g.sync();
    if (lane == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            if constexpr (std::is_same<V, FF>::value) red[i * 32 + w] = (double)v[i].hi + (double)v[i].lo;
            else red[i * 32 + w] = (double)v[i];
        }
    }
    g.sync();
    if (g.tid() == 0) {
#pragma unroll
        for (int i = 0; i < NV; ++i) {
            double s = 0.0;
            for (int k = 0; k < nw; ++k) s += red[i * 32 + k];
            out[i] = s;
        }
    }
}

}  // namespace cb
