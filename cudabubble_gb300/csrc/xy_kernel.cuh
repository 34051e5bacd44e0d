// xy-plane pass: one CTA owns one z-plane of one instance.
//
// Input is a "partial" plane (real z, spectral ky/kx) of the half spectrum:
// P0 = IFFT_z(u-hat) and P2 = IFFT_z(-cx kz^2 u-hat).  In shared memory the
// plane is packed to nx/2 complex columns: the kx = 0 and kx = nx/2 columns
// are both Hermitian in ky, so they travel together as col0 + i*colN through
// the y transform and come out as the real and imaginary parts.  The x
// transform is a real transform done through a half-length complex FFT.
//
// Modes
//   XY_REDUCE_FULL  u, lap u -> f; FP64 sums of u, (u^2-1)^2, f^2  (V, S, E_el, E)
//   XY_REDUCE_S     u only; sums of u, (u^2-1)^2                    (V, S)
//   XY_NONLIN       u, lap u -> pointwise nonlinearity G and H, forward xy
//                   transforms, written as the partials A = G^ + beta cx (kx^2+ky^2) H^
//                   and B = H^ that the z pass turns into the nonlinear spectrum
//   XY_FUSED        (FP32 form) the sums of XY_REDUCE_FULL and, with lambda = 0,
//                   the partials of XY_NONLIN, in one pass; the z pass adds the
//                   penalty terms lambda1, lambda2 f spectrally once the sums exist
//   XY_INV_PLAIN    partial -> real plane (double out)
//   XY_FWD_PLAIN    real plane (double in) -> partial
// The pointwise formulas restate Calc.cu:153-162 (f), :171-180 (g0),
// :265-284 (nld), :358-368 (s), :410-437 (nld1/nld2).
#pragma once
#include "cb_fft.cuh"
#include "cb_inst.h"
#include "cb_kargs.h"
#include "pointwise.cuh"

namespace cb {

__device__ __forceinline__ int part_set(const Ctrl* ctrl, int role) {
    return role == R_WORK ? 2 : (role == R_STATE ? ctrl->part_state : 1 - ctrl->part_state);
}

// Finalise the FP64 scalars of one state from the per-plane sums
// (phasefield.cpp:283-325, belastic.cpp:68-86); thread 0 of the last CTA.
__device__ inline void finalize_xy(const Params& p, Ctrl* ctrl, const double* sums, int role, bool full) {
    const double ss = sums[1], sf = sums[2];
    Scal& s = ctrl->sc[role];
    s.sum_g = sums[0];
    s.sum_h = sums[3];
    const double c3 = 1.0606601717798212866;  // 3 / (2 sqrt 2)
    // V comes from the exact k = 0 mode the z pass stored in sum_u
    s.sum_s2 = ss;
    s.V = (s.sum_u * p.invN + 1.0) * 0.5 * p.L3;
    s.S = (0.5 * p.eps * s.grad2 + 0.25 * p.d_ieps * (ss * p.invN)) * c3 * p.L3;
    if (full) {
        s.sum_f2 = sf;
        s.E_el = (sf * p.invN) * (0.5 * p.d_ieps) * p.L3;
        const double ve = s.V - ctrl->alpha, se = s.S - ctrl->beta;
        s.E = p.eta * s.E_el + 0.5 * p.M1 * ve * ve + 0.5 * p.M2 * se * se;
    }
}

// Per-CTA partial sums (slot `slot` of `nslots`) of (u^2 - 1)^2, f^2 and, with
// NV = 4 (XY_FUSED), of the partials G'' and w; then the last CTA of the
// instance finalises the role's scalars; all threads call.
template <class T, int NV = 2, class V, class G = Cta>
__device__ inline void xy_sums_finalize(const InstT<T>& I, Ctrl* ctrl, const Params& p, int slot, int nslots, V* vv,
                                        double* red, int role, bool full, const G& g = G()) {
    static_assert(NV == 2 || NV == 4, "two or four sums");
    double v[NV];
    block_sum<NV>(vv, v, red, g);
    double* part = I.part_xy;
    int* last = reinterpret_cast<int*>(red + 128);
    if (g.tid() == 0) {
        part[4 * slot + 1] = v[0];
        part[4 * slot + 2] = v[1];
        if constexpr (NV == 4) {
            part[4 * slot + 0] = v[2];
            part[4 * slot + 3] = v[3];
        } else {
            part[4 * slot + 0] = 0.0;
            part[4 * slot + 3] = 0.0;
        }
        CB_FENCE();
        const unsigned done_blocks = atomicAdd(&ctrl->cnt_xy[role], 1u);
        *last = done_blocks == (unsigned)(nslots - 1);
    }
    g.sync();
    if (*last) {  // the last CTA of this instance finalises, with all its threads
        CB_FENCE();
        double sums[4];
        block_sum_parts<4>(part, nslots, sums, red, g);
        if (g.tid() == 0) {
            finalize_xy(p, ctrl, sums, role, full);
            ctrl->cnt_xy[role] = 0u;
        }
    }
}

// where a nonlinear pass leaves its two forward-transformed fields: the work
// pair A, B, or (XY_FUSED of the state / candidate) that role's G slot
// (and, for the FP32 form with curvature, its third field q in *Qo)
template <class T>
__device__ __forceinline__ void nl_outputs(const InstT<T>& I, const Ctrl* c, int mode, int role, void*& A, void*& B,
                                           void** Qo = nullptr) {
    if (mode == XY_FUSED && role != R_WORK) {
        const int sl = role == R_STATE ? c->ab_state : 1 - c->ab_state;
        A = I.G[sl][0];
        B = I.G[sl][1];
        if (Qo) *Qo = I.G[sl][2];
    } else {
        A = I.A;
        B = I.B;
        if (Qo) *Qo = I.Q;
    }
}

// NF = fields per plane: 2 for XY_REDUCE_FULL / XY_NONLIN / XY_FUSED, 1 otherwise.
// NQ = 1: the FP32 fused pass with spontaneous curvature, whose third output field q lives
// in a region of its own, [NY][M + 1] after the plane (pointwise.cuh, fused_point_u2)
//
// Plane z of instance I on this CTA, all NT threads: the body of xy_kernel (one plane per
// CTA, PDL = true: programmatic launch) and of the persistent batched kernel (mega.cuh,
// PDL = false).
template <class T, int NX, int NT, int NF, int NQ = 0, bool PDL = true, class G = Cta>
__device__ __forceinline__ void xy_body(const InstT<T>& I, const int z, const XYArgs a, unsigned char* smem_raw,
                                        const G& g = G()) {
    using C = cplx<T>;
    constexpr int M = NX / 2, NY = NX, NC = M + 1;
    constexpr int nf = NF;
    constexpr int pitch = nf * M + 1;
    constexpr int QX = M + 1, SQ = NQ ? NY * QX : 0;
    if constexpr (PDL) CB_PDL_TRIGGER();
    Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    const int tid = g.tid();
    if (z >= p.nz) return;
    C* S = reinterpret_cast<C*>(smem_raw);  // [NY][pitch]
    C* Qb = S + NY * pitch;                 // q (NQ = 1)
    C* twM = Qb + SQ;                       // W_M^m
    C* twN = twM + M;                       // W_NX^m
    C* twY = twN + NX;                      // W_NY^m
    // FP32: lo parts of the three tables (same order), FP64: unused aliases
    constexpr int ntw = sizeof(T) == 4 ? 2 : 1;
    C* twMl = twY + NY;
    C* twNl = twMl + M;
    C* twYl = twNl + NX;
    double* red = reinterpret_cast<double*>(twM + ntw * (M + NX + NY));

    {
        const C* gx = reinterpret_cast<const C*>(I.twx);
        const C* gy = reinterpret_cast<const C*>(I.twy);
        for (int i = tid; i < M + NX; i += NT) twM[i] = gx[i];  // twM and twN are contiguous
        for (int i = tid; i < NY; i += NT) twY[i] = gy[i];
        if constexpr (ntw == 2) {  // the tables' lo parts follow their hi parts
            for (int i = tid; i < M + NX; i += NT) twMl[i] = gx[M + NX + i];
            for (int i = tid; i < NY; i += NT) twYl[i] = gy[NY + i];
        }
    }
    // the twiddles (written by no kernel) are loaded; what follows reads the previous
    // kernel's results
    if constexpr (PDL) CB_PDL_WAIT();
    // the control fields in one batch of independent loads, so the CTA does not wait on a
    // chain of dependent loads before its data moves
    const int c_done = ctrl->done, c_fresh = ctrl->fresh, c_part = ctrl->part_state, c_u = ctrl->u_state;
    const bool stepping = a.mode <= XY_FUSED;
    if (stepping) {
        if (c_done) return;
        if (a.skip_if_stale && !c_fresh) return;
    }
    const T cx = PC<T>(p).cx;
    const size_t plane = (size_t)NY * NC;

    if (a.mode == XY_FWD_PLAIN) {
        // real plane in natural order -> transposed slots, as the TN transforms expect
        const double* src = a.rin + (size_t)z * NY * NX;
        for (int it = tid; it < NY * M; it += NT) {
            const int m = it % M, y = it / M;
            const double2 v = reinterpret_cast<const double2*>(src + (size_t)y * NX)[m];
            S[tpos<NY>(y) * pitch + tpos<M>(m)] = cmk<C>((T)v.x, (T)v.y);
        }
        g.sync();
    } else {
        const C* P0;
        const C* P2 = nullptr;
        if (a.mode == XY_INV_PLAIN) {
            P0 = reinterpret_cast<const C*>(a.cin) + (size_t)z * plane;
        } else {
            const int set = a.role == R_WORK ? 2 : (a.role == R_STATE ? c_part : 1 - c_part);  // part_set
            P0 = reinterpret_cast<const C*>(I.P[set][0]) + (size_t)z * plane;
            P2 = reinterpret_cast<const C*>(I.P[set][1]) + (size_t)z * plane;
        }
        // store one loaded element (and, in column 0, its Nyquist partner) into the plane
        auto put = [&](int it, C v, C w, C vN, C wN) {
            const int c = it % M, ky = it / M;
            if (c == 0) S[ky * pitch] = cmk<C>(v.x - vN.y, v.y + vN.x);  // col0 + i*colN
            else S[ky * pitch + c] = v;
            if (nf == 2) {  // laplacian partial Q = -cx (kx^2 + ky^2) P0 + P2 (Calc.cu:107-124)
                const int kyf = min(ky, NY - ky);
                if constexpr (sizeof(T) == 8) {
                    const T kyy = cx * (T)(kyf * kyf);
                    if (c == 0) {
                        const T kN = cx * (T)(M * M) + kyy;
                        const C q0 = cmk<C>(w.x - kyy * v.x, w.y - kyy * v.y);
                        const C qN = cmk<C>(wN.x - kN * vN.x, wN.y - kN * vN.y);
                        S[ky * pitch + M] = cmk<C>(q0.x - qN.y, q0.y + qN.x);
                    } else {
                        const T k2 = cx * (T)(c * c) + kyy;
                        S[ky * pitch + M + c] = cmk<C>(w.x - k2 * v.x, w.y - k2 * v.y);
                    }
                } else if (a.mode == XY_FUSED) {  // P2 holds the whole Laplacian (z_kernel.cuh)
                    if (c == 0) S[ky * pitch + M] = cmk<C>(w.x - wN.y, w.y + wN.x);
                    else S[ky * pitch + M + c] = w;
                } else {  // integer |k|^2 exact in FP32, cx folded hi + lo
                    const KC<T> kcx = PC<T>(p).k_cx;
                    auto q = [&](C ww, C vv, int kk) {
                        return cmk<C>(ww.x - kcx.mul((T)kk * vv.x), ww.y - kcx.mul((T)kk * vv.y));
                    };
                    if (c == 0) {
                        const C q0 = q(w, v, kyf * kyf), qN = q(wN, vN, M * M + kyf * kyf);
                        S[ky * pitch + M] = cmk<C>(q0.x - qN.y, q0.y + qN.x);
                    } else {
                        S[ky * pitch + M + c] = q(w, v, c * c + kyf * kyf);
                    }
                }
            }
        };
        // loads in batches of LB per thread, all issued before any is used: the
        // plane load is latency-bound with one load in flight per thread
        constexpr int LB = 4;
        constexpr int ITER = (NY * M + NT - 1) / NT;
        for (int b0 = 0; b0 < ITER; b0 += LB) {
            C v[LB], w[LB], vN[LB], wN[LB];
#pragma unroll
            for (int j = 0; j < LB; ++j) {
                const int it = tid + (b0 + j) * NT;
                v[j] = w[j] = vN[j] = wN[j] = cmk<C>(0, 0);
                if (b0 + j < ITER && it < NY * M) {
                    const int c = it % M, ky = it / M;
                    v[j] = __ldg(P0 + ky * NC + c);
                    if (nf == 2) w[j] = __ldg(P2 + ky * NC + c);
                    if (c == 0) {
                        vN[j] = __ldg(P0 + ky * NC + M);
                        if (nf == 2) wN[j] = __ldg(P2 + ky * NC + M);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < LB; ++j) {
                const int it = tid + (b0 + j) * NT;
                if (b0 + j < ITER && it < NY * M) put(it, v[j], w[j], vN[j], wN[j]);
            }
        }
        g.sync();
        // ---- y inverse (natural in, transposed out) on nf*M columns
        fft_lines_NT<NY, true, NT, nf * M>(S, LinearLines{1}, pitch, twY, twYl, g);
        g.sync();
        // ---- x C2R: half-length pre-processing, then inverse M-point FFT per row
        const PairRows<NY, pitch, M> rows;
        for (int it = tid; it < nf * NY * (M / 2 + 1); it += NT) {
            const int l = it % (nf * NY), k = it / (nf * NY);
            C* row = S + rows(l);
            if (k == 0) {
                const C v = row[0];  // X[0] + i X[M], both real
                row[0] = cmk<C>(v.x + v.y, v.x - v.y);
            } else {
                const int k2 = M - k;
                const C xk = row[k], xk2 = row[k2];
                {
                    const C e = cadd(xk, cconj(xk2));
                    const C o = twmul<true>(csub(xk, cconj(xk2)), twN, twNl, k);  // * W_N^{-k}
                    row[k] = cmk<C>(e.x - o.y, e.y + o.x);            // e + i o
                }
                if (k2 != k) {
                    const C e = cadd(xk2, cconj(xk));
                    const C o = twmul<true>(csub(xk2, cconj(xk)), twN, twNl, k2);
                    row[k2] = cmk<C>(e.x - o.y, e.y + o.x);
                }
            }
        }
        g.sync();
        fft_lines_NT<M, true, NT, nf * NY>(S, rows, 1, twM, twMl, g);
        g.sync();

        if (a.mode == XY_INV_PLAIN) {
            double* dst = a.rout + (size_t)z * NY * NX;
            for (int it = tid; it < NY * M; it += NT) {
                const int m = it % M, y = it / M;
                const C v = S[tpos<NY>(y) * pitch + tpos<M>(m)];
                reinterpret_cast<double2*>(dst + (size_t)y * NX)[m] = make_double2((double)v.x, (double)v.y);
            }
            return;
        }

        // ---- pointwise over all slots (order-free)
        const PC<T> k(p);
        if (a.mode == XY_NONLIN) {
            // lambdas formed once per CTA in FP64, broadcast in the kernel's precision
            T* lam = reinterpret_cast<T*>(red);
            const bool euler = p.method == M_EULER;
            if (tid == 0) nonlin_lambdas<T>(p, ctrl, a.role, lam);
            g.sync();
            const T g_c = lam[0];
            const T g_f = lam[1];
            for (int it = tid; it < NY * M; it += NT) {
                const int q = it % M, r = it / M;
                C* pu = S + r * pitch + q;
                C* pl = pu + M;
                const C uu = *pu, ll = *pl;
                C g, h;
                nonlin_point<T>(k, euler, g_c, g_f, uu.x, ll.x, g.x, h.x);
                nonlin_point<T>(k, euler, g_c, g_f, uu.y, ll.y, g.y, h.y);
                *pu = g;
                *pl = h;
            }
            g.sync();
        } else if (a.mode == XY_FUSED) {
            // sums of the state and its lambda-free partials G'', w in one sweep
            const bool euler = p.method == M_EULER;
            Acc<T> as, af;
            PSum<T> ag, ah;
            if constexpr (sizeof(T) == 4) {
                // u = U[u_state] + (u - u_state); the candidate pass keeps its u for the next state
                const float4* Us = reinterpret_cast<const float4*>(I.U[c_u]) + (size_t)z * NY * M;
                float4* Uo = a.role == R_CAND ? reinterpret_cast<float4*>(I.U[1 - c_u]) + (size_t)z * NY * M
                                              : nullptr;
                Acc2 as2, af2;
                PSum2 ag2, ah2;
                for (int it = tid; it < NY * M; it += NT) {
                    const int q = it % M, r = it / M;
                    const int ui = tidx<NY>(r) * M + q;  // row y, x slot q (stored in x-slot order)
                    const float4 Uv = __ldg(Us + ui);
                    C* pu = S + r * pitch + q;
                    C* pl = pu + M;
                    const C dd = *pu, ll = *pl;
                    float2 uh, ul;
                    ff_add_f2(Uv, dd, uh, ul);
                    if (Uo) Uo[ui] = make_float4(uh.x, ul.x, uh.y, ul.y);
                    float2 g, h, qv;
                    fused_point_u2<NQ == 1>(k, euler, uh, ul, ll, as2, af2, g, h, &qv);
                    ag2.add(g);
                    ah2.add(h);
                    *pu = g;
                    *pl = h;
                    if constexpr (NQ == 1) Qb[r * QX + q] = qv;
                }
                as.v = as2.part();
                af.v = af2.part();
                ag.s = ag2.s.x + ag2.s.y;
                ah.s = ah2.s.x + ah2.s.y;
            } else {
                for (int it = tid; it < NY * M; it += NT) {
                    const int q = it % M, r = it / M;
                    C* pu = S + r * pitch + q;
                    C* pl = pu + M;
                    const C uu = *pu, ll = *pl;
                    C g, h;
                    fused_point<T>(k, euler, uu.x, ll.x, as, af, g.x, h.x);
                    fused_point<T>(k, euler, uu.y, ll.y, as, af, g.y, h.y);
                    ag.add(g.x); ag.add(g.y);
                    ah.add(h.x); ah.add(h.y);
                    *pu = g;
                    *pl = h;
                }
            }
            auto pv = as.part();
            decltype(pv) vv[4] = {pv, af.part(), ag.part(), ah.part()};
            xy_sums_finalize<T, 4>(I, ctrl, p, z, p.nz, vv, red, a.role, true, g);
            g.sync();
        } else {
            // reductions (XY_REDUCE_FULL / XY_REDUCE_S)
            const bool full = a.mode == XY_REDUCE_FULL;
            Acc<T> as, af;
            for (int it = tid; it < NY * M; it += NT) {
                const int q = it % M, r = it / M;
                const C uu = S[r * pitch + q];
                const C ll = full ? S[r * pitch + M + q] : cmk<C>(0, 0);
                reduce_point<T>(k, full, uu.x, ll.x, as, af);
                reduce_point<T>(k, full, uu.y, ll.y, as, af);
            }
            auto pv = as.part();
            decltype(pv) vv[2] = {pv, af.part()};
            xy_sums_finalize<T>(I, ctrl, p, z, p.nz, vv, red, a.role, full, g);
            return;
        }
    }

    // ---- forward xy: x R2C (transposed in, natural out) then y (transposed in, natural out)
    constexpr int nfo = NF + NQ;  // XY_NONLIN / XY_FUSED (2 fields, 3 with q) or XY_FWD_PLAIN (1)
    const PairRows<NY, pitch, M> rows;
    const TripleRows<NY, pitch, M, NY * pitch, QX> rows3;
    auto xrow = [&](int l) { return NQ ? rows3(l) : rows(l); };
    if constexpr (NQ == 1) fft_lines_TN<M, false, NT, 3 * NY>(S, rows3, 1, twM, twMl, g);
    else fft_lines_TN<M, false, NT, nfo * NY>(S, rows, 1, twM, twMl, g);
    g.sync();
    for (int it = tid; it < nfo * NY * (M / 2 + 1); it += NT) {
        const int l = it % (nfo * NY), k = it / (nfo * NY);
        C* row = S + xrow(l);
        if (k == 0) {
            const C z0 = row[0];
            row[0] = cmk<C>(z0.x + z0.y, z0.x - z0.y);  // X[0] + i X[M]
        } else {
            const int k2 = M - k;
            const C zk = row[k], zk2 = row[k2];
            const T h = (T)0.5;
            {
                const C e = cadd(zk, cconj(zk2));
                const C d = twmul<false>(csub(zk, cconj(zk2)), twN, twNl, k);
                row[k] = cmk<C>(h * (e.x + d.y), h * (e.y - d.x));  // (e - i d) / 2
            }
            if (k2 != k) {
                const C e = cadd(zk2, cconj(zk));
                const C d = twmul<false>(csub(zk2, cconj(zk)), twN, twNl, k2);
                row[k2] = cmk<C>(h * (e.x + d.y), h * (e.y - d.x));
            }
        }
    }
    g.sync();
    fft_lines_TN<NY, false, NT, NF * M>(S, LinearLines{1}, pitch, twY, twYl, g);
    if constexpr (NQ == 1) {
        g.sync();
        fft_lines_TN<NY, false, NT, M>(Qb, LinearLines{1}, QX, twY, twYl, g);
    }
    g.sync();

    // ---- store (natural ky, kx), unpacking the kx = 0 / nx/2 column pair
    C* outA;
    C* outB = nullptr;
    C* outQ = nullptr;
    if (a.mode == XY_NONLIN || a.mode == XY_FUSED) {
        void *oa, *ob, *oq;
        nl_outputs<T>(I, ctrl, a.mode, a.role, oa, ob, &oq);
        outA = reinterpret_cast<C*>(oa) + (size_t)z * plane;
        outB = reinterpret_cast<C*>(ob) + (size_t)z * plane;
        if constexpr (NQ == 1) outQ = reinterpret_cast<C*>(oq) + (size_t)z * plane;
    } else {
        outA = reinterpret_cast<C*>(a.cout) + (size_t)z * plane;
    }
    const PC<T> kst(p);
    // g + beta cx |k_xy|^2 h: FP64 as the reference; FP32 with beta cx folded hi + lo
    auto add_bnl = [&](C g, C hh, int kk) {
        if constexpr (sizeof(T) == 8) {
            const T mm = kst.bnl * (T)kk;
            return cmk<C>(g.x + mm * hh.x, g.y + mm * hh.y);
        } else {
            return cmk<C>(g.x + kst.k_bnl.mul((T)kk * hh.x), g.y + kst.k_bnl.mul((T)kk * hh.y));
        }
    };
    for (int it = tid; it < NY * M; it += NT) {
        const int c = it % M, ky = it / M;
        const C zg = S[ky * pitch + c];
        const int kyf = min(ky, NY - ky);
        if (c == 0) {
            const int kym = (NY - ky) % NY;
            const C zg2 = S[kym * pitch];
            const T h = (T)0.5;
            const C g0 = cmk<C>(h * (zg.x + zg2.x), h * (zg.y - zg2.y));
            const C gN = cmk<C>(h * (zg.y + zg2.y), h * (zg2.x - zg.x));  // -i/2 (z - conj z2)
            if (outB) {
                const C zh = S[ky * pitch + M], zh2 = S[kym * pitch + M];
                const C h0 = cmk<C>(h * (zh.x + zh2.x), h * (zh.y - zh2.y));
                const C hN = cmk<C>(h * (zh.y + zh2.y), h * (zh2.x - zh.x));
                if constexpr (NQ == 1) {  // q takes H's multiplier: A = G + beta cx |k_xy|^2 (H + q)
                    const C zq = Qb[ky * QX], zq2 = Qb[kym * QX];
                    const C q0 = cmk<C>(h * (zq.x + zq2.x), h * (zq.y - zq2.y));
                    const C qN = cmk<C>(h * (zq.y + zq2.y), h * (zq2.x - zq.x));
                    outA[ky * NC] = add_bnl(g0, cadd(h0, q0), kyf * kyf);
                    outA[ky * NC + M] = add_bnl(gN, cadd(hN, qN), M * M + kyf * kyf);
                    outQ[ky * NC] = q0;
                    outQ[ky * NC + M] = qN;
                } else {
                    outA[ky * NC] = add_bnl(g0, h0, kyf * kyf);
                    outA[ky * NC + M] = add_bnl(gN, hN, M * M + kyf * kyf);
                }
                outB[ky * NC] = h0;
                outB[ky * NC + M] = hN;
            } else {
                outA[ky * NC] = g0;
                outA[ky * NC + M] = gN;
            }
        } else {
            if (outB) {
                const C zh = S[ky * pitch + M + c];
                if constexpr (NQ == 1) {
                    const C zq = Qb[ky * QX + c];
                    outA[ky * NC + c] = add_bnl(zg, cadd(zh, zq), c * c + kyf * kyf);
                    outQ[ky * NC + c] = zq;
                } else {
                    outA[ky * NC + c] = add_bnl(zg, zh, c * c + kyf * kyf);
                }
                outB[ky * NC + c] = zh;
            } else {
                outA[ky * NC + c] = zg;
            }
        }
    }
}

template <class T, int NX, int NT, int NF, int NQ = 0>
__global__ void __launch_bounds__(NT) xy_kernel(const InstT<T>* __restrict__ insts, XYArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    xy_body<T, NX, NT, NF, NQ, true>(insts[blockIdx.y], blockIdx.x, a, smem_raw);
}

template <class T, int NX> __host__ __device__ constexpr size_t xy_smem_bytes(int nf, int nq = 0) {
    constexpr size_t ntw = sizeof(T) == 4 ? 2 : 1;
    return sizeof(cplx<T>) * ((size_t)NX * (nf * (NX / 2) + 1) + (nq ? (size_t)NX * (NX / 2 + 1) : 0) +
                              ntw * (NX / 2 + NX + NX)) +
           (32 * 4 + 2) * sizeof(double);
}

}  // namespace cb
