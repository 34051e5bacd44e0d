// The FP32 form's fused xy pass (XY_FUSED) on a cluster of two CTAs per
// z-plane.  One CTA per plane leaves a fifth of GB300's 152 SMs idle at 128
// planes and runs the latency-bound plane FFTs with one CTA's warps; a pair
// halves each CTA's share and doubles the CTAs in flight.
//
//   y stage:  CTA r holds packed columns [r M/2, (r+1) M/2) of both fields for
//             every row slot: load, Laplacian partial, inverse y-FFT;
//   exchange: through distributed shared memory, CTA r gathers row slots
//             [r NY/2, (r+1) NY/2) with all M columns (its own half from its
//             shared memory, the other from the partner's);
//   x stage:  x C2R, pointwise sums and lambda-free partials, x R2C on its rows;
//   exchange back, forward y-FFT of its columns, store.
//
// Each exchange reads into registers between two cluster barriers, so no CTA
// overwrites shared memory its partner still reads.  The arithmetic of every
// step is that of xy_kernel.cuh.
#pragma once
#include <cooperative_groups.h>

#include "xy_kernel.cuh"

namespace cb {

// NQ = 1 (the FP32 form with spontaneous curvature): a third output field q, transformed
// forward in a shared-memory region of its own ([NH][M + 1] in the x stage, [NY][MH + 1]
// in the y stage) and exchanged in a round of its own, so the register-staged exchange of
// the two main fields keeps its size
template <int NX, int NQ = 0> struct XYC {
    static constexpr int M = NX / 2, NY = NX, NC = M + 1, MH = M / 2, NH = NY / 2;
    static constexpr int PY = 2 * MH + 1;  // y layout: [NY][field 0 | field 1 of own columns]
    static constexpr int PX = 2 * M + 1;   // x layout: [NH][field 0 | field 1 of all columns]
    static constexpr int SZ = (NY * PY > NH * PX) ? NY * PY : NH * PX;
    static constexpr int QX = M + 1, QY = MH + 1;  // pitches of the q region
    static constexpr int SQ = NQ ? ((NH * QX > NY * QY) ? NH * QX : NY * QY) : 0;
};
template <class T, int NX, int NQ = 0> constexpr size_t xyc_smem_bytes() {
    using Q = XYC<NX, NQ>;
    constexpr size_t ntw = sizeof(T) == 4 ? 2 : 1;
    return sizeof(cplx<T>) * ((size_t)Q::SZ + Q::SQ + ntw * (Q::M + NX + NX)) + (32 * 4 + 2) * sizeof(double);
}

// Plane z of instance I on this CTA's two-CTA cluster, all NT threads of both CTAs: the
// body of xyc_fused_kernel (one plane per cluster, PDL = true: programmatic launch) and of
// the persistent batched kernel (mega.cuh, PDL = false).
template <class T, int NX, int NT, int NQ = 0, bool PDL = true>
__device__ __forceinline__ void xyc_body(const InstT<T>& I, const int z, const XYArgs a, unsigned char* smem_raw) {
    namespace cg = cooperative_groups;
    using C = cplx<T>;
    using Q = XYC<NX, NQ>;
    constexpr int M = Q::M, NY = Q::NY, NC = Q::NC, MH = Q::MH, NH = Q::NH, PY = Q::PY, PX = Q::PX;
    constexpr int QX = Q::QX, QY = Q::QY;
    constexpr int ntw = sizeof(T) == 4 ? 2 : 1;
    if constexpr (PDL) CB_PDL_TRIGGER();
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    const int tid = threadIdx.x;
    const void *p00 = I.P[0][0], *p01 = I.P[0][1], *p10 = I.P[1][0], *p11 = I.P[1][1], *p20 = I.P[2][0],
               *p21 = I.P[2][1];
    // both CTAs of a cluster hold the same plane of the same instance: they leave together
    if (z >= p.nz) return;
    C* S = reinterpret_cast<C*>(smem_raw);
    C* Qb = S + Q::SZ;  // the q region (NQ = 1)
    C* twM = Qb + Q::SQ;
    C* twN = twM + M;
    C* twY = twN + NX;
    C* twMl = twY + NY;  // lo parts (FP32)
    C* twNl = twMl + M;
    C* twYl = twNl + NX;
    double* red = reinterpret_cast<double*>(twM + ntw * (M + NX + NY));
    {
        const C* gx = reinterpret_cast<const C*>(I.twx);
        const C* gy = reinterpret_cast<const C*>(I.twy);
        for (int i = tid; i < M + NX; i += NT) twM[i] = gx[i];
        for (int i = tid; i < NY; i += NT) twY[i] = gy[i];
        if constexpr (ntw == 2) {
            for (int i = tid; i < M + NX; i += NT) twMl[i] = gx[M + NX + i];
            for (int i = tid; i < NY; i += NT) twYl[i] = gy[NY + i];
        }
    }
    // the twiddles (written by no kernel) are loaded; the control state and the
    // partials come from the previous kernel
    if constexpr (PDL) CB_PDL_WAIT();
    // the control fields and this pass's candidate partial sets in one batch of
    // independent loads (the state-selected pointers are chosen in registers)
    const int c_done = ctrl->done, c_part = ctrl->part_state, c_u = ctrl->u_state;
    if (c_done) return;
    const PC<T> k(p);
    const size_t plane = (size_t)NY * NC;
    const int set = a.role == R_WORK ? 2 : (a.role == R_STATE ? c_part : 1 - c_part);  // part_set
    const C* P0 = reinterpret_cast<const C*>(set == 2 ? p20 : (set == 1 ? p10 : p00)) + (size_t)z * plane;
    const C* P2 = reinterpret_cast<const C*>(set == 2 ? p21 : (set == 1 ? p11 : p01)) + (size_t)z * plane;
    const int c0 = rank * MH;

    // ---- load own packed columns (col 0 = kx 0 + i kx M) and the Laplacian partial
    for (int it = tid; it < NY * MH; it += NT) {
        const int cc = it % MH, ky = it / MH, c = c0 + cc;
        // P0 holds u - u_state and P2 the whole Laplacian (z_kernel.cuh, FP32 form)
        const C v = __ldg(P0 + ky * NC + c), w = __ldg(P2 + ky * NC + c);
        if (c == 0) {
            const C vN = __ldg(P0 + ky * NC + M), wN = __ldg(P2 + ky * NC + M);
            S[ky * PY] = cmk<C>(v.x - vN.y, v.y + vN.x);
            S[ky * PY + MH] = cmk<C>(w.x - wN.y, w.y + wN.x);
        } else {
            S[ky * PY + cc] = v;
            S[ky * PY + MH + cc] = w;
        }
    }
    __syncthreads();
    fft_lines_NT<NY, true, NT, 2 * MH>(S, LinearLines{1}, PY, twY, twYl);

    // ---- exchange: row slots [rank NH, rank NH + NH) with all columns
    constexpr int NE = NH * 2 * M;  // == NY * 2 * MH
    constexpr int EPT = (NE + NT - 1) / NT;
    C rg[EPT];
    C* Sp = cl.map_shared_rank(S, rank ^ 1);
    cl.sync();  // the partner's y stage is done
#pragma unroll
    for (int e = 0; e < EPT; ++e) {
        const int idx = tid + e * NT;
        if (idx < NE) {
            const int rl = idx / (2 * M), rem = idx - rl * (2 * M), f = rem / M, c = rem - f * M, o = c / MH;
            const C* src = o == rank ? S : Sp;
            rg[e] = src[(rank * NH + rl) * PY + f * MH + (c - o * MH)];
        }
    }
    cl.sync();  // every read of both CTAs is done before either rewrites its shared memory
#pragma unroll
    for (int e = 0; e < EPT; ++e) {
        const int idx = tid + e * NT;
        if (idx < NE) {
            const int rl = idx / (2 * M), rem = idx - rl * (2 * M);
            S[rl * PX + rem] = rg[e];
        }
    }
    __syncthreads();

    // ---- x C2R (half-length pre-processing, inverse M-point FFT) on NH rows x 2 fields
    const PairRows<NH, PX, M> rows;
    for (int it = tid; it < 2 * NH * (M / 2 + 1); it += NT) {
        const int l = it % (2 * NH), kk = it / (2 * NH);
        C* row = S + rows(l);
        if (kk == 0) {
            const C v = row[0];  // X[0] + i X[M]
            row[0] = cmk<C>(v.x + v.y, v.x - v.y);
        } else {
            const int k2 = M - kk;
            const C xk = row[kk], xk2 = row[k2];
            {
                const C e = cadd(xk, cconj(xk2));
                const C o = twmul<true>(csub(xk, cconj(xk2)), twN, twNl, kk);
                row[kk] = cmk<C>(e.x - o.y, e.y + o.x);
            }
            if (k2 != kk) {
                const C e = cadd(xk2, cconj(xk));
                const C o = twmul<true>(csub(xk2, cconj(xk)), twN, twNl, k2);
                row[k2] = cmk<C>(e.x - o.y, e.y + o.x);
            }
        }
    }
    __syncthreads();
    fft_lines_NT<M, true, NT, 2 * NH>(S, rows, 1, twM, twMl);
    __syncthreads();

    // ---- sums and lambda-free partials G'', w of this CTA's rows
    {
        const bool euler = p.method == M_EULER;
        Acc<T> as, af;
        PSum<T> ag, ah;
        // u = U[u_state] + (u - u_state); the candidate pass keeps its u for the next state
        const float4* Us = reinterpret_cast<const float4*>(I.U[c_u]) + (size_t)z * NY * M;
        float4* Uo = a.role == R_CAND ? reinterpret_cast<float4*>(I.U[1 - c_u]) + (size_t)z * NY * M
                                      : nullptr;
        Acc2 as2, af2;
        PSum2 ag2, ah2;
        // row y, x slot qq of slot `it` (the field is stored in x-slot order); each
        // iteration's U load is issued one iteration ahead
        auto uidx = [&](int it) { return tidx<NY>(rank * NH + it / M) * M + it % M; };
        float4 Unext = tid < NH * M ? __ldg(Us + uidx(tid)) : make_float4(0.f, 0.f, 0.f, 0.f);
        for (int it = tid; it < NH * M; it += NT) {
            const int qq = it % M, r = it / M;
            const int ui = uidx(it);
            const float4 Uv = Unext;
            if (it + NT < NH * M) Unext = __ldg(Us + uidx(it + NT));
            C* pu = S + r * PX + qq;
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
            if constexpr (NQ == 1) Qb[r * QX + qq] = qv;
        }
        as.v = as2.part();
        af.v = af2.part();
        ag.s = ag2.s.x + ag2.s.y;
        ah.s = ah2.s.x + ah2.s.y;
        auto pv = as.part();
        decltype(pv) vv[4] = {pv, af.part(), ag.part(), ah.part()};
        xy_sums_finalize<T, 4>(I, ctrl, p, 2 * z + rank, 2 * p.nz, vv, red, a.role, true);
        __syncthreads();
    }

    // ---- x R2C: forward M-point FFT, post-processing (two fields, or three with q)
    constexpr int NFO = 2 + NQ;
    const TripleRows<NH, PX, M, Q::SZ, QX> rows3;
    auto xrow = [&](int l) { return NQ ? rows3(l) : rows(l); };
    if constexpr (NQ == 1) fft_lines_TN<M, false, NT, 3 * NH>(S, rows3, 1, twM, twMl);
    else fft_lines_TN<M, false, NT, 2 * NH>(S, rows, 1, twM, twMl);
    __syncthreads();
    for (int it = tid; it < NFO * NH * (M / 2 + 1); it += NT) {
        const int l = it % (NFO * NH), kk = it / (NFO * NH);
        C* row = S + xrow(l);
        if (kk == 0) {
            const C z0 = row[0];
            row[0] = cmk<C>(z0.x + z0.y, z0.x - z0.y);  // X[0] + i X[M]
        } else {
            const int k2 = M - kk;
            const C zk = row[kk], zk2 = row[k2];
            const T h = (T)0.5;
            {
                const C e = cadd(zk, cconj(zk2));
                const C d = twmul<false>(csub(zk, cconj(zk2)), twN, twNl, kk);
                row[kk] = cmk<C>(h * (e.x + d.y), h * (e.y - d.x));
            }
            if (k2 != kk) {
                const C e = cadd(zk2, cconj(zk));
                const C d = twmul<false>(csub(zk2, cconj(zk)), twN, twNl, k2);
                row[k2] = cmk<C>(h * (e.x + d.y), h * (e.y - d.x));
            }
        }
    }

    // ---- exchange back: own columns of every row slot
    cl.sync();  // the partner's x stage is done (and this CTA's: the barrier covers the block)
#pragma unroll
    for (int e = 0; e < EPT; ++e) {
        const int idx = tid + e * NT;
        if (idx < NE) {
            const int s = idx / (2 * MH), rem = idx - s * (2 * MH), f = rem / MH, cc = rem - f * MH, o = s / NH;
            const C* src = o == rank ? S : Sp;
            rg[e] = src[(s - o * NH) * PX + f * M + c0 + cc];
        }
    }
    cl.sync();
#pragma unroll
    for (int e = 0; e < EPT; ++e) {
        const int idx = tid + e * NT;
        if (idx < NE) {
            const int s = idx / (2 * MH), rem = idx - s * (2 * MH);
            S[s * PY + rem] = rg[e];
        }
    }
    if constexpr (NQ == 1) {
        // q: own columns of every row slot, from both CTAs' x-stage q regions (unchanged
        // since the barriers above) into this CTA's y layout [NY][QY]
        constexpr int NEQ = NY * MH, EPQ = (NEQ + NT - 1) / NT;
        C rq[EPQ];
        const C* Qp = cl.map_shared_rank(Qb, rank ^ 1);
#pragma unroll
        for (int e = 0; e < EPQ; ++e) {
            const int idx = tid + e * NT;
            if (idx < NEQ) {
                const int s = idx / MH, cc = idx - s * MH, o = s / NH;
                const C* src = o == rank ? Qb : Qp;
                rq[e] = src[(s - o * NH) * QX + c0 + cc];
            }
        }
        cl.sync();  // both CTAs have read their q before either rewrites its region
#pragma unroll
        for (int e = 0; e < EPQ; ++e) {
            const int idx = tid + e * NT;
            if (idx < NEQ) {
                const int s = idx / MH, cc = idx - s * MH;
                Qb[s * QY + cc] = rq[e];
            }
        }
    }
    __syncthreads();
    fft_lines_TN<NY, false, NT, 2 * MH>(S, LinearLines{1}, PY, twY, twYl);
    if constexpr (NQ == 1) {
        __syncthreads();
        fft_lines_TN<NY, false, NT, MH>(Qb, LinearLines{1}, QY, twY, twYl);
    }
    __syncthreads();

    // ---- store own columns, unpacking the kx = 0 / nx/2 pair (rank 0)
    void *oa, *ob, *oq;
    nl_outputs<T>(I, ctrl, XY_FUSED, a.role, oa, ob, &oq);
    C* outA = reinterpret_cast<C*>(oa) + (size_t)z * plane;
    C* outB = reinterpret_cast<C*>(ob) + (size_t)z * plane;
    C* outQ = NQ ? reinterpret_cast<C*>(oq) + (size_t)z * plane : nullptr;
    auto add_bnl = [&](C g, C hh, int kk) {
        if constexpr (sizeof(T) == 8) {
            const T mm = k.bnl * (T)kk;
            return cmk<C>(g.x + mm * hh.x, g.y + mm * hh.y);
        } else {
            return cmk<C>(g.x + k.k_bnl.mul((T)kk * hh.x), g.y + k.k_bnl.mul((T)kk * hh.y));
        }
    };
    for (int it = tid; it < NY * MH; it += NT) {
        const int cc = it % MH, ky = it / MH, c = c0 + cc;
        const C zg = S[ky * PY + cc], zh = S[ky * PY + MH + cc];
        const int kyf = min(ky, NY - ky);
        if (c == 0) {
            const int kym = (NY - ky) % NY;
            const C zg2 = S[kym * PY], zh2 = S[kym * PY + MH];
            const T h = (T)0.5;
            const C g0 = cmk<C>(h * (zg.x + zg2.x), h * (zg.y - zg2.y));
            const C gN = cmk<C>(h * (zg.y + zg2.y), h * (zg2.x - zg.x));
            const C h0 = cmk<C>(h * (zh.x + zh2.x), h * (zh.y - zh2.y));
            const C hN = cmk<C>(h * (zh.y + zh2.y), h * (zh2.x - zh.x));
            if constexpr (NQ == 1) {  // q takes H's multiplier: A = G + beta cx |k_xy|^2 (H + q)
                const C zq = Qb[ky * QY], zq2 = Qb[kym * QY];
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
            if constexpr (NQ == 1) {
                const C zq = Qb[ky * QY + cc];
                outA[ky * NC + c] = add_bnl(zg, cadd(zh, zq), c * c + kyf * kyf);
                outQ[ky * NC + c] = zq;
            } else {
                outA[ky * NC + c] = add_bnl(zg, zh, c * c + kyf * kyf);
            }
            outB[ky * NC + c] = zh;
        }
    }
}

template <class T, int NX, int NT, int NQ = 0>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(NT)
    xyc_fused_kernel(const InstT<T>* __restrict__ insts, XYArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    xyc_body<T, NX, NT, NQ, true>(insts[blockIdx.y], blockIdx.x >> 1, a, smem_raw);
}

}  // namespace cb
