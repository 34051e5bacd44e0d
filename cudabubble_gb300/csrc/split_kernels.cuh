// Split plane path: the xy pass as a y-column pass and an x-row pass, for
// planes whose two fields do not fit one CTA's shared memory (the FP64 form
// from 128^2, both forms at 192^2 and 256^2).
//
//   ycol (inverse): partials P0, P2 [z][ky][kx] -> y-inverse of u and of the
//                   Laplacian partial -> Y0, Y1 [z][y][kx]
//   xrow:           rows of Y0, Y1 -> x C2R -> pointwise (nonlinear partials
//                   or sums) -> x R2C -> rows of Y0, Y1 (in place)
//   ycol (forward): Y0, Y1 -> y-forward -> A = G + beta cx |k_xy|^2 H, B = H
//
// The y pass tiles TX consecutive kx columns of one plane (rows of TX *
// sizeof(C) bytes, like the z pass); the row pass gives each CTA RPC rows of
// NX points.  Every arithmetic step matches the single-CTA xy pass.
#pragma once
#include "cb_fft.cuh"
#include "cb_inst.h"
#include "cb_kargs.h"
#include "pointwise.cuh"
#include "xy_kernel.cuh"

namespace cb {

// ------------------------------------------------------------ y columns
template <class T, int NY, int TX, int NT>
__global__ void __launch_bounds__(NT) ycol_kernel(const InstT<T>* __restrict__ insts, YArgs a) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CB_PDL_TRIGGER();
    CB_PDL_WAIT();
    const InstT<T>& I = insts[blockIdx.y];
    const Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    const int nc = p.nc;
    const int ntx = (nc + TX - 1) / TX;
    const int z = blockIdx.x / ntx, c0 = (blockIdx.x - z * ntx) * TX;
    const int tid = threadIdx.x;
    if (z >= p.nz) return;
    if (a.stepping) {
        if (ctrl->done) return;
        if (a.skip_if_stale && !ctrl->fresh) return;
    }
    const bool inv = a.mode == Y_INV2 || a.mode == Y_INV1;
    const bool two = a.mode == Y_INV2 || a.mode == Y_FWD2;
    constexpr int W = 2 * TX;
    constexpr int ntw = sizeof(T) == 4 ? 2 : 1;
    C* S = reinterpret_cast<C*>(smem_raw);
    C* tw = S + NY * W;
    C* twl = tw + NY;
    for (int i = tid; i < ntw * NY; i += NT) tw[i] = reinterpret_cast<const C*>(I.twy)[i];
    const PC<T> k(p);
    const size_t plane = (size_t)NY * nc;
    const void *src0, *src1 = nullptr;
    void *dst0, *dst1 = nullptr;
    if (inv) {
        if (a.stepping) {
            const int set = part_set(ctrl, a.role);
            src0 = I.P[set][0];
            src1 = I.P[set][1];
        } else {
            src0 = a.cin;
        }
        dst0 = I.Y[0];
        dst1 = I.Y[1];
    } else {
        src0 = I.Y[0];
        src1 = I.Y[1];
        if (a.stepping) {
            nl_outputs<T>(I, ctrl, a.fused ? XY_FUSED : XY_NONLIN, a.role, dst0, dst1);
        } else {
            dst0 = a.cout;
        }
    }
    const C* in0 = reinterpret_cast<const C*>(src0) + (size_t)z * plane;
    const C* in1 = two ? reinterpret_cast<const C*>(src1) + (size_t)z * plane : nullptr;
    for (int it = tid; it < NY * TX; it += NT) {
        const int c = it % TX, y = it / TX, kx = c0 + c;
        C v = cmk<C>(0, 0), w = cmk<C>(0, 0);
        if (kx < nc) {
            v = in0[(size_t)y * nc + kx];
            if (two) {
                w = in1[(size_t)y * nc + kx];
                // laplacian partial Q = -cx (kx^2 + ky^2) P0 + P2 (Calc.cu:107-124); in the FP32
                // form's fused pass P2 is already the whole Laplacian (z_kernel.cuh)
                if (inv && !(sizeof(T) == 4 && a.fused)) {
                    const int kyf = min(y, NY - y);
                    const int kk = kx * kx + kyf * kyf;
                    if constexpr (sizeof(T) == 8) {
                        const T k2 = k.cx * (T)(kx * kx) + k.cx * (T)(kyf * kyf);
                        w = cmk<C>(w.x - k2 * v.x, w.y - k2 * v.y);
                    } else {
                        w = cmk<C>(w.x - k.k_cx.mul((T)kk * v.x), w.y - k.k_cx.mul((T)kk * v.y));
                    }
                }
            }
        }
        S[y * W + c] = v;
        S[y * W + TX + c] = w;
    }
    __syncthreads();
    if (inv) {
        if (two) fft_lines_NT<NY, true, NT, W>(S, LinearLines{1}, W, tw, twl);
        else fft_lines_NT<NY, true, NT, TX>(S, LinearLines{1}, W, tw, twl);
    } else {
        if (two) fft_lines_NT<NY, false, NT, W>(S, LinearLines{1}, W, tw, twl);
        else fft_lines_NT<NY, false, NT, TX>(S, LinearLines{1}, W, tw, twl);
    }
    __syncthreads();
    C* out0 = reinterpret_cast<C*>(dst0) + (size_t)z * plane;
    C* out1 = two ? reinterpret_cast<C*>(dst1) + (size_t)z * plane : nullptr;
    for (int it = tid; it < NY * TX; it += NT) {
        const int c = it % TX, r = it / TX, kx = c0 + c;
        if (kx >= nc) continue;
        const int y = tidx<NY>(r);  // slot r holds element y (real row, or ky)
        const C v = S[r * W + c];
        if (!two) {
            out0[(size_t)y * nc + kx] = v;
        } else if (inv) {
            out0[(size_t)y * nc + kx] = v;
            out1[(size_t)y * nc + kx] = S[r * W + TX + c];
        } else {  // A = G + beta cx (kx^2 + ky^2) H, B = H (Calc.cu:428-437, :265-284)
            const C h = S[r * W + TX + c];
            const int kyf = min(y, NY - y);
            const int kk = kx * kx + kyf * kyf;
            C g;
            if constexpr (sizeof(T) == 8) {
                const T mm = k.bnl * (T)kk;
                g = cmk<C>(v.x + mm * h.x, v.y + mm * h.y);
            } else {
                g = cmk<C>(v.x + k.k_bnl.mul((T)kk * h.x), v.y + k.k_bnl.mul((T)kk * h.y));
            }
            out0[(size_t)y * nc + kx] = g;
            out1[(size_t)y * nc + kx] = h;
        }
    }
}

template <class T, int NY, int TX> constexpr size_t ycol_smem_bytes() {
    constexpr size_t ntw = sizeof(T) == 4 ? 2 : 1;
    return sizeof(cplx<T>) * ((size_t)NY * 2 * TX + ntw * NY);
}

// ------------------------------------------------------------------ x rows
template <class T, int NX, int RPC, int NT>
__global__ void __launch_bounds__(NT) xrow_kernel(const InstT<T>* __restrict__ insts, XYArgs a) {
    using C = cplx<T>;
    constexpr int M = NX / 2, NC = M + 1;
    constexpr int LP = M + 1;  // line pitch in shared memory
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CB_PDL_TRIGGER();
    CB_PDL_WAIT();
    const InstT<T>& I = insts[blockIdx.y];
    Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    const int tid = threadIdx.x;
    const int nrows = p.nz * p.ny;
    const int nblk = nrows / RPC;
    const int rb = blockIdx.x;
    if (rb >= nblk) return;
    const bool stepping = a.mode <= XY_FUSED;
    if (stepping) {
        if (ctrl->done) return;
        if (a.skip_if_stale && !ctrl->fresh) return;
    }
    const int nf = (a.mode == XY_REDUCE_FULL || a.mode == XY_NONLIN || a.mode == XY_FUSED) ? 2 : 1;
    constexpr int ntw = sizeof(T) == 4 ? 2 : 1;
    C* S = reinterpret_cast<C*>(smem_raw);  // line l = f * RPC + j: field f of row j
    C* twM = S + 2 * RPC * LP;
    C* twN = twM + M;
    C* twMl = twN + NX;
    C* twNl = twMl + M;
    double* red = reinterpret_cast<double*>(twM + ntw * (M + NX));
    {
        const C* gx = reinterpret_cast<const C*>(I.twx);
        for (int i = tid; i < ntw * (M + NX); i += NT) twM[i] = gx[i];  // hi (M, NX) then lo (M, NX)
    }
    __syncthreads();  // the C2R pre-processing below reads the tables straight away
    const size_t row0 = (size_t)rb * RPC;
    C* Y0 = reinterpret_cast<C*>(I.Y[0]);
    C* Y1 = reinterpret_cast<C*>(I.Y[1]);
    const LinearLines lines{LP};

    if (a.mode == XY_FWD_PLAIN) {
        const double* src = a.rin + row0 * NX;
        for (int it = tid; it < RPC * M; it += NT) {
            const int m = it % M, j = it / M;
            const double2 v = reinterpret_cast<const double2*>(src + (size_t)j * NX)[m];
            S[j * LP + tpos<M>(m)] = cmk<C>((T)v.x, (T)v.y);
        }
        __syncthreads();
    } else {
        // ---- load + x C2R pre-processing: Z[k] = e + i o,
        //      e = X[k] + conj X[M-k], o = (X[k] - conj X[M-k]) W_N^{-k}
        for (int it = tid; it < nf * RPC * (M / 2 + 1); it += NT) {
            const int l = it % (nf * RPC), kk = it / (nf * RPC);
            const int f = l / RPC, j = l - f * RPC;
            const C* X = (f ? Y1 : Y0) + (row0 + j) * NC;
            C* row = S + l * LP;
            const int k2 = M - kk;
            const C xk = X[kk], xk2 = X[k2];
            if (kk == 0) {  // X[0], X[M] real: the imaginary parts are ignored, as a C2R does
                row[0] = cmk<C>(xk.x + xk2.x, xk.x - xk2.x);
            } else {
                const C e = cadd(xk, cconj(xk2));
                const C o = twmul<true>(csub(xk, cconj(xk2)), twN, twNl, kk);
                row[kk] = cmk<C>(e.x - o.y, e.y + o.x);
            }
            if (k2 != kk && kk != 0) {
                const C e = cadd(xk2, cconj(xk));
                const C o = twmul<true>(csub(xk2, cconj(xk)), twN, twNl, k2);
                row[k2] = cmk<C>(e.x - o.y, e.y + o.x);
            }
        }
        __syncthreads();
        if (nf == 2) fft_lines_NT<M, true, NT, 2 * RPC>(S, lines, 1, twM, twMl);
        else fft_lines_NT<M, true, NT, RPC>(S, lines, 1, twM, twMl);
        __syncthreads();

        if (a.mode == XY_INV_PLAIN) {
            double* dst = a.rout + row0 * NX;
            for (int it = tid; it < RPC * M; it += NT) {
                const int m = it % M, j = it / M;
                const C v = S[j * LP + tpos<M>(m)];
                reinterpret_cast<double2*>(dst + (size_t)j * NX)[m] = make_double2((double)v.x, (double)v.y);
            }
            return;
        }
        const PC<T> k(p);
        if (a.mode == XY_NONLIN) {
            T* lam = reinterpret_cast<T*>(red);
            const bool euler = p.method == M_EULER;
            if (tid == 0) nonlin_lambdas<T>(p, ctrl, a.role, lam);
            __syncthreads();
            const T g_c = lam[0], g_f = lam[1];
            for (int it = tid; it < RPC * M; it += NT) {
                const int q = it % M, j = it / M;
                C* pu = S + j * LP + q;
                C* pl = S + (RPC + j) * LP + q;
                const C uu = *pu, ll = *pl;
                C g, h;
                nonlin_point<T>(k, euler, g_c, g_f, uu.x, ll.x, g.x, h.x);
                nonlin_point<T>(k, euler, g_c, g_f, uu.y, ll.y, g.y, h.y);
                *pu = g;
                *pl = h;
            }
            __syncthreads();
        } else if (a.mode == XY_FUSED) {
            const bool euler = p.method == M_EULER;
            Acc<T> as, af;
            PSum<T> ag, ah;
            if constexpr (sizeof(T) == 4) {
                // u = U[u_state] + (u - u_state); the candidate pass keeps its u for the next state
                const float4* Us = reinterpret_cast<const float4*>(I.U[ctrl->u_state]) + row0 * M;
                float4* Uo = a.role == R_CAND ? reinterpret_cast<float4*>(I.U[1 - ctrl->u_state]) + row0 * M : nullptr;
                Acc2 as2, af2;
                PSum2 ag2, ah2;
                for (int it = tid; it < RPC * M; it += NT) {
                    const int q = it % M, j = it / M;
                    const int ui = j * M + q;  // row j, x slot q (the field is stored in x-slot order)
                    const float4 Uv = __ldg(Us + ui);
                    C* pu = S + j * LP + q;
                    C* pl = S + (RPC + j) * LP + q;
                    const C dd = *pu, ll = *pl;
                    float2 uh, ul;
                    ff_add_f2(Uv, dd, uh, ul);
                    if (Uo) Uo[ui] = make_float4(uh.x, ul.x, uh.y, ul.y);
                    float2 g, h;
                    fused_point_u2(k, euler, uh, ul, ll, as2, af2, g, h);
                    ag2.add(g);
                    ah2.add(h);
                    *pu = g;
                    *pl = h;
                }
                as.v = as2.part();
                af.v = af2.part();
                ag.s = ag2.s.x + ag2.s.y;
                ah.s = ah2.s.x + ah2.s.y;
            } else {
                for (int it = tid; it < RPC * M; it += NT) {
                    const int q = it % M, j = it / M;
                    C* pu = S + j * LP + q;
                    C* pl = S + (RPC + j) * LP + q;
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
            xy_sums_finalize<T, 4>(I, ctrl, p, rb, nblk, vv, red, a.role, true);
            __syncthreads();
        } else {
            const bool full = a.mode == XY_REDUCE_FULL;
            Acc<T> as, af;
            for (int it = tid; it < RPC * M; it += NT) {
                const int q = it % M, j = it / M;
                const C uu = S[j * LP + q];
                const C ll = full ? S[(RPC + j) * LP + q] : cmk<C>(0, 0);
                reduce_point<T>(k, full, uu.x, ll.x, as, af);
                reduce_point<T>(k, full, uu.y, ll.y, as, af);
            }
            auto pv = as.part();
            decltype(pv) vv[2] = {pv, af.part()};
            xy_sums_finalize<T>(I, ctrl, p, rb, nblk, vv, red, a.role, full);
            return;
        }
    }

    // ---- x R2C: forward M-point transform, then
    //      X[k] = (e - i d) / 2, e = Z[k] + conj Z[M-k], d = (Z[k] - conj Z[M-k]) W_N^k
    const int nfo = (a.mode == XY_NONLIN || a.mode == XY_FUSED) ? 2 : 1;
    if (nfo == 2) fft_lines_TN<M, false, NT, 2 * RPC>(S, lines, 1, twM, twMl);
    else fft_lines_TN<M, false, NT, RPC>(S, lines, 1, twM, twMl);
    __syncthreads();
    for (int it = tid; it < nfo * RPC * (M / 2 + 1); it += NT) {
        const int l = it % (nfo * RPC), kk = it / (nfo * RPC);
        const int f = l / RPC, j = l - f * RPC;
        C* X = (f ? Y1 : Y0) + (row0 + j) * NC;
        const C* row = S + l * LP;
        const T h = (T)0.5;
        if (kk == 0) {
            const C z0 = row[0];
            X[0] = cmk<C>(z0.x + z0.y, (T)0);
            X[M] = cmk<C>(z0.x - z0.y, (T)0);
        } else {
            const int k2 = M - kk;
            const C zk = row[kk], zk2 = row[k2];
            {
                const C e = cadd(zk, cconj(zk2));
                const C d = twmul<false>(csub(zk, cconj(zk2)), twN, twNl, kk);
                X[kk] = cmk<C>(h * (e.x + d.y), h * (e.y - d.x));
            }
            if (k2 != kk) {
                const C e = cadd(zk2, cconj(zk));
                const C d = twmul<false>(csub(zk2, cconj(zk)), twN, twNl, k2);
                X[k2] = cmk<C>(h * (e.x + d.y), h * (e.y - d.x));
            }
        }
    }
}

template <class T, int NX, int RPC> constexpr size_t xrow_smem_bytes() {
    constexpr size_t ntw = sizeof(T) == 4 ? 2 : 1;
    return sizeof(cplx<T>) * ((size_t)2 * RPC * (NX / 2 + 1) + ntw * (NX / 2 + NX)) + (32 * 4 + 2) * sizeof(double);
}

}  // namespace cb
