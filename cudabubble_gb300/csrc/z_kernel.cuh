// z-line pass: one CTA owns TX consecutive (ky, kx) columns of the
// [nz][ny*(nx/2+1)] layout, i.e. TX z-lines, for one instance.  Rows of a
// tile are TX*sizeof(C) = 128 bytes, so every global access is a full line.
//
// Stage modes read the nonlinear partials A, B, transform them along z
// (natural -> transposed), form the nonlinear spectrum
//   N-hat = (A-hat + beta cx kz^2 B-hat) / N
// (forward transforms are normalised by 1/N, Calc.cu:77-96), combine it with
// the stored spectra into the next stage spectrum u-hat, store what later
// stages need, and transform u-hat and -cx kz^2 u-hat back along z
// (transposed -> natural) into the partial set the next xy pass reads.
// The same pass accumulates mean |grad u|^2 by Parseval, with the Nyquist
// plane of every axis zeroed like the reference's gradient (Calc.cu:300-341).
#pragma once
#include "cb_fft.cuh"
#include "cb_inst.h"
#include "cb_kargs.h"
#include "xy_kernel.cuh"

namespace cb {

template <class T> __device__ __forceinline__ const void* spec_of(const InstT<T>& I, const Ctrl* c, int role) {
    return role == R_STATE ? I.spec[c->spec_state] : I.spec[1 - c->spec_state];
}

template <class T, int NZ, int TX, int NT>
__global__ void __launch_bounds__(NT) z_kernel(const InstT<T>* __restrict__ insts, ZArgs a) {
    using C = cplx<T>;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const InstT<T>& I = insts[blockIdx.y];
    Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    const int nc = p.nc, ny = p.ny, nx = p.nx;
    const int Mc = ny * nc;
    const int m0 = blockIdx.x * TX;
    const int tid = threadIdx.x;
    if (m0 >= Mc) return;
    const bool plain = a.mode == Z_FWD_PLAIN || a.mode == Z_INV_PLAIN;
    if (!plain && ctrl->done) return;
    const int ntiles = (Mc + TX - 1) / TX;
    constexpr int W = 2 * TX;  // row pitch: field 0 in [0, TX), field 1 in [TX, 2 TX)
    C* S = reinterpret_cast<C*>(smem_raw);
    C* tw = S + NZ * W;
    double* red = reinterpret_cast<double*>(tw + NZ);
    for (int i = tid; i < NZ; i += NT) tw[i] = reinterpret_cast<const C*>(I.twz)[i];

    const bool stage1 = a.mode == Z_ETD2_S1 || a.mode == Z_ETD4_S1 || a.mode == Z_EULER;
    const bool reuse = stage1 && !ctrl->fresh;  // retry of a rejected step: N_u / R-hat unchanged
    const bool need_fwd = (a.mode <= Z_EULER && !reuse) || a.mode == Z_FWD_PLAIN;

    if (need_fwd) {
        const C* gA = reinterpret_cast<const C*>(a.mode == Z_FWD_PLAIN ? a.cin : I.A);
        const C* gB = reinterpret_cast<const C*>(I.B);
        const bool two = a.mode != Z_FWD_PLAIN;
        for (int it = tid; it < NZ * TX; it += NT) {
            const int c = it % TX, zz = it / TX, m = m0 + c;
            C va = cmk<C>(0, 0), vb = cmk<C>(0, 0);
            if (m < Mc) {
                va = gA[(size_t)zz * Mc + m];
                if (two) vb = gB[(size_t)zz * Mc + m];
            }
            S[zz * W + c] = va;
            S[zz * W + TX + c] = vb;
        }
        __syncthreads();
        fft_lines_NT<NZ, false, NT>(S, two ? W : TX, LinearLines{1}, W, tw);
        __syncthreads();
    }

    const T cx = (T)p.cx;
    const T invN = (T)p.invN;
    const T bnl = (T)((p.method == M_EULER) ? p.eta : -p.eta / p.eps) * cx;

    if (a.mode == Z_FWD_PLAIN) {
        C* out = reinterpret_cast<C*>(a.cout);
        for (int it = tid; it < NZ * TX; it += NT) {
            const int c = it % TX, r = it / TX, m = m0 + c;
            if (m >= Mc) continue;
            const int kz = tidx<NZ>(r);
            const C v = S[r * W + c];
            out[(size_t)kz * Mc + m] = cmk<C>(v.x * invN, v.y * invN);
        }
        return;
    }

    // ---- combine: slot r holds kz = tidx(r)
    const C* phat = reinterpret_cast<const C*>(spec_of(I, ctrl, R_STATE));
    C* cand = reinterpret_cast<C*>(const_cast<void*>(spec_of(I, ctrl, R_CAND)));
    C* Nu = reinterpret_cast<C*>(I.Nu);
    C* Na = reinterpret_cast<C*>(I.Na);
    C* Nb = reinterpret_cast<C*>(I.Nb);
    C* ah = reinterpret_cast<C*>(I.ahat);
    const T* coef = I.coef;
    const T dtga = (T)(ctrl->dt * p.ga);
    const bool ref4 = p.etd4_ref != 0;
    Acc<T> ag, al;
    for (int it = tid; it < NZ * TX; it += NT) {
        const int c = it % TX, r = it / TX, m = m0 + c;
        if (m >= Mc) {
            S[r * W + c] = cmk<C>(0, 0);
            S[r * W + TX + c] = cmk<C>(0, 0);
            continue;
        }
        const int kz = tidx<NZ>(r);
        const int kzf = min(kz, NZ - kz);
        const int ky = m / nc, kx = m - ky * nc;
        const int kyf = min(ky, ny - ky);
        const size_t g = (size_t)kz * Mc + m;
        C nh = cmk<C>(0, 0);
        if (need_fwd) {
            const C va = S[r * W + c], vb = S[r * W + TX + c];
            const T mz = bnl * (T)(kzf * kzf);
            nh = cmk<C>((va.x + mz * vb.x) * invN, (va.y + mz * vb.y) * invN);
        }
        const T* cf = coef + 8 * (kx * kx + kyf * kyf + kzf * kzf);
        C un;
        switch (a.mode) {
            case Z_ETD2_S1: {
                if (reuse) nh = Nu[g]; else Nu[g] = nh;
                const T e1 = cf[0], c1 = cf[1];
                const C ph = phat[g];
                un = cmk<C>(e1 * ph.x + c1 * nh.x, e1 * ph.y + c1 * nh.y);
                ah[g] = un;
                break;
            }
            case Z_ETD2_S2: {
                const T c2 = cf[2];
                const C av = ah[g], nu = Nu[g];
                un = cmk<C>(av.x + c2 * (nh.x - nu.x), av.y + c2 * (nh.y - nu.y));
                cand[g] = un;
                break;
            }
            case Z_ETD4_S1: {
                if (reuse) nh = Nu[g]; else Nu[g] = nh;
                const T eh = cf[0], ch = cf[1];
                const C ph = phat[g];
                un = cmk<C>(eh * ph.x + ch * nh.x, eh * ph.y + ch * nh.y);
                ah[g] = un;
                break;
            }
            case Z_ETD4_S2: {
                Na[g] = nh;
                const T eh = cf[0], ch = cf[1];
                const C ph = phat[g];
                un = cmk<C>(eh * ph.x + ch * nh.x, eh * ph.y + ch * nh.y);
                break;
            }
            case Z_ETD4_S3: {
                Nb[g] = nh;
                const T eh = cf[0], ch = cf[1];
                const C av = ah[g], nu = Nu[g];
                un = cmk<C>(eh * av.x + ch * ((T)2 * nh.x - nu.x), eh * av.y + ch * ((T)2 * nh.y - nu.y));
                break;
            }
            case Z_ETD4_S4: {
                const T e2 = cf[2], f1 = cf[3], f2 = cf[4], f3 = cf[5];
                const C ph = phat[g], n1 = ref4 ? Na[g] : Nu[g], nb = Nb[g];
                un = cmk<C>(e2 * ph.x + f1 * n1.x + f2 * (n1.x + nb.x) + f3 * nh.x,
                            e2 * ph.y + f1 * n1.y + f2 * (n1.y + nb.y) + f3 * nh.y);
                cand[g] = un;
                break;
            }
            case Z_EULER: {
                if (reuse) nh = Nu[g]; else Nu[g] = nh;
                const C ph = phat[g];
                un = cmk<C>(ph.x - dtga * nh.x, ph.y - dtga * nh.y);
                cand[g] = un;
                const T wgt = (kx == 0 || 2 * kx == nx) ? (T)1 : (T)2;
                al.add(wgt * (nh.x * nh.x + nh.y * nh.y));
                break;
            }
            case Z_INV_STATE: {
                un = reinterpret_cast<const C*>(spec_of(I, ctrl, a.role))[g];
                break;
            }
            default: {  // Z_INV_PLAIN with an optional spectral multiplier
                const C v = reinterpret_cast<const C*>(a.cin)[g];
                if (a.mul == SM_LAP) {
                    const T mm = -cx * (T)(kx * kx + kyf * kyf + kzf * kzf);
                    un = cmk<C>(mm * v.x, mm * v.y);
                } else if (a.mul >= SM_DX) {
                    const T sq = sqrt(cx);
                    int kk;
                    if (a.mul == SM_DX) kk = (2 * kx == nx) ? 0 : kx;
                    else if (a.mul == SM_DY) kk = (2 * ky == ny) ? 0 : (ky < ny - ky ? ky : ky - ny);
                    else kk = (2 * kz == NZ) ? 0 : (kz < NZ - kz ? kz : kz - NZ);
                    const T f = sq * (T)kk;
                    un = cmk<C>(-f * v.y, f * v.x);  // i k u-hat
                } else {
                    un = v;
                }
                break;
            }
        }
        if (a.mode != Z_INV_PLAIN) {
            // Parseval: mean |grad u|^2 = sum over the full spectrum of |k_g|^2 |u-hat|^2
            const int gx = (2 * kx == nx) ? 0 : kx;
            const int gy = (2 * ky == ny) ? 0 : kyf;
            const int gz = (2 * kz == NZ) ? 0 : kzf;
            const T wgt = (kx == 0 || 2 * kx == nx) ? (T)1 : (T)2;
            ag.add(wgt * cx * (T)(gx * gx + gy * gy + gz * gz) * (un.x * un.x + un.y * un.y));
        }
        const T mz = -cx * (T)(kzf * kzf);
        S[r * W + c] = un;
        S[r * W + TX + c] = cmk<C>(mz * un.x, mz * un.y);
    }
    __syncthreads();
    const bool two = a.mode != Z_INV_PLAIN;
    fft_lines_TN<NZ, true, NT>(S, two ? W : TX, LinearLines{1}, W, tw);
    __syncthreads();

    // ---- store partials (natural z)
    C* o0;
    C* o2 = nullptr;
    if (a.mode == Z_INV_PLAIN) {
        o0 = reinterpret_cast<C*>(a.cout);
    } else {
        const int set = part_set(ctrl, a.role);
        o0 = reinterpret_cast<C*>(I.P[set][0]);
        o2 = reinterpret_cast<C*>(I.P[set][1]);
    }
    for (int it = tid; it < NZ * TX; it += NT) {
        const int c = it % TX, zz = it / TX, m = m0 + c;
        if (m >= Mc) continue;
        o0[(size_t)zz * Mc + m] = S[zz * W + c];
        if (o2) o2[(size_t)zz * Mc + m] = S[zz * W + TX + c];
    }
    if (a.mode == Z_INV_PLAIN) return;

    double v[2] = {ag.get(), al.get()};
    block_sum<2>(v, red);
    if (tid == 0) {
        double* part = I.part_z;
        part[2 * blockIdx.x + 0] = v[0];
        part[2 * blockIdx.x + 1] = v[1];
        __threadfence();
        const unsigned prev = atomicAdd(&ctrl->cnt_z[a.role], 1u);
        if (prev == (unsigned)(ntiles - 1)) {
            __threadfence();
            double s0 = 0.0, s1 = 0.0;
            for (int b = 0; b < ntiles; ++b) {
                s0 += __ldcg(part + 2 * b);
                s1 += __ldcg(part + 2 * b + 1);
            }
            ctrl->sc[a.role].grad2 = s0;
            if (a.mode == Z_EULER) ctrl->sc[a.role].lsq = s1;
            ctrl->cnt_z[a.role] = 0u;
        }
    }
}

template <class T, int NZ, int TX> constexpr size_t z_smem_bytes() {
    return sizeof(cplx<T>) * ((size_t)NZ * 2 * TX + NZ) + 32 * 2 * sizeof(double);
}

}  // namespace cb
