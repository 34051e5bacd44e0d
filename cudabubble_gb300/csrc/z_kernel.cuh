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

// ---- stepped state values.  The plain FP64 form keeps the state in FP64.
// The FP32 form keeps it as double-float pairs (hi + lo, ~48-bit mantissa):
// rounding the state itself to FP32 every step injects noise into the weakly
// damped low-|k| modes that the energy sees at first order (a ~1e-6
// relative energy drift over a few hundred steps), while the increments the
// nonlinear term contributes tolerate FP32.  Updates are
//   next = base (+) (em * base_hi + incr),   em = exp(hL) - 1 from an accurate table,
// with the (+) done in error-free FP32 arithmetic (TwoSum / FastTwoSum).
template <class T> struct State;
template <> struct State<double> {
    double2 v;
    __device__ __forceinline__ static State load(const void* p, size_t g) {
        State s;
        s.v = __ldg(reinterpret_cast<const double2*>(p) + g);
        return s;
    }
    __device__ __forceinline__ static State from(double2 w) { State s; s.v = w; return s; }
    __device__ __forceinline__ void store(void* p, size_t g) const { reinterpret_cast<double2*>(p)[g] = v; }
    __device__ __forceinline__ double2 work() const { return v; }
    __device__ __forceinline__ double re_exact() const { return v.x; }
    // e * base + incr (the reference's own form, Calc.cu:453-455)
    __device__ __forceinline__ State axpy(double e, double2 incr) const {
        return from(make_double2(e * v.x + incr.x, e * v.y + incr.y));
    }
    __device__ __forceinline__ State add(double2 incr) const {
        return from(make_double2(v.x + incr.x, v.y + incr.y));
    }
    template <class A> __device__ __forceinline__ void norm2_into(A& big, A& small, double w) const {
        big.add(w * (v.x * v.x + v.y * v.y));
    }
};

__device__ __forceinline__ void df_add(float& h, float& l, float d) {
    const float s = h + d;
    const float bp = s - h;
    float e = (h - (s - bp)) + (d - bp);  // TwoSum(h, d)
    e += l;
    h = s + e;                           // FastTwoSum(s, e)
    l = e - (h - s);
}
template <> struct State<float> {
    float2 hi, lo;
    __device__ __forceinline__ static State load(const void* p, size_t g) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(p) + g);
        State s;
        s.hi = make_float2(q.x, q.y);
        s.lo = make_float2(q.z, q.w);
        return s;
    }
    __device__ __forceinline__ static State from(float2 w) {
        State s;
        s.hi = w;
        s.lo = make_float2(0.f, 0.f);
        return s;
    }
    __device__ __forceinline__ void store(void* p, size_t g) const {
        reinterpret_cast<float4*>(p)[g] = make_float4(hi.x, hi.y, lo.x, lo.y);
    }
    __device__ __forceinline__ float2 work() const { return make_float2(hi.x + lo.x, hi.y + lo.y); }
    __device__ __forceinline__ double re_exact() const { return (double)hi.x + (double)lo.x; }
    // base (+) (em * base_hi + incr)
    __device__ __forceinline__ State axpy(float em, float2 incr) const {
        State r = *this;
        df_add(r.hi.x, r.lo.x, fmaf(em, hi.x, incr.x));
        df_add(r.hi.y, r.lo.y, fmaf(em, hi.y, incr.y));
        return r;
    }
    __device__ __forceinline__ State add(float2 incr) const {
        State r = *this;
        df_add(r.hi.x, r.lo.x, incr.x);
        df_add(r.hi.y, r.lo.y, incr.y);
        return r;
    }
    // this - o, rounded once to FP32 (a stage increment: small next to either state)
    __device__ __forceinline__ float2 diff(const State& o) const {
        return make_float2((hi.x - o.hi.x) + (lo.x - o.lo.x), (hi.y - o.hi.y) + (lo.y - o.lo.y));
    }
    // w |u|^2 with u = hi + lo: hi^2 exactly via FMA, the rest in a second sum
    // (w up to 3 (n/2)^2 times an exact square needs more than 24 bits: each product
    // is split error-free, or its rounding, ~6e-8 of the term, reaches S at ~1e-9 and
    // the area penalty's lambda2 with it)
    template <class A> __device__ __forceinline__ void norm2_into(A& big, A& small, float w) const {
        const float px = hi.x * hi.x, py = hi.y * hi.y;
        const float ex = fmaf(hi.x, hi.x, -px), ey = fmaf(hi.y, hi.y, -py);
        const float wx = w * px, wy = w * py;
        big.add(wx);
        big.add(wy);
        small.add(fmaf(w, px, -wx) + fmaf(w, py, -wy) + w * (ex + ey + 2.f * (hi.x * lo.x + hi.y * lo.y)));
    }
};

// resident threads per SM the z pass is compiled for (its register cap: 64 registers a
// thread at 1024); the pass is latency-bound, and fewer resident warps cost more than
// the registers buy (768 threads: 28 % slower at 128^3)
#ifndef CB_Z_THREADS_PER_SM
#define CB_Z_THREADS_PER_SM 1024
#endif

// Mode groups: each z_kernel instance compiles only its group's stage code, so
// the ETD-RK2 instance does not carry the registers of the ETD-RK4 combine.
enum ZGroup { ZG_ETD2 = 0, ZG_ETD4 = 1, ZG_EULER = 2, ZG_PLAIN = 3 };
__host__ __device__ constexpr int zgroup_of(int mode) {
    return (mode == Z_ETD2_S1 || mode == Z_ETD2_S2) ? ZG_ETD2
         : (mode >= Z_ETD4_S1 && mode <= Z_ETD4_S4) ? ZG_ETD4
         : mode == Z_EULER ? ZG_EULER : ZG_PLAIN;
}

// The pass over one column tile `tile` of instance I, run by all NT threads of the CTA
// on its dynamic shared memory: the body of z_kernel (one tile per CTA, PDL = true:
// programmatic launch, waiting for the previous kernel after the twiddle load) and of
// the persistent batched kernel (mega.cuh, PDL = false: its own dependency counters).
//
// NQ = 1 (FP32 stage groups with spontaneous curvature): the stage's third partial q is
// transformed with A and B and takes B's multiplier, N-hat = (A-hat + beta cx kz^2 (B-hat +
// q-hat)) / N, while f-hat keeps being rebuilt from B-hat alone
template <class T, int NZ, int TX, int NT, int MG, int NQ = 0, bool PDL = true, class G = Cta>
__device__ __forceinline__ void z_body(const InstT<T>& I, const int tile, const ZArgs a,
                                       unsigned char* smem_raw, const G& g = G()) {
    constexpr bool g2 = MG == ZG_ETD2, g4 = MG == ZG_ETD4, ge = MG == ZG_EULER, gp = MG == ZG_PLAIN;
    using C = cplx<T>;
    if constexpr (PDL) CB_PDL_TRIGGER();
    Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    const int nc = p.nc, ny = p.ny, nx = p.nx;
    const int Mc = ny * nc;
    const int m0 = tile * TX;
    const int tid = g.tid();
    if (m0 >= Mc) return;
    const void* g_a[2] = {I.G[0][0], I.G[1][0]};
    const void* g_b[2] = {I.G[0][1], I.G[1][1]};
    const void* g_q[2] = {I.G[0][2], I.G[1][2]};
    const bool plain = a.mode == Z_FWD_PLAIN || a.mode == Z_INV_PLAIN;
    const int ntiles = (Mc + TX - 1) / TX;
    constexpr int W = (2 + NQ) * TX;  // row pitch: field 0 in [0, TX), field 1 in [TX, 2 TX), q after
    C* S = reinterpret_cast<C*>(smem_raw);
    C* tw = S + NZ * W;
    constexpr int ntw = sizeof(T) == 4 ? 2 : 1;  // FP32: hi table then lo table
    C* twl = tw + NZ;
    double* red = reinterpret_cast<double*>(tw + ntw * NZ);
    for (int i = tid; i < ntw * NZ; i += NT) tw[i] = reinterpret_cast<const C*>(I.twz)[i];
    // the twiddles (written by no kernel) are loaded; what follows reads the previous
    // kernel's results
    if constexpr (PDL) CB_PDL_WAIT();
    // the control fields in one batch of independent loads (the state-selected pointer
    // is chosen in registers), so the CTA does not wait on a chain of dependent loads
    const int c_done = ctrl->done, c_fresh = ctrl->fresh, c_ab = ctrl->ab_state;
    if (!plain && c_done) return;

    const bool stage1 = a.mode == Z_ETD2_S1 || a.mode == Z_ETD4_S1 || a.mode == Z_EULER;
    const bool reuse = stage1 && !c_fresh;  // retry of a rejected step: N_u / R-hat unchanged
    const bool need_fwd = (a.mode <= Z_EULER && !reuse) || a.mode == Z_FWD_PLAIN;
    // thread 0 forms the CTA's scalars from the control state now, so its chain of global
    // loads and FP64 arithmetic runs under the forward loads and transform rather than
    // while the block waits (a barrier before the combine publishes them)
    T* bc = reinterpret_cast<T*>(red);  // dt * ga and (FP32 form) the lambda terms, once per CTA
    if (tid == 0) {
        bc[0] = (T)(ctrl->dt * p.ga);
        if constexpr (sizeof(T) == 4) {  // of the state the fused pass evaluated
            if (a.mode <= Z_EULER) {
                const int role = stage1 ? R_STATE : R_WORK;
                nonlin_lambdas<T>(p, ctrl, role, bc + 1);
                // N'(k = 0) whole, in FP64, from the fused pass's FP64 totals of G'' and
                // w (or f): its terms (mean G'', the lambda1 constant, lambda2 f-hat(0))
                // are ~1e2..1e3 and cancel to O(1), so summed in FP32 they move the
                // volume by ~1e-4 of its step-to-step change, and E with it through the
                // M1 penalty
                const Scal& sc = ctrl->sc[role];
                const bool euler = p.method == M_EULER;
                const double lam1 = p.M1 * (sc.V - ctrl->alpha), lam2 = p.M2 * (sc.S - ctrl->beta);
                const double h0 = sc.sum_h * p.invN;
                const double n0 = euler ? sc.sum_g * p.invN + 0.5 * lam1 + lam2 * h0
                                        : sc.sum_g * p.invN - 0.5 * lam1 - 1.0606601717798212866 * lam2 * h0 * p.d_ieps;
                bc[3] = (T)n0;
            }
        }
    }

    if (need_fwd) {
        // stage 1 of the FP32 form reads the state's fused-pass outputs (G slot)
        const void* srcA = I.A;
        const void* srcB = I.B;
        const void* srcQ = I.Q;
        if constexpr (sizeof(T) == 4) {
            if (stage1) {
                srcA = c_ab ? g_a[1] : g_a[0];
                srcB = c_ab ? g_b[1] : g_b[0];
                srcQ = c_ab ? g_q[1] : g_q[0];
            }
        }
        const C* gA = reinterpret_cast<const C*>(a.mode == Z_FWD_PLAIN ? a.cin : srcA);
        const C* gB = reinterpret_cast<const C*>(srcB);
        const C* gQ = reinterpret_cast<const C*>(srcQ);
        const bool two = a.mode != Z_FWD_PLAIN;
        // batches of LB loads per thread in flight before the shared-memory stores
        constexpr int LB = 4;
        constexpr int ITER = (NZ * TX + NT - 1) / NT;
        for (int b0 = 0; b0 < ITER; b0 += LB) {
            C va[LB], vb[LB], vq[LB];
#pragma unroll
            for (int j = 0; j < LB; ++j) {
                const int it = tid + (b0 + j) * NT;
                va[j] = vb[j] = vq[j] = cmk<C>(0, 0);
                const int m = m0 + it % TX;
                if (b0 + j < ITER && it < NZ * TX && m < Mc) {
                    const size_t gi = (size_t)(it / TX) * Mc + m;
                    va[j] = __ldg(gA + gi);
                    if (two) vb[j] = __ldg(gB + gi);
                    if constexpr (NQ == 1) vq[j] = __ldg(gQ + gi);
                }
            }
#pragma unroll
            for (int j = 0; j < LB; ++j) {
                const int it = tid + (b0 + j) * NT;
                if (b0 + j < ITER && it < NZ * TX) {
                    const int c = it % TX, zz = it / TX;
                    S[zz * W + c] = va[j];
                    S[zz * W + TX + c] = vb[j];
                    if constexpr (NQ == 1) S[zz * W + 2 * TX + c] = vq[j];
                }
            }
        }
        g.sync();
        if (two) fft_lines_NT<NZ, false, NT, W>(S, LinearLines{1}, W, tw, twl, g);
        else fft_lines_NT<NZ, false, NT, TX>(S, LinearLines{1}, W, tw, twl, g);
        g.sync();
    }

    const PC<T> k(p);
    const T cx = k.cx;
    const T invN = k.invN;
    const T bnl = k.bnl;

    if (a.mode == Z_FWD_PLAIN) {
        C* out = reinterpret_cast<C*>(a.cout);
        const bool to_state = (a.state_io & IO_COUT_STATE) != 0;
        for (int it = tid; it < NZ * TX; it += NT) {
            const int c = it % TX, r = it / TX, m = m0 + c;
            if (m >= Mc) continue;
            const int kz = tidx<NZ>(r);
            const C v = S[r * W + c];
            const C o = cmk<C>(k.k_invN.mul(v.x), k.k_invN.mul(v.y));
            if constexpr (sizeof(T) == 8) {
                if (a.state_io & IO_COUT_FF) {  // the FP32 form's state, split in this pass
                    const float hx = __double2float_rn(o.x), hy = __double2float_rn(o.y);
                    reinterpret_cast<float4*>(a.cout)[(size_t)kz * Mc + m] =
                        make_float4(hx, hy, __double2float_rn(o.x - (double)hx), __double2float_rn(o.y - (double)hy));
                    continue;
                }
            }
            if (to_state) State<T>::from(o).store(a.cout, (size_t)kz * Mc + m);
            else out[(size_t)kz * Mc + m] = o;
        }
        return;
    }

    // ---- combine: slot r holds kz = tidx(r)
    const void* phat = spec_of(I, ctrl, R_STATE);
    void* cand = const_cast<void*>(spec_of(I, ctrl, R_CAND));
    C* Nu = reinterpret_cast<C*>(I.Nu);
    C* Na = reinterpret_cast<C*>(I.Na);
    C* Nb = reinterpret_cast<C*>(I.Nb);
    void* ah = I.ahat;
    const T* coef = I.coef + (size_t)ctrl->tab_cur * (size_t)(p.kmax + 1) * 8;
    g.sync();
    const T dtga = bc[0];
    const T g_f = sizeof(T) == 4 ? bc[2] : (T)0;  // bc[1], the lambda1 constant, enters n0
    const T n0 = sizeof(T) == 4 ? bc[3] : (T)0;
    const bool ref4 = p.etd4_ref != 0;
    Acc<T> ag, ag2, al;
    static_assert(NT % TX == 0, "one column per thread");
    const int c = tid % TX, m = m0 + c;  // fixed column of this thread
    const int ky = m / nc, kx = m - ky * nc;
    const int kyf = min(ky, ny - ky);
    const int kxy = kx * kx + kyf * kyf;
    const T wxy = (kx == 0 || 2 * kx == nx) ? (T)1 : (T)2;
    const int gxy = ((2 * kx == nx) ? 0 : kx * kx) + ((2 * ky == ny) ? 0 : kyf * kyf);
    for (int it = tid; it < NZ * TX; it += NT) {
        const int r = it / TX;
        if (m >= Mc) {
            S[r * W + c] = cmk<C>(0, 0);
            S[r * W + TX + c] = cmk<C>(0, 0);
            continue;
        }
        const int kz = tidx<NZ>(r);
        const int kzf = min(kz, NZ - kz);
        const size_t g = (size_t)kz * Mc + m;
        C nh = cmk<C>(0, 0), wn = cmk<C>(0, 0);
        if (need_fwd) {
            const C va = S[r * W + c], vb = S[r * W + TX + c];
            if constexpr (sizeof(T) == 8) {
                const T mz = bnl * (T)(kzf * kzf);
                nh = cmk<C>((va.x + mz * vb.x) * invN, (va.y + mz * vb.y) * invN);
            } else {  // beta cx and 1/N folded hi + lo: no systematic gain on N-hat
                const T kk = (T)(kzf * kzf);
                C vm = vb;  // the field under the multiplier: B, or B + q with curvature
                if constexpr (NQ == 1) vm = cadd(vb, S[r * W + 2 * TX + c]);
                nh = cmk<C>(k.k_invN.mul(va.x + k.k_bnl.mul(kk * vm.x)), k.k_invN.mul(va.y + k.k_bnl.mul(kk * vm.y)));
                wn = cmk<C>(k.k_invN.mul(vb.x), k.k_invN.mul(vb.y));
            }
        }
        // FP32 form: the penalty terms of the fused pass's state x,
        //   + lambda-constant at k = 0 and + g_f f-hat(x), f-hat = eps cx |k|^2 x-hat + w-hat / eps (ETD)
        //   or the transformed f itself (Euler)
        const int kk_full = kxy + kzf * kzf;
        auto add_lam = [&](C& v, C xh) {
            if constexpr (sizeof(T) == 4) {
                if (m == 0 && kz == 0) {  // the whole N'(0), formed in FP64 above
                    v = cmk<C>(n0, (T)0);
                    return;
                }
                C fh;
                if (a.mode == Z_EULER) {
                    fh = wn;
                } else {
                    const T kf = (T)kk_full;
                    fh = cmk<C>(k.k_ieps.mul(wn.x) + k.k_eps.mul(k.k_cx.mul(kf * xh.x)),
                                k.k_ieps.mul(wn.y) + k.k_eps.mul(k.k_cx.mul(kf * xh.y)));
                }
                v.x = fmaf(g_f, fh.x, v.x);
                v.y = fmaf(g_f, fh.y, v.y);
            }
            (void)xh;
        };
        const T* cf = coef + 8 * (kxy + kzf * kzf);
        State<T> us;           // the new stage / state spectrum
        bool have_state = true;
        C un;
        float2 dv = make_float2(0.f, 0.f);  // FP32 form: us - state, the transformed part of u
        if constexpr (sizeof(T) == 4) {
            // the table row (8 floats, 32-byte aligned) in one or two vector loads
            float cfr[8];
            {
                const float4 q0 = __ldg(reinterpret_cast<const float4*>(cf));
                cfr[0] = q0.x; cfr[1] = q0.y; cfr[2] = q0.z; cfr[3] = q0.w;
                if constexpr (g4) {
                    const float4 q1 = __ldg(reinterpret_cast<const float4*>(cf) + 1);
                    cfr[4] = q1.x; cfr[5] = q1.y; cfr[6] = q1.z; cfr[7] = q1.w;
                } else {
                    cfr[4] = cfr[5] = cfr[6] = cfr[7] = 0.f;
                }
            }
            // FP32 form: N-hat = N'-hat + c_lin u-hat (misc_kernels.cuh, lin_coef).  nh is
            // N'-hat; the c_lin terms act on the exact double-float spectra through the
            // table, written with the stage increments d_a = a - phi, d_b = b - phi.
            switch (a.mode) {
                case Z_ETD2_S1:
                case Z_ETD4_S1: {  // a = phi (+) (em' phi + c1 N'_u)
                    if constexpr (!(g2 || g4)) break;
                    const State<T> sp = State<T>::load(phat, g);
                    if (reuse) {
                        nh = __ldg(Nu + g);
                    } else {
                        add_lam(nh, sp.work());
                        Nu[g] = nh;
                    }
                    us = sp.axpy(cfr[0], cmk<C>(cfr[1] * nh.x, cfr[1] * nh.y));
                    us.store(ah, g);
                    dv = us.diff(sp);
                    break;
                }
                case Z_ETD2_S2: {  // phi' = a (+) (c2 (N'_a - N'_u) + c2 c_lin d_a)
                    if constexpr (!g2) break;
                    const C nu = __ldg(Nu + g);
                    const State<T> sa = State<T>::load(ah, g), sp = State<T>::load(phat, g);
                    add_lam(nh, sa.work());
                    const float2 da = sa.diff(sp);
                    us = sa.add(cmk<C>(fmaf(cfr[3], da.x, cfr[2] * (nh.x - nu.x)), fmaf(cfr[3], da.y, cfr[2] * (nh.y - nu.y))));
                    us.store(cand, g);
                    dv = us.diff(sp);
                    break;
                }
                case Z_ETD4_S2:
                case Z_ETD4_S3:
                case Z_ETD4_S4: {
                    if constexpr (!g4) break;
                    const State<T> sp = State<T>::load(phat, g), sa = State<T>::load(ah, g);
                    const float2 da = sa.diff(sp);
                    const T emh = cfr[0], ch = cfr[1], chcl = cfr[6];
                    // increment of b = phi (+) (em'_h phi + c_h N'_a + c_h c_lin d_a)
                    auto inc_b = [&](C na) {
                        return cmk<C>(fmaf(chcl, da.x, ch * na.x), fmaf(chcl, da.y, ch * na.y));
                    };
                    if (a.mode == Z_ETD4_S2) {
                        add_lam(nh, sa.work());
                        Na[g] = nh;
                        us = sp.axpy(emh, inc_b(nh));
                        dv = us.diff(sp);
                        break;
                    }
                    const C na = __ldg(Na + g), nu = __ldg(Nu + g);
                    const C ib = inc_b(na);
                    const float2 db = make_float2(fmaf(emh, sp.hi.x, ib.x), fmaf(emh, sp.hi.y, ib.y));
                    const C spw = sp.work();
                    // increment of c = a (+) (em'_h a + c_h (2 N'_b - N'_u) + c_h c_lin (2 d_b - d_a))
                    auto inc_c = [&](C nb) {
                        return cmk<C>(fmaf(chcl, (T)2 * db.x - da.x, ch * ((T)2 * nb.x - nu.x)),
                                      fmaf(chcl, (T)2 * db.y - da.y, ch * ((T)2 * nb.y - nu.y)));
                    };
                    if (a.mode == Z_ETD4_S3) {
                        add_lam(nh, cmk<C>(spw.x + db.x, spw.y + db.y));  // b = phi + d_b
                        Nb[g] = nh;
                        us = sa.axpy(emh, inc_c(nh));
                        dv = us.diff(sp);
                        break;
                    }
                    // phi' = phi (+) (em'_4 phi + f1 N'_1 + f2 (N'_a + N'_b) + f3 N'_c
                    //                 + c_lin (f1 d_1 + f2 (d_a + d_b) + f3 d_c))
                    const C nb = __ldg(Nb + g);
                    const C ic = inc_c(nb);
                    const float2 dc = make_float2(da.x + fmaf(emh, sa.hi.x, ic.x), da.y + fmaf(emh, sa.hi.y, ic.y));
                    add_lam(nh, cmk<C>(spw.x + dc.x, spw.y + dc.y));  // c = phi + d_c
                    const T f1 = cfr[3], f2 = cfr[4], f3 = cfr[5], cl = cfr[7];
                    const C n1 = ref4 ? na : nu;
                    const float2 d1 = ref4 ? da : make_float2(0.f, 0.f);
                    const C inc = cmk<C>(
                        fmaf(cl, f1 * d1.x + f2 * (da.x + db.x) + f3 * dc.x, f1 * n1.x + f2 * (na.x + nb.x) + f3 * nh.x),
                        fmaf(cl, f1 * d1.y + f2 * (da.y + db.y) + f3 * dc.y, f1 * n1.y + f2 * (na.y + nb.y) + f3 * nh.y));
                    us = sp.axpy(cfr[2], inc);
                    us.store(cand, g);
                    dv = us.diff(sp);
                    break;
                }
                default: break;
            }
        }
        switch (sizeof(T) == 4 && a.mode <= Z_ETD4_S4 ? -1 : a.mode) {
            case Z_ETD2_S1: {  // a = e phi + c1 N_u (Calc.cu:453-455)
                if constexpr (!g2) break;
                if (reuse) nh = Nu[g]; else Nu[g] = nh;
                us = State<T>::load(phat, g).axpy(cf[0], cmk<C>(cf[1] * nh.x, cf[1] * nh.y));
                us.store(ah, g);
                break;
            }
            case Z_ETD2_S2: {  // phi' = a + c2 (N_a - N_u) (Calc.cu:476-477)
                if constexpr (!g2) break;
                const C nu = Nu[g];
                us = State<T>::load(ah, g).add(cmk<C>(cf[2] * (nh.x - nu.x), cf[2] * (nh.y - nu.y)));
                us.store(cand, g);
                break;
            }
            case Z_ETD4_S1: {  // a = e_h phi + c_h N_u (Calc.cu:495-497)
                if constexpr (!g4) break;
                if (reuse) nh = Nu[g]; else Nu[g] = nh;
                us = State<T>::load(phat, g).axpy(cf[0], cmk<C>(cf[1] * nh.x, cf[1] * nh.y));
                us.store(ah, g);
                break;
            }
            case Z_ETD4_S2: {  // b = e_h phi + c_h N_a (Calc.cu:516-518)
                if constexpr (!g4) break;
                Na[g] = nh;
                us = State<T>::load(phat, g).axpy(cf[0], cmk<C>(cf[1] * nh.x, cf[1] * nh.y));
                break;
            }
            case Z_ETD4_S3: {  // c = e_h a + c_h (2 N_b - N_u) (Calc.cu:537-538)
                if constexpr (!g4) break;
                Nb[g] = nh;
                const C nu = Nu[g];
                us = State<T>::load(ah, g).axpy(
                    cf[0], cmk<C>(cf[1] * ((T)2 * nh.x - nu.x), cf[1] * ((T)2 * nh.y - nu.y)));
                break;
            }
            case Z_ETD4_S4: {  // e2 phi + f1 N1 + f2 (N_a + N_b) + f3 N_c (Calc.cu:556-567)
                // N1 = N_a in the reference (belastic.cpp:550), N_u in Cox-Matthews
                if constexpr (!g4) break;
                const T f1 = cf[3], f2 = cf[4], f3 = cf[5];
                const C na = Na[g], n1 = ref4 ? na : Nu[g], nb = Nb[g];
                const C inc = cmk<C>(f1 * n1.x + f2 * (na.x + nb.x) + f3 * nh.x,
                                     f1 * n1.y + f2 * (na.y + nb.y) + f3 * nh.y);
                us = State<T>::load(phat, g).axpy(cf[2], inc);
                us.store(cand, g);
                break;
            }
            case -1: break;  // FP32 ETD stages, above
            case Z_EULER: {  // phi' = phi - dt ga R (Calc.cu:393-402)
                if constexpr (!ge) break;
                if (reuse) {
                    nh = Nu[g];
                } else {
                    add_lam(nh, cmk<C>(0, 0));
                    Nu[g] = nh;
                }
                const State<T> sp = State<T>::load(phat, g);
                us = sp.add(cmk<C>(-dtga * nh.x, -dtga * nh.y));
                us.store(cand, g);
                if constexpr (sizeof(T) == 4) dv = us.diff(sp);
                al.add(wxy * (nh.x * nh.x + nh.y * nh.y));
                break;
            }
            case Z_INV_STATE: {
                if constexpr (!gp) break;
                us = State<T>::load(spec_of(I, ctrl, a.role), g);
                if constexpr (sizeof(T) == 4)
                    if (a.role != R_STATE) dv = us.diff(State<T>::load(phat, g));
                break;
            }
            default: {  // Z_INV_PLAIN with an optional spectral multiplier
                if constexpr (!gp) break;
                have_state = false;
                C v;
                if (sizeof(T) == 8 && (a.state_io & IO_CIN_FF)) {  // the FP32 form's state, joined here
                    const float4 q = __ldg(reinterpret_cast<const float4*>(a.cin) + g);
                    v = cmk<C>((T)((double)q.x + (double)q.z), (T)((double)q.y + (double)q.w));
                } else {
                    v = (a.state_io & IO_CIN_STATE) ? State<T>::load(a.cin, g).work()
                                                    : reinterpret_cast<const C*>(a.cin)[g];
                }
                if (a.mul == SM_LAP) {
                    const int kk = kx * kx + kyf * kyf + kzf * kzf;
                    if constexpr (sizeof(T) == 8) {
                        const T mm = -cx * (T)kk;
                        un = cmk<C>(mm * v.x, mm * v.y);
                    } else {
                        un = cmk<C>(-k.k_cx.mul((T)kk * v.x), -k.k_cx.mul((T)kk * v.y));
                    }
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
        if (have_state) {
            un = us.work();
            // Parseval: mean |grad u|^2 = sum over the full spectrum of |k_g|^2 |u-hat|^2
            // (cx applied once, in FP64, when the sums are finalised)
            const int gz = (2 * kz == NZ) ? 0 : kzf;
            const T wgt = wxy * (T)(gxy + gz * gz);
            if (wgt != (T)0) us.norm2_into(ag, ag2, wgt);
            // volume from the k = 0 mode: mean u = Re u-hat(0), exactly
            if (m == 0 && kz == 0) ctrl->sc[a.role].sum_u = us.re_exact() * (double)p.N;
        }
        if constexpr (sizeof(T) == 8) {
            S[r * W + c] = un;
            const T mz = -cx * (T)(kzf * kzf);
            S[r * W + TX + c] = cmk<C>(mz * un.x, mz * un.y);
        } else {
            // FP32 form (stepping modes and Z_INV_STATE): P0 carries u - u_state, which the
            // fused xy pass adds to the state's double-float real-space field, and P2 the
            // whole Laplacian -cx |k|^2 u-hat; plain modes keep u-hat and -cx kz^2 u-hat
            S[r * W + c] = have_state ? cmk<C>(dv.x, dv.y) : un;
            const T kk = (T)(have_state ? kzf * kzf + kxy : kzf * kzf);
            S[r * W + TX + c] = cmk<C>(-k.k_cx.mul(kk * un.x), -k.k_cx.mul(kk * un.y));
        }
    }
    g.sync();
    const bool two = a.mode != Z_INV_PLAIN;
    if (two) fft_lines_TN<NZ, true, NT, 2 * TX>(S, LinearLines{1}, W, tw, twl, g);
    else fft_lines_TN<NZ, true, NT, TX>(S, LinearLines{1}, W, tw, twl, g);
    g.sync();

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

    auto g0 = ag.part();
    if constexpr (sizeof(T) == 4) g0 = ff_add(g0, ag2.part());
    else g0 += ag2.part();
    decltype(g0) vv[2] = {g0, al.part()};
    double v[2];
    g.sync();  // red held dt*ga
    block_sum<2>(vv, v, red, g);
    double* part = I.part_z;
    int* last = reinterpret_cast<int*>(red + 64);
    if (tid == 0) {
        part[2 * tile + 0] = v[0];
        part[2 * tile + 1] = v[1];
        CB_FENCE();
        const unsigned prev = atomicAdd(&ctrl->cnt_z[a.role], 1u);
        *last = prev == (unsigned)(ntiles - 1);
    }
    g.sync();
    if (*last) {  // the last CTA of this instance finalises, with all its threads
        CB_FENCE();
        double sums[2];
        block_sum_parts<2>(part, ntiles, sums, red, g);
        if (tid == 0) {
            ctrl->sc[a.role].grad2 = sums[0] * p.cx;
            if (a.mode == Z_EULER) ctrl->sc[a.role].lsq = sums[1];
            ctrl->cnt_z[a.role] = 0u;
        }
    }
}

template <class T, int NZ, int TX, int NT, int MG, int NQ = 0>
__global__ void __launch_bounds__(NT, CB_Z_THREADS_PER_SM / NT) z_kernel(const InstT<T>* __restrict__ insts, ZArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    z_body<T, NZ, TX, NT, MG, NQ, true>(insts[blockIdx.y], blockIdx.x, a, smem_raw);
}

template <class T, int NZ, int TX, int NQ = 0> __host__ __device__ constexpr size_t z_smem_bytes() {
    constexpr size_t ntw = sizeof(T) == 4 ? 2 : 1;
    return sizeof(cplx<T>) * ((size_t)NZ * (2 + NQ) * TX + ntw * NZ) + (32 * 2 + 2) * sizeof(double);
}

}  // namespace cb
