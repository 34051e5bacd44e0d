// Small kernels around the two FFT passes: ETD coefficient tables, the
// on-device accept/reject decision, and the slow-path pointwise kernels the
// field getters use.
#pragma once
#include <math.h>
#include "cb_fft.cuh"
#include "cb_inst.h"

namespace cb {

// 1 / m! (m <= 27); evaluated by the compiler wherever its argument is a constant
// expression, which phi_horner below guarantees
__host__ __device__ constexpr double rfact(int m) { return m <= 1 ? 1.0 : rfact(m - 1) / (double)m; }

// Horner steps j = J .. 0 of the three phi series; the coefficients are constexpr
// variables, so none is computed at run time (a plain loop left the recursive rfact
// to the device: hundreds of FP64 divisions per table entry)
template <int J>
__device__ __forceinline__ void phi_horner(double z, double& t1, double& t2, double& t3) {
    constexpr double c1 = rfact(J + 1), c2 = rfact(J + 2), c3 = rfact(J + 3);
    t1 = fma(t1, z, c1);
    t2 = fma(t2, z, c2);
    t3 = fma(t3, z, c3);
    if constexpr (J > 0) phi_horner<J - 1>(z, t1, t2, t3);
}

// phi_k(z) = sum_j z^j / (j+k)!, k = 1, 2, 3: Horner series for |z| < 1
// (24 terms, no divisions), closed forms otherwise
__device__ inline void phi123(double z, double& p1, double& p2, double& p3) {
    if (fabs(z) < 1.0) {
        constexpr double r24 = rfact(24), r25 = rfact(25), r26 = rfact(26);
        double t1 = r24, t2 = r25, t3 = r26;
        phi_horner<23>(z, t1, t2, t3);
        p1 = t1; p2 = t2; p3 = t3;
    } else {
        const double ez = exp(z), iz = 1.0 / z;
        p1 = (ez - 1.0) * iz;
        p2 = (p1 - 1.0) * iz;
        p3 = (p2 - 0.5) * iz;
    }
}

// The prologue's part of the control state: what it reads and what it changes.
struct ProState {
    double dt, t, sa_eng;
    int skip;          // the instance was done on entry: nothing changes
    int grow_pending, done, status, tab_cur, tab_next;
    int fill_slot;     // table slot to fill with dt (-1: none)
};

// Prologue of every attempt, as a function of the control state the previous kernel
// left (it writes nothing).  It applies a pending growth of dt (set when the accepted
// step count reached a multiple of grow_every: belastic.cpp:644-651, :376-378), so the
// step runs with the grown dt exactly as the reference's loop head grows it, then
// selects the coefficient table of the attempt's dt from the per-instance cache,
// marking a slot for filling on a miss.
__device__ inline ProState prologue_state(const Params& p, const Ctrl* c, int raw) {
    ProState s;
    s.dt = c->dt;
    s.t = c->t;
    s.sa_eng = c->sa_eng;
    s.grow_pending = c->grow_pending;
    s.done = c->done;
    s.status = c->status;
    s.tab_cur = c->tab_cur;
    s.tab_next = c->tab_next;
    s.fill_slot = -1;
    s.skip = s.done;
    if (s.skip) return s;
    if (p.sched == SCHED_SHAPE) {
        // loop head of belastic::shape_adjust (belastic.cpp:204-233), run once per
        // accepted step: advance tcur (t) by dt and count the step (the reference's
        // counter starts at 1 and is raised before the tests); test convergence when
        // dt > 1e-4 or int(tcur/dt) is a multiple of int(1e-4/dt); double dt every
        // tenth count.  The quotients are truncated in 64 bits: the reference's int
        // conversion has no defined result beyond 2^31.
        if (s.grow_pending) {
            s.grow_pending = 0;
            s.t += s.dt;
            const int count = c->steps + 2;
            if (s.dt > 1e-4 || ((long long)(s.t / s.dt)) % ((long long)(1e-4 / s.dt)) == 0) {
                const double e1 = c->E_state, e0 = s.sa_eng;
                if (e1 < 100.0 * p.eta || fabs((e0 - e1) / e0) < 0.02) {
                    s.done = 1;
                    s.status = ST_CONVERGED;
                    return s;
                }
                s.sa_eng = e1;
            }
            if (count % 10 == 0) s.dt *= 2.0;
        }
        return s;
    }
    if (!raw && s.grow_pending) {
        const double d0 = s.dt;
        s.dt = (d0 * p.cap_probe < p.dt_cap) ? d0 * p.grow_factor : p.dt_cap;
        s.grow_pending = 0;
    }
    if (p.method == M_EULER) return s;
    for (int j = 0; j < kNTab; ++j)
        if (c->tab_dt[j] == s.dt) {
            s.tab_cur = j;
            return s;
        }
    const int j = s.tab_next;
    s.tab_next = (j + 1) % kNTab;
    s.tab_cur = j;
    s.fill_slot = j;
    return s;
}

// Linear part of the ETD nonlinearity, c_lin(k) = eta kappa (D / eps^3 + cx |k|^2 / eps):
// N-hat = N'-hat + c_lin u-hat, with N' formed from G' = G - eta D kappa u / eps^3 and
// H' = H + kappa u = (u^2 - 1) u, both small where u = +-1.  The FP32 form transforms
// only G', H' and applies c_lin u-hat to the exact (double-float) spectrum through its
// table: the bulk terms of G (~eta D kappa / eps^3, thousands) otherwise carry FP32
// transform and rounding errors into the k ~ 0 modes, which the energy amplifies.
__device__ inline double lin_coef(const Params& p, int k2) {
    const double kappa = 2.0, D = 1.5;
    return p.eta * kappa * (D * p.d_ieps3 + p.cx * (double)k2 * p.d_ieps);
}

// Fills block `blk`'s share of table `slot` for time step dt (blocks 0..nblk-1 of
// blockDim.x threads together fill entries 0..kmax).
// L(k) follows Calc.cu:579-606 with c = -cx |k|^2 (kappa = 2, D = 1.5).
// accurate == 0 evaluates the reference's own closed forms (Calc.cu:446-569);
// accurate == 1 uses phi-functions, free of the small-|hL| cancellation.
// The FP32 form stores, for the split N-hat = N'-hat + c_lin u-hat (lin_coef),
//   ETD-RK2: em' = c1 L' (L' = L + c_lin), c1, c2, c2 c_lin
//   ETD-RK4: em'_h = c_h L', c_h, em'_4 = exp(hL) - 1 + c_lin (f1 + 2 f2 + f3),
//            f1, f2, f3, c_h c_lin, c_lin
// and its state update is base (+) (em' base + increment) in double-float
// arithmetic (z_kernel.cuh, State<float>).
template <class T>
__device__ inline void fill_table(const InstT<T>& I, const Params& p, int slot, double dt, int accurate, int blk,
                                  int nblk) {
    const double kappa = 2.0, D = 1.5, eps = p.eps, ie = p.d_ieps, ie2 = p.d_ieps2;
    T* tab = I.coef + (size_t)slot * (size_t)(p.kmax + 1) * 8;
    for (int idx = blk * blockDim.x + threadIdx.x; idx <= p.kmax; idx += nblk * blockDim.x) {
        const double c = -(double)idx * p.cx;
        const double L = -eps * c * c + kappa * c * ie + D * (c - kappa * ie2) * ie;
        T* out = tab + 8 * (size_t)idx;
        if (p.method == M_ETD2) {
            double x0, c1, c2;
            if (accurate) {
                double p1, p2, p3;
                phi123(dt * L, p1, p2, p3);
                c1 = dt * p1;
                c2 = dt * p2;
                x0 = (sizeof(T) == 4) ? dt * L * p1 : exp(L * dt);
            } else {
                const double e1 = exp(L * dt);
                c1 = (e1 - 1.0) / L;
                c2 = (dt * L == 0.0) ? dt / 2 : (e1 - 1.0 - dt * L) / (dt * L * L);
                x0 = (sizeof(T) == 4) ? e1 - 1.0 : e1;
            }
            if constexpr (sizeof(T) == 4) {  // the linear-split form (see lin_coef)
                const double cl = lin_coef(p, idx);
                out[0] = (T)(c1 * (L + cl));  // em' = (exp(hL) - 1) L' / L
                out[3] = (T)(c2 * cl);
            } else {
                out[0] = (T)x0;
            }
            out[1] = (T)c1; out[2] = (T)c2;
        } else {
            double x0, x2, ch, f1, f2, f3;
            if (accurate) {
                double q1, q2, q3, p1, p2, p3;
                phi123(dt * L / 2, q1, q2, q3);
                phi123(dt * L, p1, p2, p3);
                ch = dt / 2 * q1;
                f1 = dt * (p1 - 3.0 * p2 + 4.0 * p3);
                f2 = 2.0 * dt * (p2 - 2.0 * p3);
                f3 = dt * (4.0 * p3 - p2);
                x0 = (sizeof(T) == 4) ? dt * L / 2 * q1 : exp(L * dt / 2);
                x2 = (sizeof(T) == 4) ? dt * L * p1 : exp(L * dt);
            } else {
                const double eh = exp(L * dt / 2), e2 = eh * eh, h = dt;
                const double q = 1.0 / (h * h * L * L * L);
                ch = (eh - 1.0) / L;
                f1 = q * (-4.0 - h * L + e2 * (4.0 - 3.0 * h * L + h * h * L * L));
                f2 = q * 2.0 * (2.0 + h * L + e2 * (-2.0 + h * L));
                f3 = q * (-4.0 - 3.0 * h * L - h * h * L * L + e2 * (4.0 - h * L));
                x0 = (sizeof(T) == 4) ? eh - 1.0 : eh;
                x2 = (sizeof(T) == 4) ? e2 - 1.0 : e2;
            }
            if constexpr (sizeof(T) == 4) {
                const double cl = lin_coef(p, idx);
                out[0] = (T)(ch * (L + cl));                        // em'_h
                out[2] = (T)(x2 + cl * (f1 + 2.0 * f2 + f3));       // em'_4
                out[6] = (T)(ch * cl);
                out[7] = (T)cl;
            } else {
                out[0] = (T)x0; out[2] = (T)x2;
            }
            out[1] = (T)ch; out[3] = (T)f1; out[4] = (T)f2; out[5] = (T)f3;
        }
    }
}

// The prologue and the coefficient table of an attempt in one launch (grid: blocks x
// instances).  Every block derives the prologue's new state from the state the
// previous kernel left (prologue_state reads only), fills its share of the table when
// dt is new, and the last block to finish writes the new state: every block has read
// the old state before it counts itself done, so none sees a half-written one.
// Block `blk` of the nblk blocks of one instance's prologue (all threads of the CTA);
// sp and lastp point to the block's shared copies of the new state and of the
// last-block flag.
template <class T>
__device__ __forceinline__ void prologue_body(const InstT<T>& I, int blk, int nblk, int accurate, int raw,
                                              ProState* sp, int* lastp) {
    Ctrl* ctrl = I.ctrl;
    const Params& p = I.p;
    ProState& s = *sp;
    if (threadIdx.x == 0) s = prologue_state(p, ctrl, raw);
    __syncthreads();
    if (s.skip) return;
    if (s.fill_slot >= 0) fill_table<T>(I, p, s.fill_slot, s.dt, accurate, blk, nblk);
    __syncthreads();
    if (threadIdx.x == 0) {
        CB_FENCE();
        const unsigned prev = atomicAdd(&ctrl->fill_cnt, 1u);
        const int last = prev == (unsigned)(nblk - 1);
        *lastp = last;
        if (last) {
            ctrl->fill_cnt = 0u;
            ctrl->dt = s.dt;
            ctrl->t = s.t;
            ctrl->sa_eng = s.sa_eng;
            ctrl->grow_pending = s.grow_pending;
            ctrl->done = s.done;
            ctrl->status = s.status;
            ctrl->tab_cur = s.tab_cur;
            ctrl->tab_next = s.tab_next;
            if (s.fill_slot >= 0) ctrl->tab_dt[s.fill_slot] = s.dt;
            ctrl->fill_slot = -1;
        }
    }
}
template <class T>
__global__ void prologue_fill_kernel(const InstT<T>* __restrict__ insts, int accurate, int raw) {
    CB_PDL_TRIGGER();
    CB_PDL_WAIT();
    __shared__ ProState s;
    __shared__ int last;
    prologue_body<T>(insts[blockIdx.y], blockIdx.x, gridDim.x, accurate, raw, &s, &last);
}

// Accept / reject after one attempt (one thread per instance).
//   adaptive: reject when E_new > E_old, halve dt (belastic.cpp:653-668 and :380-394);
//             grow dt every grow_every accepted steps (belastic.cpp:644-651, :376-378)
//   corr:     fixed dt with M != 0 -- correct alpha/beta and redo the step once
//             from the kept state (belastic.cpp:670-691)
//   raw:      1: accept unconditionally (a single reference step body);
//             2: accept nothing and keep dt (attempts timed by the autotuner)
// Exit tests follow belastic.cpp:400-428 (Euler) and :712-740 (ETD).
// The decision on a copy of the control state (decide_one writes it back).
__device__ inline void decide_update(Ctrl* c, const Params& p, int raw) {
    c->attempts++;
    if (raw == 2) {  // a timing attempt: the state, dt and counters stay, the next attempt is fresh
        c->fresh = 1;
        return;
    }
    const Scal cs = c->sc[R_CAND];
    const double E1 = cs.E;
    c->E_last_attempt = E1;
    if (p.sched == SCHED_SHAPE) {
        // belastic.cpp:245-262: keep the attempt only if the energy fell strictly
        // (a non-finite attempt never does); otherwise halve dt, ending below dt_min
        if (!(E1 < c->E_state)) {
            c->dt *= 0.5;
            c->rejects++;
            c->fresh = 0;
            if (c->dt < p.dt_min) { c->done = 1; c->status = ST_DT_UNDERFLOW; }
            return;
        }
        c->spec_state ^= 1;
        c->part_state ^= 1;
        c->ab_state ^= 1;
        c->u_state ^= 1;
        c->sc[R_STATE] = cs;
        c->E_state = E1;
        c->fresh = 1;
        c->steps++;
        c->grow_pending = 1;  // the loop head runs before the next attempt
        if (c->steps >= c->target) { c->done = 1; c->status = ST_TARGET; }
        return;
    }
    if (!raw) {
        if (p.adaptive) {
            if (E1 > c->E_state + p.reject_tol * fabs(c->E_state)) {
                c->dt *= 0.5;
                c->rejects++;
                c->fresh = 0;
                if (c->dt < p.dt_min) { c->done = 1; c->status = ST_DT_UNDERFLOW; }
                return;
            }
        } else if (p.corr) {
            c->alpha -= (cs.V - c->alpha0);
            c->beta -= (cs.S - c->beta0);
            if (c->corr_phase == 0) {
                c->corr_phase = 1;
                c->fresh = 1;  // N_u depends on alpha, beta
                return;
            }
            c->corr_phase = 0;
        }
    }
    // accept: the candidate becomes the state
    const double E0 = c->E_state;
    c->spec_state ^= 1;
    c->part_state ^= 1;
    c->ab_state ^= 1;  // FP32 form: the candidate's fused-pass outputs become the state's
    c->u_state ^= 1;   // and its real-space field
    c->sc[R_STATE] = cs;
    if (!raw && p.corr) {  // the energy against the corrected targets (belastic.cpp:68-86)
        const double ve = cs.V - c->alpha, se = cs.S - c->beta;
        c->sc[R_STATE].E = p.eta * cs.E_el + 0.5 * p.M1 * ve * ve + 0.5 * p.M2 * se * se;
    }
    c->E_state = c->sc[R_STATE].E;
    c->fresh = 1;
    const bool nonfinite = !isfinite(E1) || !isfinite(cs.V) || !isfinite(cs.S);
    if (nonfinite) { c->done = 1; c->status = ST_NONFINITE; c->nonfinite = 1; return; }
    if (!raw) {
        if (p.method == M_EULER) {
            if (c->t > p.tmax) { c->done = 1; c->status = ST_TMAX; return; }
            if (cs.lsq * p.L3 < 1e-25) { c->done = 1; c->status = ST_CONVERGED; return; }
        } else {
            const double e0 = p.adaptive ? E0 : c->E_init;
            if (e0 < 1e-3) { c->done = 1; c->status = ST_SMALL_ENERGY; return; }
        }
    }
    c->t += c->dt;
    c->steps++;
    if (c->steps >= c->target) { c->done = 1; c->status = ST_TARGET; }
    // relaxation criterion |dE / E| < rel_tol (no counterpart in the reference loops)
    if (!raw && p.rel_tol > 0.0 && fabs(E1 - E0) < p.rel_tol * fabs(E1)) { c->done = 1; c->status = ST_CONVERGED; }
    if (!raw && p.adaptive && c->steps % p.grow_every == 0) c->grow_pending = 1;
}

// One thread per instance.  The control state and the parameters are copied in one
// batch of independent loads, the decision runs on the copies, and the state is
// written back in one batch: a chain of dependent global loads otherwise sets the
// kernel's length.
// the decision of one instance on a register copy of its control block
template <class T> __device__ __forceinline__ void decide_one(const InstT<T>& I, int raw) {
    Ctrl* g = I.ctrl;
    Ctrl c = *g;
    if (c.done) return;
    const Params p = I.p;
    decide_update(&c, p, raw);
    *g = c;
}

template <class T>
__global__ void decide_kernel(const InstT<T>* __restrict__ insts, int n, int raw) {
    CB_PDL_TRIGGER();
    CB_PDL_WAIT();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    decide_one(insts[i], raw);
}

// ---------------------------------------------------------- slow path
enum PwKind { PW_F = 0, PW_G0 = 1, PW_T = 2, PW_NLD = 3, PW_S = 4, PW_RHS = 5 };

// Pointwise field getters on FP64 real arrays (Calc.cu:153-180, :265-284, :358-368, :410-419).
static __global__ void pointwise_kernel(int kind, size_t n, double* out, const double* a, const double* b,
                                 const double* c, const double* d, double eps, double x0, double x1, double x2) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        const double u = a[i];
        switch (kind) {
            case PW_F: out[i] = -b[i] * eps + (u * u - 1.0) * u / eps; break;                   // b = lap u
            case PW_G0: out[i] = -c[i] + (3.0 * u * u - 1.0) * b[i] / (eps * eps); break;      // b = f, c = lap f
            case PW_T: out[i] = u * (u * u - 1.0 - 2.0); break;
            case PW_NLD: {                                                                     // b = f, c = t, d = lap t
                const double ie = 1.0 / eps, ie2 = ie * ie, ie3 = ie * ie2, D = 1.5;
                out[i] = -d[i] * ie + D * c[i] * ie3 + (3.0 * u * u - D - 1.0) * ie2 * b[i];
                break;
            }
            case PW_S: {  // a = u, b, c, d = grad
                const double g = b[i] * b[i] + c[i] * c[i] + d[i] * d[i];
                out[i] = 0.5 * eps * g + 0.25 / eps * (u * u - 1.0) * (u * u - 1.0);
                break;
            }
            case PW_RHS: out[i] = x0 * 0.5 + x1 * b[i] + c[i] * x2; break;                    // a unused, b = f, c = g0
        }
    }
}

// stepped-state spectrum (FP64, or double-float pairs in the FP32 form) -> complex double
template <class T>
__global__ void state_to_double_kernel(const void* __restrict__ in, double2* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        if (sizeof(T) == 4) {
            const float4 q = reinterpret_cast<const float4*>(in)[i];
            out[i] = make_double2((double)q.x + (double)q.z, (double)q.y + (double)q.w);
        } else {
            out[i] = reinterpret_cast<const double2*>(in)[i];
        }
    }
}

// full N-hat = N'-hat + c_lin u-hat of the FP32 form's split (lin_coef), in FP64,
// for the field getter; the FP64 form keeps the full N-hat in Nu
template <class T>
__global__ void nhat_full_kernel(const InstT<T>* __restrict__ insts, const void* __restrict__ spec,
                                 double2* __restrict__ out) {
    const InstT<T>& I = insts[0];
    const Params& p = I.p;
    const size_t n = (size_t)p.nz * p.ny * p.nc;
    const cplx<T>* nu = reinterpret_cast<const cplx<T>*>(I.Nu);
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
        double2 v = make_double2((double)nu[i].x, (double)nu[i].y);
        if (sizeof(T) == 4) {
            const int kx = (int)(i % p.nc), ky = (int)((i / p.nc) % p.ny), kz = (int)(i / ((size_t)p.nc * p.ny));
            const int kyf = min(ky, p.ny - ky), kzf = min(kz, p.nz - kz);
            const double cl = lin_coef(p, kx * kx + kyf * kyf + kzf * kzf);
            const float4 q = reinterpret_cast<const float4*>(spec)[i];
            v.x += cl * ((double)q.x + (double)q.z);
            v.y += cl * ((double)q.y + (double)q.w);
        }
        out[i] = v;
    }
}

template <class T>
__global__ void cplx_to_double_kernel(const cplx<T>* __restrict__ in, double2* __restrict__ out, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        out[i] = make_double2((double)in[i].x, (double)in[i].y);
}

}  // namespace cb
