// Host/device shared definitions of one stepper instance (one vesicle).
//
// HBM layout of an instance (T = float for the precision form, double for
// the plain FP64 form; C = complex T):
//   spectra      C[nz][ny][nx/2+1]  phi-hat (x2: state / candidate), a-hat,
//                                   N_u, N_a, N_b (nonlinear spectra)
//   partials     C[nz][ny][nx/2+1]  z-inverted (real z, spectral y/x) fields
//                                   P0 = IFFT_z(u-hat), P2 = IFFT_z(-kz^2 u-hat)
//                                   for three states (state / candidate / work)
//                                   and the nonlinear partials A, B
//   coef         T[(kmax+1)*8]      ETD coefficients indexed by the integer |k|^2
//   ctrl         Ctrl               FP64 scalars, dt, accept/reject state
// The forward 3-D transform is normalised by 1/N, as in the reference
// (Calc.cu:88-96); the inverse is not.
#pragma once
#include <stdint.h>

#include "cb_fft.cuh"

namespace cb {

enum Method { M_EULER = 0, M_ETD2 = 1, M_ETD4 = 2 };

// ETD coefficient tables cached per instance, one per recent dt value
// (adaptive dt moves among a handful of values: grown, capped, halved)
constexpr int kNTab = 8;

// which Scal / partial set a kernel works on
enum Role { R_STATE = 0, R_CAND = 1, R_WORK = 2, R_NROLE = 3 };

// FP64 reductions of one state.  Means are over the N grid points.
struct Scal {
    double sum_u;   // sum of u (real space)
    double sum_s2;  // sum of (u^2-1)^2
    double sum_f2;  // sum of f^2, f = -eps lap u + (u^2-1) u / eps
    double grad2;   // mean |grad u|^2 via Parseval over the half spectrum
    double lsq;     // mean R^2 of the Euler right-hand side (LSerror) via Parseval
    double V, S, E_el, E;
    // FP32 form: FP64 totals of the fused pass's real-space partials G'' and w,
    // the exact k = 0 modes of their transforms (z pass)
    double sum_g, sum_h;
    double pad;
};

struct Ctrl {
    double dt;        // time step of the next attempt
    double t;         // accepted time
    double alpha, beta, alpha0, beta0;
    double E_state;   // energy of the accepted state
    double E_init;    // energy at the start of the run (fixed-dt exit test, belastic.cpp:617,727)
    double E_last_attempt;
    double sa_eng;    // shape adjustment: energy at its last convergence check
    int steps;        // accepted steps
    int attempts;
    int rejects;
    int fresh;        // 1: stage-1 nonlinear term must be recomputed
    int done;         // 1: instance finished (kernels skip it)
    int status;       // CB_OK or an error / exit reason
    int target;       // accepted steps to take before done
    int spec_state;   // index (0/1) of the state phi-hat buffer
    int part_state;   // index (0/1) of the state partial set
    int corr_phase;   // alpha/beta correction sub-step (fixed dt, M != 0)
    int nonfinite;
    int grow_pending;  // apply the dt growth rule at the start of the next attempt
    int ab_state;      // FP32 form: G[ab_state] holds the state's fused-pass outputs
    int u_state;       // FP32 form: U[u_state] holds the state's real-space field
    int tab_cur;       // coefficient table of the current dt
    int tab_next;      // round-robin slot for the next new dt
    int fill_slot;     // table being filled this attempt (-1: none)
    unsigned fill_cnt; // last-block-done counter of the fill
    double tab_dt[kNTab];
    unsigned cnt_xy[R_NROLE];  // last-block-done counters per role
    unsigned cnt_z[R_NROLE];
    Scal sc[R_NROLE];
};

struct Params {
    int nx, ny, nz, nc;
    long long N;
    int method;         // Method
    int adaptive;       // 1: energy accept/reject with dt schedule
    int corr;           // 1: alpha/beta correction double step (fixed dt, M != 0)
    int etd4_ref;       // 1: reference combine (N_a in the first slot, belastic.cpp:550)
    int kmax;           // largest folded |k|^2 index
    int grow_every;     // grow dt every this many accepted steps
    int split;          // 1: split plane passes for every xy mode
    int sched;          // SCHED_LOOP: the time loops; SCHED_SHAPE: the shape_adjust rules
    int curv;           // FP32 form with C != 0: the fused passes carry a third field q (InstT::Q, G[.][2])
    int pad_curv;
    double eps, eta, ga, M1, M2;
    double cx;          // (2 pi / L)^2
    double L3;          // box volume
    double invN;
    double grow_factor, dt_cap, cap_probe, dt_min;
    double tmax;        // Euler loop time limit (belastic.cpp:407)
    double rel_tol;     // > 0: stop once an accepted step changes E by < rel_tol |E|
    double reject_tol;  // adaptive: reject when E_new > E_old + reject_tol |E_old|
    double C;           // spontaneous curvature (0 in the reference)
    // host-precomputed constants: GB300 runs FP64 at a small fraction of its
    // FP32 rate, so kernels read these instead of dividing per thread
    double d_ieps, d_ieps2, d_ieps3, d_bnl;  // 1/eps, 1/eps^2, 1/eps^3, beta * cx
    float f_eps, f_ieps, f_ieps2, f_ieps3, f_bnl, f_cx, f_invN, f_eta;
    // the same constants split hi + lo for the FP32 form's compensated
    // products (KC<float>): eps, 1/eps, eta/eps^2, eta D/eps^3, beta cx, 1/N, cx
    float fk[7][2];
    // FP32 form with curvature: C, the third field's factor (eps C for ETD, C for Euler)
    // and 2 eps C
    float f_C, f_qC, f_2eC, f_padc;
};
enum { FK_EPS = 0, FK_IEPS, FK_K2, FK_K3, FK_BNL, FK_INVN, FK_CX };

// the precomputed constants in the kernel's precision
template <class T> struct PC;
template <> struct PC<float> {
    float eps, ieps, ieps2, ieps3, bnl, cx, invN, eta, C, qC, e2C;
    KC<float> k_eps, k_ieps, k_K2, k_K3, k_bnl, k_invN, k_cx;
    __device__ __forceinline__ explicit PC(const Params& p)
        : eps(p.f_eps), ieps(p.f_ieps), ieps2(p.f_ieps2), ieps3(p.f_ieps3), bnl(p.f_bnl), cx(p.f_cx),
          invN(p.f_invN), eta(p.f_eta), C(p.f_C), qC(p.f_qC), e2C(p.f_2eC), k_eps{p.fk[FK_EPS][0], p.fk[FK_EPS][1]},
          k_ieps{p.fk[FK_IEPS][0], p.fk[FK_IEPS][1]}, k_K2{p.fk[FK_K2][0], p.fk[FK_K2][1]},
          k_K3{p.fk[FK_K3][0], p.fk[FK_K3][1]}, k_bnl{p.fk[FK_BNL][0], p.fk[FK_BNL][1]},
          k_invN{p.fk[FK_INVN][0], p.fk[FK_INVN][1]}, k_cx{p.fk[FK_CX][0], p.fk[FK_CX][1]} {}
};
template <> struct PC<double> {
    double eps, ieps, ieps2, ieps3, bnl, cx, invN, eta, C;
    KC<double> k_eps, k_ieps, k_K2, k_K3, k_bnl, k_invN, k_cx;
    __device__ __forceinline__ explicit PC(const Params& p)
        : eps(p.eps), ieps(p.d_ieps), ieps2(p.d_ieps2), ieps3(p.d_ieps3), bnl(p.d_bnl), cx(p.cx), invN(p.invN),
          eta(p.eta), C(p.C), k_eps{p.eps}, k_ieps{p.d_ieps}, k_K2{p.eta * p.d_ieps2}, k_K3{p.eta * 1.5 * p.d_ieps3},
          k_bnl{p.d_bnl}, k_invN{p.invN}, k_cx{p.cx} {}
};

// exit reasons kept in Ctrl::status (mirrors the public CB_* codes)
// accept / reject and dt rules of an attempt
enum { SCHED_LOOP = 0, SCHED_SHAPE = 1 };

enum { ST_RUNNING = 0, ST_TARGET = 1, ST_DT_UNDERFLOW = 2, ST_SMALL_ENERGY = 3, ST_NONFINITE = 4, ST_CONVERGED = 5,
       ST_TMAX = 6, ST_CANCELLED = 7 };

template <class T> struct InstT {
    void* spec[2];  // phi-hat state / candidate (swap via ctrl->spec_state)
    void* ahat;
    void* Nu;
    void* Na;
    void* Nb;
    void* P[3][2];  // partial sets: [0],[1] state/candidate (swap via ctrl->part_state), [2] work
    void* A;
    void* B;
    void* Y[2];       // split plane path: y-transformed fields (nullptr when unused)
    void* G[2][3];    // FP32 form: XY_FUSED outputs (G'', w, and q with curvature) of the state /
                      // candidate (ctrl->ab_state)
    void* Q;          // FP32 form with curvature: the work stage's third partial (q)
    // FP32 form: real-space u of the state / candidate as double-float pairs, rows
    // [z][y] of nx/2 float4 (two points each) in the fused passes' x-slot order
    // (ctrl->u_state).  The z pass transforms only u - u_state, and the
    // fused pass adds it to U[u_state]: u from a plain FP32 transform carries
    // ~6e-8 absolute error, which where u = +-1 + d with d below it makes
    // w = u^3 - u ~ +-2 d wrong by 100 %, with one sign over the whole far field
    void* U[2];
    T* coef;          // kNTab tables of (kmax + 1) * 8 entries
    Ctrl* ctrl;
    double* part_xy;  // [nz][4] per-plane partial sums
    double* part_z;   // [ntiles][2] per-tile partial sums
    const void* twx;  // W_{nx/2}^m (nx/2 entries) then W_nx^m (nx entries)
    const void* twy;  // W_ny^m
    const void* twz;  // W_nz^m
    Params p;
};

}  // namespace cb
