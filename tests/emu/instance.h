// Test infrastructure: FP32-form instances of the library's kernels for the emulation
// drivers (attempt.cpp, mega_attempt.cpp): every buffer an exact-size heap allocation,
// so AddressSanitizer reports an access one element outside it.
#pragma once
#include <cstdio>
#include <cstdlib>

#include "cuda_runtime.h"
#include "misc_kernels.cuh"

using namespace cb;

// twiddle tables as the stepper builds them: W_{n/2}^m then W_n^m (x), hi parts then lo parts
static void* tw_table(int n, int xkind) {
    std::vector<long double> ex;
    auto push = [&](int len) {
        for (int m = 0; m < len; ++m) {
            const long double a = 2.0L * 3.141592653589793238462643383279502884L * m / len;
            ex.push_back(cosl(a));
            ex.push_back(-sinl(a));
        }
    };
    if (xkind) push(n / 2);
    push(n);
    std::vector<float> v;
    for (auto x : ex) v.push_back((float)x);
    for (size_t i = 0; i < ex.size(); ++i) v.push_back((float)(ex[i] - (long double)v[i]));
    void* d = malloc(v.size() * sizeof(float));
    memcpy(d, v.data(), v.size() * sizeof(float));
    return d;
}

static void* zalloc(size_t b) {
    void* p = malloc(b);
    memset(p, 0, b);
    return p;
}

// the Params fields make_params (stepper.cuh) sets for an FP32-form ETD-RK2 handle
// of n x n x nz with epssize 3 (eps = 1.5 h), M1 = M2 = 1e4 and the adaptive schedule
static Params params(int n, int nz, int method) {
    Params p;
    memset(&p, 0, sizeof p);
    p.nx = p.ny = n;
    p.nz = nz;
    p.nc = n / 2 + 1;
    p.N = (long long)n * n * nz;
    p.invN = 1.0 / p.N;
    const double xlen = 2 * M_PI;
    p.cx = 1.0;
    p.L3 = xlen * xlen * xlen;
    p.eps = 1.5 * (xlen / n);
    p.eta = 1;
    p.ga = 1;
    p.M1 = 1e4;
    p.M2 = 1e4;
    p.method = method;
    p.adaptive = 1;
    p.etd4_ref = 1;
    p.kmax = 2 * (n / 2) * (n / 2) + (nz / 2) * (nz / 2);
    p.grow_every = 4;
    const bool euler = method == M_EULER;
    p.grow_factor = euler ? 1.4 : 2;
    p.dt_cap = euler ? 1e300 : 1e-3;
    p.cap_probe = euler ? 0.0 : 1.4;
    p.dt_min = 1e-23;
    p.tmax = 4;
    const double beta = euler ? p.eta : -p.eta / p.eps;
    p.d_ieps = 1 / p.eps;
    p.d_ieps2 = 1 / (p.eps * p.eps);
    p.d_ieps3 = p.d_ieps2 * p.d_ieps;
    p.d_bnl = beta * p.cx;
    p.f_eps = (float)p.eps;
    p.f_ieps = (float)p.d_ieps;
    p.f_ieps2 = (float)p.d_ieps2;
    p.f_ieps3 = (float)p.d_ieps3;
    p.f_bnl = (float)p.d_bnl;
    p.f_cx = (float)p.cx;
    p.f_invN = (float)p.invN;
    p.f_eta = (float)p.eta;
    const double k[7] = {p.eps, p.d_ieps, p.eta * p.d_ieps2, p.eta * 1.5 * p.d_ieps3, p.d_bnl, p.invN, p.cx};
    for (int i = 0; i < 7; ++i) {
        p.fk[i][0] = (float)k[i];
        p.fk[i][1] = (float)(k[i] - (double)(float)k[i]);
    }
    return p;
}

// one instance of an n x n x nz grid with a synthetic state: a smooth sphere-like
// spectrum and its real-space field; `ztx` is the z tile its partial sums are sized for
template <int N, int NZ> InstT<float> make_instance(int method, int ztx = 16) {
    using T = float;
    const Params p = params(N, NZ, method);
    const size_t ns = (size_t)NZ * N * p.nc;
    const int ntiles = (int)((N * p.nc + ztx - 1) / ztx);
    InstT<T> h;
    memset(&h, 0, sizeof h);
    for (int i = 0; i < 2; ++i) h.spec[i] = zalloc(ns * 16);
    h.ahat = zalloc(ns * 16);
    h.Nu = zalloc(ns * 8);
    if (method == M_ETD4) {  // the stepper holds N-hat_a, N-hat_b for ETD-RK4 only
        h.Na = zalloc(ns * 8);
        h.Nb = zalloc(ns * 8);
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) h.P[i][j] = zalloc(ns * 8);
    h.A = zalloc(ns * 8);
    h.B = zalloc(ns * 8);
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) h.G[i][j] = zalloc(ns * 8);
    for (int i = 0; i < 2; ++i) h.U[i] = zalloc((size_t)p.N * 8);
    h.coef = (T*)zalloc((size_t)kNTab * (p.kmax + 1) * 8 * sizeof(T));
    h.part_xy = (double*)zalloc(2 * (size_t)NZ * 4 * sizeof(double));
    h.part_z = (double*)zalloc((size_t)ntiles * 2 * sizeof(double));
    h.ctrl = (Ctrl*)zalloc(sizeof(Ctrl));
    h.twx = tw_table(N, 1);
    h.twy = tw_table(N, 0);
    h.twz = tw_table(NZ, 0);
    h.p = p;
    // a state: a smooth sphere-like spectrum (k = 0 mode and a few low modes, hi parts of
    // the double-float pairs) and its real-space field u = -1 inside, +1 outside
    {
        float* s = (float*)h.spec[0];
        s[0] = 0.5f;
        for (int m = 1; m < 6; ++m) s[4 * m] = -0.05f / m;
        float* u = (float*)h.U[0];
        for (size_t i = 0; i < (size_t)p.N; ++i) u[2 * i] = (i % 7) ? 1.f : -1.f;
    }
    Ctrl& c = *h.ctrl;
    c.dt = 1e-6;
    c.fresh = 1;
    c.target = 1 << 30;
    c.fill_slot = -1;
    c.alpha = 10;
    c.beta = 20;
    return h;
}
