// Test infrastructure (tests/test_kernel_emulation.py): one FP32-form attempt (ETD-RK2,
// ETD-RK4 or Euler) on an n x n x nz grid through the library's own kernel sources, run
// on the host by the CUDA emulation in fake/ and checked by AddressSanitizer.  Every device buffer and every
// block's shared memory is a separate heap allocation of the exact size the library
// gives it, so an index one element past any of them is reported.
//
// Sequence (as cb_set_phi and one attempt of the stepper's loop run it):
//   z Z_INV_STATE (state)   -> xy XY_FUSED (state)
//   prologue + coefficient fill -> the method's z stages, each but the last followed by
//   xy FUSED (work) -> xy FUSED (candidate) -> decide
// The xy passes run on the schedule given on the command line: 2 = one CTA per plane,
// 3 = two-CTA clusters.  The sums the passes leave are printed for comparison.
#include <cstdio>
#include <cstdlib>
#include <functional>
#include <thread>
#include <vector>

#include "cuda_runtime.h"
#include "misc_kernels.cuh"
#include "xy_cluster.cuh"
#include "xy_kernel.cuh"
#include "z_kernel.cuh"

namespace emu {
thread_local Block* t_blk = nullptr;
thread_local dim3 t_tid, t_bid;
dim3 g_bdim, g_gdim;
std::mutex g_atomic_mu;

// body() for every thread of the grid, `clus` consecutive blocks (along x) at a time;
// one OS thread per CUDA thread of a cluster, reused for every cluster of the grid
void launch(dim3 grid, int nt, size_t smem, int clus, const std::function<void()>& body) {
    g_bdim = dim3(nt);
    g_gdim = grid;
    const int total = nt * clus;
    Cluster cl;
    std::vector<Block> blocks(clus);
    for (int r = 0; r < clus; ++r) {
        blocks[r].ex = new double[nt];
        blocks[r].smem = (unsigned char*)malloc(smem ? smem : 1);
        blocks[r].smem_bytes = smem;
        blocks[r].rank = r;
        blocks[r].cl = &cl;
        cl.blocks[r] = &blocks[r];
    }
    auto reset = [&] {
        cl.bar.alive = total;
        cl.bar.arrived = 0;
        for (int r = 0; r < clus; ++r) {
            blocks[r].bar.alive = nt;
            blocks[r].bar.arrived = 0;
            memset(blocks[r].smem, 0xA5, smem);
        }
    };
    reset();
    Barrier pool;
    pool.alive = total;
    std::vector<std::thread> th;
    th.reserve(total);
    for (int t = 0; t < total; ++t)
        th.emplace_back([&, t] {
            const int r = t / nt;
            for (unsigned by = 0; by < grid.y; ++by)
                for (unsigned bx = 0; bx < grid.x; bx += clus) {
                    t_blk = &blocks[r];
                    t_tid = dim3(t % nt);
                    t_bid = dim3(bx + r, by);
                    body();
                    blocks[r].bar.drop();
                    cl.bar.drop();
                    pool.wait();  // every thread is done with this cluster
                    if (t == 0) reset();
                    pool.wait();
                }
        });
    for (auto& x : th) x.join();
    for (auto& b : blocks) {
        free(b.smem);
        delete[] b.ex;
    }
}
}  // namespace emu

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

template <int N, int NZ> int run(int path, int method) {
    using T = float;
    const Params p = params(N, NZ, method);
    const size_t ns = (size_t)NZ * N * p.nc;
    const int ntiles = (int)((N * p.nc + 15) / 16);
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
    InstT<T>* d = &h;

    auto xy = [&](int mode, int role) {
        XYArgs a;
        memset(&a, 0, sizeof a);
        a.mode = mode;
        a.role = role;
        if (path == XYP_CLUSTER) {
            if constexpr (N >= 64) {  // the cluster pass is built from 64^2 planes
                constexpr int NT = N >= 96 ? 512 : 256;
                emu::launch(dim3(2 * NZ, 1), NT, xyc_smem_bytes<T, N>(), 2, [&] { xyc_fused_kernel<T, N, NT>(d, a); });
            }
        } else {
            constexpr int NT = N <= 32 ? 128 : (N <= 64 ? 256 : 1024);
            emu::launch(dim3(NZ, 1), NT, xy_smem_bytes<T, N>(2), 1, [&] { xy_kernel<T, N, NT, 2>(d, a); });
        }
    };
    auto z = [&](int mode, int role, auto group) {
        constexpr int MG = decltype(group)::value;
        ZArgs a;
        memset(&a, 0, sizeof a);
        a.mode = mode;
        a.role = role;
        emu::launch(dim3(ntiles, 1), 256, z_smem_bytes<T, NZ, 16>(), 1, [&] { z_kernel<T, NZ, 16, 256, MG>(d, a); });
    };
    using GP = std::integral_constant<int, ZG_PLAIN>;
    using G2 = std::integral_constant<int, ZG_ETD2>;
    using G4 = std::integral_constant<int, ZG_ETD4>;
    using GE = std::integral_constant<int, ZG_EULER>;
    z(Z_INV_STATE, R_STATE, GP{});
    xy(XY_FUSED, R_STATE);
    c.E_state = c.sc[R_STATE].E;
    emu::launch(dim3(64, 1), 256, 0, 1, [&] { prologue_fill_kernel<T>(d, 1, 0); });
    if (method == M_ETD2) {
        z(Z_ETD2_S1, R_WORK, G2{});
        xy(XY_FUSED, R_WORK);
        z(Z_ETD2_S2, R_CAND, G2{});
    } else if (method == M_ETD4) {
        z(Z_ETD4_S1, R_WORK, G4{});
        xy(XY_FUSED, R_WORK);
        z(Z_ETD4_S2, R_WORK, G4{});
        xy(XY_FUSED, R_WORK);
        z(Z_ETD4_S3, R_WORK, G4{});
        xy(XY_FUSED, R_WORK);
        z(Z_ETD4_S4, R_CAND, G4{});
    } else {
        z(Z_EULER, R_CAND, GE{});
    }
    xy(XY_FUSED, R_CAND);
    emu::launch(dim3(1), 128, 0, 1, [&] { decide_kernel<T>(d, 1, 0); });
    printf("state V %.17g S %.17g E %.17g sum_g %.17g\n", c.sc[R_STATE].V, c.sc[R_STATE].S, c.sc[R_STATE].E,
           c.sc[R_STATE].sum_g);
    printf("work V %.17g S %.17g sum_g %.17g sum_h %.17g\n", c.sc[R_WORK].V, c.sc[R_WORK].S, c.sc[R_WORK].sum_g,
           c.sc[R_WORK].sum_h);
    printf("cand V %.17g S %.17g E %.17g\n", c.sc[R_CAND].V, c.sc[R_CAND].S, c.sc[R_CAND].E);
    printf("ctrl attempts %d steps %d rejects %d tab_cur %d u_state %d cnt_xy %u cnt_z %u\n", c.attempts, c.steps,
           c.rejects, c.tab_cur, c.u_state, c.cnt_xy[0] + c.cnt_xy[1] + c.cnt_xy[2],
           c.cnt_z[0] + c.cnt_z[1] + c.cnt_z[2]);
    return 0;
}

int main(int argc, char** argv) {
    const int n = argc > 1 ? atoi(argv[1]) : 32;
    const int nz = argc > 2 ? atoi(argv[2]) : n;
    const int path = argc > 3 ? atoi(argv[3]) : XYP_SINGLE;
    const int method = argc > 4 ? atoi(argv[4]) : M_ETD2;
    if (n == 16 && nz == 16) return run<16, 16>(path, method);
    if (n == 32 && nz == 32) return run<32, 32>(path, method);
    if (n == 48 && nz == 16) return run<48, 16>(path, method);
    if (n == 64 && nz == 16) return run<64, 16>(path, method);
    if (n == 96 && nz == 16) return run<96, 16>(path, method);
    fprintf(stderr, "grid %dx%dx%d not built into the emulation harness\n", n, n, nz);
    return 2;
}
