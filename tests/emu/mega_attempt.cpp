// Test infrastructure (tests/test_kernel_emulation.py): one attempt of a small batched pool
// through the persistent batched kernel (mega.cuh), run on the host by the CUDA emulation
// in fake/ and checked by AddressSanitizer, against the same attempt through the one-pass
// kernels with the persistent kernel's shapes (the one-pass z and one-CTA plane kernels'
// own shapes, 512-thread CTAs for the cluster plane pass).  Both run the same pass bodies,
// so every buffer and every control field must come out bitwise the same; the persistent
// kernel's own parts (the work list, the unit hand-over between the two CTAs of a cluster,
// the thread groups on named barriers, the dependency counters, the decision by the CTA
// that ends an instance's last phase) are what differ.
//
// The pool: a 32^3 instance (planes one per CTA), a 64 x 64 x 16 instance (planes on
// both CTAs of a cluster) and a 16^3 instance, each with its own synthetic state.  The
// emulation runs one cluster, so the units run in list order.
#define CB_MEGA_SIZES(X) X(16) X(32) X(64)

#include <cstdio>
#include <cstdlib>
#include <functional>
#include <thread>
#include <vector>

#include "cuda_runtime.h"
#include "emu_launch.h"
#include "instance.h"
#include "mega.cuh"

using T = float;

template <int N, int NZ> struct Inst {
    InstT<T> h;
    explicit Inst(int seed) : h(make_instance<N, NZ>(M_ETD2)) {  // partial sums sized as the stepper sizes them
        // instances differ: scale the state's low modes
        float* s = (float*)h.spec[0];
        for (int m = 1; m < 6; ++m) s[4 * m] *= 1.0f + 0.1f * seed;
        h.ctrl->alpha = 10 + seed;
    }
    // the set-up pass of cb_set_phi: partials and sums of the state
    void setup() {
        InstT<T>* d = &h;
        ZArgs za = {};
        za.mode = Z_INV_STATE;
        za.role = R_STATE;
        const int nt = (N * h.p.nc + 15) / 16;
        emu::launch(dim3(nt, 1), 256, z_smem_bytes<T, NZ, 16>(), 1, [&] { z_kernel<T, NZ, 16, 256, ZG_PLAIN>(d, za); });
        xy(XY_FUSED, R_STATE);
        h.ctrl->E_state = h.ctrl->sc[R_STATE].E;
    }
    void xy(int mode, int role) {
        InstT<T>* d = &h;
        XYArgs a = {};
        a.mode = mode;
        a.role = role;
        if constexpr (mega_cluster_xy(N)) {
            emu::launch(dim3(2 * NZ, 1), kMegaThreads, xyc_smem_bytes<T, N>(), 2,
                        [&] { xyc_fused_kernel<T, N, kMegaThreads>(d, a); });
        } else {
            constexpr int NT = mega_xy_threads(N);
            emu::launch(dim3(NZ, 1), NT, xy_smem_bytes<T, N>(2), 1, [&] { xy_kernel<T, N, NT, 2>(d, a); });
        }
    }
    void z(int mode, int role) {
        InstT<T>* d = &h;
        ZArgs za = {};
        za.mode = mode;
        za.role = role;
        const int nt = (N * h.p.nc + kMegaZTX - 1) / kMegaZTX;
        emu::launch(dim3(nt, 1), kMegaZThreads, z_smem_bytes<T, NZ, kMegaZTX>(), 1,
                    [&] { z_kernel<T, NZ, kMegaZTX, kMegaZThreads, ZG_ETD2>(d, za); });
    }
    // one ETD-RK2 attempt through the one-pass kernels
    void attempt() {
        InstT<T>* d = &h;
        // prologue_fill_kernel's body with its block state in the emulated block's shared
        // memory (the emulation gives a kernel's static __shared__ variables one copy per thread)
        emu::launch(dim3(64, 1), 256, 64, 1, [&] {
            unsigned char* sm = emu::t_blk->smem;
            prologue_body<T>(*d, (int)blockIdx.x, 64, 0, 0, reinterpret_cast<ProState*>(sm), reinterpret_cast<int*>(sm + 60));
        });
        z(Z_ETD2_S1, R_WORK);
        xy(XY_FUSED, R_WORK);
        z(Z_ETD2_S2, R_CAND);
        xy(XY_FUSED, R_CAND);
        emu::launch(dim3(1), 128, 0, 1, [&] { decide_kernel<T>(d, 1, 0); });
    }
};

// buffers of one instance compared byte for byte
static int compare(const char* name, const InstT<T>& a, const InstT<T>& b) {
    const Params& p = a.p;
    const size_t ns = (size_t)p.nz * p.ny * p.nc;
    struct Buf {
        const char* what;
        const void *x, *y;
        size_t n;
    };
    std::vector<Buf> bufs = {{"spec0", a.spec[0], b.spec[0], ns * 16}, {"spec1", a.spec[1], b.spec[1], ns * 16},
                             {"ahat", a.ahat, b.ahat, ns * 16},         {"Nu", a.Nu, b.Nu, ns * 8},
                             {"A", a.A, b.A, ns * 8},                   {"B", a.B, b.B, ns * 8},
                             {"U0", a.U[0], b.U[0], (size_t)p.N * 8},   {"U1", a.U[1], b.U[1], (size_t)p.N * 8}};
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 2; ++j) bufs.push_back({"P", a.P[i][j], b.P[i][j], ns * 8});
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 2; ++j) bufs.push_back({"G", a.G[i][j], b.G[i][j], ns * 8});
    bufs.push_back({"coef", a.coef, b.coef, (size_t)kNTab * (p.kmax + 1) * 8 * sizeof(T)});
    int bad = 0;
    for (auto& x : bufs)
        if (memcmp(x.x, x.y, x.n)) {
            printf("%s: %s differs\n", name, x.what);
            ++bad;
        }
    const Ctrl &c = *a.ctrl, &d = *b.ctrl;
    if (memcmp(c.sc, d.sc, sizeof c.sc)) { printf("%s: sums differ\n", name); ++bad; }
    if (c.dt != d.dt || c.attempts != d.attempts || c.steps != d.steps || c.rejects != d.rejects ||
        c.spec_state != d.spec_state || c.u_state != d.u_state || c.ab_state != d.ab_state || c.done != d.done ||
        c.E_state != d.E_state || c.tab_cur != d.tab_cur || c.fresh != d.fresh) {
        printf("%s: control state differs\n", name);
        ++bad;
    }
    printf("%s attempts %d steps %d rejects %d E %.17g cnt_xy %u cnt_z %u fill_cnt %u\n", name, c.attempts, c.steps,
           c.rejects, c.sc[R_CAND].E, c.cnt_xy[0] + c.cnt_xy[1] + c.cnt_xy[2], c.cnt_z[0] + c.cnt_z[1] + c.cnt_z[2],
           c.fill_cnt);
    return bad;
}

int main() {
    Inst<32, 32> a1(1), a2(1);
    Inst<64, 16> b1(2), b2(2);
    Inst<16, 16> c1(3), c2(3);
    a1.setup(); a2.setup();
    b1.setup(); b2.setup();
    c1.setup(); c2.setup();
    // reference: the one-pass kernels
    a1.attempt();
    b1.attempt();
    c1.attempt();
    // the persistent kernel over a pool of the three others (classes of one instance each)
    std::vector<MegaClass> cls = {{32, 32, 0, 1, 0}, {64, 16, 0, 1, 1}, {16, 16, 0, 1, 2}};
    std::vector<MegaTask> tasks;
    std::vector<unsigned> need;
    mega_plan(cls, tasks, need);
    std::vector<const InstT<T>*> insts = {&a2.h, &b2.h, &c2.h};
    std::vector<unsigned> done(need.size() + 1, 0u);
    unsigned err = 0;
    MegaArgs m = {};
    m.tasks = tasks.data();
    m.insts = insts.data();
    m.need = need.data();
    m.done = done.data();
    m.ticket = done.data() + need.size();
    m.err = &err;
    m.ntasks = (int)tasks.size();
    m.ninst = (int)insts.size();
    // the kernel's dynamic shared memory for these sizes (kernels_mega.cu, mega_smem_bytes)
    auto zb = [](size_t b) { return 2 * mega_align(b); };
    auto xb = [](int n, size_t b) { return (size_t)(kMegaThreads / mega_xy_threads(n)) * mega_align(b); };
    size_t smem = 0;
    smem = std::max(smem, std::max(zb(z_smem_bytes<T, 32, kMegaZTX>()), xb(32, xy_smem_bytes<T, 32>(2))));
    smem = std::max(smem, std::max(zb(z_smem_bytes<T, 16, kMegaZTX>()), xyc_smem_bytes<T, 64>()));
    smem = std::max(smem, std::max(zb(z_smem_bytes<T, 16, kMegaZTX>()), xb(16, xy_smem_bytes<T, 16>(2))));
    smem += kMegaHead;
    emu::launch(dim3(2), kMegaThreads, smem, 2, [&] { mega_kernel(m); });
    int bad = 0;
    bad += compare("n32", a2.h, a1.h);
    bad += compare("n64", b2.h, b1.h);
    bad += compare("n16", c2.h, c1.h);
    unsigned claimed = done[need.size()];
    printf("units %d claimed %u err %u\n", m.ntasks, claimed, err);
    for (size_t i = 0; i < need.size(); ++i)
        if (done[i] != need[i]) {
            printf("phase counter %zu: %u of %u\n", i, done[i], need[i]);
            ++bad;
        }
    if (err) ++bad;
    printf(bad ? "MISMATCH\n" : "SAME\n");
    return bad ? 1 : 0;
}
