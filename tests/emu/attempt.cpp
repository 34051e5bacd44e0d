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
#include "emu_launch.h"
#include "instance.h"
#include "misc_kernels.cuh"
#include "xy_cluster.cuh"
#include "xy_kernel.cuh"
#include "z_kernel.cuh"


using namespace cb;

template <int N, int NZ> int run(int path, int method) {
    using T = float;
    const Params p = params(N, NZ, method);
    const int ntiles = (int)((N * p.nc + 15) / 16);
    InstT<T> h = make_instance<N, NZ>(method);
    Ctrl& c = *h.ctrl;
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
