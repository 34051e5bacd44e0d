/* Test infrastructure (tests/test_host_emulation.py): a session through the C ABI of
   libcbstep, run on the host against the emulated runtime.  For each form (FP32, FP64;
   FP32 only when the third argument is 1) on an n x n x nz grid: create, set phi (an
   ellipsoid of semi-axes 1.6, 1.6, 1.6 nz / n), run, autotune, run again, read phi and
   the scalars back, destroy.  Prints one line of results per form.
   Usage: sequence n [nz] [fp32_only] */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "cbstep.h"

static int session(int n, int nz, int precision, int method) {
    cb_params p;
    cb_params_default(&p);
    p.nx = p.ny = n;
    p.nz = nz;
    p.method = method;
    p.precision = precision;
    p.M1 = 1e4;
    p.M2 = 1e4;
    p.time_step = 1e-6;
    p.fixed_time_step = 0.0;
    const size_t N = (size_t)n * n * nz;
    double* phi = (double*)malloc(N * sizeof(double));
    const double h = 2 * M_PI / n, hz = 2 * M_PI / nz, cz = (double)n / nz;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < n; ++y)
            for (int x = 0; x < n; ++x) {
                const double X = -M_PI + x * h, Y = -M_PI + y * h, Z = (-M_PI + z * hz) * cz;
                phi[((size_t)z * n + y) * n + x] = tanh((sqrt(X * X + Y * Y + Z * Z) - 1.6) / (1.5 * h));
            }
    cb_handle* hd = NULL;
    int rc = cb_create(&p, &hd);
    cb_run_stats st;
    cb_tune_result tr;
    cb_scalars sc;
    tr.path = -1;
    if (!rc) rc = cb_set_phi(hd, phi, 0);
    if (!rc) rc = cb_run(hd, 3, &st);
    if (!rc) rc = cb_autotune(hd, 1, &tr);
    if (!rc) rc = cb_run(hd, 2, &st);
    if (!rc) rc = cb_get_phi(hd, phi, 0);
    if (!rc) rc = cb_scalars_get(hd, &sc);
    if (rc) {
        printf("form %d rc %d %s\n", precision, rc, cb_last_error());
    } else {
        double mx = 0;
        for (size_t i = 0; i < N; ++i) mx = fmax(mx, fabs(phi[i]));
        printf("form %d rc 0 path %d steps %d E %.17g V %.17g S %.17g maxphi %.17g\n", precision, tr.path,
               sc.steps, sc.E, sc.V, sc.S, mx);
    }
    cb_destroy(hd);
    free(phi);
    return rc;
}

int main(int argc, char** argv) {
    const int n = argc > 1 ? atoi(argv[1]) : 16;
    const int nz = argc > 2 ? atoi(argv[2]) : n;
    const int fp32_only = argc > 3 ? atoi(argv[3]) : 0;
    int rc = session(n, nz, CB_FP32, CB_ETD2);
    if (!rc && !fp32_only) rc = session(n, nz, CB_FP64, CB_ETD2);
    return rc;
}
