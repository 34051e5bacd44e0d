// C ABI of include/cbstep.h over the stepper instances of stepper.cuh.
#include "stepper.cuh"

// ====================================================================== C ABI
struct cb_handle {
    std::unique_ptr<cb::Handle> impl;
};

extern "C" {

void cb_params_default(cb_params* p) {
    memset(p, 0, sizeof *p);
    p->nx = p->ny = p->nz = 64;
    p->lenx = 1.0;
    p->epssize = 200;
    p->eta = 1.0;
    p->ga = 1.0;
    p->alpha = -1.0;
    p->beta = -1.0;
    p->M1 = 1.0e4;
    p->M2 = 1.0e4;
    p->time_step = 1e-6;
    p->fixed_time_step = 0.0;
    p->tmax = 100.0;
    p->method = CB_ETD4;
    p->precision = CB_FP64;
    p->accurate_coefficients = -1;
    p->reject_tol = -1.0;
}

int cb_params_from_ini_line(const char* line, cb_params* p) {
    if (!line || !p) return cb::fail(CB_EINVAL, "null argument");
    cb_params_default(p);
    int ifold = 0, nx = 0, ny = 0, nz = 0, b_shape = 0, ninit = 0, nflush = 0, epssize = 2, ncur = 0, oi = 0, einit = 0;
    double xlen = 0, ylen = 0, zlen = 0, ts = 0, fts = 0, fixed = 0, surctrl = 0, angle = 0, re = 0, eta = -1, ga = 0,
           alpha = 0, beta = 0, M1 = 0, M2 = 0, M3 = 0, M4 = 0, tmax = -1, gw = 0, mk = 1, mc = 0, lt = 0, a3 = 0;
    int used = 0;
    // field order and types of fluidbase.cpp:33-35
    const int n = sscanf(line,
                         "%d %d %d %d %lf %lf %lf %d %lf %lf %lf %d %d %lf %d %d %lf %lf %lf %lf %lf %lf %lf %lf "
                         "%lf %lf %lf %d %lf %d %lf %lf %lf %lf%n",
                         &ifold, &nx, &ny, &nz, &xlen, &ylen, &zlen, &b_shape, &ts, &fts, &fixed, &ninit, &nflush,
                         &surctrl, &epssize, &ncur, &angle, &re, &eta, &ga, &alpha, &beta, &M1, &M2, &M3, &M4, &tmax,
                         &oi, &gw, &einit, &mk, &mc, &lt, &a3, &used);
    if (n < 4 || nx <= 0 || ny <= 0 || nz <= 0) return cb::fail(CB_EINVAL, "Illegal ngrid number! (%d fields read)", n);
    p->nx = nx;
    p->ny = nx;
    p->nz = nz;
    p->lenx = xlen > 0 ? xlen : 1.0;
    p->epssize = epssize;
    p->time_step = ts > 0 ? ts : 1e-6;
    p->fixed_time_step = fixed;
    p->eta = eta < 0 ? 10.0 : eta;
    p->ga = ga <= 0 ? 1.0 : ga;
    if (beta < 0) alpha = beta = 0;  // fluidbase.cpp:143
    p->alpha = alpha;
    p->beta = beta;
    p->M1 = M1;
    p->M2 = M2;
    p->tmax = tmax < 0 ? 4.0 : tmax;
    if (n == 34 && used > 0) {
        int method = -1, prec = -1;
        const int m = sscanf(line + used, "%d %d", &method, &prec);
        if (m >= 1) {
            if (method < CB_EULER || method > CB_ETD4) return cb::fail(CB_EINVAL, "bad method field %d", method);
            p->method = method;
        }
        if (m >= 2) {
            if (prec != CB_FP64 && prec != CB_FP32) return cb::fail(CB_EINVAL, "bad precision field %d", prec);
            p->precision = prec;
        }
    }
    return CB_OK;
}

double cb_params_eps(const cb_params* p) {
    cb::Eff e;
    if (!p || cb::make_params(*p, e)) return -1.0;
    return e.p.eps;
}

long long cb_instance_bytes(const cb_params* p) {
    cb::Eff e;
    if (!p || cb::make_params(*p, e)) return -1;
    return p->precision == CB_FP32 ? (long long)cb::instance_arena_bytes<float>(e.p)
                                   : (long long)cb::instance_arena_bytes<double>(e.p);
}

int cb_supported(const cb_params* p) {
    cb::Eff e;
    if (!p || cb::make_params(*p, e)) return 0;
    if (p->precision == CB_FP32)
        return cb::Launch<float>::xy_supported(p->nx) && cb::Launch<float>::z_supported(p->nz);
    return cb::Launch<double>::xy_supported(p->nx) && cb::Launch<double>::z_supported(p->nz);
}

int cb_create(const cb_params* p, cb_handle** out) {
    if (!p || !out) return cb::fail(CB_EINVAL, "null argument");
    *out = nullptr;
    std::unique_ptr<cb_handle> h(new cb_handle);
    if (p->precision == CB_FP32) h->impl.reset(new cb::Stepper<float>());
    else h->impl.reset(new cb::Stepper<double>());
    int rc = h->impl->init(*p);
    if (rc) return rc;
    *out = h.release();
    return CB_OK;
}

int cb_destroy(cb_handle* h) {
    delete h;
    return CB_OK;
}

#define CB_H(h) \
    if (!(h) || !(h)->impl) return cb::fail(CB_EINVAL, "null handle")

int cb_set_phi(cb_handle* h, const double* phi, int on_device) {
    CB_H(h);
    if (!phi) return cb::fail(CB_EINVAL, "null phi");
    return h->impl->set_phi(phi, on_device != 0);
}
int cb_get_phi(cb_handle* h, double* phi, int on_device) {
    CB_H(h);
    if (!phi) return cb::fail(CB_EINVAL, "null phi");
    return h->impl->get_phi(phi, on_device != 0);
}
int cb_scalars_get(cb_handle* h, cb_scalars* s) {
    CB_H(h);
    if (!s) return cb::fail(CB_EINVAL, "null scalars");
    return h->impl->scalars(s);
}
double cb_getstaticenergy(cb_handle* h) {
    cb_scalars s;
    if (!h || !h->impl || h->impl->scalars(&s)) return NAN;
    return s.E;
}
int cb_ETD2RK(cb_handle* h) { CB_H(h); return h->impl->raw_step(CB_ETD2); }
int cb_ETD4RK(cb_handle* h) { CB_H(h); return h->impl->raw_step(CB_ETD4); }
int cb_euler_step(cb_handle* h) { CB_H(h); return h->impl->raw_step(CB_EULER); }
int cb_run(cb_handle* h, int nsteps, cb_run_stats* st) { CB_H(h); return h->impl->run(nsteps, st); }
int cb_field(cb_handle* h, int which, double* out, int on_device) {
    CB_H(h);
    if (!out) return cb::fail(CB_EINVAL, "null output");
    return h->impl->field(which, out, on_device != 0);
}
int cb_set_dt(cb_handle* h, double dt) { CB_H(h); return h->impl->set_dt(dt); }
int cb_set_loop_state(cb_handle* h, double t, double dt, double alpha, double beta) {
    CB_H(h);
    return h->impl->set_loop_state(t, dt, alpha, beta);
}
int cb_autotune(cb_handle* h, int attempts, cb_tune_result* out) {
    CB_H(h);
    return h->impl->autotune(attempts, out);
}
int cb_shape_adjust(cb_handle* h, int max_steps, cb_adjust_stats* st) {
    CB_H(h);
    return h->impl->shape_adjust(max_steps, st);
}
int cb_synchronize(cb_handle* h) { CB_H(h); return h->impl->sync(); }
int cb_set_launch_limit(cb_handle* h, long long max_graph_launches) {
    CB_H(h);
    if (max_graph_launches < 0) return cb::fail(CB_EINVAL, "launch limit < 0");
    h->impl->set_launch_limit(max_graph_launches);
    return CB_OK;
}
int cb_run_timed(cb_handle* h, int nsteps, long long flush_bytes, double* device_ms, int* attempts) {
    CB_H(h);
    return h->impl->run_timed(nsteps, flush_bytes, device_ms, attempts);
}
int cb_profile_kernels(cb_handle* h, int nattempts, long long flush_bytes, double* ms, int* counts) {
    CB_H(h);
    if (!ms || !counts || nattempts < 0) return cb::fail(CB_EINVAL, "bad profile arguments");
    return h->impl->profile(nattempts, flush_bytes, ms, counts);
}
long long cb_handle_bytes(cb_handle* h) {
    if (!h || !h->impl) return -1;
    return h->impl->bytes();
}
const char* cb_last_error(void) { return cb::g_err.c_str(); }
const char* cb_version(void) { return "cudabubble-gb300 0.1 (sm_103a)"; }

}  // extern "C"
