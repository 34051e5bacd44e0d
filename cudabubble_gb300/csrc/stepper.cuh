// Host side of the GB300 stepper: one instance (vesicle) per handle, the
// per-attempt kernel sequence captured once into a CUDA graph, and the
// reference time loops driven from device-side accept/reject state.  The C
// ABI of include/cbstep.h is in stepper.cu; batched and served pools of
// instances are in pool.cu.
//
// Attempt sequences (every kernel reads its instance's Ctrl block, so the
// graph is replayed unchanged while dt, the state index and the accept flag
// live on the device):
//   ETD-RK2 (belastic.cpp:491-517)
//     xy NONLIN(state) -> z ETD2_S1 -> xy REDUCE_S(work) -> xy NONLIN(work)
//     -> z ETD2_S2 -> xy REDUCE_FULL(cand) -> decide -> coef
//   ETD-RK4 (belastic.cpp:519-552): four stages of the same shape
//   Euler   (belastic.cpp:52-64, 382): xy NONLIN(state) -> z EULER
//     -> xy REDUCE_FULL(cand) -> decide
// The stage-1 nonlinear spectrum does not depend on dt, so a rejected attempt
// reuses it (the xy NONLIN on the state is skipped while ctrl->fresh == 0).
//
// The FP32 form runs one xy pass per stage (XY_FUSED: the stage state's sums
// and its lambda-free nonlinear partials together); the penalty terms enter
// in the following z pass, which reads lambda from those sums:
//   ETD-RK2  z ETD2_S1 -> xy FUSED(work) -> z ETD2_S2 -> xy FUSED(cand) -> decide
// and the candidate's partials become the next state's (G slot swap on accept).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "cb_inst.h"
#include "cb_kargs.h"
#include "cbstep.h"
#include "launch.h"

namespace cb {

inline thread_local std::string g_err;

inline int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CB_CK(x)                                                                                    \
    do {                                                                                            \
        cudaError_t e_ = (x);                                                                       \
        if (e_ != cudaSuccess)                                                                      \
            return fail(CB_ECUDA, "%s failed: %s (%s:%d)", #x, cudaGetErrorString(e_), __FILE__, __LINE__); \
    } while (0)

inline constexpr double kTwoPi = 6.283185307179586476925286766559;

// ------------------------------------------------------------ twiddles
// W_n^m = exp(-2 pi i m / n), evaluated in long double and rounded once.
inline std::mutex g_tw_mu;
inline std::map<std::tuple<int, int, int, int>, void*> g_tw;

template <class T> inline void* twiddle_table(int n, int xkind, cudaError_t* err) {
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto key = std::make_tuple(dev, (int)sizeof(T), n, xkind);
    auto it = g_tw.find(key);
    if (it != g_tw.end()) return it->second;
    std::vector<T> v;
    std::vector<long double> ex;  // the exact values, for the FP32 lo parts
    auto push = [&](int len) {
        for (int m = 0; m < len; ++m) {
            const long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)m / (long double)len;
            ex.push_back(cosl(a));
            ex.push_back(-sinl(a));
        }
    };
    if (xkind) push(n / 2);  // half-length transform table, then the full one
    push(n);
    for (long double x : ex) v.push_back((T)x);
    if (sizeof(T) == 4)  // FP32: lo = fl(exact - hi), in the same order after the hi parts
        for (size_t i = 0; i < ex.size(); ++i) v.push_back((T)(ex[i] - (long double)v[i]));
    void* d = nullptr;
    *err = cudaMalloc(&d, v.size() * sizeof(T));
    if (*err != cudaSuccess) return nullptr;
    *err = cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    if (*err != cudaSuccess) return nullptr;
    g_tw[key] = d;
    return d;
}

// ------------------------------------------------------------ parameters
inline double eps_rule(int epssize, double xlen, int nx) {  // fluidbase.cpp:68-108
    const double h2 = 2 * xlen / 2.0 / nx;
    switch (epssize) {
        case 1: return 2.5 * (std::sqrt(2.) * xlen / 2.0 / nx);
        case 2: return 2.5 * h2;
        case 3: return 1.5 * h2;
        case 4: return 1.25 * h2;
        case 5: return 1.0 * h2;
        case 6: return 0.7 * h2;
        case 7: return 4.0 * h2;
        case 8: return 2.5 * (std::sqrt(2.) * xlen / 2.0 / nx) * 1.22;
        default: return epssize > 10 ? epssize / 100.0 * h2 : 2.0 * h2;
    }
}

struct Eff {
    Params p;
    double dt0;
    int accurate;
    int precision;
};

inline int make_params(const cb_params& u, Eff& e) {
    Params& p = e.p;
    memset(&p, 0, sizeof p);
    if (u.nx <= 0 || u.nz <= 0 || (u.nx & 1))
        return fail(CB_EINVAL, "grid %dx%dx%d: nx must be even and positive (Calc.cu:52-55)", u.nx, u.nx, u.nz);
    if (u.method < CB_EULER || u.method > CB_ETD4) return fail(CB_EINVAL, "unknown method %d", u.method);
    if (u.precision != CB_FP64 && u.precision != CB_FP32) return fail(CB_EINVAL, "unknown precision %d", u.precision);
    if (!std::isfinite(u.spont_c)) return fail(CB_EINVAL, "spontaneous curvature must be finite");
    p.nx = u.nx;
    p.ny = u.nx;  // Calc.cu:45-46
    p.nz = u.nz;
    p.nc = u.nx / 2 + 1;
    p.N = (long long)p.nx * p.ny * p.nz;
    p.invN = 1.0 / (double)p.N;
    const double xlen = (u.lenx > 0 ? u.lenx : 1.0) * kTwoPi;
    p.cx = (kTwoPi / xlen) * (kTwoPi / xlen);
    p.L3 = xlen * xlen * xlen;
    p.eps = u.eps > 0 ? u.eps : eps_rule(u.epssize, xlen, u.nx);
    p.eta = u.eta;
    p.ga = u.ga;
    p.M1 = u.M1;
    p.M2 = u.M2;
    p.method = u.method;
    p.adaptive = u.fixed_time_step <= 0;
    p.corr = (!p.adaptive && u.method != CB_EULER && (u.M1 != 0 || u.M2 != 0)) ? 1 : 0;
    p.etd4_ref = u.etd4_textbook ? 0 : 1;
    p.kmax = (p.nx / 2) * (p.nx / 2) + (p.ny / 2) * (p.ny / 2) + (p.nz / 2) * (p.nz / 2);
    const bool euler = u.method == CB_EULER;
    p.grow_every = u.grow_every > 0 ? u.grow_every : 4;
    if (u.xy_split < XYP_AUTO || u.xy_split > XYP_CLUSTER) return fail(CB_EINVAL, "xy_split %d: 0..3", u.xy_split);
    p.split = u.xy_split;
    p.grow_factor = u.grow_factor > 0 ? u.grow_factor : (euler ? 1.4 : 2.0);
    p.dt_cap = u.dt_cap > 0 ? u.dt_cap : (euler ? 1e300 : 1e-3);
    p.cap_probe = u.cap_probe > 0 ? u.cap_probe : (euler ? 0.0 : 1.4);
    p.dt_min = 1e-23;
    p.tmax = u.tmax >= 0 ? u.tmax : 4.0;
    p.rel_tol = u.rel_tol > 0 ? u.rel_tol : 0.0;
    // both forms default to the reference's strict E_new > E_old rejection
    // (belastic.cpp:653-668); a positive reject_tol tolerates rises below reject_tol |E|
    p.reject_tol = u.reject_tol >= 0 ? u.reject_tol : 0.0;
    p.C = u.spont_c;
    // FP32 form with curvature: the fused passes carry the third field q = (eps) C (u^2 - 1)
    p.curv = (u.precision == CB_FP32 && u.spont_c != 0.0) ? 1 : 0;
    p.f_C = (float)p.C;
    p.f_qC = (float)((euler ? 1.0 : p.eps) * p.C);
    p.f_2eC = (float)(2.0 * p.eps * p.C);
    // nonlinear term N-hat = A-hat + beta cx |k|^2 B-hat: beta = eta (Euler, -lap f in g0)
    // or -eta/eps (ETD, +lap t / eps in -eta NL)
    const double beta = euler ? p.eta : -p.eta / p.eps;
    p.d_ieps = 1.0 / p.eps;
    p.d_ieps2 = 1.0 / (p.eps * p.eps);
    p.d_ieps3 = 1.0 / (p.eps * p.eps * p.eps);
    p.d_bnl = beta * p.cx;
    p.f_eps = (float)p.eps;
    p.f_ieps = (float)p.d_ieps;
    p.f_ieps2 = (float)p.d_ieps2;
    p.f_ieps3 = (float)p.d_ieps3;
    p.f_bnl = (float)p.d_bnl;
    p.f_cx = (float)p.cx;
    p.f_invN = (float)p.invN;
    p.f_eta = (float)p.eta;
    {
        const double k[7] = {p.eps, p.d_ieps, p.eta * p.d_ieps2, p.eta * 1.5 * p.d_ieps3, p.d_bnl, p.invN, p.cx};
        for (int i = 0; i < 7; ++i) {
            const float hi = (float)k[i];
            p.fk[i][0] = hi;
            p.fk[i][1] = (float)(k[i] - (double)hi);
        }
    }
    const double ts = u.time_step > 0 ? u.time_step : 1e-6;  // fluidbase.cpp:112
    e.dt0 = p.adaptive ? ts : std::min(u.fixed_time_step, ts);  // belastic.cpp:599-602
    e.precision = u.precision;
    e.accurate = u.accurate_coefficients >= 0 ? u.accurate_coefficients : (u.precision == CB_FP32 ? 1 : 0);
    return CB_OK;
}

// ------------------------------------------------------------ instance
struct Handle {
    virtual ~Handle() {}
    virtual int init(const cb_params& u) = 0;
    virtual int set_phi(const double* phi, bool dev) = 0;
    virtual int get_phi(double* phi, bool dev) = 0;
    virtual int scalars(cb_scalars* s) = 0;
    virtual int raw_step(int method) = 0;
    virtual int run(int nsteps, cb_run_stats* st) = 0;
    virtual int field(int which, double* out, bool dev) = 0;
    virtual int set_dt(double dt) = 0;
    virtual int set_loop_state(double t, double dt, double alpha, double beta) = 0;
    virtual int shape_adjust(int max_steps, cb_adjust_stats* st) = 0;
    virtual int autotune(int attempts, cb_tune_result* out) = 0;
    virtual int sync() = 0;
    virtual long long bytes() const = 0;
    virtual int run_timed(int nsteps, long long flush_bytes, double* ms, int* attempts) = 0;
    virtual int profile(int nattempts, long long flush_bytes, double* ms, int* cnt) = 0;
    // bound on the attempt-graph launches of one run / run_timed / shape_adjust call
    // (0: the built-in no-progress bound, which returns CB_ENOTCONVERGED)
    void set_launch_limit(long long n) { launch_limit = n > 0 ? n : 0; }

   protected:
    long long launch_limit = 0;
};

// kernel kinds reported by cb_profile_kernels
enum { K_XY_NONLIN = 0, K_XY_REDUCE_S = 1, K_XY_REDUCE_FULL = 2, K_Z_STAGE = 3, K_DECIDE = 4, K_XY_FUSED = 5,
       K_NKIND = 6 };

// One attempt of the method's loop for `ninst` instances that share grid and
// method (an instance table on the device), on stream s.  With prof set, an
// event pair brackets every launch and is appended as (kind, start, end).
template <class T>
inline cudaError_t enqueue_group(int method, int nx, int nz, const InstT<T>* d, int ninst, int ntiles, int accurate,
                                 int raw, int split, int curv, cudaStream_t s,
                                 std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>>* prof = nullptr) {
    cudaError_t r = cudaSuccess;
    auto timed = [&](int kind, auto&& fn) {
        if (r != cudaSuccess) return;
        if (!prof) { r = fn(); return; }
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, s);
        r = fn();
        cudaEventRecord(b, s);
        prof->emplace_back(kind, a, b);
    };
    auto X = [&](int m, int role, int skip = 0) {
        const int kind = m == XY_NONLIN ? K_XY_NONLIN
                         : m == XY_FUSED ? K_XY_FUSED
                         : (m == XY_REDUCE_S ? K_XY_REDUCE_S : K_XY_REDUCE_FULL);
        timed(kind, [&]() {
            XYArgs a;
            memset(&a, 0, sizeof a);
            a.mode = m;
            a.role = role;
            a.skip_if_stale = skip;
            a.curv = curv;
            return Launch<T>::xy(nx, d, ninst, nz, a, s, split);
        });
    };
    auto Z = [&](int m, int role) {
        timed(K_Z_STAGE, [&]() {
            ZArgs a;
            memset(&a, 0, sizeof a);
            a.mode = m;
            a.role = role;
            a.curv = curv;
            return Launch<T>::z(nz, d, ninst, ntiles, a, s);
        });
    };
    // prologue: pending dt growth, coefficient table for the attempt's dt
    timed(K_DECIDE, [&]() { return Launch<T>::coef(d, ninst, accurate, s, raw ? 1 : 0); });
    if (sizeof(T) == 4) {
        // FP32 form: every xy pass is XY_FUSED (sums + lambda-free partials of the
        // same state); stage 1 reads the state's outputs from its G slot, left by the
        // candidate pass of the attempt that accepted it (or by cb_set_phi)
        switch (method) {
            case M_ETD2:
                Z(Z_ETD2_S1, R_WORK);
                X(XY_FUSED, R_WORK);
                Z(Z_ETD2_S2, R_CAND);
                X(XY_FUSED, R_CAND);
                break;
            case M_ETD4:
                Z(Z_ETD4_S1, R_WORK);
                X(XY_FUSED, R_WORK);
                Z(Z_ETD4_S2, R_WORK);
                X(XY_FUSED, R_WORK);
                Z(Z_ETD4_S3, R_WORK);
                X(XY_FUSED, R_WORK);
                Z(Z_ETD4_S4, R_CAND);
                X(XY_FUSED, R_CAND);
                break;
            default:
                Z(Z_EULER, R_CAND);
                X(XY_FUSED, R_CAND);
                break;
        }
    } else {
    switch (method) {
        case M_ETD2:
            X(XY_NONLIN, R_STATE, 1);
            Z(Z_ETD2_S1, R_WORK);
            X(XY_REDUCE_S, R_WORK);
            X(XY_NONLIN, R_WORK);
            Z(Z_ETD2_S2, R_CAND);
            X(XY_REDUCE_FULL, R_CAND);
            break;
        case M_ETD4:
            X(XY_NONLIN, R_STATE, 1);
            Z(Z_ETD4_S1, R_WORK);
            X(XY_REDUCE_S, R_WORK);
            X(XY_NONLIN, R_WORK);
            Z(Z_ETD4_S2, R_WORK);
            X(XY_REDUCE_S, R_WORK);
            X(XY_NONLIN, R_WORK);
            Z(Z_ETD4_S3, R_WORK);
            X(XY_REDUCE_S, R_WORK);
            X(XY_NONLIN, R_WORK);
            Z(Z_ETD4_S4, R_CAND);
            X(XY_REDUCE_FULL, R_CAND);
            break;
        default:
            X(XY_NONLIN, R_STATE, 1);
            Z(Z_EULER, R_CAND);
            X(XY_REDUCE_FULL, R_CAND);
            break;
    }
    }
    timed(K_DECIDE, [&]() { return Launch<T>::decide(d, ninst, raw, s); });
    return r;
}

// Arena of one instance.  Stepped-state spectra (phi-hat x2, a-hat) hold 16
// bytes per mode in both forms (FP64 complex, or FP32 double-float pairs);
// every other field is one complex T per mode.
// the split plane path is used for some xy mode of this precision and grid
template <class T> inline bool uses_split(const Params& p) {
    return p.split == XYP_SPLIT || !Launch<T>::xy_single(p.nx, 2) || !Launch<T>::xy_single(p.nx, 1);
}
// per-plane or per-row-block partial sums of the xy reductions
template <class T> inline size_t xy_part_slots(const Params& p) {
    size_t n = 2 * (size_t)p.nz;  // two per plane for the two-CTA fused pass
    if (uses_split<T>(p)) n = std::max(n, (size_t)p.nz * p.ny / Launch<T>::xy_rows_per_cta(p.nx));
    return n;
}

template <class T> inline size_t instance_arena_bytes(const Params& p, size_t* layout = nullptr) {
    const size_t ns = (size_t)p.nz * p.ny * p.nc;
    const int ntiles = (p.ny * p.nc + Launch<T>::z_tile() - 1) / Launch<T>::z_tile();
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t fs = al(ns * 16), fp = al(ns * sizeof(T) * 2);
    // Nu, P x6, A, B (+ Na, Nb), then the split path's Y0, Y1, then the FP32 form's G slots
    const int nplain = 9 + (p.method == M_ETD4 ? 2 : 0) + (uses_split<T>(p) ? 2 : 0) + (sizeof(T) == 4 ? 4 : 0) +
                       (p.curv ? 3 : 0);  // curvature: q of the work stage and of both G slots
    // FP32 form: the state's and the candidate's real-space u, double-float
    const size_t fu = sizeof(T) == 4 ? al((size_t)p.N * 8) : 0;
    // FP32 form: the FP64 plain transforms of set/get phi need their own Y0, Y1
    const int naux = (sizeof(T) == 4 && uses_split<double>(p)) ? 2 : 0;
    size_t off = 0;
    if (layout) layout[0] = off;
    off += (3 + naux) * fs;
    if (layout) layout[6] = off;
    off += nplain * fp;
    if (layout) layout[8] = off;
    off += 2 * fu;
    if (layout) layout[1] = off;
    off += al((size_t)kNTab * (p.kmax + 1) * 8 * sizeof(T));
    if (layout) layout[2] = off;
    off += al(xy_part_slots<T>(p) * 4 * sizeof(double));
    if (layout) layout[3] = off;
    off += al((size_t)ntiles * 2 * sizeof(double));
    if (layout) layout[4] = off;
    off += al(sizeof(Ctrl));
    if (layout) layout[5] = off;
    off += al(sizeof(InstT<T>));
    if (layout) layout[7] = off;
    off += al(sizeof(InstT<double>));  // FP64 descriptor for exact set/get of phi (FP32 form)
    return off;
}

template <class T> class Stepper final : public Handle {
   public:
    ~Stepper() override {
        if (st) cudaStreamSynchronize(st);
        if (g_loop) cudaGraphExecDestroy(g_loop);
        if (g_raw) cudaGraphExecDestroy(g_raw);
        if (g_shape) cudaGraphExecDestroy(g_shape);
        if (!ext_arena) cudaFree(arena);
        cudaFree(scratch);
        cudaFree(cbuf);
        cudaFree(flush_buf);
        if (st && !ext_stream) cudaStreamDestroy(st);
    }

    int init(const cb_params& u) override { return init_in(u, nullptr, nullptr); }

    // init on caller-owned memory: `mem` (instance_arena_bytes, 256-byte aligned) and
    // stream `s` are used instead of a cudaMalloc and a new stream, and stay the
    // caller's (the served pool admits requests into arenas it carved up front)
    int init_in(const cb_params& u, void* mem, cudaStream_t s) {
        up = u;
        int rc = make_params(u, e);
        if (rc) return rc;
        p = e.p;
        if (!Launch<T>::xy_supported(p.nx) || !Launch<T>::z_supported(p.nz))
            return fail(CB_EUNSUPPORTED, "grid %dx%dx%d not built for %s", p.nx, p.ny, p.nz,
                        sizeof(T) == 4 ? "FP32" : "FP64");
        if (p.curv && !Launch<T>::fused_curv_ok(p.nx, p.split))
            return fail(CB_EUNSUPPORTED,
                        "spontaneous curvature in the FP32 form runs on the cluster and one-CTA plane passes "
                        "(planes up to 128^2, not the split passes); use CB_FP64 for %dx%d planes", p.nx, p.ny);
        ns = (size_t)p.nz * p.ny * p.nc;
        ntiles = (p.ny * p.nc + Launch<T>::z_tile() - 1) / Launch<T>::z_tile();
        size_t lay[9];
        arena_bytes = instance_arena_bytes<T>(p, lay);
        if (s) {
            st = s;
            ext_stream = true;
        } else {
            CB_CK(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
        }
        if (mem) {
            if (reinterpret_cast<uintptr_t>(mem) % 256) return fail(CB_EINVAL, "arena not 256-byte aligned");
            arena = mem;
            ext_arena = true;
        } else if (cudaMalloc(&arena, arena_bytes) != cudaSuccess) {
            cudaGetLastError();
            return fail(CB_ENOMEM, "cudaMalloc of %zu bytes failed", arena_bytes);
        }
        CB_CK(cudaMemsetAsync(arena, 0, arena_bytes, st));
        char* base = (char*)arena;
        const size_t fs = ((ns * 16) + 255) & ~(size_t)255;
        const size_t fp = ((ns * sizeof(T) * 2) + 255) & ~(size_t)255;
        void** fst[3] = {&h.spec[0], &h.spec[1], &h.ahat};
        for (int i = 0; i < 3; ++i) *fst[i] = base + lay[0] + i * fs;
        void** f[11] = {&h.Nu, &h.P[0][0], &h.P[0][1], &h.P[1][0], &h.P[1][1], &h.P[2][0], &h.P[2][1],
                        &h.A, &h.B, &h.Na, &h.Nb};
        const int nplain = 9 + (p.method == M_ETD4 ? 2 : 0);
        for (int i = 0; i < nplain; ++i) *f[i] = base + lay[6] + i * fp;
        int nextf = nplain;
        if (uses_split<T>(p))
            for (int i = 0; i < 2; ++i) h.Y[i] = base + lay[6] + (nextf++) * fp;
        if (sizeof(T) == 4) {
            for (int i = 0; i < 4; ++i) h.G[i / 2][i % 2] = base + lay[6] + (nextf++) * fp;
            if (p.curv) {
                h.G[0][2] = base + lay[6] + (nextf++) * fp;
                h.G[1][2] = base + lay[6] + (nextf++) * fp;
                h.Q = base + lay[6] + (nextf++) * fp;
            }
            const size_t fu = ((size_t)p.N * 8 + 255) & ~(size_t)255;
            for (int i = 0; i < 2; ++i) h.U[i] = base + lay[8] + i * fu;
        }
        h.coef = reinterpret_cast<T*>(base + lay[1]);
        h.part_xy = reinterpret_cast<double*>(base + lay[2]);
        h.part_z = reinterpret_cast<double*>(base + lay[3]);
        h.ctrl = reinterpret_cast<Ctrl*>(base + lay[4]);
        d = reinterpret_cast<InstT<T>*>(base + lay[5]);
        cudaError_t err = cudaSuccess;
        h.twx = twiddle_table<T>(p.nx, 1, &err);
        if (!h.twx) return fail(CB_ECUDA, "twiddles: %s", cudaGetErrorString(err));
        h.twy = twiddle_table<T>(p.ny, 0, &err);
        if (!h.twy) return fail(CB_ECUDA, "twiddles: %s", cudaGetErrorString(err));
        h.twz = twiddle_table<T>(p.nz, 0, &err);
        if (!h.twz) return fail(CB_ECUDA, "twiddles: %s", cudaGetErrorString(err));
        h.p = p;
        CB_CK(cudaMemcpyAsync(d, &h, sizeof h, cudaMemcpyHostToDevice, st));
        if (sizeof(T) == 4 && Launch<double>::xy_plain_supported(p.nx)) {
            // the FP32 form reads and writes phi through FP64 plain transforms, so
            // its double-float state starts exact (an FP32 forward FFT of phi0
            // alone costs ~6e-7 of the energy at 128^3)
            InstT<double> x;
            memset(&x, 0, sizeof x);
            x.ctrl = h.ctrl;
            x.coef = nullptr;
            x.p = p;
            x.part_xy = h.part_xy;  // plain modes write no sums; kept valid all the same
            if (uses_split<double>(p))
                for (int i = 0; i < 2; ++i) x.Y[i] = base + lay[0] + (3 + i) * fs;
            x.twx = twiddle_table<double>(p.nx, 1, &err);
            x.twy = twiddle_table<double>(p.ny, 0, &err);
            x.twz = twiddle_table<double>(p.nz, 0, &err);
            if (!x.twx || !x.twy || !x.twz) return fail(CB_ECUDA, "twiddles: %s", cudaGetErrorString(err));
            aux = reinterpret_cast<InstT<double>*>(base + lay[7]);
            aux_h = x;
            CB_CK(cudaMemcpyAsync(aux, &aux_h, sizeof aux_h, cudaMemcpyHostToDevice, st));
        }
        memset(&hc, 0, sizeof hc);
        reset_ctrl();
        CB_CK(push());
        return CB_OK;
    }

    long long bytes() const override { return (long long)arena_bytes; }

    // ---- used by the batched / served pools (pool.cu)
    const InstT<T>& inst() const { return h; }
    const Params& params() const { return p; }
    int accurate() const { return e.accurate; }
    int tiles() const { return ntiles; }
    // arm the device loop state for `nsteps` more accepted steps (as run() does)
    int prepare_run(int nsteps) {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        CB_CK(pull());
        hc.target = hc.steps + nsteps;
        hc.done = nsteps == 0 ? 1 : 0;
        hc.status = nsteps == 0 ? ST_TARGET : ST_RUNNING;
        CB_CK(push());
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }
    // after a pooled run: record the exit reason and leave the instance live
    int finish_run(int* status) {
        CB_CK(pull());
        last_status = hc.status;
        if (status) *status = hc.status;
        hc.done = 0;
        CB_CK(push());
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    // phi staging buffer: the two work partials are contiguous in the arena and
    // hold at least N doubles; A is the transform intermediate.  Both are
    // free between attempts, so set/get_phi allocate nothing.
    double* stage() const { return reinterpret_cast<double*>(h.P[2][0]); }

    int set_phi(const double* phi, bool dev) override {
        const double* src = phi;
        if (!dev) {
            CB_CK(cudaMemcpyAsync(stage(), phi, (size_t)p.N * sizeof(double), cudaMemcpyHostToDevice, st));
            src = stage();
        }
        reset_ctrl();
        CB_CK(push());
        // FP32 form: the state's real-space field, exact as a double-float pair
        if (sizeof(T) == 4) CB_CK(launch_real_to_ff(src, h.U[0], (size_t)p.nz * p.ny, p.nx, st));
        if (aux) {  // exact spectrum: FP64 transform, split hi/lo into the state by its z pass
            CB_CK(fwd3d_f64(src, h.spec[0], h.ahat));
        } else {
            CB_CK(fwd3d(src, h.spec[0], h.A, true));
        }
        CB_CK(zpass(Z_INV_STATE, R_STATE));
        // FP32 form: the fused pass also leaves the state's nonlinear partials in its G slot
        CB_CK(xypass(sizeof(T) == 4 ? XY_FUSED : XY_REDUCE_FULL, R_STATE));
        CB_CK(pull());
        // alpha/beta from t = 0 when beta <= 0 (fluidbase.cpp:143, belastic.cpp:588-591)
        if (!(up.beta > 0.0)) {
            hc.alpha = hc.sc[R_STATE].V;
            hc.beta = hc.sc[R_STATE].S;
        } else {
            hc.alpha = up.alpha;
            hc.beta = up.beta;
        }
        hc.alpha0 = hc.alpha;
        hc.beta0 = hc.beta;
        Scal& s = hc.sc[R_STATE];
        const double ve = s.V - hc.alpha, se = s.S - hc.beta;
        s.E = p.eta * s.E_el + 0.5 * p.M1 * ve * ve + 0.5 * p.M2 * se * se;
        hc.E_state = hc.E_init = s.E;
        hc.grow_pending = p.adaptive ? 1 : 0;  // the loop grows dt before its first step
        CB_CK(push());
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        have_state = true;
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    int get_phi(double* out, bool dev) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        CB_CK(pull());
        double* dst = dev ? out : stage();
        if (aux) {  // FP64 transform of the state, joined from its hi/lo pairs by its z pass
            CB_CK(inv3d_f64(h.spec[hc.spec_state], dst, h.ahat));
        } else {
            CB_CK(inv3d(h.spec[hc.spec_state], SM_NONE, dst, h.A, true));
        }
        if (!dev) CB_CK(cudaMemcpyAsync(out, stage(), (size_t)p.N * sizeof(double), cudaMemcpyDeviceToHost, st));
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    int scalars(cb_scalars* s) override {
        CB_CK(pull());
        const Scal& sc = hc.sc[R_STATE];
        s->V = sc.V;
        s->S = sc.S;
        s->E_el = sc.E_el;
        s->E = hc.E_state;
        s->alpha = hc.alpha;
        s->beta = hc.beta;
        s->lamb1 = p.M1 * (sc.V - hc.alpha);
        s->lamb2 = p.M2 * (sc.S - hc.beta);
        s->dt = hc.dt;
        s->t = hc.t;
        s->lserror = sc.lsq * p.L3;
        s->steps = hc.steps;
        s->attempts = hc.attempts;
        s->rejects = hc.rejects;
        s->status = last_status;
        s->E_attempt = hc.E_last_attempt;
        return CB_OK;
    }

    int set_dt(double dt) override {
        if (!(dt > 0)) return fail(CB_EINVAL, "dt must be positive");
        CB_CK(pull());
        hc.dt = dt;
        CB_CK(push());
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    // resume a run: accepted time, dt and the volume / area targets of the
    // reference's .info file (fluidbase.cpp:2797-2826), the state set before
    int set_loop_state(double t, double dt, double alpha, double beta) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        if (!(dt > 0)) return fail(CB_EINVAL, "dt must be positive");
        CB_CK(pull());
        hc.t = t;
        hc.dt = dt;
        hc.alpha = hc.alpha0 = alpha;
        hc.beta = hc.beta0 = beta;
        Scal& s = hc.sc[R_STATE];
        const double ve = s.V - alpha, se = s.S - beta;
        s.E = p.eta * s.E_el + 0.5 * p.M1 * ve * ve + 0.5 * p.M2 * se * se;
        hc.E_state = hc.E_init = s.E;
        hc.fresh = 1;
        CB_CK(push());
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    int sync() override {
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    // the xy paths this handle can run: the split passes need the y buffers the arena
    // holds only where the handle was created for them
    bool path_ok(int path) const {
        switch (path) {
            case XYP_SPLIT: return !p.curv && h.Y[0] != nullptr && Launch<T>::xy_split_supported(p.nx);
            case XYP_SINGLE: return Launch<T>::xy_single(p.nx, 2, p.curv);
            case XYP_CLUSTER: return sizeof(T) == 4 && Launch<T>::xy_cluster_ok(p.nx, p.curv);
            default: return false;
        }
    }

    // Times one attempt of the handle's method on every xy path it can run and keeps
    // the fastest.  The timed attempts start from the current state and accept nothing
    // (decide's timing mode), so state, dt, counters and coefficient tables are as
    // before; the loop graphs are re-captured for the chosen path.
    int autotune(int attempts, cb_tune_result* out) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        if (attempts < 1) return fail(CB_EINVAL, "attempts must be positive");
        CB_CK(pull());
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
            if (e0) cudaEventDestroy(e0);
            return fail(CB_ECUDA, "autotune: event creation failed");
        }
        const Ctrl saved = hc;
        hc.target = INT_MAX;
        hc.done = 0;
        hc.fresh = 1;
        const int keep = p.split;
        const int cands[3] = {XYP_CLUSTER, XYP_SINGLE, XYP_SPLIT};
        cb_tune_result r{};
        r.path = -1;
        double best = 1e300;
        int rc = CB_OK;
        {
            const cudaError_t e = push();
            if (e != cudaSuccess) rc = fail(CB_ECUDA, "autotune: push failed: %s", cudaGetErrorString(e));
        }
        // every error in the loop ends it through the restore below (path, control state,
        // events, cached graphs), not by an early return
        auto ck = [&](cudaError_t e, const char* what) {
            if (e != cudaSuccess && rc == CB_OK) rc = fail(CB_ECUDA, "autotune: %s failed: %s", what, cudaGetErrorString(e));
            return rc == CB_OK;
        };
        for (int path : cands) {
            if (rc) break;
            if (!path_ok(path)) continue;
            p.split = path;
            cudaGraphExec_t g = nullptr;
            rc = capture(2, &g);
            if (rc) break;
            bool ok = true;
            for (int i = 0; ok && i < 2; ++i) ok = ck(cudaGraphLaunch(g, st), "warm-up launch");
            ok = ok && ck(cudaEventRecord(e0, st), "event record");
            for (int i = 0; ok && i < attempts; ++i) ok = ck(cudaGraphLaunch(g, st), "timed launch");
            ok = ok && ck(cudaEventRecord(e1, st), "event record") && ck(cudaEventSynchronize(e1), "event sync");
            float ms = 0.f;
            if (ok) ck(cudaEventElapsedTime(&ms, e0, e1), "elapsed time");
            cudaGraphExecDestroy(g);
            if (rc) break;
            const double per = ms / attempts;
            r.paths[r.npaths] = path;
            r.ms_per_attempt[r.npaths] = per;
            r.npaths++;
            if (per < best) {
                best = per;
                r.path = path;
            }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        p.split = r.path >= 0 ? r.path : keep;
        for (cudaGraphExec_t* gp : {&g_loop, &g_raw, &g_shape})
            if (*gp) {
                cudaGraphExecDestroy(*gp);
                *gp = nullptr;
            }
        hc = saved;
        const cudaError_t pe = push();
        const cudaError_t se = cudaStreamSynchronize(st);
        if (rc) return rc;
        CB_CK(pe);
        CB_CK(se);
        if (r.npaths == 0) return fail(CB_EUNSUPPORTED, "no xy path to time");
        if (out) *out = r;
        return CB_OK;
    }

    // belastic::shape_adjust (belastic.cpp:174-284): forward Euler on g0 alone
    // from the current state, under the adjustment's accept and dt rules
    // (SCHED_SHAPE in the prologue and decide kernels).  It runs the Euler
    // attempt of this precision with M1 = M2 = 0 and ga = 3 / eta, so that
    // phi' = phi - dt ga (eta g0) = phi - 3 dt g0 and the energy is eta E_el.
    // The loop's own dt, time and counters are kept (belastic.cpp:280: the
    // adjustment restores time_step and does not advance time_current).  The
    // volume and area targets are taken again from the adjusted state when the
    // handle takes them from the state (beta <= 0): run_static_fEIF and
    // run_static read them after the adjustment (belastic.cpp:558-591, :289-325).
    int shape_adjust(int max_steps, cb_adjust_stats* out) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        if (!(p.eta > 0)) return fail(CB_EINVAL, "shape adjustment needs eta > 0");
        if (max_steps < 0) return fail(CB_EINVAL, "max_steps < 0");
        cb_params u = up;
        u.method = CB_EULER;
        u.M1 = u.M2 = 0.0;
        u.ga = 3.0 / p.eta;
        u.fixed_time_step = 0.0;
        u.rel_tol = 0.0;
        u.reject_tol = 0.0;
        Eff es{};
        int rc = make_params(u, es);
        if (rc) return rc;
        Params ps = es.p;
        ps.sched = SCHED_SHAPE;
        ps.dt_min = 1e-13;  // belastic.cpp:260
        CB_CK(pull());
        const Ctrl saved = hc;
        CB_CK(cudaMemcpyAsync(&d->p, &ps, sizeof ps, cudaMemcpyHostToDevice, st));
        // the state's sums and, in the FP32 form, its Euler partials (G slot)
        if (sizeof(T) == 4) {
            CB_CK(zpass(Z_INV_STATE, R_STATE));
            CB_CK(xypass(XY_FUSED, R_STATE));
        }
        CB_CK(pull());
        const double E_start = p.eta * hc.sc[R_STATE].E_el;
        hc.sc[R_STATE].E = E_start;
        hc.E_state = hc.E_init = hc.sa_eng = E_start;
        hc.dt = 1e-7;  // belastic.cpp:185
        hc.t = 0.0;
        hc.steps = hc.attempts = hc.rejects = 0;
        hc.target = max_steps > 0 ? max_steps : 1000000;
        hc.done = 0;
        hc.status = ST_RUNNING;
        hc.grow_pending = 1;  // the loop head runs before the first attempt
        hc.fresh = 1;
        hc.nonfinite = 0;
        CB_CK(push());
        if (!g_shape) {
            rc = capture(false, &g_shape, M_EULER);
            if (rc) {
                cudaMemcpy(&d->p, &p, sizeof p, cudaMemcpyHostToDevice);
                return rc;
            }
        }
        cudaEvent_t e0, e1;
        CB_CK(cudaEventCreate(&e0));
        CB_CK(cudaEventCreate(&e1));
        CB_CK(cudaEventRecord(e0, st));
        long long launches = 0;
        const long long limit = 70LL * (hc.target + 1LL) + 1000;
        bool timed_out = false;
        while (!hc.done && launches <= limit) {
            long long chunk = 64;
            if (launch_limit > 0) {
                if (launches >= launch_limit) { timed_out = true; break; }
                chunk = std::min(chunk, launch_limit - launches);
            }
            for (long long i = 0; i < chunk; ++i) CB_CK(cudaGraphLaunch(g_shape, st));
            launches += chunk;
            CB_CK(pull());
        }
        CB_CK(cudaEventRecord(e1, st));
        CB_CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        const Ctrl fin = hc;
        // back to the loop: its parameters, counters and dt, on the adjusted state
        CB_CK(cudaMemcpyAsync(&d->p, &p, sizeof p, cudaMemcpyHostToDevice, st));
        hc = saved;
        hc.spec_state = fin.spec_state;
        hc.part_state = fin.part_state;
        hc.ab_state = fin.ab_state;
        hc.u_state = fin.u_state;
        hc.sc[R_STATE] = fin.sc[R_STATE];
        hc.fresh = 1;
        hc.done = 0;
        CB_CK(push());
        CB_CK(zpass(Z_INV_STATE, R_STATE));
        CB_CK(xypass(sizeof(T) == 4 ? XY_FUSED : XY_REDUCE_FULL, R_STATE));
        CB_CK(pull());
        if (!(up.beta > 0.0)) {
            hc.alpha = hc.alpha0 = hc.sc[R_STATE].V;
            hc.beta = hc.beta0 = hc.sc[R_STATE].S;
        }
        Scal& sc = hc.sc[R_STATE];
        const double ve = sc.V - hc.alpha, se = sc.S - hc.beta;
        sc.E = p.eta * sc.E_el + 0.5 * p.M1 * ve * ve + 0.5 * p.M2 * se * se;
        hc.E_state = hc.E_init = sc.E;
        CB_CK(push());
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        CB_CK(cudaStreamSynchronize(st));
        if (out) {
            out->steps = fin.steps;
            out->attempts = fin.attempts;
            out->status = fin.done ? fin.status : ST_RUNNING;
            out->graph_launches = (int)launches;
            out->t = fin.t;
            out->E_start = E_start;
            out->E_end = fin.E_state;
            out->device_ms = ms;
        }
        if (timed_out && !fin.done)
            return fail(CB_ETIMEOUT, "shape adjustment stopped at the launch limit (%lld attempts)", launches);
        if (!fin.done) return fail(CB_ENOTCONVERGED, "shape adjustment made no progress after %lld attempts", launches);
        return CB_OK;
    }

    int raw_step(int method) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        if (method != p.method) return fail(CB_EINVAL, "handle was created for method %d, not %d", p.method, method);
        CB_CK(pull());
        hc.target = INT_MAX;
        hc.done = 0;
        CB_CK(push());
        if (!g_raw) {
            int rc = capture(true, &g_raw);
            if (rc) return rc;
        }
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        CB_CK(cudaGraphLaunch(g_raw, st));
        CB_CK(pull());
        last_status = hc.status;
        if (hc.nonfinite) return fail(CB_ENONFINITE, "state is no longer finite");
        return CB_OK;
    }

    int run(int nsteps, cb_run_stats* stt) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        if (nsteps < 0) return fail(CB_EINVAL, "nsteps < 0");
        CB_CK(pull());
        const int steps0 = hc.steps, att0 = hc.attempts;
        hc.target = hc.steps + nsteps;
        hc.done = nsteps == 0 ? 1 : 0;
        hc.status = nsteps == 0 ? ST_TARGET : ST_RUNNING;
        CB_CK(push());
        if (!g_loop) {
            int rc = capture(false, &g_loop);
            if (rc) return rc;
        }
        cudaEvent_t e0, e1;
        CB_CK(cudaEventCreate(&e0));
        CB_CK(cudaEventCreate(&e1));
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        CB_CK(cudaEventRecord(e0, st));
        int launches = 0;
        const long long limit = 70LL * (nsteps + 1) * (p.corr ? 2 : 1) + 1000;
        int stop = CB_OK;  // CB_ETIMEOUT at the caller's launch limit, CB_ENOTCONVERGED at the built-in one
        while (!hc.done) {
            const int remaining = hc.target - hc.steps;
            int chunk = remaining * (p.corr ? 2 : 1) + remaining / 8 + 1;
            chunk = std::max(1, std::min(chunk, 512));
            if (launch_limit > 0) {
                if (launches >= launch_limit) { stop = CB_ETIMEOUT; break; }
                chunk = (int)std::min<long long>(chunk, launch_limit - launches);
            }
            for (int i = 0; i < chunk; ++i) CB_CK(cudaGraphLaunch(g_loop, st));
            launches += chunk;
            CB_CK(pull());
            if (!hc.done && launches > limit) { stop = CB_ENOTCONVERGED; break; }
        }
        CB_CK(cudaEventRecord(e1, st));
        CB_CK(cudaEventSynchronize(e1));
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        last_status = hc.status;
        if (stt) {
            stt->steps = hc.steps - steps0;
            stt->attempts = hc.attempts - att0;
            stt->status = hc.status;
            stt->graph_launches = launches;
            stt->device_ms = ms;
        }
        // leave the instance live for getters and further runs
        hc.done = 0;
        CB_CK(push());
        CB_CK(cudaStreamSynchronize(st));
        // a stopped call ends between attempts: the state is the last accepted one and a
        // further cb_run continues the same trajectory
        if (stop == CB_ETIMEOUT)
            return fail(CB_ETIMEOUT, "stopped at the launch limit of %lld attempts (%d of %d steps taken)",
                        launch_limit, hc.steps - steps0, nsteps);
        if (stop == CB_ENOTCONVERGED) return fail(CB_ENOTCONVERGED, "no progress after %d attempts", launches);
        switch (last_status) {
            case ST_NONFINITE: return fail(CB_ENONFINITE, "state blew up (non-finite energy)");
            case ST_DT_UNDERFLOW: return fail(CB_EDTUNDERFLOW, "adaptive dt fell below %g", p.dt_min);
            default: return CB_OK;
        }
    }

    int field(int which, double* out, bool dev) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        int rc = ensure_scratch();
        if (rc) return rc;
        CB_CK(pull());
        const size_t N = (size_t)p.N;
        const bool cplx_out = which == CB_FIELD_FD || which == CB_FIELD_NLD_HAT;
        const size_t out_doubles = cplx_out ? 2 * ns : N;
        double* dst = dev ? out : rbuf[5];
        if (cplx_out && !dev) {
            if (!cbuf) CB_CK(cudaMalloc(&cbuf, 2 * ns * sizeof(double)));
            dst = cbuf;
        }
        const void* phat = h.spec[hc.spec_state];
        double* phi = rbuf[0];
        auto need_phi = [&]() { return inv3d(phat, SM_NONE, phi, nullptr, true); };
        const double eps = p.eps;
        switch (which) {
            case CB_FIELD_PHI: CB_CK(inv3d(phat, SM_NONE, dst, nullptr, true)); break;
            case CB_FIELD_FD: CB_CK(Launch<T>::state_to_double(phat, dst, ns, st)); break;
            case CB_FIELD_LAP: CB_CK(inv3d(phat, SM_LAP, dst, nullptr, true)); break;
            case CB_FIELD_DX: CB_CK(inv3d(phat, SM_DX, dst, nullptr, true)); break;
            case CB_FIELD_DY: CB_CK(inv3d(phat, SM_DY, dst, nullptr, true)); break;
            case CB_FIELD_DZ: CB_CK(inv3d(phat, SM_DZ, dst, nullptr, true)); break;
            case CB_FIELD_F:
            case CB_FIELD_G0:
            case CB_FIELD_NLD: {
                CB_CK(need_phi());
                CB_CK(inv3d(phat, SM_LAP, rbuf[1], nullptr, true));
                double* f = which == CB_FIELD_F ? dst : rbuf[2];
                CB_CK(launch_pointwise(0, N, f, phi, rbuf[1], nullptr, nullptr, eps, 0, 0, 0, st));
                if (which == CB_FIELD_G0) {  // Calc.cu:171-188: g0 = -lap f + (3 phi^2 - 1) f / eps^2
                    CB_CK(fwd3d(f, tmpS));
                    CB_CK(inv3d(tmpS, SM_LAP, rbuf[3]));
                    CB_CK(launch_pointwise(1, N, dst, phi, f, rbuf[3], nullptr, eps, 0, 0, 0, st));
                } else if (which == CB_FIELD_NLD) {  // Calc.cu:265-297
                    CB_CK(launch_pointwise(2, N, rbuf[3], phi, nullptr, nullptr, nullptr, eps, 0, 0, 0, st));
                    CB_CK(fwd3d(rbuf[3], tmpS));
                    CB_CK(inv3d(tmpS, SM_LAP, rbuf[4]));
                    CB_CK(launch_pointwise(3, N, dst, phi, f, rbuf[3], rbuf[4], eps, 0, 0, 0, st));
                }
                break;
            }
            case CB_FIELD_S: {  // Calc.cu:358-374
                CB_CK(need_phi());
                CB_CK(inv3d(phat, SM_DX, rbuf[1], nullptr, true));
                CB_CK(inv3d(phat, SM_DY, rbuf[2], nullptr, true));
                CB_CK(inv3d(phat, SM_DZ, rbuf[3], nullptr, true));
                CB_CK(launch_pointwise(4, N, dst, phi, rbuf[1], rbuf[2], rbuf[3], eps, 0, 0, 0, st));
                break;
            }
            case CB_FIELD_NLD_HAT:
            case CB_FIELD_RHS: {
                // the hot-path kernels themselves: xy NONLIN on the state, then the
                // stage-1 z pass leaves N_u (ETD) or R-hat (Euler) in the Nu buffer
                const bool etd = p.method != M_EULER;
                if ((which == CB_FIELD_NLD_HAT) != etd)
                    return fail(CB_EINVAL, "field %d needs a %s handle", which, etd ? "Euler" : "ETD");
                hc.fresh = 1;
                hc.done = 0;
                CB_CK(push());
                CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
                if (sizeof(T) == 8) CB_CK(xypass(XY_NONLIN, R_STATE));  // FP32: the state's G slot holds them
                CB_CK(zpass(etd ? (p.method == M_ETD2 ? Z_ETD2_S1 : Z_ETD4_S1) : Z_EULER, etd ? R_WORK : R_CAND));
                if (etd) CB_CK(Launch<T>::nhat_full(d, h.spec[hc.spec_state], dst, ns, st));
                else CB_CK(inv3d(h.Nu, SM_NONE, dst));
                break;
            }
            default: return fail(CB_EINVAL, "unknown field %d", which);
        }
        if (!dev) CB_CK(cudaMemcpyAsync(out, dst, out_doubles * sizeof(double), cudaMemcpyDeviceToHost, st));
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

    // Same loop as run(), one attempt at a time, each bracketed by CUDA events
    // on the handle's stream; an optional L2 flush (memset of flush_bytes)
    // runs between attempts, outside the timed events.
    int run_timed(int nsteps, long long flush_bytes, double* ms_out, int* att_out) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        CB_CK(pull());
        hc.target = hc.steps + nsteps;
        hc.done = nsteps == 0 ? 1 : 0;
        hc.status = ST_RUNNING;
        CB_CK(push());
        if (!g_loop) {
            int rc = capture(false, &g_loop);
            if (rc) return rc;
        }
        if (flush_bytes > 0 && flush_bytes != flush_size) {
            cudaFree(flush_buf);
            flush_buf = nullptr;
            CB_CK(cudaMalloc(&flush_buf, (size_t)flush_bytes));
            flush_size = flush_bytes;
        }
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        cudaEvent_t e0, e1;
        CB_CK(cudaEventCreate(&e0));
        CB_CK(cudaEventCreate(&e1));
        double total = 0.0;
        int att = 0;
        const long long limit = 70LL * (nsteps + 1) * (p.corr ? 2 : 1) + 1000;
        bool timed_out = false;
        while (!hc.done && att < limit) {
            if (launch_limit > 0 && att >= launch_limit) { timed_out = true; break; }
            if (flush_bytes > 0) CB_CK(cudaMemsetAsync(flush_buf, att & 0xff, (size_t)flush_bytes, st));
            CB_CK(cudaEventRecord(e0, st));
            CB_CK(cudaGraphLaunch(g_loop, st));
            CB_CK(cudaEventRecord(e1, st));
            CB_CK(cudaEventSynchronize(e1));
            float ms = 0.f;
            CB_CK(cudaEventElapsedTime(&ms, e0, e1));
            total += ms;
            ++att;
            CB_CK(pull());
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        last_status = hc.status;
        hc.done = 0;
        CB_CK(push());
        CB_CK(cudaStreamSynchronize(st));
        if (ms_out) *ms_out = total;
        if (att_out) *att_out = att;
        if (timed_out) return fail(CB_ETIMEOUT, "stopped at the launch limit of %lld attempts", launch_limit);
        if (last_status == ST_NONFINITE) return fail(CB_ENONFINITE, "state blew up");
        if (att >= limit) return fail(CB_ENOTCONVERGED, "no progress after %d attempts", att);
        return CB_OK;
    }

    // nattempts loop attempts launched kernel by kernel (not from the graph),
    // with an event pair around every launch; per kind, the summed device time
    // and launch count.  Kernels that exit early (skipped stage 1) still count.
    int profile(int nattempts, long long flush_bytes, double* ms, int* cnt) override {
        if (!have_state) return fail(CB_EINVAL, "no state: call cb_set_phi first");
        for (int k = 0; k < K_NKIND; ++k) { ms[k] = 0.0; cnt[k] = 0; }
        CB_CK(pull());
        hc.target = INT_MAX;
        hc.done = 0;
        CB_CK(push());
        if (flush_bytes > 0 && flush_bytes != flush_size) {
            cudaFree(flush_buf);
            flush_buf = nullptr;
            CB_CK(cudaMalloc(&flush_buf, (size_t)flush_bytes));
            flush_size = flush_bytes;
        }
        CB_CK(Launch<T>::coef(d, 1, e.accurate, st));
        for (int a = 0; a < nattempts; ++a) {
            if (flush_bytes > 0) CB_CK(cudaMemsetAsync(flush_buf, a & 0xff, (size_t)flush_bytes, st));
            std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>> prof;
            int rc = enqueue_attempt(false, &prof);
            if (rc) return rc;
            CB_CK(cudaStreamSynchronize(st));
            for (auto& t : prof) {
                float m = 0.f;
                cudaEventElapsedTime(&m, std::get<1>(t), std::get<2>(t));
                ms[std::get<0>(t)] += m;
                cnt[std::get<0>(t)] += 1;
                cudaEventDestroy(std::get<1>(t));
                cudaEventDestroy(std::get<2>(t));
            }
        }
        CB_CK(pull());
        hc.done = 0;
        CB_CK(push());
        CB_CK(cudaStreamSynchronize(st));
        return CB_OK;
    }

   private:
    void reset_ctrl() {
        Ctrl c;
        memset(&c, 0, sizeof c);
        c.dt = e.dt0;
        c.alpha = up.alpha;
        c.beta = up.beta;
        c.fresh = 1;
        c.target = INT_MAX;
        c.fill_slot = -1;
        hc = c;
        last_status = ST_RUNNING;
    }
    cudaError_t push() { return cudaMemcpyAsync(h.ctrl, &hc, sizeof hc, cudaMemcpyHostToDevice, st); }
    cudaError_t pull() {
        cudaError_t r = cudaMemcpyAsync(&hc, h.ctrl, sizeof hc, cudaMemcpyDeviceToHost, st);
        if (r != cudaSuccess) return r;
        return cudaStreamSynchronize(st);
    }
    cudaError_t xypass(int mode, int role, int skip = 0) {
        XYArgs a;
        memset(&a, 0, sizeof a);
        a.mode = mode;
        a.role = role;
        a.skip_if_stale = skip;
        a.curv = p.curv;
        return Launch<T>::xy(p.nx, d, 1, p.nz, a, st, p.split);
    }
    cudaError_t zpass(int mode, int role) {
        ZArgs a;
        memset(&a, 0, sizeof a);
        a.mode = mode;
        a.role = role;
        a.curv = p.curv;
        return Launch<T>::z(p.nz, d, 1, ntiles, a, st);
    }
    // real double field -> spectrum (x 1/N), through the partial buffer `part`
    cudaError_t fwd3d(const double* src, void* spec, void* part = nullptr, bool to_state = false) {
        if (!part) part = tmpP;
        XYArgs a;
        memset(&a, 0, sizeof a);
        a.mode = XY_FWD_PLAIN;
        a.rin = src;
        a.cout = part;
        cudaError_t r = Launch<T>::xy(p.nx, d, 1, p.nz, a, st, p.split);
        if (r != cudaSuccess) return r;
        ZArgs z;
        memset(&z, 0, sizeof z);
        z.mode = Z_FWD_PLAIN;
        z.state_io = to_state ? IO_COUT_STATE : 0;
        z.cin = part;
        z.cout = spec;
        return Launch<T>::z(p.nz, d, 1, ntiles, z, st);
    }
    // FP64 plain transforms over the auxiliary descriptor (FP32 form only), between the
    // real double field and the FP32 form's double-float state spectrum
    cudaError_t fwd3d_f64(const double* src, void* state, void* part64) {
        XYArgs a;
        memset(&a, 0, sizeof a);
        a.mode = XY_FWD_PLAIN;
        a.rin = src;
        a.cout = part64;
        cudaError_t r = Launch<double>::xy(p.nx, aux, 1, p.nz, a, st, p.split);
        if (r != cudaSuccess) return r;
        ZArgs z;
        memset(&z, 0, sizeof z);
        z.mode = Z_FWD_PLAIN;
        z.state_io = IO_COUT_FF;
        z.cin = part64;
        z.cout = state;
        return Launch<double>::z(p.nz, aux, 1, ntiles64(), z, st);
    }
    cudaError_t inv3d_f64(const void* state, double* dst, void* part64) {
        ZArgs z;
        memset(&z, 0, sizeof z);
        z.mode = Z_INV_PLAIN;
        z.state_io = IO_CIN_FF;
        z.cin = state;
        z.cout = part64;
        cudaError_t r = Launch<double>::z(p.nz, aux, 1, ntiles64(), z, st);
        if (r != cudaSuccess) return r;
        XYArgs a;
        memset(&a, 0, sizeof a);
        a.mode = XY_INV_PLAIN;
        a.cin = part64;
        a.rout = dst;
        return Launch<double>::xy(p.nx, aux, 1, p.nz, a, st, p.split);
    }
    int ntiles64() const { return (p.ny * p.nc + Launch<double>::z_tile() - 1) / Launch<double>::z_tile(); }
    // spectrum (x multiplier) -> real double field, through `part`
    cudaError_t inv3d(const void* spec, int mul, double* dst, void* part = nullptr, bool from_state = false) {
        if (!part) part = tmpP;
        ZArgs z;
        memset(&z, 0, sizeof z);
        z.mode = Z_INV_PLAIN;
        z.mul = mul;
        z.state_io = from_state ? IO_CIN_STATE : 0;
        z.cin = spec;
        z.cout = part;
        cudaError_t r = Launch<T>::z(p.nz, d, 1, ntiles, z, st);
        if (r != cudaSuccess) return r;
        XYArgs a;
        memset(&a, 0, sizeof a);
        a.mode = XY_INV_PLAIN;
        a.cin = part;
        a.rout = dst;
        return Launch<T>::xy(p.nx, d, 1, p.nz, a, st, p.split);
    }
    int ensure_scratch() {
        if (scratch) return CB_OK;
        const size_t N = (size_t)p.N;
        const size_t cb = ((ns * sizeof(T) * 2) + 255) & ~(size_t)255;
        const size_t rb = ((N * sizeof(double)) + 255) & ~(size_t)255;
        if (cudaMalloc(&scratch, 2 * cb + 6 * rb) != cudaSuccess) {
            cudaGetLastError();
            return fail(CB_ENOMEM, "scratch allocation failed");
        }
        tmpP = scratch;
        tmpS = (char*)scratch + cb;
        for (int i = 0; i < 6; ++i) rbuf[i] = reinterpret_cast<double*>((char*)scratch + 2 * cb + i * rb);
        return CB_OK;
    }
    // prof != nullptr: record an event pair around every launch (profiling; not captured)
    int enqueue_attempt(int raw, std::vector<std::tuple<int, cudaEvent_t, cudaEvent_t>>* prof = nullptr,
                        int method = -1) {
        cudaError_t r = enqueue_group<T>(method < 0 ? p.method : method, p.nx, p.nz, d, 1, ntiles, e.accurate, raw,
                                         p.split, p.curv, st, prof);
        if (r != cudaSuccess) return fail(CB_ECUDA, "enqueue attempt: %s", cudaGetErrorString(r));
        return CB_OK;
    }
    int capture(int raw, cudaGraphExec_t* out, int method = -1) {
        cudaGraph_t g = nullptr;
        CB_CK(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_attempt(raw, nullptr, method);
        cudaError_t ce = cudaStreamEndCapture(st, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        CB_CK(ce);
        cudaError_t ie = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        CB_CK(ie);
        return CB_OK;
    }

    cb_params up{};
    Eff e{};
    Params p{};
    InstT<T> h{};
    InstT<T>* d = nullptr;
    Ctrl hc{};
    void* arena = nullptr;
    size_t arena_bytes = 0;
    void* scratch = nullptr;
    void* tmpP = nullptr;
    void* tmpS = nullptr;
    double* rbuf[6] = {};
    double* cbuf = nullptr;
    size_t ns = 0;
    int ntiles = 0;
    cudaStream_t st = nullptr;
    bool ext_arena = false, ext_stream = false;
    InstT<double>* aux = nullptr;  // FP64 descriptor for exact set/get of phi (FP32 form)
    InstT<double> aux_h{};
    cudaGraphExec_t g_loop = nullptr, g_raw = nullptr, g_shape = nullptr;
    void* flush_buf = nullptr;
    long long flush_size = 0;
    bool have_state = false;
    int last_status = ST_RUNNING;
};

}  // namespace cb

