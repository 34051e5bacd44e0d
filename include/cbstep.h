/* cbstep.h -- C ABI of the GB300 pseudo-spectral Allen-Cahn stepper.
 *
 * Drop-in replacement for the per-step call surface of CudaBubble's
 * vesicle relaxation (phase-field elastic bending energy with volume and
 * surface-area penalties on a periodic [-pi, pi]^3 grid).  The reference has
 * no plugin or FFI layer; it is one executable whose time loops call
 * (citations are file:line in the reference tree):
 *
 *   belastic::ETD2RK(Het)              belastic.cpp:491-517   -> cb_ETD2RK
 *   belastic::ETD4RK(Het)              belastic.cpp:519-552   -> cb_ETD4RK
 *   get_sum_fgqterm + time_diff_solve_phi
 *                                      belastic.cpp:52-64, phasefield.cpp:89-93
 *                                                             -> cb_euler_step
 *   belastic::getstaticenergy          belastic.cpp:68-86     -> cb_getstaticenergy
 *   belastic::run_static   (Euler)     belastic.cpp:286-470   -> cb_run (method CB_EULER)
 *   belastic::run_static_fEIF (ETD)    belastic.cpp:554-786   -> cb_run (CB_ETD2 / CB_ETD4)
 *   phasefield getters fd/lap/f/g0/nld/gradient/s/vol/surface/elastic_eng
 *                                      phasefield.cpp:130-325 -> cb_field, cb_scalars
 *   fluidbase ini first line (34 fields)
 *                                      fluidbase.cpp:33-35    -> cb_params_from_ini_line
 *
 * Conventions: real fields are double[nz][ny][nx] with x fastest (the
 * reference's .out layout, tool.cpp:118-132); spectra are complex double
 * [nz][ny][nx/2+1] (cuFFT D2Z layout, forward-normalised by 1/N as in
 * Calc.cu:88-96).  Every call returns CB_OK or a negative CB_E* code and
 * never exits the process (the reference exit()s, Calc.cu:52-55).
 * A handle owns one CUDA stream; calls on one handle are not thread-safe.
 */
#ifndef CBSTEP_H
#define CBSTEP_H

#ifdef __cplusplus
extern "C" {
#endif

enum {
    CB_OK = 0,
    CB_EINVAL = -1,         /* bad argument or unsupported grid */
    CB_ENOMEM = -2,         /* device allocation failed / over budget */
    CB_ECUDA = -3,          /* CUDA runtime error (see cb_last_error) */
    CB_ENONFINITE = -4,     /* the state blew up (non-finite energy) */
    CB_ENOTCONVERGED = -5,  /* step / attempt limit reached */
    CB_ETIMEOUT = -6,       /* a bounded wait ran out */
    CB_EDTUNDERFLOW = -7,   /* adaptive dt fell below 1e-23 (belastic.cpp:713) */
    CB_EUNSUPPORTED = -8    /* combination not built (grid size / precision) */
};

enum { CB_EULER = 0, CB_ETD2 = 1, CB_ETD4 = 2 };
enum { CB_FP64 = 0, CB_FP32 = 1 };

/* exit reasons reported in cb_scalars.status */
enum {
    CB_RUNNING = 0, CB_DONE_TARGET = 1, CB_DONE_DT_UNDERFLOW = 2, CB_DONE_SMALL_ENERGY = 3,
    CB_DONE_NONFINITE = 4, CB_DONE_CONVERGED = 5, CB_DONE_TMAX = 6,
    CB_DONE_CANCELLED = 7   /* served request cancelled by its client (cb_request.cancel_ms) */
};

/* field selectors for cb_field (phasefield.cpp getters) */
enum {
    CB_FIELD_PHI = 0,     /* phi (real)                              phasefield::d        */
    CB_FIELD_FD = 1,      /* phi-hat (complex, half spectrum)        phasefield::fd       */
    CB_FIELD_LAP = 2,     /* lap phi                                 phasefield::lap      */
    CB_FIELD_F = 3,       /* f = -eps lap phi + (phi^2-1) phi / eps  phasefield::f        */
    CB_FIELD_G0 = 4,      /* g0 = -lap f + (3 phi^2 - 1) f / eps^2   phasefield::g0       */
    CB_FIELD_NLD = 5,     /* ETD nonlinearity                        phasefield::nld      */
    CB_FIELD_DX = 6,      /* spectral gradient, Nyquist zeroed       phasefield::gradient */
    CB_FIELD_DY = 7,
    CB_FIELD_DZ = 8,
    CB_FIELD_S = 9,       /* surface density                         phasefield::s        */
    CB_FIELD_NLD_HAT = 10,/* N-hat of the ETD step (complex)         belastic::get_nld_term   (ETD handles) */
    CB_FIELD_RHS = 11     /* Euler right-hand side (real)            belastic::get_sum_fgqterm (Euler handles) */
};

typedef struct cb_params {
    int nx, ny, nz;          /* ny is forced to nx, as Calc.cu:45-46 does; nx even */
    double lenx;             /* box edge in units of 2*pi (ini "lenx", fluidbase.cpp:52-57) */
    int epssize;             /* ini "epssize": eps rule of fluidbase.cpp:68-108 */
    double eps;              /* > 0 overrides the epssize rule */
    double eta, ga;          /* bending rigidity, Euler mobility */
    double alpha, beta;      /* volume / area targets; beta <= 0: take them from t = 0 */
    double M1, M2;           /* volume / area penalty coefficients */
    double time_step;        /* initial dt */
    double fixed_time_step;  /* > 0: fixed dt = min(fixed_time_step, time_step) */
    double tmax;             /* Euler loop time limit */
    int method;              /* CB_EULER / CB_ETD2 / CB_ETD4 */
    int precision;           /* CB_FP64 (plain form) / CB_FP32 (FP32 FFT + FP64 reductions) */
    /* adaptive-dt schedule; defaults reproduce belastic.cpp:644-651 (ETD) and :376-378 (Euler) */
    int grow_every;          /* 0: method default (4) */
    double grow_factor;      /* 0: method default (2.0 ETD, 1.4 Euler) */
    double dt_cap;           /* 0: method default (1e-3 ETD, none for Euler) */
    double cap_probe;        /* 0: method default (1.4 ETD) */
    int etd4_textbook;       /* 1: Cox-Matthews combine with N_u; 0: the reference's N_a (belastic.cpp:550) */
    int accurate_coefficients; /* -1: default (FP32 form: phi-function series; FP64 form: reference closed forms) */
    double rel_tol;          /* > 0: cb_run stops (CB_DONE_CONVERGED) once an accepted step changes
                                E by less than rel_tol |E|; not in the reference loops */
    int xy_split;            /* xy pass path: 0 the size rule (one CTA per plane where a plane's two fields
                                fit, two-CTA clusters for the FP32 form from 64^2, else the split passes);
                                1 the split (y-column + x-row) passes; 2 one CTA per plane; 3 two-CTA
                                clusters (FP32 form, 64^2..192^2); cb_autotune picks among them */
    int pad0;
    double reject_tol;       /* adaptive loops reject an attempt when E_new > E_old + reject_tol |E_old|;
                                < 0: default 0, the reference rule (belastic.cpp:653-668), for both forms */
    double spont_c;          /* spontaneous curvature C of fc = f + (phi^2 - 1) C, from the reference's
                                commented-out formulas (phasefield.cpp:183-250); 0 (the reference, whose
                                curvature field is NULL, fluidbase.cpp:150) or any value: CB_FP64 on every
                                grid, CB_FP32 where the plane passes run as clusters or one CTA per plane
                                (planes up to 128^2; the split passes return CB_EUNSUPPORTED) */
} cb_params;

typedef struct cb_scalars {
    double V, S, E_el, E;    /* volume, area, elastic energy, total static energy */
    double lamb1, lamb2;     /* M1 (V - alpha), M2 (S - beta) */
    double alpha, beta;
    double dt, t;
    double lserror;          /* Euler LSerror of the last step (belastic.cpp:414) */
    int steps, attempts, rejects, status;
    double E_attempt;        /* energy of the last attempted candidate (accepted or not) */
} cb_scalars;

typedef struct cb_run_stats {
    int steps;               /* accepted steps taken by this call */
    int attempts;            /* attempts (accepted + rejected) */
    int status;              /* CB_DONE_* exit reason */
    int graph_launches;
    double device_ms;        /* CUDA-event time of the call's device work */
} cb_run_stats;

typedef struct cb_tune_result {
    int path;                /* the chosen xy path (cb_params.xy_split code) */
    int npaths;              /* paths timed */
    int paths[3];
    double ms_per_attempt[3];
} cb_tune_result;

typedef struct cb_adjust_stats {
    int steps;               /* accepted adjustment steps */
    int attempts;            /* attempts (accepted + rejected) */
    int status;              /* CB_DONE_CONVERGED (energy below 100 eta or changed < 2 % between
                                checks), CB_DONE_DT_UNDERFLOW (dt < 1e-13) or CB_DONE_TARGET */
    int graph_launches;
    double t;                /* adjustment time reached (not added to the run's time) */
    double E_start, E_end;   /* unconstrained energy eta E_el before and after */
    double device_ms;
} cb_adjust_stats;

typedef struct cb_handle cb_handle;

/* defaults for every field (FP64 ETD4 on 64^3, the reference's main path) */
void cb_params_default(cb_params* p);
/* parse the reference's ini first line (fluidbase.cpp:33-35 field order and
 * defaults); an optional 35th field selects the method and a 36th the
 * precision.  Returns CB_OK or CB_EINVAL. */
int cb_params_from_ini_line(const char* line, cb_params* p);
/* eps the instance will use (fluidbase.cpp:68-108) */
double cb_params_eps(const cb_params* p);
/* HBM bytes one instance needs */
long long cb_instance_bytes(const cb_params* p);
/* 1 when the (grid, precision, method) combination is built */
int cb_supported(const cb_params* p);

int cb_create(const cb_params* p, cb_handle** out);
int cb_destroy(cb_handle* h);
/* phi in the .out layout; on_device != 0 means a device pointer */
int cb_set_phi(cb_handle* h, const double* phi, int on_device);
int cb_get_phi(cb_handle* h, double* phi, int on_device);
int cb_scalars_get(cb_handle* h, cb_scalars* s);
double cb_getstaticenergy(cb_handle* h);
/* single reference step bodies at the current dt, always accepted */
int cb_ETD2RK(cb_handle* h);
int cb_ETD4RK(cb_handle* h);
int cb_euler_step(cb_handle* h);
/* the reference time loop of the handle's method until nsteps more accepted steps */
int cb_run(cb_handle* h, int nsteps, cb_run_stats* st);
/* derived fields; real fields N doubles, complex fields 2*Nc doubles */
int cb_field(cb_handle* h, int which, double* out, int on_device);
/* set the time step (and drop the cached coefficient table) */
int cb_set_dt(cb_handle* h, double dt);
/* resume: accepted time, dt and the volume / area targets alpha, beta of a
 * reference run (the .info file of fluidbase::load_info, fluidbase.cpp:2797-2826);
 * call after cb_set_phi, which otherwise takes alpha, beta from the new state */
int cb_set_loop_state(cb_handle* h, double t, double dt, double alpha, double beta);
/* belastic::shape_adjust (belastic.cpp:174-284): unconstrained pre-relaxation of the
 * current state, phi <- phi - 3 dt g0, kept only where eta E_el falls strictly, dt
 * from 1e-7 (halved on a rise, doubled every 10 steps); ends when eta E_el < 100 eta,
 * when it changed by < 2 % since the last check (checks at multiples of 1e-4 of
 * adjustment time), or when dt < 1e-13.  The loop's dt, time and counters are kept;
 * alpha, beta are taken again from the adjusted state when the parameters' beta <= 0.
 * max_steps > 0 bounds the accepted steps (0: 1,000,000). */
int cb_shape_adjust(cb_handle* h, int max_steps, cb_adjust_stats* st);
/* no counterpart in the reference: times `attempts` attempts of the handle's method on
 * each xy path it can run (2-CTA clusters, one CTA per plane, and the split passes when
 * the handle was created with them), from the current state without accepting any,
 * and keeps the fastest for this handle; the state, dt and counters are unchanged */
int cb_autotune(cb_handle* h, int attempts, cb_tune_result* out);
int cb_synchronize(cb_handle* h);
/* no counterpart in the reference, whose loops run until their own exit tests
 * (belastic.cpp:400-428, :712-740): bounds the attempts (graph launches) that one
 * cb_run, cb_run_timed or cb_shape_adjust call on this handle may make.  A call that
 * reaches the bound before its loop ends returns CB_ETIMEOUT; it stops between two
 * attempts, so the state is the last accepted one and a further call continues the
 * same trajectory.  0 (the default) keeps only the built-in no-progress bound, which
 * returns CB_ENOTCONVERGED. */
int cb_set_launch_limit(cb_handle* h, long long max_graph_launches);
/* HBM bytes held by the handle's stepping state */
long long cb_handle_bytes(cb_handle* h);

/* ---- measurement (no counterpart in the reference) ------------------------
 * cb_run_timed: cb_run, but one attempt per CUDA-event pair on the handle's
 * stream; flush_bytes > 0 writes that many bytes between attempts (outside
 * the timed pairs) so every attempt starts with a cold L2.  device_ms is the
 * summed attempt time.
 * cb_profile_kernels: nattempts loop attempts launched kernel by kernel with
 * an event pair around each launch; ms[k] / counts[k] (6 entries each) per
 * kernel kind k = 0 xy nonlinear pass, 1 xy reduce (S only), 2 xy reduce
 * (full), 3 z pass, 4 decide + coefficient table, 5 xy fused pass (FP32). */
int cb_run_timed(cb_handle* h, int nsteps, long long flush_bytes, double* device_ms, int* attempts);
int cb_profile_kernels(cb_handle* h, int nattempts, long long flush_bytes, double* ms, int* counts);

/* ---- batched vesicles (no counterpart in the reference, which runs one grid
 * per process, main.cpp:17-18).  Instances of uneven grids advance together:
 * one launch per pass covers every instance of a grid size, and one CUDA
 * graph runs an attempt of every instance.  Each instance keeps its own dt,
 * accept/reject state and exit test.  All instances share one precision. */
typedef struct cb_batch cb_batch;
int cb_batch_create(const cb_params* params, int n, cb_batch** out);
/* flags = CB_BATCH_PERSISTENT: one persistent kernel runs each attempt of every
 * instance, walking a device work list of (instance, pass, tile or plane) units with
 * per-instance dependency counters, instead of one launch per pass and grid size.
 * FP32 form, ETD-RK2, grids of 32, 48, 64, 96 or 128 per edge, no spontaneous
 * curvature, the default xy path; otherwise CB_EUNSUPPORTED.  Each instance's
 * decisions are its own as in the default mode, and its results are the default mode's
 * bit for bit, except on 64^2 planes, which the kernel runs on 512-thread CTAs (256 in
 * the default mode) and whose sums therefore differ in summation order.
 * A dependency wait that runs out of its bound makes cb_batch_run return CB_ETIMEOUT. */
#define CB_BATCH_PERSISTENT 1
int cb_batch_create_ex(const cb_params* params, int n, int flags, cb_batch** out);
int cb_batch_destroy(cb_batch* b);
int cb_batch_set_phi(cb_batch* b, int i, const double* phi, int on_device);
int cb_batch_get_phi(cb_batch* b, int i, double* phi, int on_device);
int cb_batch_scalars(cb_batch* b, int i, cb_scalars* s);
/* every instance takes nsteps more accepted steps (or stops at its own exit test) */
int cb_batch_run(cb_batch* b, int nsteps, cb_run_stats* st);
/* same, one attempt per CUDA-event pair with an L2 flush of flush_bytes between */
int cb_batch_run_timed(cb_batch* b, int nsteps, long long flush_bytes, double* device_ms, cb_run_stats* st);

/* ---- served relaxations (no counterpart in the reference).  A request is a
 * relaxation of a seeded ellipsoid phi0 = tanh(d / (sqrt(2) eps)) until an
 * accepted step changes E by less than params.rel_tol |E| (CB_DONE_CONVERGED)
 * or max_steps accepted steps pass (CB_DONE_TARGET: not converged).
 * cb_serve_trace replays an arrival trace in real time with continuous
 * batching.  Requests of one (grid, method) form a size class with its own
 * slot table, attempt graph and stream, so classes advance independently and
 * their work overlaps on the device.  Arrivals queue in arrival order; each
 * pass admits every queued request whose class has a free slot (a full class
 * is passed over) while hbm_budget_bytes holds its state (a request the
 * budget cannot hold stops admission behind it).  Instances live in arenas
 * carved from one device region reserved before the trace starts, so
 * admission allocates nothing.  A class runs `quantum` attempts per batch
 * (more for grids below 128^3, whose attempts are short), retires the
 * requests that finished or were cancelled, admits new ones and starts its
 * next batch at once. */
typedef struct cb_request {
    cb_params params;
    double axes[3], centre[3];    /* ellipsoid semi-axes and centre */
    double axes2[3], centre2[3];  /* optional second ellipsoid (union) when axes2[0] > 0 */
    double arrival_s;             /* arrival time from the start of the trace */
    int max_steps;
    int cancel_ms;                /* > 0: the client cancels the request this many ms after its arrival */
} cb_request;

typedef struct cb_result {
    double arrival_s, admitted_s, finished_s, latency_s;
    double E, V, S;
    int steps, attempts, status, pad;
    long long bytes;
} cb_result;

typedef struct cb_serve_stats {
    double wall_s;
    double point_steps;       /* sum over requests of grid points x accepted steps */
    int completed;
    int graph_launches;
    long long peak_bytes;     /* largest admitted stepping state */
} cb_serve_stats;

/* phi_out: NULL, or n pointers (NULL entries skip) that receive each request's final phi */
int cb_serve_trace(const cb_request* reqs, int n, long long hbm_budget_bytes, int max_slots_per_class, int quantum,
                   cb_result* results, double** phi_out, cb_serve_stats* stats);

/* No counterpart in the reference: an allocation-free volume integral.
 * Computes (mean(u) + addition) * multiply * volume of a device-resident real
 * field d_u[nz][ny][nx] and writes it to the device double *d_val on `stream`
 * (a cudaStream_t; NULL is the legacy default stream).  With addition 1 and
 * multiply 1/2 it is the vesicle volume; with addition 0 it integrates a
 * density (the surface term, f^2).  It allocates nothing: its per-plane
 * partial sums live in a fixed file-scope device array of 4096 planes
 * (32 KiB), so nz > 4096 returns CB_EINVAL.  It is meant for callers that may
 * not allocate device memory at the point of the call (a carved-up memory
 * pool, a host that forbids allocations after start-up).  The first call on
 * each device (and after a context rebuild) clears the array's counter
 * synchronously: make it before any stream capture.  All calls on a device
 * share the one array and each call leaves it ready for the next, so calls
 * that overlap in time (other streams, other host threads) race; serialise
 * them. */
int cb_intf_noalloc(const double* d_u, int nx, int ny, int nz, double addition, double multiply, double volume,
                    double* d_val, void* stream);

const char* cb_last_error(void);
const char* cb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* CBSTEP_H */
