/* cstep.c -- plain FP64 host C restatement of CudaBubble's spectral step.
 *
 * TEST INFRASTRUCTURE ONLY (part of the oracle): the timed CPU baseline of
 * bench.py and a second, compiled check of oracle/oracle.py.  Nothing in the
 * product links it.
 *
 * It follows the reference's algorithm and operation order, not the GPU
 * stepper's: every derived field goes through a real-space round trip as in
 * phasefield.cpp (update_fd = C2R, fd = R2C), the Laplacian keeps the Nyquist
 * modes (Calc.cu:107-124), the gradient zeroes them (Calc.cu:300-341), the
 * forward transform is normalised by 1/N (Calc.cu:88-96), and the ETD update
 * kernels are Calc.cu:446-577.  FFTs are this file's own mixed-radix (2, 3, 4)
 * complex transforms; the x axis is a real transform through a half-length
 * complex FFT.  Loops are parallelised with OpenMP over lines / points.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { double re, im; } cx;

static inline cx cmul(cx a, cx b) { cx r = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re}; return r; }
static inline cx cadd(cx a, cx b) { cx r = {a.re + b.re, a.im + b.im}; return r; }
static inline cx csub(cx a, cx b) { cx r = {a.re - b.re, a.im - b.im}; return r; }
static inline cx cconj(cx a) { cx r = {a.re, -a.im}; return r; }

/* ------------------------------------------------------------- 1-D FFT */
typedef struct {
    int n;
    int nf;
    int f[32];  /* radix factors */
    cx* w;      /* W_n^e = exp(-2 pi i e / n), e in [0, n) */
} plan1;

static int plan_init(plan1* p, int n) {
    p->n = n;
    p->nf = 0;
    int m = n;
    while (m % 4 == 0) { p->f[p->nf++] = 4; m /= 4; }
    while (m % 2 == 0) { p->f[p->nf++] = 2; m /= 2; }
    while (m % 3 == 0) { p->f[p->nf++] = 3; m /= 3; }
    if (m != 1) return -1;
    p->w = (cx*)malloc(sizeof(cx) * (size_t)n);
    for (int e = 0; e < n; ++e) {
        long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)e / (long double)n;
        p->w[e].re = (double)cosl(a);
        p->w[e].im = (double)-sinl(a);
    }
    return 0;
}

/* recursive decimation in time: out[0..n) = DFT of in[0], in[s], in[2s], ...
 * sign = -1 forward, +1 inverse (unnormalised) */
static void fft_rec(const cx* in, int s, cx* out, int n, const plan1* P, int lvl, int sign) {
    if (n == 1) { out[0] = in[0]; return; }
    const int p = P->f[lvl], m = n / p, N = P->n, step = N / n;
    for (int q = 0; q < p; ++q) fft_rec(in + (size_t)q * s, s * p, out + (size_t)q * m, m, P, lvl + 1, sign);
    for (int k = 0; k < m; ++k) {
        cx t[4];
        for (int q = 0; q < p; ++q) {
            cx w = P->w[(size_t)((q * k) % n) * step];
            if (sign > 0) w.im = -w.im;
            t[q] = q ? cmul(out[q * m + k], w) : out[k];
        }
        if (p == 2) {
            out[k] = cadd(t[0], t[1]);
            out[k + m] = csub(t[0], t[1]);
        } else if (p == 4) {
            cx s0 = cadd(t[0], t[2]), d0 = csub(t[0], t[2]), s1 = cadd(t[1], t[3]), d1 = csub(t[1], t[3]);
            cx jd1 = sign < 0 ? (cx){d1.im, -d1.re} : (cx){-d1.im, d1.re};
            out[k] = cadd(s0, s1);
            out[k + 2 * m] = csub(s0, s1);
            out[k + m] = cadd(d0, jd1);
            out[k + 3 * m] = csub(d0, jd1);
        } else { /* 3 */
            const double h = 0.86602540378443864676;
            cx su = cadd(t[1], t[2]), df = csub(t[1], t[2]);
            cx mm = {t[0].re - 0.5 * su.re, t[0].im - 0.5 * su.im};
            cx r = sign < 0 ? (cx){df.im, -df.re} : (cx){-df.im, df.re};
            out[k] = cadd(t[0], su);
            out[k + m] = (cx){mm.re + h * r.re, mm.im + h * r.im};
            out[k + 2 * m] = (cx){mm.re - h * r.re, mm.im - h * r.im};
        }
    }
}

/* ------------------------------------------------------------- 3-D R2C / C2R */
typedef struct {
    int nx, ny, nz, nc;
    size_t N, Nc;
    plan1 px2, py, pz;  /* half-length x, y, z */
    cx* wx;             /* W_nx^k, k in [0, nx) */
} fft3;

static int fft3_init(fft3* F, int nx, int ny, int nz) {
    F->nx = nx; F->ny = ny; F->nz = nz; F->nc = nx / 2 + 1;
    F->N = (size_t)nx * ny * nz;
    F->Nc = (size_t)F->nc * ny * nz;
    if (plan_init(&F->px2, nx / 2) || plan_init(&F->py, ny) || plan_init(&F->pz, nz)) return -1;
    F->wx = (cx*)malloc(sizeof(cx) * (size_t)nx);
    for (int e = 0; e < nx; ++e) {
        long double a = 2.0L * 3.141592653589793238462643383279502884L * (long double)e / (long double)nx;
        F->wx[e].re = (double)cosl(a);
        F->wx[e].im = (double)-sinl(a);
    }
    return 0;
}

/* forward, normalised by 1/N (Calc.cu:88-96) */
static void r2c(const fft3* F, const double* u, cx* s) {
    const int nx = F->nx, ny = F->ny, nz = F->nz, nc = F->nc, M = nx / 2;
    const double inv = 1.0 / (double)F->N;
#pragma omp parallel
    {
        cx* a = (cx*)malloc(sizeof(cx) * (size_t)(nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz)) * 2);
        cx* b = a + (nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz));
#pragma omp for schedule(static)
        for (long r = 0; r < (long)ny * nz; ++r) {
            const double* row = u + (size_t)r * nx;
            for (int m = 0; m < M; ++m) { a[m].re = row[2 * m]; a[m].im = row[2 * m + 1]; }
            fft_rec(a, 1, b, M, &F->px2, 0, -1);
            cx* o = s + (size_t)r * nc;
            for (int k = 0; k <= M; ++k) {
                cx zk = b[k % M], zm = cconj(b[(M - k) % M]);
                cx e = {0.5 * (zk.re + zm.re), 0.5 * (zk.im + zm.im)};
                cx d = cmul(csub(zk, zm), F->wx[k % nx]);
                o[k].re = e.re + 0.5 * d.im;
                o[k].im = e.im - 0.5 * d.re;
            }
        }
#pragma omp for schedule(static)
        for (long l = 0; l < (long)nz * nc; ++l) {
            const int z = (int)(l / nc), kx = (int)(l % nc);
            cx* base = s + (size_t)z * ny * nc + kx;
            for (int y = 0; y < ny; ++y) a[y] = base[(size_t)y * nc];
            fft_rec(a, 1, b, ny, &F->py, 0, -1);
            for (int y = 0; y < ny; ++y) base[(size_t)y * nc] = b[y];
        }
#pragma omp for schedule(static)
        for (long l = 0; l < (long)ny * nc; ++l) {
            cx* base = s + l;
            const size_t st = (size_t)ny * nc;
            for (int z = 0; z < nz; ++z) a[z] = base[z * st];
            fft_rec(a, 1, b, nz, &F->pz, 0, -1);
            for (int z = 0; z < nz; ++z) { base[z * st].re = b[z].re * inv; base[z * st].im = b[z].im * inv; }
        }
        free(a);
    }
}

/* inverse, unnormalised (Calc.cu:99-104); s is left unchanged */
static void c2r(const fft3* F, const cx* s, double* u, cx* tmp) {
    const int nx = F->nx, ny = F->ny, nz = F->nz, nc = F->nc, M = nx / 2;
    memcpy(tmp, s, sizeof(cx) * F->Nc);
#pragma omp parallel
    {
        const int mx = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
        cx* a = (cx*)malloc(sizeof(cx) * (size_t)mx * 2);
        cx* b = a + mx;
#pragma omp for schedule(static)
        for (long l = 0; l < (long)ny * nc; ++l) {
            cx* base = tmp + l;
            const size_t st = (size_t)ny * nc;
            for (int z = 0; z < nz; ++z) a[z] = base[z * st];
            fft_rec(a, 1, b, nz, &F->pz, 0, +1);
            for (int z = 0; z < nz; ++z) base[z * st] = b[z];
        }
#pragma omp for schedule(static)
        for (long l = 0; l < (long)nz * nc; ++l) {
            const int z = (int)(l / nc), kx = (int)(l % nc);
            cx* base = tmp + (size_t)z * ny * nc + kx;
            for (int y = 0; y < ny; ++y) a[y] = base[(size_t)y * nc];
            fft_rec(a, 1, b, ny, &F->py, 0, +1);
            for (int y = 0; y < ny; ++y) base[(size_t)y * nc] = b[y];
        }
#pragma omp for schedule(static)
        for (long r = 0; r < (long)ny * nz; ++r) {
            const cx* X = tmp + (size_t)r * nc;
            for (int k = 0; k < M; ++k) {
                cx xk = X[k], xm = cconj(X[M - k]);
                if (k == 0) { xk.im = 0; xm.re = X[M].re; xm.im = 0; }
                cx e = cadd(xk, xm);
                cx o = cmul(csub(xk, xm), cconj(F->wx[k]));
                a[k].re = e.re - o.im;
                a[k].im = e.im + o.re;
            }
            fft_rec(a, 1, b, M, &F->px2, 0, +1);
            double* row = u + (size_t)r * nx;
            for (int m = 0; m < M; ++m) { row[2 * m] = b[m].re; row[2 * m + 1] = b[m].im; }
        }
        free(a);
    }
}

/* ------------------------------------------------------------- stepper */
typedef struct {
    fft3 F;
    int nx, ny, nz;
    double xlen, eps, eta, ga, M1, M2, alpha, beta, alpha0, beta0, dt, L3;
    double *lapm, *gx, *gy, *gz, *het;  /* spectral multipliers, L(k) */
    double *d, *t0, *t1, *t2, *t3, *t4, *t5, *od;  /* real work arrays */
    cx *c0, *c1, *c2, *c3, *c4, *c5, *c6, *ctmp;   /* spectra */
    int steps, rejects;
    double tcur;
} cstep;

static double mean(const cstep* h, const double* u) {
    double s = 0.0;
#pragma omp parallel for reduction(+ : s) schedule(static)
    for (long i = 0; i < (long)h->F.N; ++i) s += u[i];
    return s / (double)h->F.N;
}

/* lap of a spectrum into a real field (Calc.cu:139-144) */
static void lap_spec(cstep* h, const cx* fd, double* out) {
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)h->F.Nc; ++i) {
        h->c6[i].re = fd[i].re * h->lapm[i];
        h->c6[i].im = fd[i].im * h->lapm[i];
    }
    c2r(&h->F, h->c6, out, h->ctmp);
}

/* derived fields of the state h->d: V, S, E_el and (optionally) f, NL */
typedef struct { double V, S, Eel; } scal3;

static scal3 state_scalars(cstep* h, const double* d, cx* fd, double* f, double* lap) {
    const size_t N = h->F.N, Nc = h->F.Nc;
    const double eps = h->eps;
    r2c(&h->F, d, fd);                               /* phasefield::fd */
    lap_spec(h, fd, lap);                             /* phasefield::lap */
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) f[i] = -lap[i] * eps + (d[i] * d[i] - 1.0) * d[i] / eps;  /* Calc.cu:160 */
    /* gradient, three Z2D (Calc.cu:300-356), then s (Calc.cu:358-368) */
    double* g[3] = {h->t3, h->t4, h->t5};
    const double* mult[3] = {h->gx, h->gy, h->gz};
    for (int a = 0; a < 3; ++a) {
#pragma omp parallel for schedule(static)
        for (long i = 0; i < (long)Nc; ++i) {
            const double m = mult[a][i];
            h->c6[i].re = -fd[i].im * m;
            h->c6[i].im = fd[i].re * m;
        }
        c2r(&h->F, h->c6, g[a], h->ctmp);
    }
    double ss = 0.0, sf = 0.0, su = 0.0;
#pragma omp parallel for reduction(+ : ss, sf, su) schedule(static)
    for (long i = 0; i < (long)N; ++i) {
        const double u = d[i], q = u * u - 1.0;
        ss += 0.5 * eps * (g[0][i] * g[0][i] + g[1][i] * g[1][i] + g[2][i] * g[2][i]) + 0.25 / eps * q * q;
        sf += f[i] * f[i];
        su += u;
    }
    scal3 r;
    r.V = (su / (double)N + 1.0) * 0.5 * h->L3;                         /* phasefield.cpp:283-289 */
    r.S = (ss / (double)N) * (3.0 / (2.0 * sqrt(2.0))) * h->L3;         /* phasefield.cpp:310-316 */
    r.Eel = (sf / (double)N) * (1.0 / (eps * 2.0)) * h->L3;             /* phasefield.cpp:318-325 */
    return r;
}

static double energy(const cstep* h, scal3 s) {  /* belastic.cpp:68-86 */
    const double ve = s.V - h->alpha, se = s.S - h->beta;
    return s.Eel * h->eta + 0.5 * h->M1 * ve * ve + 0.5 * h->M2 * se * se;
}

/* N-hat of state d (belastic.cpp:473-489); returns the scalars of d */
static scal3 nld_term(cstep* h, const double* d, cx* fd, cx* nhat) {
    const size_t N = h->F.N;
    const double eps = h->eps, kappa = 2.0, D = 1.5;
    double *f = h->t0, *lap = h->t1, *tt = h->t2, *lt = h->t3;
    scal3 s = state_scalars(h, d, fd, f, lap);
    const double l1 = h->M1 * (s.V - h->alpha), l2 = h->M2 * (s.S - h->beta);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) tt[i] = d[i] * (d[i] * d[i] - 1.0 - kappa);  /* nld_kernel1 */
    r2c(&h->F, tt, h->c5);
    lap_spec(h, h->c5, lt);
    const double ie = 1.0 / eps, ie2 = ie * ie, ie3 = ie * ie2;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) {
        const double nl = -lt[i] * ie + D * tt[i] * ie3 + (3 * d[i] * d[i] - D - 1) * ie2 * f[i];  /* nld_kernel2 */
        lap[i] = -l1 * 0.5 - l2 * f[i] * 3.0 / (2.0 * sqrt(2.0)) - nl * h->eta;                   /* nld2_kernel */
    }
    r2c(&h->F, lap, nhat);
    return s;
}

static void etd2_step(cstep* h) {  /* belastic.cpp:491-517 */
    const size_t Nc = h->F.Nc;
    const double dt = h->dt;
    cx *fd = h->c0, *nl = h->c1, *a = h->c2, *nn = h->c3, *fa = h->c4;
    nld_term(h, h->d, fd, nl);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)Nc; ++i) {  /* etd1_kernel */
        const double L = h->het[i], c = exp(L * dt);
        a[i].re = c * fd[i].re + (c - 1.0) * nl[i].re / L;
        a[i].im = c * fd[i].im + (c - 1.0) * nl[i].im / L;
    }
    c2r(&h->F, a, h->od + h->F.N, h->ctmp); /* m_pa->update_fd(a): a real-space */
    double* ar = h->od + h->F.N;
    nld_term(h, ar, fa, nn);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)Nc; ++i) {  /* etd2_kernel */
        const double L = h->het[i];
        double c = exp(L * dt);
        if (dt * L == 0) c = dt / 2;
        else c = (c - 1.0 - dt * L) / (dt * L * L);
        a[i].re = fa[i].re + c * (nn[i].re - nl[i].re);
        a[i].im = fa[i].im + c * (nn[i].im - nl[i].im);
    }
    c2r(&h->F, a, h->d, h->ctmp);
}

static void etd4_step(cstep* h, int textbook) {  /* belastic.cpp:519-552 */
    const size_t Nc = h->F.Nc, N = h->F.N;
    const double dt = h->dt;
    cx *fd = h->c0, *nl = h->c1, *nla = h->c2, *nlb = h->c3, *fa = h->c4;
    cx* ch = (cx*)malloc(sizeof(cx) * Nc);
    cx* bb = (cx*)malloc(sizeof(cx) * Nc);
    double* ar = h->od + N;
    nld_term(h, h->d, fd, nl);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)Nc; ++i) {  /* etd41 */
        const double L = h->het[i], e1 = exp(L * dt / 2);
        bb[i].re = e1 * fd[i].re + (e1 - 1.0) * nl[i].re / L;
        bb[i].im = e1 * fd[i].im + (e1 - 1.0) * nl[i].im / L;
    }
    c2r(&h->F, bb, ar, h->ctmp);
    nld_term(h, ar, fa, nla);
    memcpy(ch, fa, sizeof(cx) * Nc);  /* c = m_pa->fd() */
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)Nc; ++i) {  /* etd42 */
        const double L = h->het[i], e1 = exp(L * dt / 2);
        bb[i].re = e1 * fd[i].re + (e1 - 1.0) * nla[i].re / L;
        bb[i].im = e1 * fd[i].im + (e1 - 1.0) * nla[i].im / L;
    }
    c2r(&h->F, bb, ar, h->ctmp);
    nld_term(h, ar, fa, nlb);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)Nc; ++i) {  /* etd43 */
        const double L = h->het[i], e1 = exp(L * dt / 2);
        ch[i].re = ch[i].re * e1 + (e1 - 1.0) * (2 * nlb[i].re - nl[i].re) / L;
        ch[i].im = ch[i].im * e1 + (e1 - 1.0) * (2 * nlb[i].im - nl[i].im) / L;
    }
    c2r(&h->F, ch, ar, h->ctmp);
    nld_term(h, ar, fa, bb); /* bb = nldc */
    /* the reference passes nlda in the first slot too (belastic.cpp:550);
       Cox-Matthews has N_u there: f1 N_u + f2 (N_a + N_b) + f3 N_c */
    const cx* n1 = textbook ? nl : nla;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)Nc; ++i) {  /* etd44 */
        const double L = h->het[i], e1 = exp(L * dt / 2), e2 = e1 * e1, hh = dt;
        const double q = 1.0 / (hh * hh * L * L * L);
        const double a1 = -4.0 - hh * L + e2 * (4.0 - 3.0 * hh * L + hh * hh * L * L);
        const double a2 = 2.0 + hh * L + e2 * (-2 + hh * L);
        const double a3 = -4 - 3 * hh * L - hh * hh * L * L + e2 * (4 - hh * L);
        ch[i].re = e2 * fd[i].re + q * (n1[i].re * a1 + 2 * (nla[i].re + nlb[i].re) * a2 + bb[i].re * a3);
        ch[i].im = e2 * fd[i].im + q * (n1[i].im * a1 + 2 * (nla[i].im + nlb[i].im) * a2 + bb[i].im * a3);
    }
    c2r(&h->F, ch, h->d, h->ctmp);
    free(ch);
    free(bb);
}

/* Euler right-hand side of state d (belastic.cpp:52-64) into R */
static scal3 euler_rhs(cstep* h, const double* d, double* R) {
    const size_t N = h->F.N;
    const double eps = h->eps;
    double *f = h->t0, *lap = h->t1, *lf = h->t2;
    scal3 s = state_scalars(h, d, h->c0, f, lap);
    const double l1 = h->M1 * (s.V - h->alpha), l2 = h->M2 * (s.S - h->beta);
    r2c(&h->F, f, h->c5);
    lap_spec(h, h->c5, lf);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < (long)N; ++i) {
        const double g = -lf[i] + (3.0 * d[i] * d[i] - 1.0) * f[i] / (eps * eps);  /* g0_kernel */
        R[i] = l1 * 0.5 + l2 * f[i] + g * h->eta;                                   /* nld1_kernel */
    }
    return s;
}

/* ------------------------------------------------------------- API */
void* cs_create(int nx, int nz, double xlen, double eps, double eta, double ga, double M1, double M2) {
    cstep* h = (cstep*)calloc(1, sizeof(cstep));
    h->nx = nx; h->ny = nx; h->nz = nz;
    if (fft3_init(&h->F, nx, nx, nz)) { free(h); return 0; }
    h->xlen = xlen; h->eps = eps; h->eta = eta; h->ga = ga; h->M1 = M1; h->M2 = M2;
    h->L3 = xlen * xlen * xlen;
    const size_t N = h->F.N, Nc = h->F.Nc;
    const int nc = h->F.nc;
    h->lapm = (double*)malloc(5 * Nc * sizeof(double));
    h->gx = h->lapm + Nc; h->gy = h->gx + Nc; h->gz = h->gy + Nc; h->het = h->gz + Nc;
    const double c2 = (2.0 * 3.1415926535897932384626433832795 / xlen);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < nx; ++y)
            for (int x = 0; x < nc; ++x) {
                const size_t i = ((size_t)z * nx + y) * nc + x;
                const int zf = z < nz - z ? z : nz - z, yf = y < nx - y ? y : nx - y, xf = x < nx - x ? x : nx - x;
                const double c = -(zf * zf * c2 * c2 + yf * yf * c2 * c2 + xf * xf * c2 * c2);
                h->lapm[i] = c;  /* laplace_kernel */
                h->gx[i] = (x == nx / 2) ? 0.0 : x * c2;
                h->gy[i] = (y == nx / 2) ? 0.0 : (y < nx - y ? y : y - nx) * c2;
                h->gz[i] = (z == nz / 2) ? 0.0 : (z < nz - z ? z : z - nz) * c2;
                h->het[i] = -eps * c * c + 2.0 * c / eps + 1.5 * (c - 2.0 / (eps * eps)) / eps;  /* init_fEIF */
            }
    double* r = (double*)malloc(9 * N * sizeof(double));
    h->d = r; h->t0 = r + N; h->t1 = r + 2 * N; h->t2 = r + 3 * N; h->t3 = r + 4 * N; h->t4 = r + 5 * N;
    h->t5 = r + 6 * N; h->od = r + 7 * N;  /* od holds two fields */
    cx* c = (cx*)malloc(8 * Nc * sizeof(cx));
    h->c0 = c; h->c1 = c + Nc; h->c2 = c + 2 * Nc; h->c3 = c + 3 * Nc; h->c4 = c + 4 * Nc; h->c5 = c + 5 * Nc;
    h->c6 = c + 6 * Nc; h->ctmp = c + 7 * Nc;
    return h;
}

void cs_destroy(void* p) {
    cstep* h = (cstep*)p;
    if (!h) return;
    free(h->lapm); free(h->d); free(h->c0);
    free(h->F.px2.w); free(h->F.py.w); free(h->F.pz.w); free(h->F.wx);
    free(h);
}

int cs_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void cs_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

void cs_set_phi(void* p, const double* phi) {
    cstep* h = (cstep*)p;
    memcpy(h->d, phi, h->F.N * sizeof(double));
    h->steps = h->rejects = 0;
    h->tcur = 0.0;
}
void cs_get_phi(void* p, double* phi) { cstep* h = (cstep*)p; memcpy(phi, h->d, h->F.N * sizeof(double)); }

/* out: V, S, E_el, E, alpha, beta, dt, steps, rejects */
void cs_scalars(void* p, double* out) {
    cstep* h = (cstep*)p;
    scal3 s = state_scalars(h, h->d, h->c0, h->t0, h->t1);
    out[0] = s.V; out[1] = s.S; out[2] = s.Eel; out[3] = energy(h, s);
    out[4] = h->alpha; out[5] = h->beta; out[6] = h->dt; out[7] = h->steps; out[8] = h->rejects;
}

/* forward / inverse transforms exposed for tests */
void cs_r2c(void* p, const double* u, double* s) { cstep* h = (cstep*)p; r2c(&h->F, u, (cx*)s); }
void cs_c2r(void* p, const double* s, double* u) { cstep* h = (cstep*)p; c2r(&h->F, (const cx*)s, u, h->ctmp); }

/* run: method 0 Euler (run_static), 1 ETD2, 2 ETD4 (run_static_fEIF loop);
 * fixed <= 0 adaptive.  alpha/beta from t = 0 when beta <= 0.
 * Returns accepted steps; exit code in *why (0 max, 1 dt underflow, 2 small
 * energy, 3 blow-up, 4 converged). */
int cs_run(void* p, int method, int nsteps, double time_step, double fixed, double alpha, double beta,
           int etd4_textbook, int* why) {
    cstep* h = (cstep*)p;
    const size_t N = h->F.N;
    scal3 s = state_scalars(h, h->d, h->c0, h->t0, h->t1);
    if (h->steps == 0) {
        h->alpha = alpha; h->beta = beta;
        if (beta <= 0.0) { h->alpha = s.V; h->beta = s.S; }
        h->alpha0 = h->alpha; h->beta0 = h->beta;
        h->dt = time_step;
        if (fixed > 0) h->dt = fixed < time_step ? fixed : time_step;
    }
    double* od = h->od;
    double* R = (double*)malloc(N * sizeof(double));
    *why = 0;
    double eng0 = energy(h, s), eng1;
    if (method == 0) euler_rhs(h, h->d, R);
    const int target = h->steps + nsteps;
    while (h->steps < target) {
        if (fixed <= 0) {
            eng0 = energy(h, state_scalars(h, h->d, h->c0, h->t0, h->t1));
            memcpy(od, h->d, N * sizeof(double));
            if (h->steps % 4 == 0) {
                if (method == 0) h->dt *= 1.4;
                else h->dt = (h->dt * 1.4 < 0.001) ? h->dt * 2 : 0.001;
            }
            for (;;) {
                if (h->dt < 1e-23) break;
                if (method == 0) {
#pragma omp parallel for schedule(static)
                    for (long i = 0; i < (long)N; ++i) h->d[i] += -h->dt * h->ga * R[i];
                } else if (method == 1) etd2_step(h);
                else etd4_step(h, etd4_textbook);
                eng1 = energy(h, state_scalars(h, h->d, h->c0, h->t0, h->t1));
                if (eng1 > eng0) {
                    memcpy(h->d, od, N * sizeof(double));
                    h->dt /= 2;
                    h->rejects++;
                    continue;
                }
                break;
            }
        } else if (method != 0 && (h->M1 != 0 || h->M2 != 0)) {
            memcpy(od, h->d, N * sizeof(double));
            for (int rep = 0; rep < 2; ++rep) {
                if (rep) memcpy(h->d, od, N * sizeof(double));
                if (method == 1) etd2_step(h); else etd4_step(h, etd4_textbook);
                scal3 q = state_scalars(h, h->d, h->c0, h->t0, h->t1);
                h->alpha -= q.V - h->alpha0;
                h->beta -= q.S - h->beta0;
            }
        } else {
            if (method == 0) {
#pragma omp parallel for schedule(static)
                for (long i = 0; i < (long)N; ++i) h->d[i] += -h->dt * h->ga * R[i];
            } else if (method == 1) etd2_step(h);
            else etd4_step(h, etd4_textbook);
        }
        if (h->dt < 1e-23) { *why = 1; break; }
        if (method != 0 && eng0 < 1e-3) { *why = 2; break; }
        if (!isfinite(h->d[((size_t)(h->nz / 2) * h->ny + h->ny / 2) * h->nx + h->nx / 2])) { *why = 3; break; }
        h->tcur += h->dt;
        h->steps++;
        if (method == 0) euler_rhs(h, h->d, R);
    }
    free(R);
    return h->steps;
}
