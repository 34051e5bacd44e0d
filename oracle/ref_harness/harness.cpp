// Reference harness: drives the UNMODIFIED reference classes (belastic,
// phasefield, Calc) step by step so that the reference's own FP64 cuFFT path
// produces golden vectors and per-step timings on a GPU.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle).  Compiled by
// oracle/ref_harness/build_ref.sh with -Dprivate=public -Dprotected=public so
// the private step bodies are reachable; nothing in the product links it.
//
// The time loops below restate belastic.cpp:286-470 (run_static, forward
// Euler) and belastic.cpp:554-786 (run_static_fEIF) without their wall-clock
// output cadence, check_folder() stop and shape_adjust(); every numerical
// call inside them is the reference's own (ETD2RK, ETD4RK,
// get_sum_fgqterm, time_diff_solve_phi, getstaticenergy, vol, surface).
//
// The adjust mode calls the reference's own belastic::shape_adjust()
// (belastic.cpp:174-284) once and dumps the relaxed phi.
//
// usage:
//   refstep fields <workdir> <nx> <nz> <epssize> <dt> <phi0.out> <outdir>
//   refstep adjust <workdir> <nx> <nz> <epssize> <phi0.out> <outdir>
//   refstep run    <workdir> <euler|etd2|etd4> <nx> <nz> <epssize> <time_step>
//                  <fixed_dt> <M1> <M2> <nsteps> <phi0.out> <outdir> <snap_every>
// Standard headers first: the reference's tool.h defines min/max macros.
#include <cuda_runtime.h>
#include <sys/stat.h>
#include <unistd.h>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>
#include "belastic.h"
#include "mem_array.h"

static void die(const char* m) { fprintf(stderr, "refstep: %s\n", m); exit(2); }

static std::vector<double> read_raw(const char* path, size_t n) {
    std::vector<double> v(n);
    FILE* f = fopen(path, "rb");
    if (!f) die("cannot open phi0");
    if (fread(v.data(), sizeof(double), n, f) != n) die("short phi0");
    fclose(f);
    return v;
}

static void write_raw(const std::string& path, const void* p, size_t bytes) {
    FILE* f = fopen(path.c_str(), "wb");
    if (!f) die("cannot write output");
    fwrite(p, 1, bytes, f);
    fclose(f);
}

static void dump_dev(const std::string& path, const void* dptr, size_t bytes) {
    std::vector<char> h(bytes);
    cudaDeviceSynchronize();
    cudaMemcpy(h.data(), dptr, bytes, cudaMemcpyDeviceToHost);
    write_raw(path, h.data(), bytes);
}

// Lays out ./results/ini0.dat, ./results/<folder>/ and the ninit=7 phi0 file
// exactly where fluidbase::fluidbase / fluidbase::init look for them
// (fluidbase.cpp:27-48, :560-567, :230-238).
static void stage_workdir(const char* workdir, int nx, int nz, int epssize, double time_step,
                          double fixed_dt, double M1, double M2, const std::vector<double>& phi0) {
    mkdir(workdir, 0755);
    if (chdir(workdir) != 0) die("chdir");
    mkdir("results", 0755);
    const int folder = 7001;
    char dir[64];
    snprintf(dir, sizeof dir, "results/%d", folder);
    mkdir(dir, 0755);
    char info[128];
    snprintf(info, sizeof info, "%s/%dx%dx%d.info", dir, nx, nx, nz);
    unlink(info);  // a stale .info would trigger load_info() resume
    FILE* f = fopen("results/ini0.dat", "w");
    if (!f) die("ini");
    // folder nx ny nz lenx leny lenz shape time_step fluid_time_step fixed_time_step ninit nflush
    // surctrl epssize ncur angle Re eta gamma alpha beta M1 M2 M3 M4 tmax output_interval gweight
    // einit k c lineten alpha_3
    fprintf(f, "%d %d %d %d 1 1 1 0 %.17g 5e-6 %.17g 7 -1 1 %d 0 30 1.0 1 1 -1 -1 %.17g %.17g 0 0 100 30 0 0 30 70 10 -1\n",
            folder, nx, nx, nz, time_step, fixed_dt, epssize, M1, M2);
    fclose(f);
    char phif[128];
    size_t n = (size_t)nx * nx * nz;
    if (n * 8 > 100000)
        snprintf(phif, sizeof phif, "%s/d%dx%dx%d.out", dir, nx, nx, nz);
    else
        snprintf(phif, sizeof phif, "%s/d%dx%dx%d_%08d.out", dir, nx, nx, nz, 0);
    write_raw(phif, phi0.data(), n * sizeof(double));
}

static double dget(double* dptr) {
    double v;
    cudaMemcpy(&v, dptr, sizeof(double), cudaMemcpyDeviceToHost);
    return v;
}

static int mode_fields(int argc, char** argv) {
    if (argc < 9) die("fields args");
    const char* workdir = argv[2];
    int nx = atoi(argv[3]), nz = atoi(argv[4]), epssize = atoi(argv[5]);
    double dt = atof(argv[6]);
    size_t n = (size_t)nx * nx * nz, nc = (size_t)(nx / 2 + 1) * nx * nz;
    std::vector<double> phi0 = read_raw(argv[7], n);
    std::string out = argv[8];
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) die("getcwd");
    if (out[0] != '/') out = std::string(cwd) + "/" + out;
    stage_workdir(workdir, nx, nz, epssize, dt, dt, 1e4, 1e4, phi0);

    belastic t(0);
    phasefield* pd = t.m_pd;
    if (t.beta <= 0.0) {  // belastic.cpp:588-591
        t.alpha = dget(pd->vol());
        t.beta = dget(pd->surface());
    }
    FILE* js = fopen((out + "/scalars.json").c_str(), "w");
    double V = dget(pd->vol()), S = dget(pd->surface()), Eel = dget(pd->elastic_eng());
    double E = t.getstaticenergy(pd);
    fprintf(js, "{\"nx\": %d, \"nz\": %d, \"eps\": %.17g, \"alpha\": %.17g, \"beta\": %.17g, \"V\": %.17g, \"S\": %.17g, \"E_el\": %.17g, \"E\": %.17g, \"dt\": %.17g",
            nx, nz, t.eps, t.alpha, t.beta, V, S, Eel, E, dt);
    dump_dev(out + "/fd.bin", pd->fd(), nc * sizeof(cufftDoubleComplex));
    dump_dev(out + "/lap.bin", pd->lap(), n * 8);
    dump_dev(out + "/f.bin", pd->f(), n * 8);
    dump_dev(out + "/g0.bin", pd->g0(), n * 8);
    dump_dev(out + "/nld.bin", pd->nld(), n * 8);
    pd->gradient();
    dump_dev(out + "/dx.bin", pd->m_dx, n * 8);
    dump_dev(out + "/dy.bin", pd->m_dy, n * 8);
    dump_dev(out + "/dz.bin", pd->m_dz, n * 8);
    dump_dev(out + "/s.bin", pd->s(), n * 8);
    {
        double* R;
        cudaMalloc(&R, n * 8);
        t.get_sum_fgqterm(pd, R);  // belastic.cpp:52-64
        dump_dev(out + "/rhs_euler.bin", R, n * 8);
        double err = dget(pd->LSerror(R));
        fprintf(js, ", \"LSerror\": %.17g", err);
        cudaFree(R);
    }
    {
        cufftDoubleComplex* nl;
        cudaMalloc(&nl, nc * sizeof(cufftDoubleComplex));
        t.get_nld_term(pd, nl);  // belastic.cpp:473-489
        dump_dev(out + "/nld_hat.bin", nl, nc * sizeof(cufftDoubleComplex));
        cudaFree(nl);
    }
    double* Het;
    cudaMalloc(&Het, n * 8);
    t.calc->init_fEIF(Het, t.eps);  // Calc.cu:579-606
    dump_dev(out + "/Het.bin", Het, nc * 8);
    t.time_step = dt;
    double* od;
    cudaMalloc(&od, n * 8);
    cudaMemcpy(od, pd->d(), n * 8, cudaMemcpyDeviceToDevice);
    // one forward-Euler step (belastic.cpp:382)
    {
        double* R;
        cudaMalloc(&R, n * 8);
        t.get_sum_fgqterm(pd, R);
        pd->time_diff_solve_phi(R, -dt * t.ga);
        dump_dev(out + "/euler1.bin", pd->d(), n * 8);
        cudaFree(R);
    }
    cudaMemcpy(pd->d(), od, n * 8, cudaMemcpyDeviceToDevice);
    pd->update_d();
    t.ETD2RK(Het);
    dump_dev(out + "/etd2_1.bin", pd->d(), n * 8);
    cudaMemcpy(pd->d(), od, n * 8, cudaMemcpyDeviceToDevice);
    pd->update_d();
    t.ETD4RK(Het);
    dump_dev(out + "/etd4_1.bin", pd->d(), n * 8);
    fprintf(js, "}\n");
    fclose(js);
    cudaFree(od);
    cudaFree(Het);
    return 0;
}

static int mode_run(int argc, char** argv) {
    if (argc < 15) die("run args");
    const char* workdir = argv[2];
    std::string method = argv[3];
    int nx = atoi(argv[4]), nz = atoi(argv[5]), epssize = atoi(argv[6]);
    double time_step = atof(argv[7]), fixed_dt = atof(argv[8]);
    double M1 = atof(argv[9]), M2 = atof(argv[10]);
    int nsteps = atoi(argv[11]);
    size_t n = (size_t)nx * nx * nz;
    std::vector<double> phi0 = read_raw(argv[12], n);
    std::string out = argv[13];
    int snap_every = atoi(argv[14]);
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) die("getcwd");
    if (out[0] != '/') out = std::string(cwd) + "/" + out;
    stage_workdir(workdir, nx, nz, epssize, time_step, fixed_dt, M1, M2, phi0);

    belastic t(0);
    phasefield* pd = t.m_pd;
    FILE* js = fopen((out + "/steps.jsonl").c_str(), "w");
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);

    if (t.beta <= 0.0) {
        t.alpha = dget(pd->vol());
        t.beta = dget(pd->surface());
    }
    double alpha0 = t.alpha, beta0 = t.beta;
    if (t.fixed_time_step > 0) t.time_step = fmin(t.fixed_time_step, t.time_step);
    double* Het = nullptr;
    double* od;
    cudaMalloc(&od, n * 8);
    double* nld1 = nullptr;
    bool euler = method == "euler";
    if (euler) {
        cudaMalloc(&nld1, n * 8);
        t.get_sum_fgqterm(pd, nld1);
    } else {
        cudaMalloc(&Het, n * 8);
        t.calc->init_fEIF(Het, t.eps);
    }
    auto step_body = [&]() {
        if (method == "etd2") t.ETD2RK(Het);
        else t.ETD4RK(Het);
    };
    double eng0 = t.getstaticenergy(pd), eng1 = eng0;
    int steps = 0, rejects = 0;
    double tcur = 0.0;
    std::string reason = "max_steps";
    auto snap = [&](int s, float ms) {
        double V = dget(pd->vol()), S = dget(pd->surface()), Eel = dget(pd->elastic_eng());
        double E = t.getstaticenergy(pd);
        fprintf(js, "{\"step\": %d, \"dt\": %.17g, \"t\": %.17g, \"V\": %.17g, \"S\": %.17g, \"E_el\": %.17g, \"E\": %.17g, \"alpha\": %.17g, \"beta\": %.17g, \"rejects\": %d, \"ms\": %.6f}\n",
                s, t.time_step, tcur, V, S, Eel, E, t.alpha, t.beta, rejects, ms);
        if (snap_every > 0 && (s % snap_every == 0 || s == nsteps)) {
            char nm[64];
            snprintf(nm, sizeof nm, "/phi_%06d.bin", s);
            dump_dev(out + nm, pd->d(), n * 8);
        }
    };
    snap(0, 0.f);
    while (steps < nsteps) {
        cudaEventRecord(e0);
        if (euler) {
            // belastic.cpp:371-398
            if (t.fixed_time_step <= 0) {
                eng0 = t.getstaticenergy(pd);
                pd->copy_array(od, pd->d());
                if (steps % 4 == 0) t.time_step = t.time_step * 1.4;
                for (;;) {
                    if (t.time_step < 1e-23) break;
                    pd->time_diff_solve_phi(nld1, -t.time_step * t.ga);
                    eng1 = t.getstaticenergy(pd);
                    if (eng1 > eng0) {
                        pd->copy_array(pd->d(), od);
                        pd->update_d();
                        t.time_step /= 2;
                        rejects++;
                        continue;
                    }
                    break;
                }
            } else {
                pd->time_diff_solve_phi(nld1, -t.time_step * t.ga);
            }
        } else {
            // belastic.cpp:639-710
            if (t.fixed_time_step <= 0) {
                eng0 = t.getstaticenergy(pd);
                pd->copy_array(od, pd->d());
                if (steps % 4 == 0) {
                    if (t.time_step * 1.4 < 0.001) t.time_step = t.time_step * 2;
                    else t.time_step = 0.001;
                }
                for (;;) {
                    if (t.time_step < 1e-23) break;
                    step_body();
                    eng1 = t.getstaticenergy(pd);
                    if (eng1 > eng0) {
                        pd->copy_array(pd->d(), od);
                        pd->update_d();
                        t.time_step /= 2;
                        rejects++;
                        continue;
                    }
                    break;
                }
            } else if (t.M1 != 0 || t.M2 != 0) {
                double v, s;
                pd->copy_array(od, pd->d());
                step_body();
                v = dget(pd->vol());
                s = dget(pd->surface());
                t.alpha -= (v - alpha0);
                t.beta -= (s - beta0);
                pd->copy_array(pd->d(), od);
                pd->update_d();
                step_body();
                v = dget(pd->vol());
                s = dget(pd->surface());
                t.alpha -= (v - alpha0);
                t.beta -= (s - beta0);
            } else {
                step_body();
            }
        }
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (t.time_step < 1e-23) { reason = "dt_underflow"; break; }
        double centre;
        cudaMemcpy(&centre, pd->d() + ((size_t)(nz / 2) * nx + nx / 2) * nx + nx / 2, 8, cudaMemcpyDeviceToHost);
        if (!std::isfinite(centre)) { reason = "blowup"; break; }
        tcur += t.time_step;
        steps++;
        if (euler) t.get_sum_fgqterm(pd, nld1);  // belastic.cpp:436
        snap(steps, ms);
    }
    fprintf(js, "{\"end\": \"%s\", \"steps\": %d, \"rejects\": %d}\n", reason.c_str(), steps, rejects);
    fclose(js);
    return 0;
}

static int mode_adjust(int argc, char** argv) {
    if (argc < 8) die("adjust args");
    const char* workdir = argv[2];
    int nx = atoi(argv[3]), nz = atoi(argv[4]), epssize = atoi(argv[5]);
    size_t n = (size_t)nx * nx * nz;
    std::vector<double> phi0 = read_raw(argv[6], n);
    std::string out = argv[7];
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) die("getcwd");
    if (out[0] != '/') out = std::string(cwd) + "/" + out;
    stage_workdir(workdir, nx, nz, epssize, 1e-6, 0.0, 1e4, 1e4, phi0);

    belastic t(0);
    phasefield* pd = t.m_pd;
    const double E0 = t.getstaticenergy(pd, false);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0);
    t.shape_adjust();  // the reference's own loop; its messages go to stdout
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    dump_dev(out + "/phi_adjust.bin", pd->d(), n * 8);
    const double V = dget(pd->vol()), S = dget(pd->surface()), Eel = dget(pd->elastic_eng());
    FILE* js = fopen((out + "/scalars.json").c_str(), "w");
    fprintf(js, "{\"E0\": %.17g, \"E\": %.17g, \"E_el\": %.17g, \"V\": %.17g, \"S\": %.17g, \"dt\": %.17g, \"ms\": %.6f}\n",
            E0, t.getstaticenergy(pd, false), Eel, V, S, t.time_step, ms);
    fclose(js);
    return 0;
}

int main(int argc, char** argv) {
    if (argc < 2) die("mode");
    if (!strcmp(argv[1], "fields")) return mode_fields(argc, argv);
    if (!strcmp(argv[1], "run")) return mode_run(argc, argv);
    if (!strcmp(argv[1], "adjust")) return mode_adjust(argc, argv);
    die("unknown mode");
    return 2;
}
