/*
 * solver_main.c — the `solver` program: the reference's command line
 * (GetCMLArgs, utils.c:34-237), time loop (SpectralSolve, solver.c:50-208),
 * output naming (GetOutputDirPath, hdf5_funcs.c:330-485) and dataset names
 * (hdf5_funcs.c:33-326, 492-779, 1028-1225) on top of the GPU C ABI.
 *
 * libhdf5 is not available, so each HDF5 file of the reference becomes a
 * directory container `<name>.ns3d/` holding one raw little-endian array per
 * dataset under the same group/dataset path (Iter_00000/u_hat.bin, ...) and an
 * index.json with dtype, shape and attributes (TimeValue, TimeStep).
 *
 * Flags of the reference: -o dir (twice: file-only), -n N (x3), -s t0, -e T,
 * -h dt, -c CFL, -v nu, -d ekman (parsed, unused as in the reference), -i IC,
 * -t tag, -p SAVE_EVERY, -f ZERO|NONE|SHELL, -z checkpoint to resume from.
 * Switches that the reference sets at compile time: -I ifrk4|rk4cn,
 * -P fp64|fp32, -H (nu k^4), -a (CFL step), -S seed, -k k0, -E energy,
 * -F force_k, -R (write real-space u), -x (no field output).
 */
#define _GNU_SOURCE
#include <errno.h>
#include <getopt.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <time.h>
#include <unistd.h>

#include "../../include/ns3d.h"

typedef struct {
    char output_dir[512], output_tag[64], input_file[512], u0[64], forcing[64];
    int file_only, N[3], save_every, force_k, hyper, integ, prec, adaptive, real_out, no_fields;
    double t0, T, dt, cfl, nu, ekman, k0, energy;
    unsigned long long seed;
} opts_t;

static void usage_exit(void) {
    fprintf(stderr, "Use -o output dir, -n N (x3), -s t0, -e T, -h dt, -c CFL, -v nu, -i IC, -t tag, -f forcing,\n"
                    "    -p save every, -z checkpoint; -I rk4cn|ifrk4|rk5cn|dp5cn (default rk4cn), -P fp64|fp32,\n"
                    "    -H (nu k^4, default) | -L (nu k^2), -a, -S seed, -k k0,\n"
                    "    -E energy, -F force_k, -R, -x\n"
                    "Example: ./solver -o ../Data/Tmp -n 64 -n 64 -n 64 -s 0.0 -e 1.0 -h 0.001 -v 0.0025 -i TAYLOR_GREEN\n");
    exit(1);
}

/* GetCMLArgs, utils.c:34-237: same defaults, same checks */
static void parse(int argc, char** argv, opts_t* o) {
    memset(o, 0, sizeof(*o));
    strcpy(o->input_file, "NONE");
    strcpy(o->output_dir, "./Data/Tmp/");
    strcpy(o->output_tag, "NO_TAG");
    o->N[0] = o->N[1] = o->N[2] = 64;
    o->t0 = 0.0;
    o->dt = 1e-3;
    o->T = 1.0;
    o->cfl = sqrt(3);
    strcpy(o->u0, "TG_VORT");
    strcpy(o->forcing, "NONE");
    o->nu = 1.0;
    o->save_every = 100;
    o->force_k = 2;
    o->k0 = 4.0;
    o->energy = 1.0;
    /* the reference's default build (Makefile:44, data_types.h:57-71): RK4 +
       Crank-Nicolson with hyperviscosity nu k^4 */
    o->integ = NS3D_RK4CN;
    o->hyper = 1;
    int c, dim = 0, outdir = 0;
    while ((c = getopt(argc, argv, "o:h:n:d:s:e:t:v:i:c:p:f:z:I:P:HLaS:k:E:F:Rx")) != -1) {
        switch (c) {
            case 'o':
                if (outdir == 0) {
                    snprintf(o->output_dir, sizeof(o->output_dir), "%s", optarg);
                    outdir++;
                } else {
                    o->file_only = 1;
                }
                break;
            case 'n':
                if (dim > 2) usage_exit();
                o->N[dim] = atoi(optarg);
                if (o->N[dim] <= 2) {
                    fprintf(stderr, "\n[ERROR] The minimum dimension size of [%d] must be greater than 2\n", o->N[dim]);
                    exit(1);
                } else if (o->N[dim] % 2 != 0) {
                    fprintf(stderr, "\n[ERROR] The system dimension of [%d] must be a multiple of 2\n", o->N[dim]);
                    exit(1);
                }
                dim++;
                break;
            case 's':
                o->t0 = atof(optarg);
                if (o->t0 < 0) { fprintf(stderr, "\n[ERROR] The integration start time must be positive\n"); exit(1); }
                break;
            case 'e':
                o->T = atof(optarg);
                if (o->T < 0 || o->T < o->t0) { fprintf(stderr, "\n[ERROR] Bad end time [%lf]\n", o->T); exit(1); }
                break;
            case 'h':
                o->dt = atof(optarg);
                if (o->dt <= 0) { fprintf(stderr, "\n[ERROR] The timestep must be strictly positive\n"); exit(1); }
                break;
            case 'c':
                o->cfl = atof(optarg);
                if (o->cfl <= 0) { fprintf(stderr, "\n[ERROR] The CFL constant must be strictly positive\n"); exit(1); }
                break;
            case 'v':
                o->nu = atof(optarg);
                if (o->nu <= 0) { fprintf(stderr, "\n[ERROR] The viscosity must be strictly positive\n"); exit(1); }
                break;
            case 'd':
                o->ekman = atof(optarg);
                if (o->ekman <= 0) { fprintf(stderr, "\n[ERROR] The Ekman friction must be strictly positive\n"); exit(1); }
                break;
            case 'i':
                if (!strcmp(optarg, "TAYLOR_GREEN") || !strcmp(optarg, "SHAPIRO") || !strcmp(optarg, "TESTING") ||
                    !strcmp(optarg, "RANDOM") || !strcmp(optarg, "SPECTRUM"))
                    snprintf(o->u0, sizeof(o->u0), "%s", optarg);
                else
                    strcpy(o->u0, "NONE");   /* falls back to random modes (utils.c:181-185) */
                break;
            case 't': snprintf(o->output_tag, sizeof(o->output_tag), "%s", optarg); break;
            case 'p': o->save_every = atoi(optarg); break;
            case 'f':
                if (!strcmp(optarg, "ZERO")) strcpy(o->forcing, "ZERO");
                else if (!strcmp(optarg, "SHELL")) strcpy(o->forcing, "SHELL");
                else strcpy(o->forcing, "NONE");
                break;
            case 'z':
                snprintf(o->input_file, sizeof(o->input_file), "%s", optarg);
                if (access(o->input_file, F_OK) != 0) {
                    fprintf(stderr, "\n[ERROR] The input file [%s] cannot be found\n", o->input_file);
                    exit(1);
                }
                break;
            case 'I':
                o->integ = !strcmp(optarg, "ifrk4")   ? NS3D_IFRK4
                           : !strcmp(optarg, "rk5cn") ? NS3D_RK5CN
                           : !strcmp(optarg, "dp5cn") ? NS3D_DP5CN
                                                      : NS3D_RK4CN;
                break;
            case 'P': o->prec = !strcmp(optarg, "fp32") ? NS3D_FP32 : NS3D_FP64; break;
            case 'H': o->hyper = 1; break;
            case 'L': o->hyper = 0; break;   /* nu k^2: the reference's "solver_test" build */
            case 'a': o->adaptive = 1; break;
            case 'S': o->seed = strtoull(optarg, NULL, 10); break;
            case 'k': o->k0 = atof(optarg); break;
            case 'E': o->energy = atof(optarg); break;
            case 'F': o->force_k = atoi(optarg); break;
            case 'R': o->real_out = 1; break;
            case 'x': o->no_fields = 1; break;
            default: usage_exit();
        }
    }
    if (o->save_every <= 0) o->save_every = 1;
}

static void mkdir_or_die(const char* d) {
    struct stat st;
    if (stat(d, &st) == -1 && mkdir(d, 0700) == -1 && errno != EEXIST) {
        fprintf(stderr, "\n[ERROR] --- Unable to create directory [%s]\n-->> Exiting...\n", d);
        exit(1);
    }
}

/* --------------------------------------------------------------------- */
/* raw + JSON dataset container                                            */
/* --------------------------------------------------------------------- */
typedef struct {
    char dir[1100];
    FILE* index;
    int first;
} container_t;

static void cont_open(container_t* c, const char* path) {
    snprintf(c->dir, sizeof(c->dir), "%s", path);
    mkdir_or_die(c->dir);
    char p[1200];
    snprintf(p, sizeof(p), "%s/index.json", c->dir);
    c->index = fopen(p, "w");
    if (!c->index) { fprintf(stderr, "[ERROR] cannot write %s\n", p); exit(1); }
    fprintf(c->index, "{\"format\": \"ns3d raw little-endian datasets\", \"datasets\": [\n");
    c->first = 1;
}

static void cont_write(container_t* c, const char* group, const char* name, const char* dtype, const void* data,
                       size_t elem, int rank, const long* shape, double tval, double tstep, long iters) {
    char rel[256], p[1400];
    size_t n = 1;
    for (int i = 0; i < rank; ++i) n *= (size_t)shape[i];
    if (group) {
        snprintf(p, sizeof(p), "%s/%s", c->dir, group);
        mkdir_or_die(p);
        snprintf(rel, sizeof(rel), "%s/%s.bin", group, name);
    } else {
        snprintf(rel, sizeof(rel), "%s.bin", name);
    }
    snprintf(p, sizeof(p), "%s/%s", c->dir, rel);
    FILE* f = fopen(p, "wb");
    if (!f || fwrite(data, elem, n, f) != n) { fprintf(stderr, "[ERROR] cannot write %s\n", p); exit(1); }
    fclose(f);
    fprintf(c->index, "%s  {\"path\": \"/%s%s%s\", \"file\": \"%s\", \"dtype\": \"%s\", \"shape\": [", c->first ? "" : ",\n",
            group ? group : "", group ? "/" : "", name, rel, dtype);
    for (int i = 0; i < rank; ++i) fprintf(c->index, "%s%ld", i ? ", " : "", shape[i]);
    fprintf(c->index, "]");
    if (group) fprintf(c->index, ", \"attrs\": {\"TimeValue\": %.17g, \"TimeStep\": %.17g, \"Iter\": %ld}", tval, tstep, iters);
    fprintf(c->index, "}");
    c->first = 0;
}

static void cont_close(container_t* c) {
    if (c->index) {
        fprintf(c->index, "\n]}\n");
        fclose(c->index);
        c->index = NULL;
    }
}

/* --------------------------------------------------------------------- */
/* checkpoint: header + u_hat in the reference layout                      */
/* --------------------------------------------------------------------- */
typedef struct {
    char magic[8];
    int32_t version, N, precision, integrator, visc_pow, forcing;
    double nu, t, dt, force_target, cfl;
    int64_t iters;
} ckpt_header;

static void ckpt_write(const char* path, ns3d_ctx* ctx, const ns3d_params* p, double* u_hat, size_t nd) {
    ckpt_header h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, "NS3DCKPT", 8);
    h.version = 1;
    h.N = p->N;
    h.precision = p->precision;
    h.integrator = p->integrator;
    h.visc_pow = p->visc_pow;
    h.forcing = p->forcing;
    h.nu = p->nu;
    h.cfl = p->cfl;
    long it = 0;
    ns3d_get_time(ctx, &h.t, &h.dt, &it);
    h.iters = it;
    ns3d_get_forcing_target(ctx, &h.force_target);
    ns3d_get_state_host(ctx, u_hat);
    FILE* f = fopen(path, "wb");
    if (!f || fwrite(&h, sizeof(h), 1, f) != 1 || fwrite(u_hat, sizeof(double), nd, f) != nd) {
        fprintf(stderr, "[ERROR] cannot write checkpoint %s\n", path);
        exit(1);
    }
    fclose(f);
}

static void ckpt_read(const char* path, ns3d_ctx* ctx, const ns3d_params* p, double* u_hat, size_t nd) {
    ckpt_header h;
    FILE* f = fopen(path, "rb");
    if (!f || fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, "NS3DCKPT", 8) != 0 || h.N != p->N) {
        fprintf(stderr, "[ERROR] %s is not a checkpoint of an N=%d run\n", path, p->N);
        exit(1);
    }
    if (fread(u_hat, sizeof(double), nd, f) != nd) {
        fprintf(stderr, "[ERROR] truncated checkpoint %s\n", path);
        exit(1);
    }
    fclose(f);
    if (ns3d_set_state_host(ctx, u_hat) != NS3D_OK || ns3d_set_time(ctx, h.t, h.dt, (long)h.iters) != NS3D_OK ||
        ns3d_set_forcing_target(ctx, h.force_target) != NS3D_OK) {
        fprintf(stderr, "[ERROR] cannot restore checkpoint: %s\n", ns3d_last_error(ctx));
        exit(1);
    }
}

static void check(ns3d_ctx* ctx, ns3d_status s, const char* what) {
    if (s != NS3D_OK) {
        fprintf(stderr, "\n[ERROR] --- %s: %s (%s)\n-->> Exiting!!!\n", what, ns3d_status_string(s),
                ctx ? ns3d_last_error(ctx) : "");
        exit(1);
    }
}

/* RecordSystemMeasures + WriteDataToFile (solver.c:1283-1305, hdf5_funcs.c:492-779) */
typedef struct {
    ns3d_ctx* ctx;
    const opts_t* o;
    container_t *cm, *cs;
    double *u_hat, *ureal, *Ek, *Ok, *Ts, *En, *Ens, *Pal, *Hel, *Dis;
    long cap, nsave;
    const long *fshape, *rshape, *sshape;
} rec_t;

static void record(rec_t* r, long it) {
    ns3d_measures m;
    double tt, tdt;
    long ii;
    check(r->ctx, ns3d_get_time(r->ctx, &tt, &tdt, &ii), "ns3d_get_time");
    check(r->ctx, ns3d_measurables(r->ctx, &m, r->Ek, r->Ok), "ComputeSystemMeasurables");
    if (r->nsave < r->cap) {
        r->Ts[r->nsave] = tt;
        r->En[r->nsave] = m.energy;
        r->Ens[r->nsave] = m.enstrophy;
        r->Pal[r->nsave] = m.palinstrophy;
        r->Hel[r->nsave] = m.helicity;
        r->Dis[r->nsave] = m.dissipation;
    }
    char g[32];
    snprintf(g, sizeof(g), "Iter_%05d", (int)it);
    if (!r->o->no_fields) {
        check(r->ctx, ns3d_get_state_host(r->ctx, r->u_hat), "get_state");
        cont_write(r->cm, g, "u_hat", "complex128", r->u_hat, 16, 4, r->fshape, tt, tdt, it);
        if (r->ureal) {
            check(r->ctx, ns3d_real_space_host(r->ctx, r->ureal, NULL), "real_space");
            cont_write(r->cm, g, "u", "float64", r->ureal, 8, 4, r->rshape, tt, tdt, it);
        }
    }
    cont_write(r->cs, g, "EnergySpectrum", "float64", r->Ek, 8, 1, r->sshape, tt, tdt, it);
    cont_write(r->cs, g, "EnstrophySpectrum", "float64", r->Ok, 8, 1, r->sshape, tt, tdt, it);
    printf("Iter: %ld\tt: %1.6lf\tdt: %1.6g\tKE: %1.8e\tENS: %1.8e\tDISS: %1.8e\n", it, tt, tdt, m.energy,
           m.enstrophy, m.dissipation);
    r->nsave++;
}

int main(int argc, char** argv) {
    opts_t o;
    parse(argc, argv, &o);
    struct timespec w0, w1;
    clock_gettime(CLOCK_MONOTONIC, &w0);
    if (o.N[0] != o.N[1] || o.N[0] != o.N[2]) {
        fprintf(stderr, "\n[ERROR] only cubic grids are supported (N = [%d,%d,%d])\n", o.N[0], o.N[1], o.N[2]);
        return 1;
    }
    const int N = o.N[0], NF = N / 2 + 1, ns = ns3d_n_spect(N);
    ns3d_params p;
    memset(&p, 0, sizeof(p));
    p.N = N;
    p.nu = o.nu;
    p.dt = o.dt;
    p.t0 = o.t0;
    p.visc_pow = o.hyper ? 2 : 1;
    p.integrator = o.integ;
    p.precision = o.prec;
    p.cfl = (o.adaptive && o.integ != NS3D_DP5CN) ? o.cfl : 0.0;   /* DP5CN controls its own step */
    p.forcing = !strcmp(o.forcing, "SHELL") ? NS3D_FORCE_SHELL : NS3D_FORCE_NONE;
    p.force_k = o.force_k;
    ns3d_ctx* ctx = NULL;
    check(NULL, ns3d_create(&p, &ctx), "ns3d_create");

    const size_t nd = (size_t)N * N * NF * 3 * 2;
    double* u_hat = (double*)malloc(sizeof(double) * nd);
    if (!u_hat) { fprintf(stderr, "[ERROR] out of host memory\n"); return 1; }
    if (strcmp(o.input_file, "NONE") != 0) {
        ckpt_read(o.input_file, ctx, &p, u_hat, nd);
        printf("Resumed from %s\n", o.input_file);
    } else {
        check(ctx, ns3d_initial_condition(ctx, o.u0, o.seed, o.k0, o.energy), "InitialConditions");
    }

    /* InitializeIntegrationVariables, solver.c:1314-1363 */
    double t = 0, dt = 0;
    long iters0 = 0;
    check(ctx, ns3d_get_time(ctx, &t, &dt, &iters0), "ns3d_get_time");
    const long num_t_steps = (long)((o.T - o.t0) / o.dt);
    const long num_print_steps = (num_t_steps >= o.save_every ? num_t_steps / o.save_every : num_t_steps) + 1;
    printf("Total Iters: %ld\t Saving Iters: %ld\n", num_t_steps, num_print_steps);

    /* GetOutputDirPath, hdf5_funcs.c:330-485 */
    char dir[1024], main_path[1100], spec_path[1100], ckpt_path[1100];
    mkdir_or_die(o.output_dir);
    snprintf(dir, sizeof(dir), "%s", o.output_dir);
    if (dir[strlen(dir) - 1] != '/') strcat(dir, "/");
    /* solver-type tag of GetOutputDirPath (hdf5_funcs.c:372-380) */
    const char* solv = o.integ == NS3D_RK4CN ? "RK4" : o.integ == NS3D_RK5CN ? "RK5" : o.integ == NS3D_DP5CN ? "DP5" : "IFRK4";
    if (o.file_only) {
        char fd[512];
        snprintf(fd, sizeof(fd), "_SIM[NAV-%s-FULL]_N[%d,%d]_T[%d-%d]_NU[%1.10lf]_CFL[%1.2lf]_u0[%s]", solv, N, N,
                 (int)o.t0, (int)o.T, o.nu, o.cfl, o.u0);
        snprintf(main_path, sizeof(main_path), "%sMain_HDF_Data%s.ns3d", dir, fd);
        snprintf(spec_path, sizeof(spec_path), "%sSpectra_HDF_Data%s.ns3d", dir, fd);
        snprintf(ckpt_path, sizeof(ckpt_path), "%sCheckpoint%s.ns3d", dir, fd);
    } else {
        char sub[512];
        snprintf(sub, sizeof(sub), "SIM_DATA_NAVIER_%s_FULL_N[%d,%d]_T[%d-%d]_NU[%1.10lf]_CFL[%1.2lf]_u0[%s]_TAG[%s]/",
                 solv, N, N, (int)o.t0, (int)o.T, o.nu, o.cfl, o.u0, o.output_tag);
        strncat(dir, sub, sizeof(dir) - strlen(dir) - 1);
        mkdir_or_die(dir);
        snprintf(main_path, sizeof(main_path), "%sMain_HDF_Data.ns3d", dir);
        snprintf(spec_path, sizeof(spec_path), "%sSpectra_HDF_Data.ns3d", dir);
        snprintf(ckpt_path, sizeof(ckpt_path), "%sCheckpoint.ns3d", dir);
    }
    printf("\nMain Output File: %s\n\n", main_path);
    container_t cm, cs;
    cont_open(&cm, main_path);
    cont_open(&cs, spec_path);

    /* time series (hdf5_funcs.c:1111-1165) */
    const long cap = num_print_steps + 2;
    double *Ts = calloc(cap, 8), *En = calloc(cap, 8), *Ens = calloc(cap, 8), *Pal = calloc(cap, 8),
           *Hel = calloc(cap, 8), *Dis = calloc(cap, 8), *Ek = calloc(ns, 8), *Ok = calloc(ns, 8);
    double* ureal = o.real_out ? (double*)malloc(sizeof(double) * (size_t)N * N * (N + 2) * 3) : NULL;
    const long fshape[4] = {N, N, NF, 3};
    const long rshape[4] = {N, N, N + 2, 3};
    const long sshape[1] = {ns};

    rec_t R = {ctx, &o, &cm, &cs, u_hat, ureal, Ek, Ok, Ts, En, Ens, Pal, Hel, Dis, cap, 0, fshape, rshape, sshape};
    record(&R, iters0);
    /* the time loop (solver.c:125-194): t = t0 + iters * dt while t <= T */
    long iters = iters0;
    if (p.cfl > 0 || p.integrator == NS3D_DP5CN) {
        for (;;) {
            check(ctx, ns3d_get_time(ctx, &t, &dt, &iters), "ns3d_get_time");
            if (t + dt > o.T + 1e-12 * o.T) break;
            check(ctx, ns3d_step(ctx, 1), p.integrator >= NS3D_RK5CN ? "RK5DPStep" : "RK4Step");
            if ((iters + 1) % o.save_every == 0) record(&R, iters + 1);
        }
    } else {
        long last = iters0;
        while (o.t0 + (double)(last + 1) * o.dt <= o.T) last++;
        while (iters < last) {
            long next = (iters / o.save_every + 1) * o.save_every;
            if (next > last) next = last;
            check(ctx, ns3d_step(ctx, (int)(next - iters)), "RK4Step");
            iters = next;
            if (iters % o.save_every == 0) record(&R, iters);
        }
    }

    /* FinalWriteAndCloseOutputFile, hdf5_funcs.c:1028-1225 */
    int* kk = malloc(sizeof(int) * N);
    double* xx = malloc(sizeof(double) * N);
    for (int i = 0; i < N; ++i) {
        kk[i] = i <= N / 2 ? i : i - N;
        xx[i] = 2.0 * M_PI * i / N;
    }
    const long nsave = R.nsave;
    const long nN[1] = {N}, nF[1] = {NF}, nT[1] = {nsave};
    int* kz = malloc(sizeof(int) * NF);
    for (int i = 0; i < NF; ++i) kz[i] = i;
    cont_write(&cm, NULL, "kx", "int32", kk, 4, 1, nN, 0, 0, 0);
    cont_write(&cm, NULL, "ky", "int32", kk, 4, 1, nN, 0, 0, 0);
    cont_write(&cm, NULL, "kz", "int32", kz, 4, 1, nF, 0, 0, 0);
    cont_write(&cm, NULL, "x", "float64", xx, 8, 1, nN, 0, 0, 0);
    cont_write(&cm, NULL, "y", "float64", xx, 8, 1, nN, 0, 0, 0);
    cont_write(&cm, NULL, "z", "float64", xx, 8, 1, nN, 0, 0, 0);
    cont_write(&cm, NULL, "Time", "float64", Ts, 8, 1, nT, 0, 0, 0);
    cont_write(&cm, NULL, "TotalEnergy", "float64", En, 8, 1, nT, 0, 0, 0);
    cont_write(&cm, NULL, "TotalEnstrophy", "float64", Ens, 8, 1, nT, 0, 0, 0);
    cont_write(&cm, NULL, "TotalPalinstrophy", "float64", Pal, 8, 1, nT, 0, 0, 0);
    cont_write(&cm, NULL, "TotalHelicity", "float64", Hel, 8, 1, nT, 0, 0, 0);
    cont_write(&cm, NULL, "EnergyDissipation", "float64", Dis, 8, 1, nT, 0, 0, 0);
    cont_close(&cm);
    cont_close(&cs);
    ckpt_write(ckpt_path, ctx, &p, u_hat, nd);

    clock_gettime(CLOCK_MONOTONIC, &w1);
    const double spent = (w1.tv_sec - w0.tv_sec) + 1e-9 * (w1.tv_nsec - w0.tv_nsec);
    printf("\n\nTotal Execution Time: [%5.10lf] --> %d hrs : %d mins : %d secs\n\n", spent, (int)spent / 3600,
           ((int)spent % 3600) / 60, (int)spent % 60);
    printf("Checkpoint: %s\n", ckpt_path);
    ns3d_destroy(ctx);
    free(u_hat);
    free(Ts); free(En); free(Ens); free(Pal); free(Hel); free(Dis); free(Ek); free(Ok); free(ureal);
    free(kk); free(xx); free(kz);
    return 0;
}
