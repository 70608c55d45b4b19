/*
 * Reference driver: runs the reference solver's own C sources (compiled
 * unmodified from the reference tree against the stand-ins in ref_shim/)
 * through its public API, and dumps raw arrays for the golden fixtures.
 * Test infrastructure only; built into oracle/_ref by oracle/Makefile.
 *
 * Usage: ref_driver <case-file> <out-dir>
 *
 * Case file: whitespace separated "key value..." lines, '#' comments.
 *   grid NX NY NZ                      sizes
 *   xf f0 ... fNX  (and yf, zf)        face coordinates
 *   re RE   dt DT   tol TOL
 *   calls n1 n2 ...                    IBMSolver_iterate(n1), then (n2), ...
 *   bc FACE TYPE [values]              FACE in W E S N D U; TYPE one of
 *                                      vel u v w | press p | wall | slip |
 *                                      sym | per | velper p
 *   force f1 f2 f3
 *   smag CS
 *   stl PATH                           obstacle (omit for none)
 *   init const u v w p | init field    field: smooth analytic field below
 *   init raw DIR                       u1.f64 u2.f64 u3.f64 p.f64 in DIR: padded
 *                                      (N+4)^3 arrays written into the solver
 *                                      after init_flow_const (what the GPU
 *                                      library's IBMSolver_init_flow_array does)
 *   bcfunc FACE TYPE KIND              VAL_FUNC boundary values: TYPE vel
 *                                      (KIND pulse) or press / velper
 *                                      (KIND ramp); functions below
 *   forcefunc KIND                     VAL_FUNC body force (KIND swirl)
 *   export NAME                        after the last call,
 *                                      IBMSolver_export_result(out-dir/NAME)
 *
 * Dumped (little-endian raw, padded (N+4)^3 cell layout, k fastest):
 *   flag.i32 lvset.f64 coeffsum.f64 ghost.txt  after IBMSolver_assemble
 *   u1_0.f64 u2_0.f64 u3_0.f64 p_0.f64          initial fields
 *   after call c=1..: u1_c u2_c u3_c p_c U1_c U2_c U3_c u1star_c u2star_c
 *   u3star_c U1star_c U2star_c U3star_c pprime_c N1_c N2_c N3_c  (.f64;
 *   the *star/pprime/N arrays hold the last step of that call)
 *   calls.txt: call index, steps, hypre stand-in iteration total, time
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ibm3d.h"
#include "geo3d.h"

extern int shim_hypre_total_iterations(void);

static int face_dir(const char *f) {
    switch (f[0]) {
    case 'N': return DIR_NORTH;
    case 'E': return DIR_EAST;
    case 'S': return DIR_SOUTH;
    case 'W': return DIR_WEST;
    case 'D': return DIR_DOWN;
    case 'U': return DIR_UP;
    }
    fprintf(stderr, "bad face %s\n", f);
    exit(2);
}

static void dump(const char *dir, const char *name, const void *p, size_t bytes) {
    char path[1024];
    snprintf(path, sizeof path, "%s/%s", dir, name);
    FILE *f = fopen(path, "wb");
    if (!f) { perror(path); exit(2); }
    fwrite(p, 1, bytes, f);
    fclose(f);
}

/* Smooth, non-trivial initial field used by "init field" cases.  It only has
   to be deterministic: the fixture stores the resulting arrays. */
static double fx_u(double x, double y, double z) { return 0.3 * sin(2.1 * x + 0.4) * cos(1.3 * y) + 0.1 * z; }
static double fx_v(double x, double y, double z) { return 0.2 * cos(1.7 * x) * sin(2.3 * z + 0.2) - 0.05 * y; }
static double fx_w(double x, double y, double z) { return 0.25 * sin(1.1 * y + 0.3) * cos(0.9 * x) + 0.05 * x * z; }
static double fx_p(double x, double y, double z) { return 0.1 * cos(x + 0.5 * y) + 0.05 * z * z; }

/* Time-dependent boundary values and force for the VAL_FUNC cases.  Only
   +, -, * so that the same expressions evaluated elsewhere (the GPU tests'
   callbacks) give the same doubles. */
static double pulse_u(double t, double x, double y, double z) { (void)x; return (1.0 + 3.0 * t) * (1.0 - 0.2 * y * y) * (1.0 - 0.25 * z * z); }
static double pulse_v(double t, double x, double y, double z) { (void)x; (void)y; return 0.2 * t * z; }
static double pulse_w(double t, double x, double y, double z) { (void)z; return -0.1 * t * y + 0.05 * x; }
static double ramp_p(double t, double x, double y, double z) { (void)x; return 0.5 * t + 0.1 * y - 0.05 * z * t; }
static double swirl_f1(double t, double x, double y, double z) { (void)x; (void)z; return 0.02 * (1.0 + t) * y; }
static double swirl_f2(double t, double x, double y, double z) { (void)y; return -0.03 * x * t + 0.01 * z; }
static double swirl_f3(double t, double x, double y, double z) { (void)z; return 0.01 * (x - y) * t; }

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s case-file out-dir\n", argv[0]);
        return 2;
    }
    FILE *cf = fopen(argv[1], "r");
    if (!cf) { perror(argv[1]); return 2; }
    const char *out = argv[2];

    int NX = 0, NY = 0, NZ = 0;
    int calls[64], ncalls = 0;
    double *xf = NULL, *yf = NULL, *zf = NULL;
    double Re = 100, dt = 1e-3, tol = 1e-12, cs = -1;
    double f1 = 0, f2 = 0, f3 = 0;
    char stl[1024] = "";
    int init_field = 0;
    char init_dir[1024] = "";
    char export_name[256] = "";
    double iu = 0, iv = 0, iw = 0, ip = 0;

    struct { int dir, type; double a, b, c; int func; } bcs[16];
    int nbc = 0;
    int force_func = 0;

    char key[64];
    while (fscanf(cf, "%63s", key) == 1) {
        if (key[0] == '#') { int ch; while ((ch = fgetc(cf)) != '\n' && ch != EOF); continue; }
        if (!strcmp(key, "grid")) {
            if (fscanf(cf, "%d %d %d", &NX, &NY, &NZ) != 3) return 2;
        } else if (!strcmp(key, "xf") || !strcmp(key, "yf") || !strcmp(key, "zf")) {
            int n = key[0] == 'x' ? NX : key[0] == 'y' ? NY : NZ;
            double *a = malloc(sizeof(double) * (n + 1));
            for (int i = 0; i <= n; i++) if (fscanf(cf, "%lf", &a[i]) != 1) return 2;
            if (key[0] == 'x') xf = a; else if (key[0] == 'y') yf = a; else zf = a;
        } else if (!strcmp(key, "re")) { if (fscanf(cf, "%lf", &Re) != 1) return 2; }
        else if (!strcmp(key, "dt")) { if (fscanf(cf, "%lf", &dt) != 1) return 2; }
        else if (!strcmp(key, "calls")) {
            int n;
            while (ncalls < 64 && fscanf(cf, "%d", &n) == 1) calls[ncalls++] = n;
        }
        else if (!strcmp(key, "tol")) { if (fscanf(cf, "%lf", &tol) != 1) return 2; }
        else if (!strcmp(key, "force")) { if (fscanf(cf, "%lf %lf %lf", &f1, &f2, &f3) != 3) return 2; }
        else if (!strcmp(key, "smag")) { if (fscanf(cf, "%lf", &cs) != 1) return 2; }
        else if (!strcmp(key, "stl")) { if (fscanf(cf, "%1023s", stl) != 1) return 2; }
        else if (!strcmp(key, "init")) {
            char kind[32];
            if (fscanf(cf, "%31s", kind) != 1) return 2;
            if (!strcmp(kind, "field")) init_field = 1;
            else if (!strcmp(kind, "raw")) { if (fscanf(cf, "%1023s", init_dir) != 1) return 2; }
            else if (fscanf(cf, "%lf %lf %lf %lf", &iu, &iv, &iw, &ip) != 4) return 2;
        } else if (!strcmp(key, "bcfunc")) {
            char face[8], type[16], kind[16];
            if (fscanf(cf, "%7s %15s %15s", face, type, kind) != 3) return 2;
            bcs[nbc].dir = face_dir(face);
            bcs[nbc].a = bcs[nbc].b = bcs[nbc].c = 0;
            bcs[nbc].func = 1;
            if (!strcmp(type, "vel") && !strcmp(kind, "pulse")) bcs[nbc].type = BC_VELOCITY_COMPONENT;
            else if (!strcmp(type, "press") && !strcmp(kind, "ramp")) bcs[nbc].type = BC_PRESSURE;
            else if (!strcmp(type, "velper") && !strcmp(kind, "ramp")) bcs[nbc].type = BC_VELOCITY_PERIODIC;
            else { fprintf(stderr, "bad bcfunc %s %s\n", type, kind); return 2; }
            nbc++;
        } else if (!strcmp(key, "export")) {
            if (fscanf(cf, "%255s", export_name) != 1) return 2;
        } else if (!strcmp(key, "forcefunc")) {
            char kind[16];
            if (fscanf(cf, "%15s", kind) != 1 || strcmp(kind, "swirl")) return 2;
            force_func = 1;
        } else if (!strcmp(key, "bc")) {
            char face[8], type[16];
            if (fscanf(cf, "%7s %15s", face, type) != 2) return 2;
            bcs[nbc].dir = face_dir(face);
            bcs[nbc].a = bcs[nbc].b = bcs[nbc].c = 0;
            bcs[nbc].func = 0;
            if (!strcmp(type, "vel")) {
                bcs[nbc].type = BC_VELOCITY_COMPONENT;
                if (fscanf(cf, "%lf %lf %lf", &bcs[nbc].a, &bcs[nbc].b, &bcs[nbc].c) != 3) return 2;
            } else if (!strcmp(type, "press")) {
                bcs[nbc].type = BC_PRESSURE;
                if (fscanf(cf, "%lf", &bcs[nbc].a) != 1) return 2;
            } else if (!strcmp(type, "velper")) {
                bcs[nbc].type = BC_VELOCITY_PERIODIC;
                if (fscanf(cf, "%lf", &bcs[nbc].a) != 1) return 2;
            } else if (!strcmp(type, "wall")) bcs[nbc].type = BC_STATIONARY_WALL;
            else if (!strcmp(type, "slip")) bcs[nbc].type = BC_FREE_SLIP_WALL;
            else if (!strcmp(type, "sym")) bcs[nbc].type = BC_SYMMETRIC;
            else if (!strcmp(type, "per")) bcs[nbc].type = BC_ALL_PERIODIC;
            else { fprintf(stderr, "bad bc %s\n", type); return 2; }
            nbc++;
        } else {
            fprintf(stderr, "unknown key %s\n", key);
            return 2;
        }
    }
    fclose(cf);

    MPI_Init(&argc, &argv);
    HYPRE_Init();

    IBMSolver *solver = IBMSolver_new(1, 0, 1, 1, 1);
    IBMSolver_set_grid(solver, NX, NY, NZ, xf, yf, zf);
    IBMSolver_set_params(solver, Re, dt);
    if (force_func) IBMSolver_set_ext_force(solver, VAL_FUNC, swirl_f1, swirl_f2, swirl_f3);
    else IBMSolver_set_ext_force(solver, VAL_CONST, f1, f2, f3);
    if (cs >= 0) IBMSolver_set_turb_model(solver, TURBMODEL_SMAGORINSKY, cs);
    for (int b = 0; b < nbc; b++) {
        if (bcs[b].func) {
            if (bcs[b].type == BC_VELOCITY_COMPONENT)
                IBMSolver_set_bc(solver, bcs[b].dir, BC_VELOCITY_COMPONENT, VAL_FUNC, pulse_u, pulse_v, pulse_w);
            else
                IBMSolver_set_bc(solver, bcs[b].dir, bcs[b].type, VAL_FUNC, ramp_p);
            continue;
        }
        switch (bcs[b].type) {
        case BC_VELOCITY_COMPONENT:
            IBMSolver_set_bc(solver, bcs[b].dir, BC_VELOCITY_COMPONENT, VAL_CONST, bcs[b].a, bcs[b].b, bcs[b].c);
            break;
        case BC_PRESSURE:
        case BC_VELOCITY_PERIODIC:
            IBMSolver_set_bc(solver, bcs[b].dir, bcs[b].type, VAL_CONST, bcs[b].a);
            break;
        default:
            IBMSolver_set_bc(solver, bcs[b].dir, bcs[b].type);
        }
    }
    Polyhedron *poly = NULL;
    if (stl[0]) {
        FILE *fp = fopen(stl, "rb");
        if (!fp) { perror(stl); return 2; }
        poly = Polyhedron_new();
        Polyhedron_read_stl(poly, fp);
        fclose(fp);
    }
    IBMSolver_set_obstacle(solver, poly);
    IBMSolver_set_linear_solver(solver, SOLVER_BiCGSTAB, PRECOND_AMG, tol);
    IBMSolver_set_autosave(solver, "unused", 0);
    IBMSolver_assemble(solver);
    if (poly) Polyhedron_destroy(poly);

    const size_t nc = (size_t)(NX + 4) * (NY + 4) * (NZ + 4);
    const size_t nu = (size_t)(NX + 1) * (NY + 4) * (NZ + 4);
    const size_t nv = (size_t)(NX + 4) * (NY + 1) * (NZ + 4);
    const size_t nw = (size_t)(NX + 4) * (NY + 4) * (NZ + 1);

    dump(out, "flag.i32", solver->flag, nc * sizeof(int));
    dump(out, "lvset.f64", solver->lvset, nc * sizeof(double));
    dump(out, "coeffsum.f64", solver->p_coeffsum, nc * sizeof(double));

    /* Ghost-cell interpolation stencils through the public entry point. */
    {
        char path[1024];
        snprintf(path, sizeof path, "%s/ghost.txt", out);
        FILE *g = fopen(path, "w");
        int idx[8][3];
        double coeff[8];
        for (int i = 0; i < NX; i++)
            for (int j = 0; j < NY; j++)
                for (int k = 0; k < NZ; k++) {
                    int f = solver->flag[(NY + 4) * (NZ + 4) * (i + 2) + (NZ + 4) * (j + 2) + k + 2];
                    if (f != FLAG_GHOST) continue;
                    IBMSolver_ghost_interp(solver, i, j, k, idx, coeff);
                    fprintf(g, "%d %d %d", i, j, k);
                    for (int l = 0; l < 8; l++) fprintf(g, " %d %d %d", idx[l][0], idx[l][1], idx[l][2]);
                    for (int l = 0; l < 8; l++) fprintf(g, " %a", coeff[l]);
                    fprintf(g, "\n");
                }
        fclose(g);
    }

    if (init_field) IBMSolver_init_flow_func(solver, fx_u, fx_v, fx_w, fx_p);
    else IBMSolver_init_flow_const(solver, iu, iv, iw, ip);
    if (init_dir[0]) {
        double *dst[4] = {solver->u1, solver->u2, solver->u3, solver->p};
        const char *names[4] = {"u1.f64", "u2.f64", "u3.f64", "p.f64"};
        for (int q = 0; q < 4; q++) {
            char path[1100];
            snprintf(path, sizeof path, "%s/%s", init_dir, names[q]);
            FILE *fp = fopen(path, "rb");
            if (!fp || fread(dst[q], sizeof(double), nc, fp) != nc) { perror(path); return 2; }
            fclose(fp);
        }
    }

    dump(out, "u1_0.f64", solver->u1, nc * sizeof(double));
    dump(out, "u2_0.f64", solver->u2, nc * sizeof(double));
    dump(out, "u3_0.f64", solver->u3, nc * sizeof(double));
    dump(out, "p_0.f64", solver->p, nc * sizeof(double));

    char path[1024];
    snprintf(path, sizeof path, "%s/calls.txt", out);
    FILE *rf = fopen(path, "w");
    for (int s = 1; s <= ncalls; s++) {
        IBMSolver_iterate(solver, calls[s - 1], false);
        char name[64];
#define DUMP(fld, n, tag) do { snprintf(name, sizeof name, "%s_%d.f64", tag, s); \
        dump(out, name, solver->fld, (n) * sizeof(double)); } while (0)
        DUMP(u1, nc, "u1"); DUMP(u2, nc, "u2"); DUMP(u3, nc, "u3"); DUMP(p, nc, "p");
        DUMP(U1, nu, "U1"); DUMP(U2, nv, "U2"); DUMP(U3, nw, "U3");
        DUMP(u1_star, nc, "u1star"); DUMP(u2_star, nc, "u2star"); DUMP(u3_star, nc, "u3star");
        DUMP(U1_star, nu, "U1star"); DUMP(U2_star, nv, "U2star"); DUMP(U3_star, nw, "U3star");
        DUMP(p_prime, nc, "pprime");
        DUMP(N1_prev, nc, "N1"); DUMP(N2_prev, nc, "N2"); DUMP(N3_prev, nc, "N3");
#undef DUMP
        fprintf(rf, "%d %d %d %.17g\n", s, calls[s - 1], shim_hypre_total_iterations(), solver->time);
    }
    fclose(rf);
    if (export_name[0]) {
        snprintf(path, sizeof path, "%s/%s", out, export_name);
        IBMSolver_export_result(solver, path);
    }

    IBMSolver_destroy(solver);
    HYPRE_Finalize();
    MPI_Finalize();
    return 0;
}
