/*
 * A case driver written against the public C API only, in the shape of the
 * reference's drivers (src/main.c, cavity.c, channel.c): MPI/hypre start-up,
 * IBMSolver_new with the drivers' 16x1x1 decomposition, the variadic
 * set_bc / set_ext_force / set_turb_model calls, an STL obstacle read with
 * fopen_check, assemble, init_flow_const, iterate with the per-step log,
 * export_result.  It links against libibm3d_gb300.so; the tests build and
 * run it and compare what it writes with the CPU oracle.
 *
 *   ibm3d_driver cavity  N STEPS OUT          lid-driven cavity, N^3
 *   ibm3d_driver channel N STEPS OUT          periodic channel, LES
 *   ibm3d_driver sphere  N STEPS OUT STL      body in a uniform stream
 *
 * Writes OUT.nc and OUT.ibm3d (export_result) and OUT_u1.f64, OUT_u2.f64,
 * OUT_u3.f64, OUT_p.f64 (padded (N+4)^3 arrays, read back with the
 * IBMSolver_get_field extension).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "geo3d.h"
#include "ibm3d.h"
#include "ibm3d_gb300.h"
#include "utils.h"

static void faces(double *f, int n, double lo, double hi) {
    for (int i = 0; i <= n; i++) f[i] = lo + (hi - lo) * i / n;
}

static void dump(const char *out, const char *name, IBMSolver *s, int field, size_t n) {
    double *buf = malloc(sizeof(double) * n);
    char path[1024];
    IBMSolver_get_field(s, field, buf);
    snprintf(path, sizeof path, "%s_%s.f64", out, name);
    FILE *fp = fopen_check(path, "wb");
    fwrite(buf, sizeof(double), n, fp);
    fclose(fp);
    free(buf);
}

int main(int argc, char **argv) {
    if (argc < 5) {
        fprintf(stderr, "usage: %s cavity|channel|sphere N STEPS OUT [STL]\n", argv[0]);
        return 2;
    }
    const char *kind = argv[1], *out = argv[4];
    const int N = atoi(argv[2]), steps = atoi(argv[3]);
    const int Nx = N, Ny = N, Nz = N;
    int num_process, rank;

    MPI_Init(&argc, &argv);
    MPI_Comm_size(MPI_COMM_WORLD, &num_process);
    MPI_Comm_rank(MPI_COMM_WORLD, &rank);
    HYPRE_Init();

    IBMSolver *solver = IBMSolver_new(num_process, rank, 16, 1, 1);
    double *xf = malloc(sizeof(double) * (Nx + 1)), *yf = malloc(sizeof(double) * (Ny + 1)),
           *zf = malloc(sizeof(double) * (Nz + 1));
    Polyhedron *poly = NULL;
    double Re, dt, u0 = 0.0;

    if (!strcmp(kind, "cavity")) {
        Re = 400.0, dt = 2e-3;
        faces(xf, Nx, 0, 1), faces(yf, Ny, 0, 1), faces(zf, Nz, 0, 1);
        IBMSolver_set_grid(solver, Nx, Ny, Nz, xf, yf, zf);
        IBMSolver_set_params(solver, Re, dt);
        IBMSolver_set_bc(solver, DIR_UP, BC_VELOCITY_COMPONENT, VAL_CONST, 1., 0., 0.);
        IBMSolver_set_bc(solver, DIR_WEST | DIR_EAST | DIR_SOUTH | DIR_NORTH | DIR_DOWN, BC_STATIONARY_WALL);
        IBMSolver_set_ext_force(solver, VAL_CONST, 0., 0., 0.);
        IBMSolver_set_turb_model(solver, TURBMODEL_NONE);
    } else if (!strcmp(kind, "channel")) {
        Re = 3000.0, dt = 5e-3, u0 = 1.0;
        faces(xf, Nx, 0, 2 * M_PI), faces(zf, Nz, 0, M_PI);
        for (int j = 0; j <= Ny; j++) yf[j] = tanh(2.0 * (2.0 * j / Ny - 1)) / tanh(2.0);
        IBMSolver_set_grid(solver, Nx, Ny, Nz, xf, yf, zf);
        IBMSolver_set_params(solver, Re, dt);
        IBMSolver_set_bc(solver, DIR_WEST | DIR_EAST | DIR_DOWN | DIR_UP, BC_ALL_PERIODIC);
        IBMSolver_set_bc(solver, DIR_SOUTH | DIR_NORTH, BC_STATIONARY_WALL);
        IBMSolver_set_ext_force(solver, VAL_CONST, 2.0 / Re, 0., 0.);
        IBMSolver_set_turb_model(solver, TURBMODEL_SMAGORINSKY, 0.1);
    } else if (!strcmp(kind, "sphere") && argc > 5) {
        Re = 100.0, dt = 1e-2, u0 = 1.0;
        faces(xf, Nx, -1.5, 2.5), faces(yf, Ny, -1.5, 1.5), faces(zf, Nz, -1.5, 1.5);
        IBMSolver_set_grid(solver, Nx, Ny, Nz, xf, yf, zf);
        IBMSolver_set_params(solver, Re, dt);
        IBMSolver_set_bc(solver, DIR_WEST, BC_VELOCITY_COMPONENT, VAL_CONST, 1., 0., 0.);
        IBMSolver_set_bc(solver, DIR_EAST, BC_PRESSURE, VAL_CONST, 0.);
        IBMSolver_set_bc(solver, DIR_NORTH | DIR_SOUTH | DIR_DOWN | DIR_UP, BC_FREE_SLIP_WALL);
        IBMSolver_set_ext_force(solver, VAL_CONST, 0., 0., 0.);
        FILE *fp = fopen_check(argv[5], "rb");
        poly = Polyhedron_new();
        Polyhedron_read_stl(poly, fp);
        fclose(fp);
        if (rank == 0) Polyhedron_print_stats(poly);
    } else {
        fprintf(stderr, "unknown case %s\n", kind);
        return 2;
    }
    IBMSolver_set_obstacle(solver, poly);
    IBMSolver_set_linear_solver(solver, SOLVER_BiCGSTAB, PRECOND_AMG, 1e-12);
    IBMSolver_set_autosave(solver, out, 0);
    IBMSolver_assemble(solver);
    if (poly) Polyhedron_destroy(poly);

    if (rank == 0) {
        printf("\nInput mesh size: %d x %d x %d\n", Nx, Ny, Nz);
        printf("Reynolds no.: %.6lf\ndelta t     : %.6lf\n", Re, dt);
    }
    IBMSolver_init_flow_const(solver, u0, 0., 0., 0.);
    IBMSolver_iterate(solver, steps, true);
    IBMSolver_export_result(solver, out);

    const size_t nc = (size_t)(Nx + 4) * (Ny + 4) * (Nz + 4);
    dump(out, "u1", solver, IBM3D_F_U1, nc);
    dump(out, "u2", solver, IBM3D_F_U2, nc);
    dump(out, "u3", solver, IBM3D_F_U3, nc);
    dump(out, "p", solver, IBM3D_F_P, nc);
    const int status = IBMSolver_last_status(solver);

    IBMSolver_destroy(solver);
    free(xf), free(yf), free(zf);
    HYPRE_Finalize();
    MPI_Finalize();
    return status;
}
