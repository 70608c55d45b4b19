/*
 * ibm3d-gb300 public C ABI: drop-in for the reference solver's public
 * header (src/ibm3d.h:1-221 of thecasterian/2020ResearchProject).
 *
 * Types, enums and enum values are kept exactly as the reference defines
 * them (src/ibm3d.h:14-98) so existing drivers compile unchanged.  The
 * solver struct keeps the reference's field names where they still mean
 * something on one GPU; its layout is not part of the ABI (no reference
 * driver touches the fields), and the device state hangs off `dev`.
 *
 * The whole domain is one subdomain on one GPU: IBMSolver_new accepts the
 * reference's (num_process, rank, Px, Py, Pz) arguments and collapses any
 * decomposition to 1x1x1.
 */
#ifndef IBM3D_H
#define IBM3D_H

#include <stdbool.h>

#include "ibm3d_mpi.h"
#include "geo3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* (x, y, z) => init value.  (src/ibm3d.h:14) */
typedef double (*IBMSolverInitFunc)(double, double, double);

typedef enum _linear_solver_type {
    SOLVER_AMG,
    SOLVER_PCG,
    SOLVER_BiCGSTAB,
    SOLVER_GMRES,
} IBMSolverLinearSolverType;

typedef enum _precond_type {
    PRECOND_NONE,
    PRECOND_AMG,
} IBMSolverPrecondType;

typedef enum _direction {
    DIR_NORTH = 1 << 0,
    DIR_EAST  = 1 << 1,
    DIR_SOUTH = 1 << 2,
    DIR_WEST  = 1 << 3,
    DIR_DOWN  = 1 << 4,
    DIR_UP    = 1 << 5
} IBMSolverDirection;

typedef enum _bc_type {
    BC_VELOCITY_COMPONENT,
    BC_PRESSURE,
    BC_STATIONARY_WALL,
    BC_FREE_SLIP_WALL,
    BC_SYMMETRIC,
    BC_ALL_PERIODIC,
    BC_VELOCITY_PERIODIC,
} IBMSolverBCType;

typedef enum _val_type {
    VAL_CONST,
    VAL_FUNC,
} IBMSolverValType;

/* (t, x, y, z) => boundary value */
typedef double (*IBMSolverBCValFunc)(double, double, double, double);

typedef struct _bc {
    IBMSolverBCType type;
    IBMSolverValType val_type;
    union {
        struct {
            double const_u1, const_u2, const_u3, const_p;
        };
        struct {
            IBMSolverBCValFunc func_u1, func_u2, func_u3, func_p;
        };
    };
} IBMSolverBC;

/* (t, x, y, z) => force value */
typedef double (*IBMSolverForceFunc)(double, double, double, double);

typedef struct _force {
    IBMSolverValType val_type;
    union {
        struct {
            double const_f1, const_f2, const_f3;
        };
        struct {
            IBMSolverForceFunc func_f1, func_f2, func_f3;
        };
    };
} IBMSolverForce;

typedef enum _turb_model_type {
    TURBMODEL_NONE,
    TURBMODEL_SMAGORINSKY,
    TURBMODEL_WALE,
} IBMSolverTurbModelType;

typedef struct _turb_model {
    IBMSolverTurbModelType type;
    double Cs;
} IBMSolverTurbModel;

enum {
    FLAG_FLUID = 1,
    FLAG_GHOST,
    FLAG_SOLID
};

struct ibm3d_device;

typedef struct _ibm_solver {
    /* Decomposition as passed by the caller, and as used (always 1x1x1). */
    int num_process;
    int Px, Py, Pz;
    int rank;
    int ri, rj, rk;

    /* Grid dimensions (global == local on one GPU). */
    int Nx_global, Ny_global, Nz_global;
    int Nx, Ny, Nz;

    double Re;
    double dt;

    int iter;
    double time;

    const char *autosave_filename;
    int autosave_period;

    /* Host copies, reference layout: 1-D arrays of length N+4 indexed i+2. */
    double *dx, *dy, *dz;
    double *xc, *yc, *zc;
    double xmin, xmax, ymin, ymax, zmin, zmax;
    double *kx_W, *kx_E, *ky_S, *ky_N, *kz_D, *kz_U;

    /* Boundary conditions: north, east, south, west, down, up. */
    IBMSolverBC bc[6];

    Polyhedron *poly;

    /* Host mirrors of device fields, padded (N+4)^3 layout, k fastest.
       Valid after IBMSolver_assemble (flag, lvset, p_coeffsum) and after
       IBMSolver_sync_host (u1, u2, u3, p). */
    int *flag;
    double *lvset;
    double *u1, *u2, *u3, *p;
    double *p_coeffsum;

    IBMSolverForce ext_force;
    IBMSolverTurbModel turb_model;

    IBMSolverLinearSolverType linear_solver_type;
    IBMSolverPrecondType precond_type;
    double tol;

    struct ibm3d_device *dev;
} IBMSolver;

#ifdef __cplusplus
}
#endif

#include "ibm3d_setup.h"
#include "ibm3d_init.h"
#include "ibm3d_fracstep.h"
#include "ibm3d_turb.h"
#include "ibm3d_export.h"

#endif
