/* Solver construction and assembly: replaces src/ibm3d_setup.h:6-31. */
#ifndef IBM3D_SETUP_H
#define IBM3D_SETUP_H

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/ibm3d_setup.c:48-104.  Any Px*Py*Pz is accepted; one GPU holds the
   whole domain, so the decomposition collapses to 1x1x1. */
IBMSolver *IBMSolver_new(const int num_process, const int rank, const int Px, const int Py, const int Pz);
/* src/ibm3d_setup.c:111-187: frees host and device memory. */
void IBMSolver_destroy(IBMSolver *);

/* src/ibm3d_setup.c:203-284: copies xf/yf/zf (Nx+1, Ny+1, Nz+1 faces). */
void IBMSolver_set_grid(
    IBMSolver *,
    const int Nx_global, const int Ny_global, const int Nz_global,
    const double *xf, const double *yf, const double *zf
);
/* src/ibm3d_setup.c:294-297 */
void IBMSolver_set_params(IBMSolver *, const double Re, const double dt);
/* src/ibm3d_setup.c:306-327: VAL_CONST, f1, f2, f3 | VAL_FUNC, func1..3 */
void IBMSolver_set_ext_force(IBMSolver *, IBMSolverValType, ...);
/* src/ibm3d_setup.c:336-356: TURBMODEL_NONE | TURBMODEL_SMAGORINSKY, Cs */
void IBMSolver_set_turb_model(IBMSolver *, IBMSolverTurbModelType, ...);
/* src/ibm3d_setup.c:367-439: same variadic conventions; STATIONARY_WALL
   becomes a zero velocity BC and SYMMETRIC becomes a free-slip wall. */
void IBMSolver_set_bc(IBMSolver *, IBMSolverDirection, IBMSolverBCType, ...);
/* src/ibm3d_setup.c:448-450: borrowed until IBMSolver_assemble returns. */
void IBMSolver_set_obstacle(IBMSolver *, Polyhedron *);
/* src/ibm3d_setup.c:461-470 */
void IBMSolver_set_linear_solver(IBMSolver *, IBMSolverLinearSolverType, IBMSolverPrecondType, const double tol);
/* src/ibm3d_setup.c:484-491: filename is borrowed for the solver lifetime. */
void IBMSolver_set_autosave(IBMSolver *, const char *, int);

/* src/ibm3d_setup.c:499-639: ghost widths, Crank-Nicolson coefficients,
   level set and flags, ghost-cell stencils and the pressure multigrid
   hierarchy, all built on the GPU. */
void IBMSolver_assemble(IBMSolver *);

/* src/utils.c:111-171: the 8-point trilinear mirror-point stencil of cell
   (i, j, k), evaluated on the host from the assembled level set. */
void IBMSolver_ghost_interp(
    IBMSolver *,
    const int i, const int j, const int k,
    int interp_idx[][3], double interp_coeff[]
);

#ifdef __cplusplus
}
#endif

#endif
