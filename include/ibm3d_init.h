/* Flow initialisation: replaces src/ibm3d_init.h:6-8. */
#ifndef IBM3D_INIT_H
#define IBM3D_INIT_H

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/ibm3d_init.c:15-37 */
void IBMSolver_init_flow_const(IBMSolver *, const double u1, const double u2, const double u3, const double p);
/* src/ibm3d_init.c:45-224: reads the state written by IBMSolver_export_result
   (file name without extension). */
void IBMSolver_init_flow_file(IBMSolver *, const char *);
/* src/ibm3d_init.c:237-262: host callbacks sampled at cell centroids. */
void IBMSolver_init_flow_func(IBMSolver *, IBMSolverInitFunc, IBMSolverInitFunc, IBMSolverInitFunc, IBMSolverInitFunc);

#ifdef __cplusplus
}
#endif

#endif
