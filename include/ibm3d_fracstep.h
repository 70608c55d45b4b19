/* Time stepping: replaces src/ibm3d_fracstep.h:6. */
#ifndef IBM3D_FRACSTEP_H
#define IBM3D_FRACSTEP_H

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/ibm3d_fracstep.c:38-115: advances num_time_steps fractional steps on
   the GPU; with verbose, prints the reference's per-step table. */
void IBMSolver_iterate(IBMSolver *, int num_time_steps, bool verbose);

#ifdef __cplusplus
}
#endif

#endif
