/* Smagorinsky subgrid stress: replaces src/ibm3d_turb.h:6. */
#ifndef IBM3D_TURB_H
#define IBM3D_TURB_H

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/ibm3d_turb.c:8-45: tau_r = -2 l^2 |S| S on fluid cells (GPU). */
void IBMSolver_calc_tau_r(IBMSolver *);

#ifdef __cplusplus
}
#endif

#endif
