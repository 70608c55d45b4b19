/* Result export: replaces src/ibm3d_export.h:6-9. */
#ifndef IBM3D_EXPORT_H
#define IBM3D_EXPORT_H

#include "ibm3d.h"

#ifdef __cplusplus
extern "C" {
#endif

/* src/ibm3d_export.c:16-253.  libnetcdf is not a dependency here: the
   state (time, iter, u1, u2, u3, p in the padded layout, FP64) is written
   as a raw little-endian file "<name>.ibm3d" that IBMSolver_init_flow_file
   reads back exactly. */
void IBMSolver_export_result(IBMSolver *, const char *);
/* src/ibm3d_export.c:262-435: "<name>.lvset_flag" (lvset f64, flag i32). */
void IBMSolver_export_lvset_flag(IBMSolver *, const char *);
/* src/ibm3d_export.c:437-650: "<name>.intermediate" (u*, U*, p'). */
void IBMSolver_export_intermediate(IBMSolver *, const char *);

#ifdef __cplusplus
}
#endif

#endif
