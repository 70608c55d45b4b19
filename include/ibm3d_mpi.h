/*
 * ibm3d-gb300: single-process stand-ins for the MPI and hypre start-up
 * calls of the reference's case drivers, so that those drivers compile
 * against this library unchanged.  The reference's ibm3d.h pulls these
 * declarations in through HYPRE.h (src/ibm3d.h:6-9), and the drivers call
 * MPI_Init, MPI_Comm_size, MPI_Comm_rank, MPI_Finalize, HYPRE_Init and
 * HYPRE_Finalize (src/main.c:20-25, 178-181; src/cavity.c:39-43, 95-96).
 *
 * One GPU holds the whole domain, so the driver is one process: size 1,
 * rank 0.  A host that runs real MPI (for its own purposes) defines
 * IBM3D_USE_MPI before including ibm3d.h to get <mpi.h> instead; one that
 * links hypre defines IBM3D_USE_HYPRE to get "HYPRE.h".
 */
#ifndef IBM3D_MPI_H
#define IBM3D_MPI_H

#include <stdlib.h>

#ifdef IBM3D_USE_MPI
#include <mpi.h>
#else
typedef int MPI_Comm;
#define MPI_COMM_WORLD ((MPI_Comm)0x44000000)
static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }
static inline int MPI_Abort(MPI_Comm comm, int code) { (void)comm; exit(code & 0xff); return code; }
#endif

#ifdef IBM3D_USE_HYPRE
#include "HYPRE.h"
#else
static inline int HYPRE_Init(void) { return 0; }
static inline int HYPRE_Finalize(void) { return 0; }
#endif

#endif
