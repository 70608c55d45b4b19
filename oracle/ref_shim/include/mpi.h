/*
 * Single-rank MPI stand-in used only to compile the reference solver's own
 * C sources on a machine without an MPI installation.  Test infrastructure:
 * it is linked into the reference build under oracle/_ref and nowhere else.
 *
 * With one rank and a 1x1x1 decomposition every point-to-point branch of the
 * reference is dead code (ri == 0 == Px-1 and the Px == 1 periodic copies are
 * taken, src/ibm3d_fracstep.c:950-960), so Send/Recv abort loudly if reached.
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_DOUBLE ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)2)
#define MPI_DOUBLE_INT ((MPI_Datatype)3)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm, MPI_Status *status);

#ifdef __cplusplus
}
#endif

#endif
