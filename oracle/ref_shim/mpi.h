/* Single-process stand-in for the few MPI names the DTCF leaf sources use
 * (communicator type, world communicator, rank and size).  Test
 * infrastructure for building the reference leaves under oracle/_ref only. */
#ifndef ORACLE_REF_SHIM_MPI_H
#define ORACLE_REF_SHIM_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline double MPI_Wtime(void) { return 0.0; }
static inline int MPI_Intercomm_create(MPI_Comm, int, MPI_Comm, int, int, MPI_Comm* c) { *c = 0; return 0; }
#endif
