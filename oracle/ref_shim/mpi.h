/* Single-rank stand-in for <mpi.h>, written for this project.
 *
 * Test infrastructure only: it lets the reference's own C++ sources be compiled
 * as the oracle on a machine without MPI.  Semantics are those of a world of
 * size 1: rank 0, broadcasts and barriers do nothing, gathers and scatters copy
 * the send buffer into the receive buffer.  Point-to-point calls are never
 * reached with one rank (every particle is local); they report an error.
 *
 * Symbols follow the MPI-3 standard names used by the reference
 * (src/mpi.cc:15-16,142-158,397-472,545-573,635-646,916-939).
 */
#ifndef BEEP_ORACLE_MPI_SHIM_H
#define BEEP_ORACLE_MPI_SHIM_H

#include <stddef.h>
#include <string.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int source, tag, error; } MPI_Status;
typedef int MPI_Request;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

/* The datatype value is the element size in bytes. */
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_UNSIGNED ((MPI_Datatype)sizeof(unsigned int))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_CXX_BOOL ((MPI_Datatype)sizeof(bool))
#define MPI_INT ((MPI_Datatype)sizeof(int))

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Gather(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf,
               int rcount, MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Scatter(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf,
                int rcount, MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Send(const void *buf, int count, MPI_Datatype type, int dest, int tag,
             MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype type, int src, int tag,
             MPI_Comm comm, MPI_Status *st);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *stats);

#ifdef __cplusplus
}
#endif

#endif
