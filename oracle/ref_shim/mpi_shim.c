/* Single-rank MPI stand-in (see mpi.h in this folder).  Test infrastructure
 * for building the reference as the oracle; never linked into the product. */
#include "mpi.h"

#include <stdio.h>
#include <stdlib.h>

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return 0; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return 0; }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return 0; }

int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm)
{
	(void)buf; (void)count; (void)type; (void)root; (void)comm;
	return 0;
}

static int copy_buf(const void *s, int sc, MPI_Datatype st, void *r)
{
	if (s != r && sc > 0) memmove(r, s, (size_t)sc * (size_t)st);
	return 0;
}

int MPI_Gather(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf,
               int rcount, MPI_Datatype rtype, int root, MPI_Comm comm)
{
	(void)rcount; (void)rtype; (void)root; (void)comm;
	return copy_buf(sbuf, scount, stype, rbuf);
}

int MPI_Scatter(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf,
                int rcount, MPI_Datatype rtype, int root, MPI_Comm comm)
{
	(void)rcount; (void)rtype; (void)root; (void)comm;
	return copy_buf(sbuf, scount, stype, rbuf);
}

static int p2p_unreachable(const char *name)
{
	fprintf(stderr, "oracle mpi shim: %s called with a single rank\n", name);
	abort();
}

int MPI_Send(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m)
{ (void)b; (void)c; (void)t; (void)d; (void)g; (void)m; return p2p_unreachable("MPI_Send"); }
int MPI_Recv(void *b, int c, MPI_Datatype t, int s, int g, MPI_Comm m, MPI_Status *st)
{ (void)b; (void)c; (void)t; (void)s; (void)g; (void)m; (void)st; return p2p_unreachable("MPI_Recv"); }
int MPI_Isend(const void *b, int c, MPI_Datatype t, int d, int g, MPI_Comm m, MPI_Request *r)
{ (void)b; (void)c; (void)t; (void)d; (void)g; (void)m; (void)r; return p2p_unreachable("MPI_Isend"); }
int MPI_Irecv(void *b, int c, MPI_Datatype t, int s, int g, MPI_Comm m, MPI_Request *r)
{ (void)b; (void)c; (void)t; (void)s; (void)g; (void)m; (void)r; return p2p_unreachable("MPI_Irecv"); }
int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *stats)
{ (void)reqs; (void)stats; return n == 0 ? 0 : p2p_unreachable("MPI_Waitall"); }
