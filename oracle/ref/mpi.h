/*
 * Single-rank stand-in for <mpi.h>, used only to compile the reference
 * mantle-convection code from its own sources as a CPU oracle (test
 * infrastructure; nothing in the product includes this file).
 *
 * With one rank every collective is a copy, and every point-to-point call is
 * a bug: the reference only issues them when a rank has neighbours
 * (G.smpi[lev].nshareip > 0), so they abort loudly instead of returning junk.
 */
#ifndef MCLG_ORACLE_MPI_STUB_H
#define MCLG_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

static inline size_t mclg_stub_type_size(MPI_Datatype t)
{
	return t == MPI_DOUBLE ? sizeof(double) : sizeof(int);
}

static inline void mclg_stub_abort(const char *what)
{
	fprintf(stderr, "mpi stub: %s called on a single rank (unexpected)\n", what);
	abort();
}

static inline int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm c, int *r) { (void)c; *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm c, int *s) { (void)c; *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }

static inline double MPI_Wtime(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
	(void)op; (void)c;
	memmove(r, s, (size_t)n * mclg_stub_type_size(t));
	return 0;
}

static inline int MPI_Allgather(const void *s, int ns, MPI_Datatype ts, void *r, int nr, MPI_Datatype tr, MPI_Comm c)
{
	(void)nr; (void)tr; (void)c;
	memmove(r, s, (size_t)ns * mclg_stub_type_size(ts));
	return 0;
}

static inline int MPI_Allgatherv(const void *s, int ns, MPI_Datatype ts, void *r, const int *nr, const int *displ, MPI_Datatype tr, MPI_Comm c)
{
	(void)nr; (void)c;
	memmove((char *)r + (size_t)displ[0] * mclg_stub_type_size(tr), s, (size_t)ns * mclg_stub_type_size(ts));
	return 0;
}

static inline int MPI_Send(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; mclg_stub_abort("MPI_Send"); return 1; }
static inline int MPI_Recv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)st; mclg_stub_abort("MPI_Recv"); return 1; }
static inline int MPI_Probe(int s, int tag, MPI_Comm c, MPI_Status *st)
{ (void)s; (void)tag; (void)c; (void)st; mclg_stub_abort("MPI_Probe"); return 1; }
static inline int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *n)
{ (void)st; (void)t; (void)n; mclg_stub_abort("MPI_Get_count"); return 1; }
static inline int MPI_Isend(const void *b, int n, MPI_Datatype t, int d, int tag, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)d; (void)tag; (void)c; (void)q; mclg_stub_abort("MPI_Isend"); return 1; }
static inline int MPI_Irecv(void *b, int n, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Request *q)
{ (void)b; (void)n; (void)t; (void)s; (void)tag; (void)c; (void)q; mclg_stub_abort("MPI_Irecv"); return 1; }
static inline int MPI_Waitall(int n, MPI_Request *q, MPI_Status *st)
{
	(void)q; (void)st;
	if (n != 0)
		mclg_stub_abort("MPI_Waitall");
	return 0;
}

#endif
