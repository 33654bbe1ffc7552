/*
 * Single-rank stand-in for the MPI-1 subset that the photoNs-2.0 FMM
 * sources call (src/fmm.c, src/remotes.c, src/toptree.c, src/domains.c).
 *
 * Test infrastructure only: it exists so the reference's own C sources can
 * be compiled unmodified as a one-rank CPU oracle.  With one rank every
 * point-to-point message is a self-send (src/remotes.c:728-746 ships the
 * periodic-image tree to itself), so Isend records the buffer and the
 * matching Recv copies it.  Collectives reduce to copies.
 *
 * A datatype is represented by its size in bytes; MPI_Type_contiguous of
 * N MPI_CHARs therefore yields N, which is how the reference builds its
 * RemoteNode / RemoteBody types (src/initial.c:234-241).
 */
#ifndef ORACLE_MPISTUB_H
#define ORACLE_MPISTUB_H

#include <stddef.h>

typedef int MPI_Comm;
typedef long MPI_Datatype;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef int MPI_Op;

#define MPI_COMM_WORLD 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_SUCCESS 0

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_LONG ((MPI_Datatype)sizeof(long))
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm c, int *size);
int MPI_Comm_rank(MPI_Comm c, int *rank);
int MPI_Comm_dup(MPI_Comm c, MPI_Comm *out);
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out);
int MPI_Type_commit(MPI_Datatype *t);
int MPI_Type_free(MPI_Datatype *t);
int MPI_Barrier(MPI_Comm c);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c, MPI_Request *req);
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st);
int MPI_Wait(MPI_Request *req, MPI_Status *st);
int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, int rcount, MPI_Datatype rt, MPI_Comm c);
int MPI_Alltoall(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, int rcount, MPI_Datatype rt, MPI_Comm c);
int MPI_Alltoallv(const void *sbuf, const int *scounts, const int *sdispls, MPI_Datatype st,
                  void *rbuf, const int *rcounts, const int *rdispls, MPI_Datatype rt, MPI_Comm c);
int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c);

/* Harness hook: called after every completed self-receive with its tag. */
extern void (*oracle_mpi_recv_hook)(int tag, void *buf, int count);

#endif
