/*
 * Single-rank MPI stand-in (see mpi.h).  Test infrastructure for the
 * reference oracle build only.
 */
#include "mpi.h"
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

void (*oracle_mpi_recv_hook)(int tag, void *buf, int count) = 0;

#define MAX_PENDING 16
static struct { const void *buf; size_t bytes; int tag; int live; } pending[MAX_PENDING];

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return 0; }
int MPI_Finalize(void) { return 0; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return 0; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return 0; }
int MPI_Comm_dup(MPI_Comm c, MPI_Comm *out) { *out = c; return 0; }
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype *out) { *out = (MPI_Datatype)count * old; return 0; }
int MPI_Type_commit(MPI_Datatype *t) { (void)t; return 0; }
int MPI_Type_free(MPI_Datatype *t) { (void)t; return 0; }
int MPI_Barrier(MPI_Comm c) { (void)c; return 0; }
int MPI_Abort(MPI_Comm c, int code) { (void)c; fprintf(stderr, "MPI_Abort(%d)\n", code); exit(code); }

int MPI_Isend(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c, MPI_Request *req)
{
    (void)dest; (void)c;
    for (int i = 0; i < MAX_PENDING; i++) {
        if (!pending[i].live) {
            pending[i].buf = buf;
            pending[i].bytes = (size_t)count * (size_t)t;
            pending[i].tag = tag;
            pending[i].live = 1;
            *req = i;
            return 0;
        }
    }
    fprintf(stderr, "mpistub: too many pending sends\n");
    exit(3);
}

int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st)
{
    (void)src; (void)c; (void)st;
    for (int i = 0; i < MAX_PENDING; i++) {
        if (pending[i].live && pending[i].tag == tag) {
            size_t want = (size_t)count * (size_t)t;
            if (want != pending[i].bytes) {
                fprintf(stderr, "mpistub: size mismatch on tag %d (%zu vs %zu)\n", tag, want, pending[i].bytes);
                exit(3);
            }
            if (want) memmove(buf, pending[i].buf, want);
            pending[i].live = 0;
            if (oracle_mpi_recv_hook) oracle_mpi_recv_hook(tag, buf, count);
            return 0;
        }
    }
    fprintf(stderr, "mpistub: receive on tag %d without a matching self-send\n", tag);
    exit(3);
}

int MPI_Wait(MPI_Request *req, MPI_Status *st) { (void)req; (void)st; return 0; }

int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, int rcount, MPI_Datatype rt, MPI_Comm c)
{
    (void)rcount; (void)rt; (void)c;
    memmove(rbuf, sbuf, (size_t)scount * (size_t)st);
    return 0;
}

int MPI_Alltoall(const void *sbuf, int scount, MPI_Datatype st, void *rbuf, int rcount, MPI_Datatype rt, MPI_Comm c)
{
    (void)rcount; (void)rt; (void)c;
    memmove(rbuf, sbuf, (size_t)scount * (size_t)st);
    return 0;
}

int MPI_Alltoallv(const void *sbuf, const int *scounts, const int *sdispls, MPI_Datatype st,
                  void *rbuf, const int *rcounts, const int *rdispls, MPI_Datatype rt, MPI_Comm c)
{
    (void)rcounts; (void)c;
    memmove((char *)rbuf + (size_t)rdispls[0] * (size_t)rt,
            (const char *)sbuf + (size_t)sdispls[0] * (size_t)st, (size_t)scounts[0] * (size_t)st);
    return 0;
}

int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype t, MPI_Op op, MPI_Comm c)
{
    (void)op; (void)c;
    memmove(rbuf, sbuf, (size_t)count * (size_t)t);
    return 0;
}
