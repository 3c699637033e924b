/*
 * Single-rank MPI stand-in used ONLY to compile the reference's own C sources
 * into the CPU oracle (oracle/_ref).  It is test infrastructure, never linked
 * into the product library.
 *
 * With one rank every collective is a copy from the send buffer to the receive
 * buffer, and point-to-point messages can only go to self (periodic meshes on
 * one rank send their ghost layers to themselves, src/meshcore_iga.c:152-192).
 * Self messages are matched FIFO by tag, as MPI's non-overtaking rule requires.
 */
#ifndef IGAP_ORACLE_STUB_MPI_H
#define IGAP_ORACLE_STUB_MPI_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Scatter(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount,
                MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Scatterv(const void *sbuf, const int *scounts, const int *displs, MPI_Datatype stype,
                 void *rbuf, int rcount, MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Gather(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, int rcount,
               MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Gatherv(const void *sbuf, int scount, MPI_Datatype stype, void *rbuf, const int *rcounts,
                const int *displs, MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Isend(const void *buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
              MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *status);
int MPI_Barrier(MPI_Comm comm);

#ifdef __cplusplus
}
#endif
#endif
