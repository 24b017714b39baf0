/*
 * Single-process MPI stand-in used ONLY to compile the reference's own
 * FP64 sources (Palabos + src/fsi) as a test oracle.  It is test
 * infrastructure, not part of the product.
 *
 * The reference's fsi module calls MPI directly (src/fsi/CommunicationBuffer.hh:44-103,
 * src/fsi/ImmersedBoundaryDynamics.hh:553,566) and therefore has to be built with
 * PLB_MPI_PARALLEL; no MPI library exists in this image.  With one rank every
 * collective is a copy, every broadcast a no-op and point-to-point messages go to a
 * tag-matched mailbox of the single rank.  MPI-IO is reported as unsupported.
 */
#ifndef BIB_ORACLE_MPI_SHIM_H
#define BIB_ORACLE_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; int count; } MPI_Status;
typedef struct bib_mpi_file* MPI_File;

#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_INFO_NULL 0
#define MPI_REQUEST_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_SEEK_SET 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2
#define MPI_MODE_RDONLY 4

/* datatypes carry their size in bytes */
#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_BYTE ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_LONG ((MPI_Datatype)(0x100 | sizeof(long)))
#define MPI_LONG_LONG ((MPI_Datatype)(0x200 | sizeof(long long)))
#define MPI_UNSIGNED_LONG_LONG ((MPI_Datatype)(0x300 | sizeof(unsigned long long)))
#define MPI_FLOAT ((MPI_Datatype)(0x400 | sizeof(float)))
#define MPI_DOUBLE ((MPI_Datatype)(0x500 | sizeof(double)))
#define MPI_LONG_DOUBLE ((MPI_Datatype)(0x600 | sizeof(long double)))

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_LAND 4
#define MPI_PROD 5

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Initialized(int* flag);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);

int MPI_Send(void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Rsend(void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Isend(void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Recv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Sendrecv(void* sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status* status);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);
int MPI_Request_free(MPI_Request* req);
int MPI_Get_count(MPI_Status* status, MPI_Datatype type, int* count);

int MPI_Reduce(void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Scatterv(void* sendbuf, int* sendcounts, int* displs, MPI_Datatype sendtype,
                 void* recvbuf, int recvcount, MPI_Datatype recvtype, int root, MPI_Comm comm);
int MPI_Gatherv(void* sendbuf, int sendcount, MPI_Datatype sendtype,
                void* recvbuf, int* recvcounts, int* displs, MPI_Datatype recvtype, int root, MPI_Comm comm);

int MPI_File_open(MPI_Comm comm, char* name, int mode, MPI_Info info, MPI_File* fh);
int MPI_File_close(MPI_File* fh);
int MPI_File_seek(MPI_File fh, MPI_Offset offset, int whence);
int MPI_File_write(MPI_File fh, void* buf, int count, MPI_Datatype type, MPI_Status* status);
int MPI_File_read(MPI_File fh, void* buf, int count, MPI_Datatype type, MPI_Status* status);

#ifdef __cplusplus
}
#endif
#endif
