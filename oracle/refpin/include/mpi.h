// Single-rank stand-in for the MPI interface the reference calls (TEST INFRASTRUCTURE ONLY).
//
// Lets the reference's unmodified sources compile and run as one process of rank 0 in a
// communicator of size 1: collectives copy their send buffer to the receive buffer, point-to-
// point messages to oneself are queued and matched by (tag), and MPI-IO writes go to a plain
// file at the requested offset.  Implemented in oracle/refpin/refpin_runtime.cpp.
#pragma once
#include <cstddef>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef long long MPI_Offset;
struct MPI_Status { int MPI_SOURCE, MPI_TAG, MPI_ERROR; int count; };
struct refpin_file;
typedef refpin_file* MPI_File;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_CHAR 1
#define MPI_INT 2
#define MPI_DOUBLE 3
#define MPI_LONG 4
#define MPI_UNSIGNED_LONG 5
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_INFO_NULL 0
#define MPI_MODE_RDWR 1
#define MPI_MODE_CREATE 2
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_IN_PLACE ((void*)1)

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize();
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Reduce(const void* sendbuf, void* recvbuf, int count, MPI_Datatype type, MPI_Op op, int root, MPI_Comm comm);
int MPI_Allgather(const void* sendbuf, int scount, MPI_Datatype stype, void* recvbuf, int rcount, MPI_Datatype rtype,
                  MPI_Comm comm);
int MPI_Scatter(const void* sendbuf, int scount, MPI_Datatype stype, void* recvbuf, int rcount, MPI_Datatype rtype,
                int root, MPI_Comm comm);
int MPI_Scatterv(const void* sendbuf, const int* scounts, const int* displs, MPI_Datatype stype, void* recvbuf,
                 int rcount, MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Gatherv(const void* sendbuf, int scount, MPI_Datatype stype, void* recvbuf, const int* rcounts,
                const int* displs, MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Issend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Isend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Bsend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Request* req);
int MPI_Recv(void* buf, int count, MPI_Datatype type, int source, int tag, MPI_Comm comm, MPI_Status* status);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Waitall(int count, MPI_Request* reqs, MPI_Status* statuses);
int MPI_Get_address(const void* location, MPI_Aint* address);
int MPI_Type_create_struct(int count, const int* lens, const MPI_Aint* displs, const MPI_Datatype* types,
                           MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Buffer_attach(void* buf, int size);
int MPI_File_open(MPI_Comm comm, const char* name, int amode, MPI_Info info, MPI_File* fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype etype, MPI_Datatype filetype, const char* rep,
                      MPI_Info info);
int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype type, MPI_Status* status);
int MPI_File_close(MPI_File* fh);
double MPI_Wtime();
