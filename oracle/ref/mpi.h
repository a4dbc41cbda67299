/*
 * mpi.h - thread-rank MPI shim. TEST INFRASTRUCTURE (oracle only).
 *
 * Just enough of the MPI C interface to compile and run the reference's own
 * CPU sort path (HykSort / SampleSort / HyperQuickSort with the OpenMP merge
 * sort) in one process: ranks are threads started by shim_run_ranks(),
 * collectives meet at per-communicator barriers and copy from each other's
 * buffers, point-to-point messages go through per-rank mailboxes (sends are
 * buffered, so they complete at once). Written for the oracle build in
 * oracle/ref/Makefile; never linked into the engine.
 */
#ifndef GS_ORACLE_MPI_SHIM_H_
#define GS_ORACLE_MPI_SHIM_H_

#ifdef __cplusplus
extern "C" {
#endif

typedef struct shim_comm* MPI_Comm;
typedef struct shim_group* MPI_Group;
typedef struct shim_type* MPI_Datatype;
typedef struct shim_request* MPI_Request;
typedef int MPI_Op;

typedef struct MPI_Status {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  long long count_bytes;
} MPI_Status;

extern struct shim_type shim_type_char, shim_type_uchar, shim_type_short, shim_type_ushort,
    shim_type_int, shim_type_unsigned, shim_type_long, shim_type_ulong, shim_type_float,
    shim_type_double, shim_type_long_double, shim_type_long_long, shim_type_byte;

#define MPI_CHAR (&shim_type_char)
#define MPI_UNSIGNED_CHAR (&shim_type_uchar)
#define MPI_SHORT (&shim_type_short)
#define MPI_UNSIGNED_SHORT (&shim_type_ushort)
#define MPI_INT (&shim_type_int)
#define MPI_UNSIGNED (&shim_type_unsigned)
#define MPI_LONG (&shim_type_long)
#define MPI_UNSIGNED_LONG (&shim_type_ulong)
#define MPI_FLOAT (&shim_type_float)
#define MPI_DOUBLE (&shim_type_double)
#define MPI_LONG_DOUBLE (&shim_type_long_double)
#define MPI_LONG_LONG_INT (&shim_type_long_long)
#define MPI_BYTE (&shim_type_byte)

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_MAXLOC 4

#define MPI_SUCCESS 0
#define MPI_ERR_BUFFER 1
#define MPI_ERR_COUNT 2
#define MPI_ERR_TYPE 3
#define MPI_ERR_TAG 4
#define MPI_ERR_COMM 5
#define MPI_ERR_RANK 6
#define MPI_ERR_REQUEST 7
#define MPI_ERR_ROOT 8
#define MPI_ERR_OP 9
#define MPI_ERR_ARG 12
#define MPI_ERR_OTHER 15
#define MPI_ERR_INTERN 16
#define MPI_ERR_IN_STATUS 17

#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_COMM_NULL ((MPI_Comm)0)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)

MPI_Comm shim_comm_world(void);
#define MPI_COMM_WORLD (shim_comm_world())

/* Run fn(arg, rank) on `nranks` threads, each one an MPI rank of
 * MPI_COMM_WORLD; returns when all have returned. */
void shim_run_ranks(int nranks, void (*fn)(void* arg, int rank), void* arg);

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Abort(MPI_Comm comm, int code);
int MPI_Comm_rank(MPI_Comm comm, int* rank);
int MPI_Comm_size(MPI_Comm comm, int* size);
int MPI_Comm_split(MPI_Comm comm, int color, int key, MPI_Comm* newcomm);
int MPI_Comm_group(MPI_Comm comm, MPI_Group* group);
int MPI_Group_incl(MPI_Group group, int n, const int* ranks, MPI_Group* newgroup);
int MPI_Comm_create(MPI_Comm comm, MPI_Group group, MPI_Comm* newcomm);
int MPI_Comm_free(MPI_Comm* comm);
int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* newtype);
int MPI_Type_commit(MPI_Datatype* type);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void* buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Gather(const void* sbuf, int scount, MPI_Datatype stype, void* rbuf, int rcount,
               MPI_Datatype rtype, int root, MPI_Comm comm);
int MPI_Allgather(const void* sbuf, int scount, MPI_Datatype stype, void* rbuf, int rcount,
                  MPI_Datatype rtype, MPI_Comm comm);
int MPI_Allgatherv(const void* sbuf, int scount, MPI_Datatype stype, void* rbuf,
                   const int* rcounts, const int* displs, MPI_Datatype rtype, MPI_Comm comm);
int MPI_Allreduce(const void* sbuf, void* rbuf, int count, MPI_Datatype type, MPI_Op op,
                  MPI_Comm comm);
int MPI_Scan(const void* sbuf, void* rbuf, int count, MPI_Datatype type, MPI_Op op,
             MPI_Comm comm);
int MPI_Alltoall(const void* sbuf, int scount, MPI_Datatype stype, void* rbuf, int rcount,
                 MPI_Datatype rtype, MPI_Comm comm);
int MPI_Alltoallv(const void* sbuf, const int* scounts, const int* sdispls, MPI_Datatype stype,
                  void* rbuf, const int* rcounts, const int* rdispls, MPI_Datatype rtype,
                  MPI_Comm comm);
int MPI_Send(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm);
int MPI_Recv(void* buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
             MPI_Status* status);
int MPI_Sendrecv(const void* sbuf, int scount, MPI_Datatype stype, int dest, int stag,
                 void* rbuf, int rcount, MPI_Datatype rtype, int src, int rtag, MPI_Comm comm,
                 MPI_Status* status);
int MPI_Issend(const void* buf, int count, MPI_Datatype type, int dest, int tag, MPI_Comm comm,
               MPI_Request* req);
int MPI_Irecv(void* buf, int count, MPI_Datatype type, int src, int tag, MPI_Comm comm,
              MPI_Request* req);
int MPI_Test(MPI_Request* req, int* flag, MPI_Status* status);
int MPI_Wait(MPI_Request* req, MPI_Status* status);
int MPI_Waitall(int n, MPI_Request* reqs, MPI_Status* statuses);

#ifdef __cplusplus
}
#endif

#endif /* GS_ORACLE_MPI_SHIM_H_ */
