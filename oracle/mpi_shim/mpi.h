/*
 * Single-rank MPI shim: test infrastructure for building the reference
 * PLSQR3 CPU path in a container that has no MPI library.
 *
 * Only the oracle build uses this header.  It declares the subset of MPI-1/2
 * that the reference sources call (collectives, point-to-point, RMA windows,
 * MPI-IO, derived datatypes) with the semantics those calls have when the
 * communicator holds exactly one process:
 *   - Allreduce / Reduce / Bcast / Allgather / Scatterv become copies,
 *   - Barrier, Win_fence and the unused point-to-point calls are no-ops,
 *   - MPI_File_* map to open/pread/pwrite with the datatype extent,
 *   - MPI_Type_struct computes the extent the way MPI does for a struct of
 *     basic types (upper bound rounded up to the largest member alignment).
 */
#ifndef ORACLE_MPI_SHIM_H
#define ORACLE_MPI_SHIM_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_Request;
typedef int MPI_Win;
typedef long long MPI_Offset;
typedef long MPI_Aint;
typedef struct { int fd; int amode; } *MPI_File;

typedef struct {
  int MPI_SOURCE;
  int MPI_TAG;
  int MPI_ERROR;
  long long count_bytes;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_ERR_FILE 27
#define MPI_INFO_NULL 0
#define MPI_PROC_NULL (-2)
#define MPI_ANY_SOURCE (-1)
#define MPI_ANY_TAG (-1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
#define MPI_STATUSES_IGNORE ((MPI_Status *)0)
#define MPI_IN_PLACE ((void *)1)
#define MPI_MAX_ERROR_STRING 256

/* basic datatypes: handle value indexes the shim's datatype table */
#define MPI_CHAR 1
#define MPI_BYTE 2
#define MPI_INT 3
#define MPI_FLOAT 4
#define MPI_DOUBLE 5
#define MPI_LONG_LONG 6
#define MPI_LONG 7
#define MPI_UNSIGNED 8

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

#define MPI_MODE_RDONLY 2
#define MPI_MODE_RDWR 8
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Barrier(MPI_Comm comm);
int MPI_Abort(MPI_Comm comm, int code);
double MPI_Wtime(void);
int MPI_Error_string(int err, char *str, int *len);
int MPI_Error_class(int err, int *cls);

int MPI_Reduce(const void *sbuf, void *rbuf, int count, MPI_Datatype dt,
               MPI_Op op, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sbuf, void *rbuf, int count, MPI_Datatype dt,
                  MPI_Op op, MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype dt, int root, MPI_Comm comm);
int MPI_Allgather(const void *sbuf, int scount, MPI_Datatype sdt, void *rbuf,
                  int rcount, MPI_Datatype rdt, MPI_Comm comm);
int MPI_Scatter(const void *sbuf, int scount, MPI_Datatype sdt, void *rbuf,
                int rcount, MPI_Datatype rdt, int root, MPI_Comm comm);
int MPI_Scatterv(const void *sbuf, const int *scounts, const int *displs,
                 MPI_Datatype sdt, void *rbuf, int rcount, MPI_Datatype rdt,
                 int root, MPI_Comm comm);

int MPI_Send(const void *buf, int count, MPI_Datatype dt, int dest, int tag,
             MPI_Comm comm);
int MPI_Recv(void *buf, int count, MPI_Datatype dt, int src, int tag,
             MPI_Comm comm, MPI_Status *st);
int MPI_Isend(const void *buf, int count, MPI_Datatype dt, int dest, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Irecv(void *buf, int count, MPI_Datatype dt, int src, int tag,
              MPI_Comm comm, MPI_Request *req);
int MPI_Wait(MPI_Request *req, MPI_Status *st);
int MPI_Waitall(int count, MPI_Request *reqs, MPI_Status *sts);

int MPI_Alloc_mem(MPI_Aint size, MPI_Info info, void *baseptr);
int MPI_Free_mem(void *base);
int MPI_Win_create(void *base, MPI_Aint size, int disp_unit, MPI_Info info,
                   MPI_Comm comm, MPI_Win *win);
int MPI_Win_fence(int assert_, MPI_Win win);
int MPI_Win_free(MPI_Win *win);
int MPI_Put(const void *obuf, int ocount, MPI_Datatype odt, int trank,
            MPI_Aint tdisp, int tcount, MPI_Datatype tdt, MPI_Win win);
int MPI_Get(void *obuf, int ocount, MPI_Datatype odt, int trank,
            MPI_Aint tdisp, int tcount, MPI_Datatype tdt, MPI_Win win);

int MPI_Type_extent(MPI_Datatype dt, MPI_Aint *extent);
int MPI_Type_struct(int count, int *blocklens, MPI_Aint *disps,
                    MPI_Datatype *types, MPI_Datatype *newtype);
int MPI_Type_commit(MPI_Datatype *dt);
int MPI_Type_free(MPI_Datatype *dt);

int MPI_File_open(MPI_Comm comm, const char *name, int amode, MPI_Info info,
                  MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_read_at(MPI_File fh, MPI_Offset off, void *buf, int count,
                     MPI_Datatype dt, MPI_Status *st);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int count,
                         MPI_Datatype dt, MPI_Status *st);
int MPI_File_write_at(MPI_File fh, MPI_Offset off, const void *buf, int count,
                      MPI_Datatype dt, MPI_Status *st);
int MPI_File_get_size(MPI_File fh, MPI_Offset *size);
int MPI_File_preallocate(MPI_File fh, MPI_Offset size);
int MPI_File_delete(const char *name, MPI_Info info);

#ifdef __cplusplus
}
#endif
#endif
