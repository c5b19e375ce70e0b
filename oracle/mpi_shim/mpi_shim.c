/*
 * Single-rank MPI shim (test infrastructure; see mpi.h).
 *
 * With one process every collective is a copy from the send buffer to the
 * receive buffer, every point-to-point call would address a peer that does
 * not exist (the reference never issues one when numProc == 1), and MPI-IO
 * is plain positional file I/O whose offsets are bytes (no file view is ever
 * set by the reference, so the etype is MPI_BYTE).
 */
#define _GNU_SOURCE
#include "mpi.h"

#include <errno.h>
#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>
#include <sys/time.h>
#include <unistd.h>

#define SHIM_MAX_TYPES 256

static MPI_Aint type_extent[SHIM_MAX_TYPES] = {
    0, /* 0: invalid */
    1, /* MPI_CHAR */
    1, /* MPI_BYTE */
    4, /* MPI_INT */
    4, /* MPI_FLOAT */
    8, /* MPI_DOUBLE */
    8, /* MPI_LONG_LONG */
    8, /* MPI_LONG */
    4, /* MPI_UNSIGNED */
};
static MPI_Aint type_align[SHIM_MAX_TYPES] = {0, 1, 1, 4, 4, 8, 8, 8, 4};
static int type_next = 9;

static MPI_Aint extent_of(MPI_Datatype dt) {
  if (dt <= 0 || dt >= type_next) {
    fprintf(stderr, "mpi_shim: invalid datatype handle %d\n", dt);
    abort();
  }
  return type_extent[dt];
}

static void copy_buf(const void *s, void *r, long long count, MPI_Datatype dt) {
  if (s == MPI_IN_PLACE || s == r || count <= 0) return;
  memcpy(r, s, (size_t)(count * extent_of(dt)));
}

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm c, int *size) { (void)c; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm c, int *rank) { (void)c; *rank = 0; return MPI_SUCCESS; }
int MPI_Barrier(MPI_Comm c) { (void)c; return MPI_SUCCESS; }
int MPI_Abort(MPI_Comm c, int code) { (void)c; fflush(stdout); exit(code ? code : 1); }

double MPI_Wtime(void) {
  struct timeval tv;
  gettimeofday(&tv, NULL);
  return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}

int MPI_Error_string(int err, char *str, int *len) {
  int n = snprintf(str, MPI_MAX_ERROR_STRING, "mpi_shim error %d", err);
  if (len) *len = n;
  return MPI_SUCCESS;
}
int MPI_Error_class(int err, int *cls) { *cls = err; return MPI_SUCCESS; }

int MPI_Reduce(const void *s, void *r, int count, MPI_Datatype dt, MPI_Op op,
               int root, MPI_Comm c) {
  (void)op; (void)root; (void)c;
  copy_buf(s, r, count, dt);
  return MPI_SUCCESS;
}
int MPI_Allreduce(const void *s, void *r, int count, MPI_Datatype dt, MPI_Op op,
                  MPI_Comm c) {
  (void)op; (void)c;
  copy_buf(s, r, count, dt);
  return MPI_SUCCESS;
}
int MPI_Bcast(void *b, int count, MPI_Datatype dt, int root, MPI_Comm c) {
  (void)b; (void)count; (void)dt; (void)root; (void)c;
  return MPI_SUCCESS;
}
int MPI_Allgather(const void *s, int sc, MPI_Datatype sdt, void *r, int rc,
                  MPI_Datatype rdt, MPI_Comm c) {
  (void)rc; (void)rdt; (void)c;
  copy_buf(s, r, sc, sdt);
  return MPI_SUCCESS;
}
int MPI_Scatter(const void *s, int sc, MPI_Datatype sdt, void *r, int rc, MPI_Datatype rdt,
                int root, MPI_Comm c) {
  (void)rc; (void)rdt; (void)root; (void)c;
  if (s == MPI_IN_PLACE) return MPI_SUCCESS;
  memcpy(r, s, (size_t)sc * (size_t)extent_of(sdt));
  return MPI_SUCCESS;
}

int MPI_Scatterv(const void *s, const int *scounts, const int *displs,
                 MPI_Datatype sdt, void *r, int rc, MPI_Datatype rdt, int root,
                 MPI_Comm c) {
  (void)rc; (void)rdt; (void)root; (void)c;
  if (s == MPI_IN_PLACE) return MPI_SUCCESS;
  memcpy(r, (const char *)s + (size_t)displs[0] * (size_t)extent_of(sdt),
         (size_t)scounts[0] * (size_t)extent_of(sdt));
  return MPI_SUCCESS;
}

/* No peer exists; the reference guards every send/receive with numProc > 1
 * or with a neighbour list that is empty on one rank.  Reaching one of these
 * means the shim is being used outside its single-rank contract. */
static int no_peer(const char *what) {
  fprintf(stderr, "mpi_shim: %s called with a single rank\n", what);
  return MPI_ERR_OTHER;
}
int MPI_Send(const void *b, int n, MPI_Datatype dt, int d, int t, MPI_Comm c) {
  (void)b; (void)n; (void)dt; (void)t; (void)c;
  return d == MPI_PROC_NULL ? MPI_SUCCESS : no_peer("MPI_Send");
}
int MPI_Recv(void *b, int n, MPI_Datatype dt, int s, int t, MPI_Comm c,
             MPI_Status *st) {
  (void)b; (void)n; (void)dt; (void)t; (void)c; (void)st;
  return s == MPI_PROC_NULL ? MPI_SUCCESS : no_peer("MPI_Recv");
}
int MPI_Isend(const void *b, int n, MPI_Datatype dt, int d, int t, MPI_Comm c,
              MPI_Request *rq) {
  (void)b; (void)n; (void)dt; (void)t; (void)c;
  *rq = 0;
  return d == MPI_PROC_NULL ? MPI_SUCCESS : no_peer("MPI_Isend");
}
int MPI_Irecv(void *b, int n, MPI_Datatype dt, int s, int t, MPI_Comm c,
              MPI_Request *rq) {
  (void)b; (void)n; (void)dt; (void)t; (void)c;
  *rq = 0;
  return s == MPI_PROC_NULL ? MPI_SUCCESS : no_peer("MPI_Irecv");
}
int MPI_Wait(MPI_Request *rq, MPI_Status *st) { (void)rq; (void)st; return MPI_SUCCESS; }
int MPI_Waitall(int n, MPI_Request *rq, MPI_Status *st) {
  (void)n; (void)rq; (void)st;
  return MPI_SUCCESS;
}

int MPI_Alloc_mem(MPI_Aint size, MPI_Info info, void *baseptr) {
  (void)info;
  void *p = malloc(size > 0 ? (size_t)size : 1);
  if (!p) return MPI_ERR_OTHER;
  *(void **)baseptr = p;
  return MPI_SUCCESS;
}
int MPI_Free_mem(void *base) { free(base); return MPI_SUCCESS; }
int MPI_Win_create(void *base, MPI_Aint size, int du, MPI_Info info, MPI_Comm c,
                   MPI_Win *win) {
  (void)base; (void)size; (void)du; (void)info; (void)c;
  *win = 1;
  return MPI_SUCCESS;
}
int MPI_Win_fence(int a, MPI_Win w) { (void)a; (void)w; return MPI_SUCCESS; }
int MPI_Win_free(MPI_Win *w) { *w = 0; return MPI_SUCCESS; }
int MPI_Put(const void *o, int oc, MPI_Datatype odt, int tr, MPI_Aint td,
            int tc, MPI_Datatype tdt, MPI_Win w) {
  (void)o; (void)oc; (void)odt; (void)td; (void)tc; (void)tdt; (void)w;
  return tr == MPI_PROC_NULL ? MPI_SUCCESS : no_peer("MPI_Put");
}
int MPI_Get(void *o, int oc, MPI_Datatype odt, int tr, MPI_Aint td, int tc,
            MPI_Datatype tdt, MPI_Win w) {
  (void)o; (void)oc; (void)odt; (void)td; (void)tc; (void)tdt; (void)w;
  return tr == MPI_PROC_NULL ? MPI_SUCCESS : no_peer("MPI_Get");
}

int MPI_Type_extent(MPI_Datatype dt, MPI_Aint *extent) {
  *extent = extent_of(dt);
  return MPI_SUCCESS;
}
int MPI_Type_struct(int count, int *blocklens, MPI_Aint *disps,
                    MPI_Datatype *types, MPI_Datatype *newtype) {
  MPI_Aint ub = 0, align = 1;
  for (int i = 0; i < count; ++i) {
    MPI_Aint end = disps[i] + (MPI_Aint)blocklens[i] * extent_of(types[i]);
    if (end > ub) ub = end;
    if (type_align[types[i]] > align) align = type_align[types[i]];
  }
  if (type_next >= SHIM_MAX_TYPES) return MPI_ERR_OTHER;
  ub = (ub + align - 1) / align * align;
  type_extent[type_next] = ub;
  type_align[type_next] = align;
  *newtype = type_next++;
  return MPI_SUCCESS;
}
int MPI_Type_commit(MPI_Datatype *dt) { (void)dt; return MPI_SUCCESS; }
int MPI_Type_free(MPI_Datatype *dt) { *dt = 0; return MPI_SUCCESS; }

int MPI_File_open(MPI_Comm c, const char *name, int amode, MPI_Info info,
                  MPI_File *fh) {
  (void)c; (void)info;
  int flags = (amode & MPI_MODE_WRONLY) ? O_WRONLY
              : (amode & MPI_MODE_RDWR) ? O_RDWR : O_RDONLY;
  if (amode & MPI_MODE_CREATE) flags |= O_CREAT;
  int fd = open(name, flags, 0644);
  if (fd < 0) return MPI_ERR_FILE;
  *fh = malloc(sizeof(**fh));
  (*fh)->fd = fd;
  (*fh)->amode = amode;
  return MPI_SUCCESS;
}
int MPI_File_close(MPI_File *fh) {
  if (!fh || !*fh) return MPI_ERR_FILE;
  close((*fh)->fd);
  free(*fh);
  *fh = NULL;
  return MPI_SUCCESS;
}
static int rw_at(MPI_File fh, MPI_Offset off, void *buf, long long count,
                 MPI_Datatype dt, MPI_Status *st, int write) {
  long long want = count * (long long)extent_of(dt), done = 0;
  while (done < want) {
    ssize_t k = write ? pwrite(fh->fd, (char *)buf + done, (size_t)(want - done), off + done)
                      : pread(fh->fd, (char *)buf + done, (size_t)(want - done), off + done);
    if (k < 0) {
      if (errno == EINTR) continue;
      return MPI_ERR_FILE;
    }
    if (k == 0) break; /* end of file: MPI reports a short count, not an error */
    done += k;
  }
  if (st && st != MPI_STATUS_IGNORE) st->count_bytes = done;
  return MPI_SUCCESS;
}
int MPI_File_read_at(MPI_File fh, MPI_Offset off, void *buf, int count,
                     MPI_Datatype dt, MPI_Status *st) {
  return rw_at(fh, off, buf, count, dt, st, 0);
}
int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int count,
                         MPI_Datatype dt, MPI_Status *st) {
  return rw_at(fh, off, buf, count, dt, st, 0);
}
int MPI_File_write_at(MPI_File fh, MPI_Offset off, const void *buf, int count,
                      MPI_Datatype dt, MPI_Status *st) {
  return rw_at(fh, off, (void *)buf, count, dt, st, 1);
}
int MPI_File_get_size(MPI_File fh, MPI_Offset *size) {
  struct stat sb;
  if (fstat(fh->fd, &sb) != 0) return MPI_ERR_FILE;
  *size = (MPI_Offset)sb.st_size;
  return MPI_SUCCESS;
}
int MPI_File_preallocate(MPI_File fh, MPI_Offset size) {
  struct stat sb;
  if (fstat(fh->fd, &sb) != 0) return MPI_ERR_FILE;
  if (sb.st_size < size && ftruncate(fh->fd, size) != 0) return MPI_ERR_FILE;
  return MPI_SUCCESS;
}
int MPI_File_delete(const char *name, MPI_Info info) {
  (void)info;
  return unlink(name) == 0 ? MPI_SUCCESS : MPI_ERR_FILE;
}
