/*
 * Single-rank loopback MPI, just enough to compile and run the reference
 * solver's particle path (particle.cpp, tensor0.cpp, tensor1.cpp,
 * communicator.cpp, gridsize.cpp, proc.cpp, params.cpp) in one process.
 *
 * Test infrastructure only: it exists so that oracle/_ref can be built from
 * the reference sources and used as the checker. Nothing in the product
 * links it.
 *
 * Semantics on one rank (every neighbour is this rank):
 *  - MPI_Isend snapshots the message (tag, bytes) into a FIFO;
 *  - MPI_Irecv records (tag, destination, capacity);
 *  - MPI_Waitall delivers each pending receive from the oldest queued send
 *    with the same tag. The reference posts Irecv before it fills the send
 *    buffer (particle.cpp:751-755), so matching happens at Waitall time.
 *  - reductions, broadcasts, gathers and scatters are copies.
 *  - MPI-IO is plain stdio on the one file: open (MPI_MODE_EXCL refuses an existing
 *    file), read/write at a byte offset, close; the views and collectives reduce to
 *    that on one rank.
 */
#ifndef PSTEP_ORACLE_MPI_STUB_H
#define PSTEP_ORACLE_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Group;
typedef int MPI_Info;
typedef int MPI_Request;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef FILE *MPI_File;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_INFO_NULL 0
#define MPI_ANY_SOURCE (-1)
#define MPI_ORDER_C 0
#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_MODE_EXCL 64
#define MPI_MODE_APPEND 128
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

#ifdef __cplusplus
extern "C" {
#endif

static inline size_t mpistub_size(MPI_Datatype t) { return t == MPI_DOUBLE ? sizeof(double) : sizeof(int); }

enum { MPISTUB_MAXQ = 64 };
typedef struct { int used, tag; long seq; size_t bytes; char *data; } mpistub_msg;
typedef struct { int used, is_recv, tag; size_t cap; void *dst; } mpistub_req;
static mpistub_msg mpistub_q[MPISTUB_MAXQ];
static mpistub_req mpistub_r[MPISTUB_MAXQ];
static long mpistub_seq = 0;

static inline void mpistub_fail(const char *what) {
  fprintf(stderr, "mpi stub: %s\n", what);
  abort();
}

static inline int mpistub_new_req(int is_recv, int tag, size_t cap, void *dst) {
  for (int i = 0; i < MPISTUB_MAXQ; ++i)
    if (!mpistub_r[i].used) {
      mpistub_r[i].used = 1; mpistub_r[i].is_recv = is_recv; mpistub_r[i].tag = tag;
      mpistub_r[i].cap = cap; mpistub_r[i].dst = dst;
      return i;
    }
  mpistub_fail("request table full");
  return -1;
}

static inline int MPI_Init(int *, char ***) { return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Comm_group(MPI_Comm, MPI_Group *g) { *g = 1; return 0; }
static inline int MPI_Group_incl(MPI_Group, int, const int *, MPI_Group *g) { *g = 1; return 0; }
static inline int MPI_Comm_create(MPI_Comm, MPI_Group, MPI_Comm *c) { *c = MPI_COMM_WORLD; return 0; }
static inline int MPI_Comm_free(MPI_Comm *) { return 0; }
static inline int MPI_Group_free(MPI_Group *) { return 0; }
static inline int MPI_Type_create_subarray(int, const int *, const int *, const int *, int, MPI_Datatype,
                                           MPI_Datatype *t) { *t = 100; return 0; }
static inline int MPI_Type_commit(MPI_Datatype *) { return 0; }
static inline int MPI_Type_free(MPI_Datatype *) { return 0; }

static inline int MPI_Isend(const void *buf, int count, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  size_t bytes = (size_t)count * mpistub_size(t);
  for (int i = 0; i < MPISTUB_MAXQ; ++i)
    if (!mpistub_q[i].used) {
      mpistub_q[i].used = 1; mpistub_q[i].tag = tag; mpistub_q[i].bytes = bytes; mpistub_q[i].seq = mpistub_seq++;
      mpistub_q[i].data = (char *)malloc(bytes ? bytes : 1);
      if (bytes) memcpy(mpistub_q[i].data, buf, bytes);
      *req = mpistub_new_req(0, tag, 0, 0);
      return 0;
    }
  mpistub_fail("send queue full");
  return 1;
}

static inline int MPI_Irecv(void *buf, int count, MPI_Datatype t, int, int tag, MPI_Comm, MPI_Request *req) {
  *req = mpistub_new_req(1, tag, (size_t)(count < 0 ? 0 : count) * mpistub_size(t), buf);
  return 0;
}

static inline void mpistub_complete(MPI_Request r) {
  mpistub_req *q = &mpistub_r[r];
  if (!q->used) return;
  if (q->is_recv) {
    int best = -1;
    for (int i = 0; i < MPISTUB_MAXQ; ++i)  /* FIFO per tag: the oldest queued send */
      if (mpistub_q[i].used && mpistub_q[i].tag == q->tag && (best < 0 || mpistub_q[i].seq < mpistub_q[best].seq)) best = i;
    if (best < 0) mpistub_fail("receive with no matching send (would deadlock)");
    if (mpistub_q[best].bytes > q->cap) mpistub_fail("message larger than receive buffer");
    if (mpistub_q[best].bytes) memcpy(q->dst, mpistub_q[best].data, mpistub_q[best].bytes);
    free(mpistub_q[best].data);
    mpistub_q[best].used = 0;
  }
  q->used = 0;
}

static inline int MPI_Waitall(int n, MPI_Request *reqs, MPI_Status *) {
  for (int i = 0; i < n; ++i) mpistub_complete(reqs[i]);
  return 0;
}
static inline int MPI_Send(const void *buf, int count, MPI_Datatype t, int d, int tag, MPI_Comm c) {
  MPI_Request r; return MPI_Isend(buf, count, t, d, tag, c, &r);
}
static inline int MPI_Recv(void *buf, int count, MPI_Datatype t, int s, int tag, MPI_Comm c, MPI_Status *) {
  MPI_Request r; MPI_Irecv(buf, count, t, s, tag, c, &r); mpistub_complete(r); return 0;
}

static inline int MPI_Reduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
  memmove(r, s, (size_t)n * mpistub_size(t)); return 0;
}
static inline int MPI_Allreduce(const void *s, void *r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
  memmove(r, s, (size_t)n * mpistub_size(t)); return 0;
}
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Gather(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm) {
  memmove(r, s, (size_t)n * mpistub_size(t)); return 0;
}
static inline int MPI_Scatter(const void *s, int n, MPI_Datatype t, void *r, int, MPI_Datatype, int, MPI_Comm) {
  memmove(r, s, (size_t)n * mpistub_size(t)); return 0;
}

static inline int MPI_File_open(MPI_Comm, const char *name, int amode, MPI_Info, MPI_File *fh) {
  const char *mode = (amode & MPI_MODE_RDONLY) ? "rb" : ((amode & MPI_MODE_EXCL) ? "wbx" : "wb");
  *fh = fopen(name, mode);
  return *fh ? MPI_SUCCESS : 1;
}
static inline int MPI_File_close(MPI_File *fh) {
  if (*fh) fclose(*fh);
  *fh = NULL;
  return MPI_SUCCESS;
}
static inline int MPI_File_set_view(MPI_File, MPI_Offset, MPI_Datatype, MPI_Datatype, const char *, MPI_Info) { mpistub_fail("MPI-IO views"); return 1; }
static inline int MPI_File_read_all(MPI_File, void *, int, MPI_Datatype, MPI_Status *) { mpistub_fail("MPI-IO read_all"); return 1; }
static inline int MPI_File_write_all(MPI_File, const void *, int, MPI_Datatype, MPI_Status *) { mpistub_fail("MPI-IO write_all"); return 1; }
static inline int MPI_File_read_at_all(MPI_File fh, MPI_Offset off, void *buf, int n, MPI_Datatype t, MPI_Status *) {
  if (!fh) mpistub_fail("read from a file that did not open");
  if (fseek(fh, (long)off, SEEK_SET) != 0) return 1;
  return fread(buf, mpistub_size(t), (size_t)n, fh) == (size_t)n ? MPI_SUCCESS : 1;
}
static inline int MPI_File_write_at_all(MPI_File fh, MPI_Offset off, const void *buf, int n, MPI_Datatype t, MPI_Status *) {
  if (!fh) mpistub_fail("write to a file that did not open");
  if (fseek(fh, (long)off, SEEK_SET) != 0) return 1;
  return fwrite(buf, mpistub_size(t), (size_t)n, fh) == (size_t)n ? MPI_SUCCESS : 1;
}
static inline int MPI_File_get_size(MPI_File, MPI_Offset *) { mpistub_fail("MPI-IO"); return 1; }

#ifdef __cplusplus
}
#endif
#endif
