/*
 * TEST INFRASTRUCTURE ONLY -- single-rank MPI stand-in (see mpi.h).
 */
#define _GNU_SOURCE
#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include <unistd.h>
#include "mpi.h"

struct oracle_mpi_file_s { int fd; };

int MPI_Init(int *argc, char ***argv) { (void)argc; (void)argv; return MPI_SUCCESS; }
int MPI_Finalize(void) { return MPI_SUCCESS; }
int MPI_Comm_size(MPI_Comm comm, int *size) { (void)comm; *size = 1; return MPI_SUCCESS; }
int MPI_Comm_rank(MPI_Comm comm, int *rank) { (void)comm; *rank = 0; return MPI_SUCCESS; }

double MPI_Wtime(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

int MPI_Abort(MPI_Comm comm, int errorcode) { (void)comm; (void)errorcode; abort(); }
int MPI_Barrier(MPI_Comm comm) { (void)comm; return MPI_SUCCESS; }

int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm) {
  (void)buf; (void)count; (void)type; (void)root; (void)comm;
  return MPI_SUCCESS;
}

int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm) {
  (void)op; (void)comm;
  if (sendbuf != MPI_IN_PLACE) memcpy(recvbuf, sendbuf, (size_t)count * (size_t)type);
  return MPI_SUCCESS;
}

int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status) {
  (void)dest; (void)sendtag; (void)source; (void)recvtag; (void)comm; (void)status; (void)recvtype;
  size_t bytes = (size_t)sendcount * (size_t)sendtype;
  size_t cap = (size_t)recvcount * (size_t)recvtype;
  memmove(recvbuf, sendbuf, bytes < cap ? bytes : cap);
  return MPI_SUCCESS;
}

int MPI_Error_string(int errorcode, char *string, int *resultlen) {
  int n = snprintf(string, MPI_MAX_ERROR_STRING, "single-rank MPI stand-in error %d", errorcode);
  *resultlen = n;
  return MPI_SUCCESS;
}

int MPI_File_open(MPI_Comm comm, const char *filename, int amode, MPI_Info info, MPI_File *fh) {
  (void)comm; (void)info;
  int flags = (amode & MPI_MODE_RDONLY) ? O_RDONLY : O_WRONLY;
  if (amode & MPI_MODE_CREATE) flags |= O_CREAT;
  /* MPI_MODE_APPEND only moves the initial file pointer; explicit-offset
   * writes below address the file directly, so O_APPEND is not used. */
  int fd = open(filename, flags, 0644);
  if (fd < 0) { *fh = NULL; return MPI_ERR_FILE; }
  *fh = (MPI_File)malloc(sizeof(struct oracle_mpi_file_s));
  (*fh)->fd = fd;
  return MPI_SUCCESS;
}

int MPI_File_close(MPI_File *fh) {
  if (*fh) { close((*fh)->fd); free(*fh); *fh = NULL; }
  return MPI_SUCCESS;
}

int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void *buf, int count, MPI_Datatype type, MPI_Status *status) {
  (void)status;
  size_t want = (size_t)count * (size_t)type;
  ssize_t got = pread(fh->fd, buf, want, (off_t)offset);
  return got == (ssize_t)want ? MPI_SUCCESS : MPI_ERR_FILE;
}

int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void *buf, int count, MPI_Datatype type, MPI_Status *status) {
  (void)status;
  size_t want = (size_t)count * (size_t)type;
  ssize_t put = pwrite(fh->fd, buf, want, (off_t)offset);
  return put == (ssize_t)want ? MPI_SUCCESS : MPI_ERR_FILE;
}
