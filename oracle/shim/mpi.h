/*
 * TEST INFRASTRUCTURE ONLY -- single-rank MPI stand-in used to compile the
 * reference's own C sources into the CPU oracle (oracle/_ref). No MPI library
 * exists in this image. Every call behaves as MPI does for a communicator of
 * size 1: reductions and broadcasts are identities, Sendrecv to oneself is a
 * copy, MPI-IO maps to pread/pwrite. Only the subset the reference uses is
 * declared (names and signatures follow the MPI standard).
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H

#include <stddef.h>

typedef int MPI_Comm;
typedef int MPI_Datatype; /* value = element size in bytes */
typedef int MPI_Op;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef long long MPI_Offset;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef struct oracle_mpi_file_s *MPI_File;

#define MPI_COMM_WORLD 0
#define MPI_SUCCESS 0
#define MPI_ERR_FILE 30
#define MPI_MAX_ERROR_STRING 256
#define MPI_INFO_NULL 0
#define MPI_IN_PLACE ((void *)1)
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

#define MPI_BYTE 1
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_C_DOUBLE_COMPLEX 16

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

#define MPI_MODE_RDONLY 2
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1
#define MPI_MODE_APPEND 128

int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm comm, int *size);
int MPI_Comm_rank(MPI_Comm comm, int *rank);
double MPI_Wtime(void);
int MPI_Abort(MPI_Comm comm, int errorcode);
int MPI_Barrier(MPI_Comm comm);
int MPI_Bcast(void *buf, int count, MPI_Datatype type, int root, MPI_Comm comm);
int MPI_Allreduce(const void *sendbuf, void *recvbuf, int count, MPI_Datatype type, MPI_Op op, MPI_Comm comm);
int MPI_Sendrecv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, int dest, int sendtag,
                 void *recvbuf, int recvcount, MPI_Datatype recvtype, int source, int recvtag,
                 MPI_Comm comm, MPI_Status *status);
int MPI_Error_string(int errorcode, char *string, int *resultlen);
int MPI_File_open(MPI_Comm comm, const char *filename, int amode, MPI_Info info, MPI_File *fh);
int MPI_File_close(MPI_File *fh);
int MPI_File_read_at_all(MPI_File fh, MPI_Offset offset, void *buf, int count, MPI_Datatype type, MPI_Status *status);
int MPI_File_write_at_all(MPI_File fh, MPI_Offset offset, const void *buf, int count, MPI_Datatype type, MPI_Status *status);

#endif
