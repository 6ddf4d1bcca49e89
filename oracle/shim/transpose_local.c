/*
 * TEST INFRASTRUCTURE ONLY -- single-rank replacement for the reference's
 * parallel_transpose (src/parallel/transpose.c:6-85), the one reference file
 * not compiled into the oracle. With one rank the MPI_Alltoallw over hvector
 * datatypes reduces to a local matrix transpose of g_jsize rows by g_isize
 * columns (row-major, x fastest) into g_isize rows by g_jsize columns:
 *   recv[i * g_jsize + j] = send[j * g_isize + i].
 */
#include <string.h>
#include "mpi.h"
#include "parallel.h"

int parallel_transpose(const int g_isize, const int g_jsize, const size_t dtypesize,
                       const MPI_Datatype mpi_dtype, const void *sendbuf, void *recvbuf) {
  (void)mpi_dtype;
  const char *src = (const char *)sendbuf;
  char *dst = (char *)recvbuf;
  for (int i = 0; i < g_isize; i++)
    for (int j = 0; j < g_jsize; j++)
      memcpy(dst + ((size_t)i * g_jsize + j) * dtypesize, src + ((size_t)j * g_isize + i) * dtypesize, dtypesize);
  return 0;
}
