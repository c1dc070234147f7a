/*
 * Single-rank stand-in for the MPI API, used only to compile the CPU
 * reference solver (src/tLBM.cpp, src/Problem.cpp, src/TLBM_Partition.cpp)
 * into a test oracle on a machine without an MPI installation.
 *
 * It supports exactly what that solver uses at one rank with an all-zero
 * parts.lbm: the communicator is size 1 / rank 0, point-to-point calls are
 * never reached (no halo neighbours exist) and refuse to run if they are,
 * and MPI-IO maps to open(O_CREAT|O_WRONLY) + pwrite at the byte offset,
 * which keeps MPI_File_write_at's "no truncation" semantics.
 *
 * Test infrastructure only: nothing in the product links this header.
 */
#ifndef TLBM_ORACLE_MPI_STUB_H
#define TLBM_ORACLE_MPI_STUB_H

#include <fcntl.h>
#include <stdio.h>
#include <stdlib.h>
#include <sys/time.h>
#include <unistd.h>

typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Info;
typedef int MPI_Datatype; /* value = element size in bytes */
typedef int MPI_File;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_INFO_NULL 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2
#define MPI_FLOAT ((MPI_Datatype)sizeof(float))
#define MPI_DOUBLE ((MPI_Datatype)sizeof(double))
#define MPI_INT ((MPI_Datatype)sizeof(int))
#define MPI_ANY_TAG (-1)
#define MPI_SUCCESS 0

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline double MPI_Wtime() {
  struct timeval tv;
  gettimeofday(&tv, 0);
  return (double)tv.tv_sec + 1e-6 * (double)tv.tv_usec;
}
static inline int mpi_stub_no_p2p() {
  fprintf(stderr, "mpi stub: point-to-point traffic is not available at one rank\n");
  abort();
  return 1;
}
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) {
  return mpi_stub_no_p2p();
}
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) {
  return mpi_stub_no_p2p();
}
static inline int MPI_Waitall(int n, MPI_Request*, MPI_Status*) {
  return n == 0 ? MPI_SUCCESS : mpi_stub_no_p2p();
}
static inline int MPI_File_open(MPI_Comm, const char* name, int amode, MPI_Info, MPI_File* fh) {
  int flags = O_WRONLY;
  if (amode & MPI_MODE_CREATE) flags |= O_CREAT;
  *fh = open(name, flags, 0644);
  return *fh < 0 ? 1 : MPI_SUCCESS;
}
static inline int MPI_File_write_at(MPI_File fh, long offset, const void* buf, int count,
                                    MPI_Datatype dt, MPI_Status*) {
  size_t bytes = (size_t)count * (size_t)dt;
  ssize_t w = pwrite(fh, buf, bytes, (off_t)offset);
  return (w == (ssize_t)bytes) ? MPI_SUCCESS : 1;
}
static inline int MPI_File_close(MPI_File* fh) {
  close(*fh);
  *fh = -1;
  return MPI_SUCCESS;
}

#endif
