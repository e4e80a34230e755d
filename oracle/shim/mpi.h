/* mpi.h — single-rank stand-in for the MPI calls of the reference's
 * cpu/InitFuncs.cpp and cpu/OutputFuncs.cpp (test infrastructure: lets those
 * files compile where they lie, without an MPI library, for the oracle
 * library oracle/_ref/libsrsref_io.so).
 *
 * One process, rank 0.  MPI_File_* write through stdio: MPI_MODE_APPEND
 * appends; otherwise an existing file is opened without truncation at
 * offset 0, as MPI_File_open does, and a missing one is created.
 * MPI_Abort prints the code and exits the process. */
#ifndef SRS_ORACLE_MPI_SHIM_H
#define SRS_ORACLE_MPI_SHIM_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Info;
typedef int MPI_Datatype;
typedef FILE* MPI_File;
typedef struct {
  int count;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_COMM_SELF 1
#define MPI_INFO_NULL 0
#define MPI_SUCCESS 0
#define MPI_ERR_OTHER 15
#define MPI_CHAR 1
#define MPI_FLOAT 2
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_MODE_APPEND 128
#define MPI_MAX_ERROR_STRING 256

static inline int MPI_Abort(MPI_Comm, int code) {
  fprintf(stderr, "MPI_Abort(%d) from the single-rank MPI stand-in\n", code);
  exit(code ? code : 1);
  return code;
}

static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }

static inline int MPI_Error_string(int code, char* s, int* len) {
  *len = snprintf(s, MPI_MAX_ERROR_STRING, "MPI stand-in error %d", code);
  return MPI_SUCCESS;
}

static inline int MPI_File_open(MPI_Comm, const char* name, int amode, MPI_Info, MPI_File* fh) {
  FILE* f = NULL;
  if (amode & MPI_MODE_APPEND) {
    f = fopen(name, "ab");
  } else {
    f = fopen(name, "r+b");
    if (!f && (amode & MPI_MODE_CREATE)) f = fopen(name, "wb");
  }
  *fh = f;
  return f ? MPI_SUCCESS : MPI_ERR_OTHER;
}

static inline int MPI_File_write(MPI_File fh, const void* buf, int count, MPI_Datatype type,
                                 MPI_Status* st) {
  size_t size = type == MPI_FLOAT ? sizeof(float) : 1;
  size_t n = fwrite(buf, size, (size_t)count, fh);
  if (st) st->count = (int)n;
  return n == (size_t)count ? MPI_SUCCESS : MPI_ERR_OTHER;
}

static inline int MPI_File_close(MPI_File* fh) {
  int rc = (*fh && fclose(*fh) == 0) ? MPI_SUCCESS : MPI_ERR_OTHER;
  *fh = NULL;
  return rc;
}

static inline int MPI_File_delete(const char* name, MPI_Info) {
  return remove(name) == 0 ? MPI_SUCCESS : MPI_ERR_OTHER;
}

#endif
