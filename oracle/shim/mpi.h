/*
 * TEST INFRASTRUCTURE ONLY. Single-rank stand-in for the MPI calls made by the
 * reference STZ code (the reference needs an MPI library that is not installed
 * here). One process, rank 0 of 1: collectives copy, point-to-point calls
 * are no-ops, MPI-IO writes a plain file.
 */
#ifndef STZ_SHIM_MPI_H
#define STZ_SHIM_MPI_H
#include <stdio.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
typedef FILE* MPI_File;
typedef long long MPI_Offset;

#define MPI_COMM_WORLD 0
#define MPI_INT 1
#define MPI_DOUBLE 2
#define MPI_FLOAT 3
#define MPI_SUM 0
#define MPI_INFO_NULL 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 2

int MPI_Init(int* argc, char*** argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm c, int* size);
int MPI_Comm_rank(MPI_Comm c, int* rank);
int MPI_Barrier(MPI_Comm c);
int MPI_Allreduce(const void* in, void* out, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Send(const void* buf, int n, MPI_Datatype t, int dest, int tag, MPI_Comm c);
int MPI_Recv(void* buf, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status* st);
int MPI_Abort(MPI_Comm c, int code);
int MPI_File_open(MPI_Comm c, const char* name, int mode, MPI_Info info, MPI_File* fh);
int MPI_File_set_view(MPI_File fh, MPI_Offset disp, MPI_Datatype et, MPI_Datatype ft,
                      const char* rep, MPI_Info info);
int MPI_File_write(MPI_File fh, const void* buf, int n, MPI_Datatype t, MPI_Status* st);
int MPI_File_close(MPI_File* fh);
#endif
