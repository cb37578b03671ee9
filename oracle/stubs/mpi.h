/*
 * mpi.h stand-in: a single-rank MPI for building the reference's host code
 * under oracle/_ref.  TEST INFRASTRUCTURE.  With one rank, the reference
 * never reaches a point-to-point call (transportroutines.c:107-155 skips
 * them on rank 0 of 1), so Send/Recv print an error and abort.
 */
#ifndef ORACLE_STUB_MPI_H
#define ORACLE_STUB_MPI_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR, count; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_CHAR 3
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_size(MPI_Comm c, int *size);
int MPI_Comm_rank(MPI_Comm c, int *rank);
double MPI_Wtime(void);
int MPI_Barrier(MPI_Comm c);
int MPI_Bcast(void *buf, int count, MPI_Datatype t, int root, MPI_Comm c);
int MPI_Send(const void *buf, int count, MPI_Datatype t, int dest, int tag, MPI_Comm c);
int MPI_Recv(void *buf, int count, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *st);
int MPI_Get_count(const MPI_Status *st, MPI_Datatype t, int *count);
#ifdef __cplusplus
}
#endif
#endif
