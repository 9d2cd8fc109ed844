/* Single-process stand-in for the few MPI calls the reference 2LPT code makes
   (test infrastructure: used only to compile the reference's own sources for
   the oracle).  Rank 0 of 1; collectives copy, the halo self-message copies. */
#ifndef AAR_SHIM_MPI_H
#define AAR_SHIM_MPI_H
#include <stddef.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int source, tag; } MPI_Status;
#define MPI_COMM_WORLD 0
#define MPI_CHAR 1
#define MPI_BYTE 2
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_STATUS_IGNORE ((MPI_Status *)0)
int MPI_Init(int *argc, char ***argv);
int MPI_Finalize(void);
int MPI_Comm_rank(MPI_Comm c, int *r);
int MPI_Comm_size(MPI_Comm c, int *s);
int MPI_Barrier(MPI_Comm c);
int MPI_Abort(MPI_Comm c, int code);
int MPI_Bcast(void *buf, int n, MPI_Datatype t, int root, MPI_Comm c);
int MPI_Allgather(const void *sb, int sn, MPI_Datatype st, void *rb, int rn, MPI_Datatype rt, MPI_Comm c);
int MPI_Allreduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, MPI_Comm c);
int MPI_Reduce(const void *sb, void *rb, int n, MPI_Datatype t, MPI_Op op, int root, MPI_Comm c);
int MPI_Send(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c);
int MPI_Isend(const void *b, int n, MPI_Datatype t, int dst, int tag, MPI_Comm c, MPI_Request *r);
int MPI_Recv(void *b, int n, MPI_Datatype t, int src, int tag, MPI_Comm c, MPI_Status *s);
int MPI_Wait(MPI_Request *r, MPI_Status *s);
#endif
