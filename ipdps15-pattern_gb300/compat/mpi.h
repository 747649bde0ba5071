// mpi.h -- the single-process subset of MPI the drivers call.  With one
// process, a barrier returns at once, the rank is 0 and a reduction over
// ranks copies its input.
#ifndef IRR_COMPAT_MPI_H_
#define IRR_COMPAT_MPI_H_
#include <string.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_COMM_WORLD 0
#define MPI_INT 4
#define MPI_DOUBLE 8
#define MPI_SUM 0
#define MPI_MAX 1
#define MPI_SUCCESS 0

static inline int MPI_Init(int *argc, char ***argv)
{
    (void)argc;
    (void)argv;
    return MPI_SUCCESS;
}
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm c)
{
    (void)c;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_rank(MPI_Comm c, int *rank)
{
    (void)c;
    *rank = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm c, int *size)
{
    (void)c;
    *size = 1;
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void *in, void *out, int count, MPI_Datatype type,
                                MPI_Op op, MPI_Comm c)
{
    (void)op;
    (void)c;
    if (in != out) memcpy(out, in, (size_t)count * (size_t)type);
    return MPI_SUCCESS;
}

#endif
