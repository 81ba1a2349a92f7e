/*
 * Single-task stand-in for <mpi.h>, used only to compile the reference's
 * hot-path translation units into the oracle's pinning library
 * (oracle/build_ref.sh).  Test infrastructure, never linked into the product.
 * Semantics: one task; reductions copy; point-to-point calls abort.
 */
#ifndef ORACLE_SHIM_MPI_H
#define ORACLE_SHIM_MPI_H
#include <cstdio>
#include <cstdlib>
#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_NULL 0
#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_STATUSES_IGNORE ((MPI_Status*)0)
#define MPI_MAX_PROCESSOR_NAME 256
#define MPI_UNDEFINED (-32766)
#define MPI_IN_PLACE ((void*)1)

#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_FLOAT 5
#define MPI_DOUBLE 8
#define MPI_SHORT 2
#define MPI_UNSIGNED 6
#define MPI_LONG 9
#define MPI_UNSIGNED_LONG 10
#define MPI_LONG_LONG 11
#define MPI_UNSIGNED_SHORT 12
#define MPI_C_BOOL 13
#define MPI_BYTE 14
#define MPI_DOUBLE_INT 15
#define MPI_FLOAT_INT 16
#define MPI_2INT 17

#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_MIN 3
#define MPI_PROD 4
#define MPI_LOR 5
#define MPI_LAND 6
#define MPI_MINLOC 7
#define MPI_MAXLOC 8
#define MPI_BOR 9

static inline size_t oracle_mpi_size(MPI_Datatype t)
{
    switch (t)
    {
        case MPI_CHAR: case MPI_BYTE: case MPI_C_BOOL: return 1;
        case MPI_SHORT: case MPI_UNSIGNED_SHORT: return 2;
        case MPI_INT: case MPI_UNSIGNED: case MPI_FLOAT: return 4;
        case MPI_DOUBLE_INT: return 16;
        case MPI_FLOAT_INT: case MPI_2INT: return 8;
        default: return 8;
    }
}
static inline void oracle_mpi_copy(const void* s, void* r, int n, MPI_Datatype t)
{
    if (s != MPI_IN_PLACE && s != r) memcpy(r, s, (size_t)n * oracle_mpi_size(t));
}
static inline int oracle_mpi_unsupported(const char* what)
{
    fprintf(stderr, "oracle mpi shim: %s is not available with one task\n", what);
    abort();
    return 1;
}

static inline int MPI_Init(int*, char***) { return 0; }
static inline int MPI_Finalize() { return 0; }
static inline int MPI_Initialized(int* f) { *f = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_split(MPI_Comm c, int, int, MPI_Comm* n) { *n = c; return 0; }
static inline int MPI_Comm_dup(MPI_Comm c, MPI_Comm* n) { *n = c; return 0; }
static inline int MPI_Comm_free(MPI_Comm* c) { *c = MPI_COMM_NULL; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline int MPI_Abort(MPI_Comm, int e) { fprintf(stderr, "MPI_Abort(%d)\n", e); abort(); return e; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) { oracle_mpi_copy(s, r, n, t); return 0; }
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) { oracle_mpi_copy(s, r, n, t); return 0; }
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) { oracle_mpi_copy(s, r, n, t); return 0; }
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) { oracle_mpi_copy(s, r, n, t); return 0; }
static inline int MPI_Gatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int* d, MPI_Datatype, int, MPI_Comm) { oracle_mpi_copy(s, (char*)r + (size_t)d[0] * oracle_mpi_size(t), n, t); return 0; }
static inline int MPI_Scatterv(const void* s, const int* c, const int* d, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) { oracle_mpi_copy((const char*)s + (size_t)d[0] * oracle_mpi_size(t), r, c[0], t); return 0; }
static inline int MPI_Scatter(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) { oracle_mpi_copy(s, r, n, t); return 0; }
static inline int MPI_Allgatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int* d, MPI_Datatype, MPI_Comm) { oracle_mpi_copy(s, (char*)r + (size_t)d[0] * oracle_mpi_size(t), n, t); return 0; }
static inline int MPI_Alltoallv(const void* s, const int* sc, const int* sd, MPI_Datatype t, void* r, const int*, const int* rd, MPI_Datatype, MPI_Comm) { memcpy((char*)r + (size_t)rd[0] * oracle_mpi_size(t), (const char*)s + (size_t)sd[0] * oracle_mpi_size(t), (size_t)sc[0] * oracle_mpi_size(t)); return 0; }
static inline int MPI_Isend(const void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return oracle_mpi_unsupported("MPI_Isend"); }
static inline int MPI_Irecv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Request*) { return oracle_mpi_unsupported("MPI_Irecv"); }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return oracle_mpi_unsupported("MPI_Send"); }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return oracle_mpi_unsupported("MPI_Recv"); }
static inline int MPI_Wait(MPI_Request*, MPI_Status*) { return 0; }
static inline int MPI_Waitall(int, MPI_Request*, MPI_Status*) { return 0; }
static inline int PMPI_Get_processor_name(char* n, int* l) { strcpy(n, "oracle"); *l = 6; return 0; }
static inline int MPI_Get_processor_name(char* n, int* l) { strcpy(n, "oracle"); *l = 6; return 0; }
static inline int MPI_Cart_create(MPI_Comm c, int, const int*, const int*, int, MPI_Comm* n) { *n = c; return 0; }
static inline int MPI_Cart_coords(MPI_Comm, int, int nd, int* co) { for (int i = 0; i < nd; i++) co[i] = 0; return 0; }
static inline int MPI_Cart_rank(MPI_Comm, const int*, int* r) { *r = 0; return 0; }
static inline int MPI_Cart_shift(MPI_Comm, int, int, int* s, int* d) { *s = 0; *d = 0; return 0; }
static inline int MPI_Cart_sub(MPI_Comm c, const int*, MPI_Comm* n) { *n = c; return 0; }
static inline double MPI_Wtime() { return 0.; }
#endif
