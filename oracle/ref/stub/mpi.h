/* Single-rank stand-in for the MPI API, used only to compile the reference's
 * CPU training path in this container (there is no MPI installation here).
 *
 * Test infrastructure: nothing in the product links this header.
 *
 * Semantics: one process, rank 0 of a world of size 1.  A datatype handle is
 * the size in bytes of one element, so collectives reduce to local copies:
 * Allgather/Gatherv copy the send buffer to the receive buffer, Allreduce with
 * MPI_IN_PLACE is the identity, and MPI-IO writes go to a stdio FILE.  Point to
 * point calls are never reached with one rank and fail loudly if they are.
 */
#ifndef ORACLE_REF_MPI_STUB_H
#define ORACLE_REF_MPI_STUB_H

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef long MPI_Datatype;   /* bytes per element */
typedef int MPI_Comm;
typedef int MPI_Op;
typedef int MPI_Info;
typedef long MPI_Aint;
typedef long long MPI_Offset;
typedef FILE* MPI_File;
typedef struct { int MPI_SOURCE; int MPI_TAG; int MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 0
#define MPI_THREAD_FUNNELED 1
#define MPI_INFO_NULL 0
#define MPI_MODE_CREATE 1
#define MPI_MODE_WRONLY 4
#define MPI_ANY_TAG (-1)
#define MPI_SUM 1
#define MPI_MAX 2
#define MPI_IN_PLACE ((void*)1)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)

#define MPI_CHAR ((MPI_Datatype)1)
#define MPI_INT ((MPI_Datatype)4)
#define MPI_FLOAT ((MPI_Datatype)4)
#define MPI_UNSIGNED_LONG ((MPI_Datatype)8)
#define MPI_OFFSET ((MPI_Datatype)8)

static inline int MPI_Init_thread(int*, char***, int required, int* provided) { *provided = required; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Abort(MPI_Comm, int code) { fprintf(stderr, "MPI_Abort(%d)\n", code); exit(code); return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* n) { *n = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }

static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* out) { *out = count * old; return 0; }
static inline int MPI_Type_create_struct(int n, const int* lens, const MPI_Aint* offs, const MPI_Datatype* types, MPI_Datatype* out) {
    long extent = 0;
    for (int i = 0; i < n; i++) {
        long end = (long)offs[i] + (long)lens[i] * (long)types[i];
        if (end > extent) extent = end;
    }
    *out = extent;
    return 0;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }
static inline int MPI_Type_free(MPI_Datatype*) { return 0; }

static inline int MPI_Allreduce(const void* send, void* recv, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (send != MPI_IN_PLACE) memcpy(recv, send, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Allgather(const void* send, int count, MPI_Datatype t, void* recv, int, MPI_Datatype, MPI_Comm) {
    memcpy(recv, send, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Allgatherv(const void* send, int count, MPI_Datatype t, void* recv, const int*, const int* displs, MPI_Datatype rt, MPI_Comm) {
    memcpy((char*)recv + (size_t)displs[0] * (size_t)rt, send, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Gatherv(const void* send, int count, MPI_Datatype t, void* recv, const int*, const int* displs, MPI_Datatype rt, int, MPI_Comm) {
    memcpy((char*)recv + (size_t)displs[0] * (size_t)rt, send, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Exscan(const void*, void* recv, int count, MPI_Datatype t, MPI_Op, MPI_Comm) {
    memset(recv, 0, (size_t)count * (size_t)t);
    return 0;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) {
    fprintf(stderr, "single-rank MPI stub: MPI_Send is unreachable with one rank\n");
    exit(3);
    return 0;
}
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
    fprintf(stderr, "single-rank MPI stub: MPI_Recv is unreachable with one rank\n");
    exit(3);
    return 0;
}

static inline int MPI_File_open(MPI_Comm, const char* path, int, MPI_Info, MPI_File* f) {
    *f = fopen(path, "w");
    return *f ? 0 : 1;
}
static inline int MPI_File_write_at_all(MPI_File f, MPI_Offset off, const void* buf, int count, MPI_Datatype t, MPI_Status*) {
    fseek(f, (long)off, SEEK_SET);
    fwrite(buf, (size_t)t, (size_t)count, f);
    return 0;
}
static inline int MPI_File_close(MPI_File* f) { fclose(*f); return 0; }

#endif /* ORACLE_REF_MPI_STUB_H */
