/*
 * Single-rank stand-in for <mpi.h>, used ONLY to compile the SCORE reference
 * sources as a CPU oracle (test infrastructure; never linked into the product).
 *
 * Semantics: exactly one rank (rank 0 of size 1).  Collectives copy the send
 * buffer into the receive buffer; point-to-point calls are no-ops; MPI-IO calls
 * are no-ops that report success.  The reference only calls MPI at start-up
 * (parameter validation) and in post-processing, never inside the growth step,
 * so these semantics do not touch the path under test.
 */
#ifndef SCORE_ORACLE_STUB_MPI_H
#define SCORE_ORACLE_STUB_MPI_H

#include <stdint.h>
#include <string.h>
#include <omp.h>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Info;
typedef int MPI_File;
typedef long long MPI_Offset;
typedef long long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_COMM_WORLD 1
#define MPI_COMM_SELF 2
#define MPI_INFO_NULL 0
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUCCESS 0
#define MPI_THREAD_FUNNELED 1
#define MPI_SEEK_SET 0
#define MPI_MODE_WRONLY 4
#define MPI_MODE_CREATE 1

/* built-in datatypes encode their byte size; derived types start at 1000 */
#define MPI_CHAR 1
#define MPI_INT 4
#define MPI_UNSIGNED 104
#define MPI_LONG 8
#define MPI_DOUBLE 108

#define MPI_SUM 1
#define MPI_MIN 2
#define MPI_MAX 3

static int score_stub_derived_size[64];
static int score_stub_nderived = 0;

static inline size_t score_stub_typesize(MPI_Datatype t) {
    if (t >= 1000 && t - 1000 < score_stub_nderived) return (size_t)score_stub_derived_size[t - 1000];
    return (size_t)(t % 100);
}

static inline int MPI_Init_thread(int*, char***, int, int* provided) { if (provided) *provided = MPI_THREAD_FUNNELED; return 0; }
static inline int MPI_Finalize(void) { return 0; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return 0; }
static inline int MPI_Barrier(MPI_Comm) { return 0; }
static inline double MPI_Wtime(void) { return omp_get_wtime(); }

static inline int MPI_Type_create_struct(int count, const int* blocklens, const MPI_Aint* displs,
                                         const MPI_Datatype* types, MPI_Datatype* newtype) {
    size_t end = 0;
    for (int i = 0; i < count; ++i) {
        size_t e = (size_t)displs[i] + (size_t)blocklens[i] * score_stub_typesize(types[i]);
        if (e > end) end = e;
    }
    if (score_stub_nderived < 64) score_stub_derived_size[score_stub_nderived] = (int)end;
    *newtype = 1000 + score_stub_nderived++;
    return 0;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return 0; }

static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    if (s != r) memcpy(r, s, (size_t)n * score_stub_typesize(t)); return 0;
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    if (r && s != r) memcpy(r, s, (size_t)n * score_stub_typesize(t)); return 0;
}
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
    if (r && s != r) memcpy(r, s, (size_t)n * score_stub_typesize(t)); return 0;
}
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) {
    if (r && s != r) memcpy(r, s, (size_t)n * score_stub_typesize(t)); return 0;
}
static inline int MPI_Gatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int* displs,
                              MPI_Datatype, int, MPI_Comm) {
    if (r && s != r) memcpy((char*)r + (size_t)(displs ? displs[0] : 0) * score_stub_typesize(t), s,
                            (size_t)n * score_stub_typesize(t));
    return 0;
}
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return 0; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return 0; }

static inline int MPI_File_open(MPI_Comm, const char*, int, MPI_Info, MPI_File* fh) { *fh = 0; return 0; }
static inline int MPI_File_close(MPI_File*) { return 0; }
static inline int MPI_File_seek(MPI_File, MPI_Offset, int) { return 0; }
static inline int MPI_File_write(MPI_File, const void*, int, MPI_Datatype, MPI_Status*) { return 0; }
static inline int MPI_File_write_at(MPI_File, MPI_Offset, const void*, int, MPI_Datatype, MPI_Status*) { return 0; }

#endif
