/*
 * Single-rank stand-in for <mpi.h>, used only to compile the reference's own
 * C++ sources as a CPU oracle (test infrastructure, never shipped).
 *
 * Semantics are those of MPI with exactly one rank:
 *   - rank 0, size 1; every Cartesian shift returns MPI_PROC_NULL;
 *   - point-to-point calls with MPI_PROC_NULL are no-ops (buffers untouched);
 *   - reductions / gathers copy the send buffer to the receive buffer.
 * The reference guards every halo exchange with `!= MPI_PROC_NULL`
 * (Simulation.cpp:258-543, ComplexGeometry.cpp:1058-1253), so with one rank
 * no communication path touches lattice data.
 */
#pragma once
#include <cstring>
#include <cstddef>

typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef long MPI_Aint;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;

#define MPI_SUCCESS 0
#define MPI_COMM_WORLD 1
#define MPI_PROC_NULL (-2)
#define MPI_STATUS_IGNORE ((MPI_Status*)0)
#define MPI_SUM 1

/* Builtin datatypes encode their byte size in the low bits (id = size | tag<<8). */
#define MPI_DATATYPE_NULL 0
#define MPI_CHAR               (1 | (1 << 8))
#define MPI_SIGNED_CHAR        (1 | (2 << 8))
#define MPI_UNSIGNED_CHAR      (1 | (3 << 8))
#define MPI_BYTE               (1 | (4 << 8))
#define MPI_C_BOOL             (1 | (5 << 8))
#define MPI_SHORT              (2 | (1 << 8))
#define MPI_UNSIGNED_SHORT     (2 | (2 << 8))
#define MPI_INT                (4 | (1 << 8))
#define MPI_UNSIGNED           (4 | (2 << 8))
#define MPI_UINT               (4 | (3 << 8))
#define MPI_WCHAR              (4 | (4 << 8))
#define MPI_FLOAT              (4 | (5 << 8))
#define MPI_LONG               (8 | (1 << 8))
#define MPI_UNSIGNED_LONG      (8 | (2 << 8))
#define MPI_LONG_LONG          (8 | (3 << 8))
#define MPI_UNSIGNED_LONG_LONG (8 | (4 << 8))
#define MPI_DOUBLE             (8 | (5 << 8))
#define MPI_C_COMPLEX          (8 | (6 << 8))
#define MPI_LONG_DOUBLE        (16 | (1 << 8))
#define MPI_C_DOUBLE_COMPLEX   (16 | (2 << 8))
#define MPI_C_LONG_DOUBLE_COMPLEX (32 | (1 << 8))

namespace mpi_single_rank {
/* Derived types (MPI_Type_contiguous) get ids from 1<<20 upward; their byte
 * sizes live in this small table. */
inline long& derived_size(int id) {
    static long table[256];
    return table[(id >> 20) & 255];
}
inline int& next_derived() { static int n = 1; return n; }
inline long type_size(MPI_Datatype t) {
    if (t >= (1 << 20)) return derived_size(t);
    return (long)(t & 0xff);
}
}  // namespace mpi_single_rank

static inline int MPI_Init(int*, char***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Comm_size(MPI_Comm, int* s) { *s = 1; return MPI_SUCCESS; }
static inline int MPI_Comm_free(MPI_Comm*) { return MPI_SUCCESS; }
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Dims_create(int, int ndims, int* dims) {
    for (int i = 0; i < ndims; ++i) if (dims[i] == 0) dims[i] = 1;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_create(MPI_Comm, int, const int*, const int*, int, MPI_Comm* c) {
    *c = 2; return MPI_SUCCESS;
}
static inline int MPI_Cart_shift(MPI_Comm, int, int, int* src, int* dst) {
    *src = MPI_PROC_NULL; *dst = MPI_PROC_NULL; return MPI_SUCCESS;
}
static inline int MPI_Cart_coords(MPI_Comm, int, int n, int* coords) {
    for (int i = 0; i < n; ++i) coords[i] = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Cart_get(MPI_Comm, int n, int* dims, int* periods, int* coords) {
    for (int i = 0; i < n; ++i) { dims[i] = 1; periods[i] = 0; coords[i] = 0; }
    return MPI_SUCCESS;
}
static inline int MPI_Cart_rank(MPI_Comm, const int*, int* r) { *r = 0; return MPI_SUCCESS; }
static inline int MPI_Type_contiguous(int count, MPI_Datatype old, MPI_Datatype* t) {
    int id = (mpi_single_rank::next_derived()++) << 20;
    mpi_single_rank::derived_size(id) = count * mpi_single_rank::type_size(old);
    *t = id; return MPI_SUCCESS;
}
static inline int MPI_Type_create_struct(int, const int*, const MPI_Aint*, const MPI_Datatype*, MPI_Datatype* t) {
    *t = MPI_BYTE; return MPI_SUCCESS;
}
static inline int MPI_Type_commit(MPI_Datatype*) { return MPI_SUCCESS; }
static inline int MPI_Type_free(MPI_Datatype*) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void*, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Send(const void*, int, MPI_Datatype, int, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Recv(void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) { return MPI_SUCCESS; }
static inline int MPI_Sendrecv(const void*, int, MPI_Datatype, int, int,
                               void*, int, MPI_Datatype, int, int, MPI_Comm, MPI_Status*) {
    return MPI_SUCCESS;
}
static inline int mpi_single_rank_copy(const void* s, void* r, int n, MPI_Datatype t) {
    if (s && r && s != r) std::memcpy(r, s, (size_t)n * (size_t)mpi_single_rank::type_size(t));
    return MPI_SUCCESS;
}
static inline int MPI_Allreduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, MPI_Comm) {
    return mpi_single_rank_copy(s, r, n, t);
}
static inline int MPI_Reduce(const void* s, void* r, int n, MPI_Datatype t, MPI_Op, int, MPI_Comm) {
    return mpi_single_rank_copy(s, r, n, t);
}
static inline int MPI_Allgather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, MPI_Comm) {
    return mpi_single_rank_copy(s, r, n, t);
}
static inline int MPI_Gather(const void* s, int n, MPI_Datatype t, void* r, int, MPI_Datatype, int, MPI_Comm) {
    return mpi_single_rank_copy(s, r, n, t);
}
static inline int MPI_Gatherv(const void* s, int n, MPI_Datatype t, void* r, const int*, const int*,
                              MPI_Datatype, int, MPI_Comm) {
    return mpi_single_rank_copy(s, r, n, t);
}
