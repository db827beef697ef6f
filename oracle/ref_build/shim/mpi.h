// Single-rank MPI stand-in for compiling the reference's sources unchanged
// into the CPU oracle (TEST INFRASTRUCTURE ONLY).  With one rank every
// collective the reference calls reduces to a local copy (Allgatherv,
// Alltoallw, Scatterv) or to nothing (Bcast, Barrier).  Written for this
// project; only the names and argument lists follow the MPI standard.
#ifndef GB300_ORACLE_MPI_STUB
#define GB300_ORACLE_MPI_STUB

#include <cstring>

typedef int MPI_Comm;
typedef int MPI_Group;
typedef int MPI_Datatype;
typedef int MPI_File;
typedef struct {
    int MPI_SOURCE, MPI_TAG, MPI_ERROR;
} MPI_Status;

#define MPI_COMM_WORLD 0
#define MPI_DOUBLE 1
#define MPI_INT 2
#define MPI_CHAR 3
#define MPI_SUCCESS 0
#define MPI_STATUS_IGNORE ((MPI_Status *)0)

static inline int mpi_stub_type_size(MPI_Datatype t) { return t == MPI_DOUBLE ? 8 : (t == MPI_INT ? 4 : 1); }

static inline int MPI_Init(int *, char ***) { return MPI_SUCCESS; }
static inline int MPI_Finalize() { return MPI_SUCCESS; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) {
    *r = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_size(MPI_Comm, int *s) {
    *s = 1;
    return MPI_SUCCESS;
}
static inline int MPI_Barrier(MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return MPI_SUCCESS; }
static inline int MPI_Allgatherv(const void *sendbuf, int sendcount, MPI_Datatype sendtype, void *recvbuf,
                                 const int * /*recvcounts*/, const int *displs, MPI_Datatype recvtype, MPI_Comm) {
    const int es = mpi_stub_type_size(recvtype);
    std::memmove((char *)recvbuf + (long)displs[0] * es, sendbuf, (size_t)sendcount * mpi_stub_type_size(sendtype));
    return MPI_SUCCESS;
}
// displacements in bytes, as MPI_Alltoallw defines them
static inline int MPI_Alltoallw(const void *sendbuf, const int sendcounts[], const int sdispls[],
                                const MPI_Datatype sendtypes[], void *recvbuf, const int /*recvcounts*/[],
                                const int rdispls[], const MPI_Datatype /*recvtypes*/[], MPI_Comm) {
    std::memmove((char *)recvbuf + rdispls[0], (const char *)sendbuf + sdispls[0],
                 (size_t)sendcounts[0] * mpi_stub_type_size(sendtypes[0]));
    return MPI_SUCCESS;
}
static inline int MPI_Scatterv(const void *sendbuf, const int sendcounts[], const int displs[], MPI_Datatype sendtype,
                               void *recvbuf, int, MPI_Datatype, int, MPI_Comm) {
    std::memmove(recvbuf, (const char *)sendbuf + (long)displs[0] * mpi_stub_type_size(sendtype),
                 (size_t)sendcounts[0] * mpi_stub_type_size(sendtype));
    return MPI_SUCCESS;
}
static inline int MPI_Comm_group(MPI_Comm, MPI_Group *g) {
    *g = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Group_incl(MPI_Group, int, const int *, MPI_Group *g) {
    *g = 0;
    return MPI_SUCCESS;
}
static inline int MPI_Comm_create(MPI_Comm, MPI_Group, MPI_Comm *c) {
    *c = 0;
    return MPI_SUCCESS;
}
static inline int MPI_File_read(MPI_File, void *, int, MPI_Datatype, MPI_Status *) { return MPI_SUCCESS; }

#endif
