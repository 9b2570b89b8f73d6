/* Single-rank MPI stand-in for the reference headers (TEST INFRASTRUCTURE ONLY).
 * With one rank MPI_Allreduce(MPI_IN_PLACE, ...) and MPI_Bcast(root 0) leave
 * the buffers unchanged, which is what these no-ops do. */
#ifndef EPH_MOCK_MPI_H
#define EPH_MOCK_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
#define MPI_IN_PLACE ((void *)1)
#define MPI_DOUBLE 0
#define MPI_SUM 0
#define MPI_COMM_WORLD 0
static inline int MPI_Allreduce(const void *, void *, int, MPI_Datatype, MPI_Op, MPI_Comm) { return 0; }
static inline int MPI_Bcast(void *, int, MPI_Datatype, int, MPI_Comm) { return 0; }
static inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = 0; return 0; }
static inline int MPI_Comm_size(MPI_Comm, int *s) { *s = 1; return 0; }
#endif
