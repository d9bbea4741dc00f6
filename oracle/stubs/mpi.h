/* Minimal stand-in for <mpi.h> so the reference's SSSP sources compile
 * without MPI.  The SSSP path only includes the header (include/graph.h:8,
 * include/timer.h:2) and never calls MPI; only MPI_Wtime is referenced
 * (utils/timer.c:45-48).  Oracle build support, not product code. */
#ifndef GBREF_MPI_STUB_H
#define GBREF_MPI_STUB_H
#include <time.h>
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Op;
typedef int MPI_Request;
typedef struct { int MPI_SOURCE, MPI_TAG, MPI_ERROR; } MPI_Status;
#define MPI_COMM_WORLD 0
static __inline__ double MPI_Wtime(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}
#endif
