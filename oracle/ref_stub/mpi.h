/* Minimal stand-in for <mpi.h> so that the reference's single-rank sources
 * (src/precomp.c, src/openmp_propagate.c, src/device_data.c) compile without
 * an MPI installation.  Only the names those files and their headers use are
 * declared; a one-rank run never calls into MPI. */
#ifndef DC_REF_STUB_MPI_H
#define DC_REF_STUB_MPI_H
typedef int MPI_Comm;
typedef int MPI_Request;
typedef int MPI_Datatype;
#define MPI_PROC_NULL (-2)
#define MPI_MAX_PROCESSOR_NAME 256
static inline int MPI_Finalize(void) { return 0; }
#endif
