/* Minimal stand-in for <mpi.h> so the reference's RCBForceTree.cxx, which
 * includes Partition.h for the rank number only, compiles without MPI.  No MPI
 * call is made on the short-range force path. */
#ifndef HSR_REF_STUB_MPI_H
#define HSR_REF_STUB_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef struct { int unused; } MPI_Status;
#define MPI_COMM_WORLD 0
#endif
