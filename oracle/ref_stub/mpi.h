/* Minimal stand-in for <mpi.h> so the reference's RCBForceTree.cxx (which
 * includes Partition.h for the rank number only) and Particles.cxx (whose
 * restart I/O declarations name MPI types) compile without MPI.  Types only:
 * no MPI call is made on the short-range force path or the sub-cycle. */
#ifndef HSR_REF_STUB_MPI_H
#define HSR_REF_STUB_MPI_H
typedef int MPI_Comm;
typedef int MPI_Datatype;
typedef int MPI_Request;
typedef int MPI_Op;
typedef struct { int unused; } MPI_Status;
typedef long MPI_Aint;
typedef int MPI_File;
#define MPI_COMM_WORLD 0
#endif
