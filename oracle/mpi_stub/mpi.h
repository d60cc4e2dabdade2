/* Minimal single-process stand-in for <mpi.h> (TEST INFRASTRUCTURE ONLY).
 *
 * It lets oracle/ref_partition.cpp compile the reference's own
 * cfdwm_mpi::partition_weighted (mpi_utils.h:46-64, built with MPI_enable)
 * without an MPI library: the communicator size that the partition reads is
 * set by the caller through refstub_size; no message is ever sent. */
#ifndef CFDWM_ORACLE_MPI_STUB_H
#define CFDWM_ORACLE_MPI_STUB_H

typedef int MPI_Comm;
typedef int MPI_Datatype;
#define MPI_COMM_WORLD 0
#define MPI_DATATYPE_NULL 0
#define MPI_DOUBLE 1
#define MPI_IN_PLACE ((void *)1)

extern int refstub_size;
extern int refstub_rank;

inline int MPI_Initialized(int *flag) { *flag = 1; return 0; }
inline int MPI_Comm_rank(MPI_Comm, int *r) { *r = refstub_rank; return 0; }
inline int MPI_Comm_size(MPI_Comm, int *s) { *s = refstub_size; return 0; }
inline int MPI_Allgatherv(const void *, int, MPI_Datatype, void *, const int *, const int *, MPI_Datatype,
                          MPI_Comm) { return 0; }

#endif
